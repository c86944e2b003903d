"""FP64 element geometry: mappings, Jacobian operators and integral factors.

Restates, for nPol = 4:
* SphericalMapping::mapping / jacobian (SOLVER/src/preloop/spectral/mapping/SphericalMapping.cpp:9-78)
* LinearMapping (LinearMapping.cpp:8-44)
* Quad::createGraident (SOLVER/src/preloop/mesh/Quad.cpp:509-525): the five operators
  dsdxii = J00/detJ, dsdeta = -J01/detJ, dzdxii = -J10/detJ, dzdeta = J11/detJ and
  inv_s = 1/s (0 on the axis)
* Quad::formIntegralFactor (Quad.cpp:527-547)
* Geodesy::theta = acos(z / r) (SOLVER/src/preloop/utilities/Geodesy.cpp:13-16)

Element nodes are a (2, 4) array of (s, z) corners in the reference's order: node 0 at
(xi, eta) = (-1, -1), 1 at (1, -1), 2 at (1, 1), 3 at (-1, 1).
"""
from __future__ import annotations

import numpy as np

from . import spectral as S

SPHERICAL, LINEAR = 0, 1

# Mapping::sOrthogQ2 (Mapping.cpp:48-53): rotates a side to position 2
_Q2 = [np.array([[-1.0, 0.0], [0.0, -1.0]]), np.array([[0.0, -1.0], [1.0, 0.0]]),
       np.array([[1.0, 0.0], [0.0, 1.0]]), np.array([[0.0, 1.0], [-1.0, 0.0]])]


def _period(p: int) -> int:
    return p % 4


def _make_close(a: float, b: float):
    """XMath::makeClose (XMath.cpp:9-16)."""
    if a - b > np.pi:
        b += 2.0 * np.pi
    if b - a > np.pi:
        a += 2.0 * np.pi
    return a, b


def _sph_params(nodes, xieta, co):
    Q2 = _Q2[co]
    n2 = Q2 @ nodes
    x2 = Q2 @ np.asarray(xieta, float)
    r = np.sqrt(n2[0] ** 2 + n2[1] ** 2)
    t = np.arctan2(n2[0], n2[1])
    r0, r3 = r[_period(co - 2)], r[_period(co + 1)]
    t0, t1, t2, t3 = t[_period(co - 2)], t[_period(co - 1)], t[_period(co)], t[_period(co + 1)]
    t2, t3 = _make_close(t2, t3)
    t0, t1 = _make_close(t0, t1)
    return Q2, x2[0], x2[1], r0, r3, t0, t1, t2, t3


def mapping(nodes, xieta, etype=SPHERICAL, co=2):
    nodes = np.asarray(nodes, float)
    if etype == LINEAR:
        xi, eta = xieta
        shp = np.array([(1 - xi) * (1 - eta), (1 + xi) * (1 - eta), (1 + xi) * (1 + eta), (1 - xi) * (1 + eta)]) / 4
        return nodes @ shp
    Q2, xi, eta, r0, r3, t0, t1, t2, t3 = _sph_params(nodes, xieta, co)
    a_out = ((1 - xi) * t3 + (1 + xi) * t2) / 2
    a_in = ((1 - xi) * t0 + (1 + xi) * t1) / 2
    sz2 = np.array([(1 + eta) * r3 / 2 * np.sin(a_out) + (1 - eta) * r0 / 2 * np.sin(a_in),
                    (1 + eta) * r3 / 2 * np.cos(a_out) + (1 - eta) * r0 / 2 * np.cos(a_in)])
    return Q2.T @ sz2


def jacobian(nodes, xieta, etype=SPHERICAL, co=2):
    nodes = np.asarray(nodes, float)
    if etype == LINEAR:
        xi, eta = xieta
        dshp = np.array([[-(1 - eta), (1 - eta), (1 + eta), -(1 + eta)],
                         [-(1 - xi), -(1 + xi), (1 + xi), (1 - xi)]]) / 4
        return nodes @ dshp.T
    Q2, xi, eta, r0, r3, t0, t1, t2, t3 = _sph_params(nodes, xieta, co)
    a_out = ((1 - xi) * t3 + (1 + xi) * t2) / 2
    a_in = ((1 - xi) * t0 + (1 + xi) * t1) / 2
    J2 = np.empty((2, 2))
    J2[0, 0] = (1 + eta) * r3 * (t2 - t3) / 4 * np.cos(a_out) + (1 - eta) * r0 * (t1 - t0) / 4 * np.cos(a_in)
    J2[0, 1] = 0.5 * (r3 * np.sin(a_out) - r0 * np.sin(a_in))
    J2[1, 0] = -(1 + eta) * r3 * (t2 - t3) / 4 * np.sin(a_out) - (1 - eta) * r0 * (t1 - t0) / 4 * np.sin(a_in)
    J2[1, 1] = 0.5 * (r3 * np.cos(a_out) - r0 * np.cos(a_in))
    return Q2.T @ J2 @ Q2


def element_geometry(nodes, axial: bool, etype=SPHERICAL, co=2):
    """Returns (geo[5, 25], ifact[25], crds[25, 2], theta[25]) in FP64.

    geo rows: dsdxii, dsdeta, dzdxii, dzdeta, inv_s (Quad::createGraident);
    ifact: Quad::formIntegralFactor; crds: GLL point (s, z); theta: colatitude."""
    geo = np.zeros((5, 25))
    ifact = np.zeros(25)
    crds = np.zeros((25, 2))
    theta = np.zeros(25)
    for ip in range(5):
        for jp in range(5):
            k = ip * 5 + jp
            xe = S.xi_eta(ip, jp, axial)
            J = jacobian(nodes, xe, etype, co)
            d = np.linalg.det(J)
            sz = mapping(nodes, xe, etype, co)
            geo[0, k] = J[0, 0] / d
            geo[1, k] = -J[0, 1] / d
            geo[2, k] = -J[1, 0] / d
            geo[3, k] = J[1, 1] / d
            geo[4, k] = 0.0 if (axial and ip == 0) else 1.0 / sz[0]
            w = S.weights(ip, jp, axial)
            wxw = w[0] * w[1]
            if axial:
                if ip == 0:
                    ifact[k] = wxw * J[0, 0] * d
                else:
                    ifact[k] = wxw * sz[0] / (1.0 + xe[0]) * d
            else:
                ifact[k] = wxw * sz[0] * d
            crds[k] = sz
            r = np.hypot(sz[0], sz[1])
            theta[k] = 0.0 if r < 1e-10 else np.arccos(sz[1] / r)
    return geo, ifact, crds, theta


def trig_tables(theta):
    """CrdTransTIsoSolid constructor (CrdTransTIsoSolid.cpp:7-12): sin t, cos t, sin 2t, cos 2t."""
    theta = np.asarray(theta, float)
    return np.stack([np.sin(theta), np.cos(theta), np.sin(2 * theta), np.cos(2 * theta)])


def cg4_weights(ifact):
    """Quad::computeWeightsCG4 (Quad.cpp:438-466) from the first-row integral factor."""
    f = np.asarray(ifact, float).reshape(5, 5)
    w = np.empty(4)
    w[0] = (f[0, 0] + f[0, 1] + f[1, 0] + f[1, 1] + 0.5 * (f[0, 2] + f[1, 2] + f[2, 0] + f[2, 1])
            + 0.25 * f[2, 2]) / f[1, 1]
    w[1] = (f[0, 3] + f[0, 4] + f[1, 3] + f[1, 4] + 0.5 * (f[0, 2] + f[1, 2] + f[2, 3] + f[2, 4])
            + 0.25 * f[2, 2]) / f[1, 3]
    w[2] = (f[3, 0] + f[3, 1] + f[4, 0] + f[4, 1] + 0.5 * (f[2, 0] + f[2, 1] + f[3, 2] + f[4, 2])
            + 0.25 * f[2, 2]) / f[3, 1]
    w[3] = (f[3, 3] + f[3, 4] + f[4, 3] + f[4, 4] + 0.5 * (f[2, 3] + f[2, 4] + f[3, 2] + f[4, 2])
            + 0.25 * f[2, 2]) / f[3, 3]
    return w


# ------------------------------------------------------------------ vectorised
SEMISPHERICAL = 2


def _batch_map_jac(nodes, XI, ETA, etype, co):
    """Mapping and Jacobian at points (XI, ETA) [E, ...] for elements of one mapping type and
    one curved side co.  nodes [E, 2, 4].  Returns s, z, J00, J01, J10, J11 (same shape as XI)."""
    E = nodes.shape[0]
    ex = (slice(None),) + (None,) * (XI.ndim - 1)
    if etype == LINEAR:
        s_ = nodes[:, 0]
        z_ = nodes[:, 1]
        shp = [(1 - XI) * (1 - ETA) / 4, (1 + XI) * (1 - ETA) / 4, (1 + XI) * (1 + ETA) / 4, (1 - XI) * (1 + ETA) / 4]
        dxi = [-(1 - ETA) / 4, (1 - ETA) / 4, (1 + ETA) / 4, -(1 + ETA) / 4]
        deta = [-(1 - XI) / 4, -(1 + XI) / 4, (1 + XI) / 4, (1 - XI) / 4]
        s = sum(s_[ex + (k,)] * shp[k] for k in range(4)) if False else sum(s_[:, k][ex] * shp[k] for k in range(4))
        z = sum(z_[:, k][ex] * shp[k] for k in range(4))
        J00 = sum(s_[:, k][ex] * dxi[k] for k in range(4))
        J01 = sum(s_[:, k][ex] * deta[k] for k in range(4))
        J10 = sum(z_[:, k][ex] * dxi[k] for k in range(4))
        J11 = sum(z_[:, k][ex] * deta[k] for k in range(4))
        return s, z, J00, J01, J10, J11
    Q2 = _Q2[co]
    n2 = np.einsum("ij,ejk->eik", Q2, nodes)
    X2 = Q2[0, 0] * XI + Q2[0, 1] * ETA
    Y2 = Q2[1, 0] * XI + Q2[1, 1] * ETA
    r = np.sqrt(n2[:, 0] ** 2 + n2[:, 1] ** 2)
    t = np.arctan2(n2[:, 0], n2[:, 1])
    i0, i1, i2, i3 = (co - 2) % 4, (co - 1) % 4, co % 4, (co + 1) % 4
    r0, r3 = r[:, i0], r[:, i3]
    t0, t1, t2, t3 = t[:, i0].copy(), t[:, i1].copy(), t[:, i2].copy(), t[:, i3].copy()
    # XMath::makeClose
    d = t2 - t3
    t3 = np.where(d > np.pi, t3 + 2 * np.pi, t3)
    t2 = np.where(t3 - t2 > np.pi, t2 + 2 * np.pi, t2)
    d = t0 - t1
    t1 = np.where(d > np.pi, t1 + 2 * np.pi, t1)
    t0 = np.where(t1 - t0 > np.pi, t0 + 2 * np.pi, t0)
    r0, r3, t0, t1, t2, t3 = (a[ex] for a in (r0, r3, t0, t1, t2, t3))
    a_out = ((1 - X2) * t3 + (1 + X2) * t2) / 2
    if etype == SPHERICAL:
        a_in = ((1 - X2) * t0 + (1 + X2) * t1) / 2
        s2 = (1 + Y2) * r3 / 2 * np.sin(a_out) + (1 - Y2) * r0 / 2 * np.sin(a_in)
        z2 = (1 + Y2) * r3 / 2 * np.cos(a_out) + (1 - Y2) * r0 / 2 * np.cos(a_in)
        K00 = (1 + Y2) * r3 * (t2 - t3) / 4 * np.cos(a_out) + (1 - Y2) * r0 * (t1 - t0) / 4 * np.cos(a_in)
        K01 = 0.5 * (r3 * np.sin(a_out) - r0 * np.sin(a_in))
        K10 = -(1 + Y2) * r3 * (t2 - t3) / 4 * np.sin(a_out) - (1 - Y2) * r0 * (t1 - t0) / 4 * np.sin(a_in)
        K11 = 0.5 * (r3 * np.cos(a_out) - r0 * np.cos(a_in))
    else:  # SemiSphericalMapping (SemiSphericalMapping.cpp:6-60)
        s0, z0 = n2[:, 0, i0][ex], n2[:, 1, i0][ex]
        s1, z1 = n2[:, 0, i1][ex], n2[:, 1, i1][ex]
        s2 = (1 + Y2) * r3 / 2 * np.sin(a_out) + (1 - Y2) / 2 * (((1 - X2) * s0 + (1 + X2) * s1) / 2)
        z2 = (1 + Y2) * r3 / 2 * np.cos(a_out) + (1 - Y2) / 2 * (((1 - X2) * z0 + (1 + X2) * z1) / 2)
        K00 = ((1 - Y2) * (s1 - s0)) / 4 + ((1 + Y2) * r3 * (t2 - t3) * np.cos(a_out)) / 4
        K01 = -((1 - X2) * s0 + (1 + X2) * s1) / 4 + r3 / 2 * np.sin(a_out)
        K10 = ((1 - Y2) * (z1 - z0)) / 4 - ((1 + Y2) * r3 * (t2 - t3) * np.sin(a_out)) / 4
        K11 = -((1 - X2) * z0 + (1 + X2) * z1) / 4 + r3 / 2 * np.cos(a_out)
    # rotate back: sz = Q2^T sz2, J = Q2^T K Q2
    s = Q2[0, 0] * s2 + Q2[1, 0] * z2
    z = Q2[0, 1] * s2 + Q2[1, 1] * z2
    K = [[K00, K01], [K10, K11]]
    J = [[sum(Q2[k, i] * K[k][l] * Q2[l, j] for k in range(2) for l in range(2)) for j in range(2)] for i in range(2)]
    return s, z, J[0][0], J[0][1], J[1][0], J[1][1]


def batch_geometry(nodes, etype, co, axial):
    """Quad::createGraident + formIntegralFactor for many elements (FP64).

    nodes [E,2,4]; etype, co, axial [E].  Returns geo [E,5,25], ifact [E,25], crds [E,25,2],
    theta [E,25] and J00 on the axis column [E,5] (for the source)."""
    E = nodes.shape[0]
    xg, wg = S.gll()[0], S.gll()[1]
    xj, wj = S.glj()[0], S.glj()[1]
    XI = np.where(axial[:, None, None], xj[None, :, None], xg[None, :, None]) * np.ones((1, 1, 5))
    ETA = np.broadcast_to(xg[None, None, :], (E, 5, 5)).copy()
    WXI = np.where(axial[:, None, None], wj[None, :, None], wg[None, :, None]) * np.ones((1, 1, 5))
    W = WXI * wg[None, None, :]
    s = np.zeros((E, 5, 5))
    z = np.zeros_like(s)
    J00 = np.zeros_like(s)
    J01 = np.zeros_like(s)
    J10 = np.zeros_like(s)
    J11 = np.zeros_like(s)
    for et in np.unique(etype):
        for c in np.unique(co[etype == et]):
            m = (etype == et) & (co == c)
            out = _batch_map_jac(nodes[m], XI[m], ETA[m], int(et), int(c))
            for arr, v in zip((s, z, J00, J01, J10, J11), out):
                arr[m] = v
    det = J00 * J11 - J01 * J10
    geo = np.empty((E, 5, 25))
    geo[:, 0] = (J00 / det).reshape(E, 25)
    geo[:, 1] = (-J01 / det).reshape(E, 25)
    geo[:, 2] = (-J10 / det).reshape(E, 25)
    geo[:, 3] = (J11 / det).reshape(E, 25)
    axrow = axial[:, None, None] & (np.arange(5)[None, :, None] == 0)
    geo[:, 4] = np.where(axrow, 0.0, 1.0 / np.where(axrow, 1.0, s)).reshape(E, 25)
    onep = np.where(XI > -1.0, 1.0 + XI, 1.0)
    ifact = np.where(axial[:, None, None], np.where(np.arange(5)[None, :, None] == 0, W * J00 * det,
                                                    W * s / onep * det), W * s * det)
    r = np.hypot(s, z)
    theta = np.where(r < 1e-10, 0.0, np.arccos(np.clip(z / np.where(r < 1e-10, 1.0, r), -1, 1)))
    crds = np.stack([s, z], -1).reshape(E, 25, 2)
    return geo, ifact.reshape(E, 25), crds, theta.reshape(E, 25), (J00, J01, J10, J11, det)
