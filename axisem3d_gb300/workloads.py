"""The element-level stiffness batching workload (vectorised builder).

n_elem independent solid elements (no shared points), nPol = 4, spherical (curvilinear)
geometry at random places in the mantle (r in [3480, 6336] km), per-element
Nu ~ round(exp(U[ln 8, ln 256])) with nr = 2 Nu + 1, transversely isotropic moduli from
Vp/Vs/rho perturbed +-5 % (uniform) per GLL point and azimuthal sample, so every element
runs in physical space (3D material), and SLS attenuation with 3 solids and Q_mu
uniform in [80, 600] per element (CG4 or full grid).  Displacement Fourier coefficients
are N(0,1) * alpha^-1.5 (order 0 real).

The geometry of a spherical element with nodes (r0, t0), (r0, t1), (r1, t1), (r1, t0)
reduces to s = r(eta) sin a(xi), z = r(eta) cos a(xi) with r(eta) the linear radius and
a(xi) the linear colatitude; its Jacobian is the closed form of
SphericalMapping::jacobian (SphericalMapping.cpp:44-78) for curvedOuter = 2, evaluated
here for all elements at once in FP64.
"""
from __future__ import annotations

import numpy as np

from . import attenuation as ATT
from . import spectral as S
from .spec import ATT_CG4, ATT_FULL, ATT_NONE, MAT_TISO, POINT_SOLID, DomainSpec

MANTLE_VP, MANTLE_VS, MANTLE_RHO = 11.0e3, 6.0e3, 4.5e3


def spherical_batch(r0, r1, t0, t1, axial):
    """geo [E,5,25], ifact [E,25], theta [E,25] for spherical elements (FP64)."""
    E = len(r0)
    xg, wg = S.gll()[0], S.gll()[1]
    xj, wj = S.glj()[0], S.glj()[1]
    xi = np.where(axial[:, None], xj[None, :], xg[None, :])      # [E,5] (ipol)
    wxi = np.where(axial[:, None], wj[None, :], wg[None, :])
    eta, weta = xg, wg                                            # [5] (jpol)
    XI = xi[:, :, None] * np.ones((1, 1, 5))                       # [E,5,5]
    ETA = np.broadcast_to(eta[None, None, :], (E, 5, 5))
    dr = (r1 - r0)[:, None, None]
    dt = (t1 - t0)[:, None, None]
    rr = ((1 + ETA) * r1[:, None, None] + (1 - ETA) * r0[:, None, None]) / 2
    a = ((1 - XI) * t0[:, None, None] + (1 + XI) * t1[:, None, None]) / 2
    J00 = rr * dt / 2 * np.cos(a)
    J01 = 0.5 * dr * np.sin(a)
    J10 = -rr * dt / 2 * np.sin(a)
    J11 = 0.5 * dr * np.cos(a)
    det = J00 * J11 - J01 * J10
    s = rr * np.sin(a)
    geo = np.empty((E, 5, 25))
    geo[:, 0] = (J00 / det).reshape(E, 25)
    geo[:, 1] = (-J01 / det).reshape(E, 25)
    geo[:, 2] = (-J10 / det).reshape(E, 25)
    geo[:, 3] = (J11 / det).reshape(E, 25)
    axial_row = axial[:, None, None] & (np.arange(5)[None, :, None] == 0)
    inv_s = np.where(axial_row, 0.0, 1.0 / np.where(axial_row, 1.0, s))
    geo[:, 4] = inv_s.reshape(E, 25)
    W = wxi[:, :, None] * weta[None, None, :]
    one_p_xi = np.where(XI > -1.0, 1.0 + XI, 1.0)  # xi = -1 only on the axis row (handled below)
    ifact = np.where(axial[:, None, None],
                     np.where(np.arange(5)[None, :, None] == 0, W * J00 * det, W * s / one_p_xi * det),
                     W * s * det)
    theta = a  # colatitude of every GLL point
    return geo, ifact.reshape(E, 25), np.broadcast_to(theta, (E, 5, 5)).reshape(E, 25).copy()


def element_benchmark(n_elem=200_000, seed=0, att=ATT_CG4, nsls=3, dt=0.05, axial_frac=0.01,
                      nu_min=8, nu_max=256, kahan=False, dtype=np.float32, in3d=True):
    rng = np.random.default_rng(seed)
    nu = np.round(np.exp(rng.uniform(np.log(nu_min), np.log(nu_max), n_elem))).astype(np.int32)
    nr = 2 * nu + 1
    # geometry: ~60-120 km elements in the mantle
    r0 = rng.uniform(3480e3, 6336e3 - 120e3, n_elem)
    r1 = r0 + rng.uniform(60e3, 120e3, n_elem)
    axial = rng.random(n_elem) < axial_frac
    dth = rng.uniform(60e3, 120e3, n_elem) / r0
    t0 = np.where(axial, 0.0, rng.uniform(0.02, np.pi - 0.04, n_elem))
    t1 = t0 + dth
    geo, ifact, theta = spherical_batch(r0, r1, t0, t1, axial)
    trig = np.stack([np.sin(theta), np.cos(theta), np.sin(2 * theta), np.cos(2 * theta)], 1)

    # SLS coefficients (one global set) and per-element Q
    alpha = beta = gamma = np.zeros(0)
    if att != ATT_NONE:
        w, y = ATT.fit_sls(nsls, 1 / 200.0, 1 / 10.0)
        f_min, f_max, f_ref = 1 / 200.0, 1 / 10.0, 1.0
        alpha, beta, gamma, _, _ = ATT.att_factors(w, y, f_min, f_max, f_ref, dt, np.ones(1), np.ones(1), True)
        qmu_e = rng.uniform(80, 600, n_elem)
    npa = 4 if att == ATT_CG4 else 25
    # material rows per element: every azimuth sample (3-D, physical-space path) or one
    # (1-D, Fourier-space path)
    rows_e = nr.astype(np.int64) if in3d else np.ones(n_elem, np.int64)
    mod_len = 5 * rows_e * 25
    att_len = (2 * rows_e * npa) if att != ATT_NONE else np.zeros(n_elem, np.int64)
    mofs = np.concatenate([[0], np.cumsum(mod_len)[:-1]]).astype(np.int64)
    aofs = np.concatenate([[0], np.cumsum(att_len)[:-1]]).astype(np.int64)
    moduli = np.empty(int(mod_len.sum()), dtype)
    attm = np.empty(int(att_len.sum()), dtype)
    inv_mass = np.empty((n_elem, 25))
    xi_ti, phi_ti, eta_ti = 1.05, 0.97, 0.98
    for r_val in np.unique(nr):
        idx = np.nonzero(nr == r_val)[0]
        m = len(idx)
        shape = (m, int(r_val) if in3d else 1, 25)
        vp = MANTLE_VP * (1 + 0.05 * rng.uniform(-1, 1, shape))
        vs = MANTLE_VS * (1 + 0.05 * rng.uniform(-1, 1, shape))
        rho = MANTLE_RHO * (1 + 0.05 * rng.uniform(-1, 1, shape))
        f = ifact[idx][:, None, :]
        A = rho * vp * vp / phi_ti * f
        C = rho * vp * vp * f
        L = rho * vs * vs * f
        N = rho * vs * vs * xi_ti * f
        F = eta_ti * (A - 2 * L)
        if att != ATT_NONE:
            kappa, mu = ATT.voigt_ti(A, C, F, L, N)
            A -= kappa + 4 / 3 * mu
            C -= kappa + 4 / 3 * mu
            F -= kappa - 2 / 3 * mu
            L -= mu
            N -= mu
            qk = np.full(shape, 57823.0)
            qm = np.broadcast_to(qmu_e[idx][:, None, None], shape)
            _, _, _, kf, mf = ATT.att_factors(w, y, f_min, f_max, f_ref, dt, qk, qm, True)
            dkf, kpa, kpn = kf
            dmf, mua, mun = mf
            if att == ATT_CG4:
                from .geometry import cg4_weights
                wcg = np.stack([cg4_weights(ifact[i]) for i in idx])  # [m,4]
                cg = list(ATT.CG4_POINTS)
                dk = wcg[:, None, :] * dkf[:, :, cg] * kappa[:, :, cg]
                dm = wcg[:, None, :] * dmf[:, :, cg] * mu[:, :, cg]
                kappa = kappa * kpn
                mu = mu * mun
                for i, p in enumerate(cg):
                    kappa[:, :, p] *= 1 + wcg[:, None, i] * (kpa[:, :, p] / kpn[:, :, p] - 1)
                    mu[:, :, p] *= 1 + wcg[:, None, i] * (mua[:, :, p] / mun[:, :, p] - 1)
            else:
                dk = dkf * kappa
                dm = dmf * mu
                kappa = kappa * kpa
                mu = mu * mua
            A += kappa + 4 / 3 * mu
            C += kappa + 4 / 3 * mu
            F += kappa - 2 / 3 * mu
            L += mu
            N += mu
            blk = np.concatenate([dk.reshape(m, -1), dm.reshape(m, -1)], 1).astype(dtype)
            pos = aofs[idx][:, None] + np.arange(blk.shape[1])[None, :]
            attm[pos] = blk
        blk = np.stack([A, C, F, L, N], 1).reshape(m, -1).astype(dtype)  # [m, 5*nr*25]
        pos = mofs[idx][:, None] + np.arange(blk.shape[1])[None, :]
        moduli[pos] = blk
        inv_mass[idx] = 1.0 / (rho[:, 0, :] * ifact[idx])  # Mass1D from the first sample
    # points: 25 per element, element-local
    P = n_elem * 25
    p_nr = np.repeat(nr, 25).astype(np.int32)
    p_axial = (axial[:, None] & (np.arange(25)[None, :] < 5)).ravel().astype(np.uint8)
    e_pts = np.arange(P, dtype=np.int32).reshape(n_elem, 25)
    spec = DomainSpec(
        dt=dt, p_nr=p_nr, p_kind=np.full(P, POINT_SOLID, np.int8), p_axial=p_axial,
        p_fsurf=np.zeros(P, np.uint8), p_mslen=np.ones(P, np.int32), p_ms=inv_mass.ravel().astype(np.float32),
        p_mflen=np.zeros(P, np.int32), p_mf=np.zeros(0, np.float32), p_sflen=np.zeros(P, np.int32),
        p_sfn=np.zeros((0, 3), np.float32), p_sfni=np.zeros((0, 3), np.float32),
        e_pts=e_pts, e_mat=np.full(n_elem, MAT_TISO, np.int8), e_axial=axial.astype(np.uint8),
        e_in3d=np.full(n_elem, int(in3d), np.uint8), e_geo=geo.astype(np.float32), e_trig=trig.astype(np.float32),
        e_mofs=mofs, e_mod=moduli, e_att=np.full(n_elem, att, np.int8), e_aofs=aofs, e_attm=attm,
        nsls=nsls if att != ATT_NONE else 0, att_alpha=alpha, att_beta=beta, att_gamma=gamma,
        att_do_kappa=True, kahan=kahan, stability_interval=0)
    return spec


def benchmark_displacement(spec: DomainSpec, seed=1, scale=1e-6):
    """N(0,1) * alpha^-1.5 complex Fourier coefficients (order 0 real), vectorised."""
    rng = np.random.default_rng(seed)
    na = spec.p_nr.astype(np.int64) // 2 + 1
    rows = int(na.sum())
    alpha = np.arange(rows) - np.repeat(np.cumsum(na) - na, na)
    amp = np.where(alpha == 0, 1.0, np.maximum(alpha, 1) ** -1.5) * scale
    u = (rng.standard_normal((rows, 3), dtype=np.float32) + 1j * rng.standard_normal((rows, 3), dtype=np.float32))
    u *= amp[:, None].astype(np.float32)
    u[alpha == 0] = u[alpha == 0].real
    return u.astype(np.complex64).ravel()


def updates_per_step(spec: DomainSpec) -> int:
    """GLL-point x azimuth updates per step, element-local count: sum_e 25 nr_e."""
    return int(25 * spec.element_nr().astype(np.int64).sum())
