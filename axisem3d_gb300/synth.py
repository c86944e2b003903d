"""Seeded synthetic domains in the reference's data model.

* `annulus_domain`: a connected meridional annulus sector meshed with spherical
  elements on an (r, theta) grid, with shared GLL points, the axis (theta = 0), optional
  fluid layers with solid-fluid boundaries, free-surface fluid points, isotropic or
  transversely isotropic 1D/3D materials, SLS attenuation (full or CG4), a source term
  and receivers.  Masses, normals and moduli follow Material / GLLPoint / Quad
  (SOLVER/src/preloop/physics/material/Material.cpp:233-379,
  SOLVER/src/preloop/mesh/GLLPoint.cpp:48-128, SOLVER/src/preloop/mesh/Quad.cpp:324-376, 661-715).
* `independent_elements`: elements that share no points, each with its own 25 GLL
  points (the element-level stiffness batching workload).

All precompute is FP64 and cast to FP32 at the boundary, like the reference's
`.cast<Real>()`.
"""
from __future__ import annotations

import numpy as np

from . import attenuation as ATT
from . import geometry as GEO
from .spec import (ATT_CG4, ATT_NONE, MAT_ACOUSTIC, MAT_ISO, MAT_TISO, POINT_FLUID,
                   POINT_SOLID, POINT_SOLID_FLUID, DomainSpec)


def _velocity_model(r, rng=None):
    """Simple three-layer Earth (km/s, g/cc) by radius in metres."""
    R = 6371e3
    if r >= R - 35e3:
        return 5.8e3, 3.2e3, 2.6e3
    if r >= 3480e3:
        x = (r - 3480e3) / (R - 35e3 - 3480e3)
        return (13.7 - 5.7 * x) * 1e3, (7.3 - 2.8 * x) * 1e3, (5.5 - 2.1 * x) * 1e3
    x = r / 3480e3
    return (11.0 - 3.0 * x) * 1e3, 0.0, (13.0 - 3.1 * x) * 1e3


def _azimuth_perturbation(rng, nr, amp, nmodes=3):
    """Smooth random perturbation over nr azimuthal samples (1 + amp * sum of modes)."""
    phi = 2 * np.pi * np.arange(nr) / nr
    out = np.ones(nr)
    for m in range(1, nmodes + 1):
        out += amp / nmodes * rng.uniform(-1, 1) * np.cos(m * phi + rng.uniform(0, 2 * np.pi))
    return out


class _Builder:
    def __init__(self, dt):
        self.dt = dt
        self.e_pts, self.e_mat, self.e_axial, self.e_in3d = [], [], [], []
        self.e_geo, self.e_trig, self.e_mod, self.e_att, self.e_attm = [], [], [], [], []

    def add_element(self, pts, mat, axial, in3d, geo, trig, mod, att, attm):
        self.e_pts.append(np.asarray(pts, np.int32))
        self.e_mat.append(mat)
        self.e_axial.append(1 if axial else 0)
        self.e_in3d.append(1 if in3d else 0)
        self.e_geo.append(np.asarray(geo, np.float32))
        self.e_trig.append(np.asarray(trig, np.float32))
        self.e_mod.append(np.asarray(mod, np.float32).ravel())
        self.e_att.append(att)
        self.e_attm.append(np.asarray(attm, np.float32).ravel())

    def element_arrays(self):
        mofs = np.cumsum([0] + [len(m) for m in self.e_mod])[:-1].astype(np.int64)
        aofs = np.cumsum([0] + [len(m) for m in self.e_attm])[:-1].astype(np.int64)
        return dict(
            e_pts=np.stack(self.e_pts).astype(np.int32), e_mat=np.array(self.e_mat, np.int8),
            e_axial=np.array(self.e_axial, np.uint8), e_in3d=np.array(self.e_in3d, np.uint8),
            e_geo=np.stack(self.e_geo).astype(np.float32), e_trig=np.stack(self.e_trig).astype(np.float32),
            e_mofs=mofs, e_mod=np.concatenate(self.e_mod).astype(np.float32) if self.e_mod else np.zeros(1, np.float32),
            e_att=np.array(self.e_att, np.int8), e_aofs=aofs,
            e_attm=(np.concatenate(self.e_attm).astype(np.float32) if self.e_attm else np.zeros(0, np.float32)))


def _solid_moduli(vp, vs, rho, ifact, tiso, xi_ti=1.05, phi_ti=0.97, eta_ti=0.98):
    """Material::createElastic (Material.cpp:313-322): A, C, F, L, N scaled by ifact.

    vp, vs, rho: arrays (nr, 25).  TI: vph = vp*sqrt(phi^-1)..., a mild anisotropy."""
    if tiso:
        vpv, vph = vp, vp * np.sqrt(1 / phi_ti)
        vsv, vsh = vs, vs * np.sqrt(xi_ti)
        eta = np.full_like(vp, eta_ti)
    else:
        vpv = vph = vp
        vsv = vsh = vs
        eta = np.ones_like(vp)
    A = rho * vph ** 2 * ifact
    C = rho * vpv ** 2 * ifact
    L = rho * vsv ** 2 * ifact
    N = rho * vsh ** 2 * ifact
    F = eta * (A - 2 * L)
    return A, C, F, L, N


def _pack_solid(mat, A, C, F, L, N, att_kind, att_info, ifact):
    """Returns (moduli array, attenuation moduli) for one solid element, 1D: (1, 25)."""
    attm = np.zeros(0)
    if att_kind != ATT_NONE:
        factors, qk, qm = att_info
        kappa, mu = ATT.voigt_ti(A, C, F, L, N)
        A, C, F, L, N = A - (kappa + 4 / 3 * mu), C - (kappa + 4 / 3 * mu), F - (kappa - 2 / 3 * mu), L - mu, N - mu
        kappa, mu, dk, dm = ATT.apply_attenuation(kappa, mu, qk, qm, ifact, att_kind == ATT_CG4, factors)
        A, C, F, L, N = A + (kappa + 4 / 3 * mu), C + (kappa + 4 / 3 * mu), F + (kappa - 2 / 3 * mu), L + mu, N + mu
        attm = np.concatenate([dk.ravel(), dm.ravel()])
    if mat == MAT_ISO:
        mod = np.stack([F, L])          # Isotropic(lambda = F, mu = L)
    elif mat == MAT_TISO:
        mod = np.stack([A, C, F, L, N])
    else:
        mod = _aniso_from_ti(A, C, F, L, N)
    return mod, attm


def _aniso_from_ti(A, C, F, L, N, eps=0.05, seed=7):
    """21 moduli (C11..C16, C22..C26, C33..C36, C44..C46, C55, C56, C66) of the TI tensor
    in the solver's strain order plus a small seeded symmetric perturbation."""
    rng = np.random.default_rng(seed)
    Z = np.zeros_like(A)
    full = [[A, A - 2 * N, F, Z, Z, Z], [A - 2 * N, A, F, Z, Z, Z], [F, F, C, Z, Z, Z],
            [Z, Z, Z, L, Z, Z], [Z, Z, Z, Z, L, Z], [Z, Z, Z, Z, Z, N]]
    out = []
    for i in range(6):
        for j in range(i, 6):
            out.append(full[i][j] + eps * L * rng.uniform(-1, 1))
    return np.stack(out)


def annulus_domain(seed=0, n_theta=4, n_r=3, r_in=3000e3, r_out=6371e3, theta_max=0.3, nu=2,
                   nu_random=False, nu_max=None, fluid_layers=(), mat=MAT_ISO, in3d=False,
                   att=ATT_NONE, nsls=3, mass3d=False, couple3d=False, dt=0.05, source=True,
                   n_receivers=3, stf_len=64, stability_interval=0, kahan=False, fluid3d=False,
                   perturb=0.04, lucky=False, surface_interval=0, ocean="", dumps=False, prt=None):
    """Connected spherical-element mesh on an (r, theta) grid.

    Element (ir, it) spans radii [rs[ir], rs[ir+1]] and colatitudes [ts[it], ts[it+1]];
    elements with it = 0 touch the axis.  fluid_layers lists the ir that are fluid.
    surface_interval > 0 records the outer surface (side 2, eta = +1, of every solid
    element of the top layer) every surface_interval steps.  ocean = "1d" puts a 3 km
    ocean on the outer surface points (MassOcean1D); "3d" varies its depth with azimuth
    and tilts the surface normal (MassOcean3D).  dumps = True flags the receivers
    dump_strain / dump_curl in turn (3, 1, 2, 0, ...).  prt = a (float) relabels every
    element with X = identity + a * noise (per point; per sample on 3-D elements, PRT_3D);
    a = 0 gives the identity map."""
    rng = np.random.default_rng(seed)
    rs = np.linspace(r_in, r_out, n_r + 1)
    ts = np.linspace(0.0, theta_max, n_theta + 1)
    NX = 4 * n_theta + 1  # GLL grid columns (theta)
    NZ = 4 * n_r + 1      # GLL grid rows (radius)
    npt = NX * NZ
    fluid_elem = np.zeros((n_r, n_theta), bool)
    for ir in fluid_layers:
        fluid_elem[ir, :] = True
    # point phases
    has_s = np.zeros(npt, bool)
    has_f = np.zeros(npt, bool)
    gid = lambda ir, it, ip, jp: (ir * 4 + jp) * NX + (it * 4 + ip)
    for ir in range(n_r):
        for it in range(n_theta):
            for ip in range(5):
                for jp in range(5):
                    (has_f if fluid_elem[ir, it] else has_s)[gid(ir, it, ip, jp)] = True
    kind = np.where(has_s & has_f, POINT_SOLID_FLUID, np.where(has_f, POINT_FLUID, POINT_SOLID)).astype(np.int8)
    # Nr per point
    if nu_random:
        nu_pt = rng.integers(0, (nu_max or 2 * nu) + 1, npt)
    else:
        nu_pt = np.full(npt, nu)
    nr_pt = 2 * nu_pt + 1
    if nu_random:  # a few even nr to exercise Nyquist handling (not on the axis)
        even = rng.random(npt) < 0.2
        nr_pt = np.where(even & (nr_pt > 2), nr_pt - 1, nr_pt)
    axial_pt = np.zeros(npt, bool)
    for jr in range(NZ):
        axial_pt[jr * NX] = True
    forced = axial_pt & (nr_pt % 2 == 0)
    nr_pt = np.where(forced, nr_pt + 1, nr_pt)  # Quad::formNrField: axis odd
    if lucky:  # FFT-friendly ring sizes (FFTW_LUCKY_NUMBER)
        from .solver import next_lucky
        nr_pt = np.array([next_lucky(int(n), bool(f)) for n, f in zip(nr_pt, forced)])
    fsurf = has_f & ~has_s & np.zeros(npt, bool)
    if fluid_layers and (n_r - 1) in fluid_layers:  # fluid at the free surface
        for ix in range(NX):
            fsurf[(NZ - 1) * NX + ix] = True

    # attenuation factors
    att_info = None
    alpha = beta = gamma = np.zeros(0)
    if att != ATT_NONE:
        w, y = ATT.fit_sls(nsls, 1 / 200.0, 1 / 10.0)
        f_min, f_max, f_ref = 1 / 200.0, 1 / 10.0, 1.0
        alpha, beta, gamma, _, _ = ATT.att_factors(w, y, f_min, f_max, f_ref, dt, np.ones(1), np.ones(1), True)

    B = _Builder(dt)
    mass_s = [dict() for _ in range(npt)]  # accumulate mass per sample later
    ms_acc = [None] * npt
    mf_acc = [None] * npt
    sfn_acc = [None] * npt
    surf_acc = [None] * npt  # summed outer-surface normals (GLLPoint::addSurfNormal)
    crds_pt = np.zeros((npt, 2))
    for ir in range(n_r):
        for it in range(n_theta):
            r0, r1, t0, t1 = rs[ir], rs[ir + 1], ts[it], ts[it + 1]
            nodes = np.array([[r0 * np.sin(t0), r0 * np.sin(t1), r1 * np.sin(t1), r1 * np.sin(t0)],
                              [r0 * np.cos(t0), r0 * np.cos(t1), r1 * np.cos(t1), r1 * np.cos(t0)]])
            axial = it == 0
            geo, ifact, crds, theta = GEO.element_geometry(nodes, axial)
            pts = [gid(ir, it, ip, jp) for ip in range(5) for jp in range(5)]
            for k, p in enumerate(pts):
                crds_pt[p] = crds[k]
            enr = int(nr_pt[pts].max())
            nr_mat = enr if (in3d or (fluid_elem[ir, it] and fluid3d)) else 1
            vp = np.zeros((nr_mat, 25))
            vs = np.zeros((nr_mat, 25))
            rho = np.zeros((nr_mat, 25))
            for k in range(25):
                a, b, c = _velocity_model(np.hypot(*crds[k]))
                vp[:, k], vs[:, k], rho[:, k] = a, b, c
            if nr_mat > 1:
                for k in range(25):
                    pert = _azimuth_perturbation(rng, nr_mat, perturb)
                    vp[:, k] *= pert
                    vs[:, k] *= pert
            if fluid_elem[ir, it]:
                K = (ifact[None, :] / rho)
                B.add_element(pts, MAT_ACOUSTIC, axial, nr_mat > 1, geo, GEO.trig_tables(theta), K, ATT_NONE, [])
                mass = ifact[None, :] / (rho * vp ** 2)  # Material::computeElementalMass (fluid)
                acc = mf_acc
            else:
                tiso = mat == MAT_TISO
                A, C, F, L, N = _solid_moduli(vp, vs, rho, ifact[None, :], tiso)
                a_info = None
                if att != ATT_NONE:
                    qk = np.full((nr_mat, 25), 57823.0)
                    qm = rng.uniform(80, 600) * np.ones((nr_mat, 25))
                    fac = ATT.att_factors(w, y, f_min, f_max, f_ref, dt, qk, qm, True)
                    a_info = ((fac[3], fac[4]), qk, qm)
                mod, attm = _pack_solid(mat, A, C, F, L, N, att, a_info, ifact)
                B.add_element(pts, mat, axial, nr_mat > 1, geo, GEO.trig_tables(theta), mod,
                              att, attm)
                mass = rho * ifact[None, :]
                acc = ms_acc
            for k, p in enumerate(pts):
                m = mass[:, k]
                if mass3d and len(m) == 1:
                    m = np.full(nr_pt[p], m[0])
                if len(m) > 1 and len(m) != nr_pt[p]:
                    m = np.full(nr_pt[p], m.mean())
                if not mass3d and len(m) > 1:
                    m = np.full(1, m.mean())
                acc[p] = m if acc[p] is None else acc[p] + m
            # solid-fluid boundary normals (Quad::computeNormal, GLLPoint::addSFNormal)
            for side, jp in ((0, 0), (2, 4)):
                irn = ir - 1 if side == 0 else ir + 1
                if not (0 <= irn < n_r) or fluid_elem[irn, it] == fluid_elem[ir, it]:
                    continue
                rsf = r0 if side == 0 else r1
                h_r_dt = 0.5 * rsf * abs(t1 - t0)
                h_r2_dt = 0.5 * rsf * rsf * abs(t1 - t0)
                for ip in range(5):
                    k = ip * 5 + jp
                    sz = crds[k]
                    sint = sz[0] / np.hypot(*sz)
                    cost = sz[1] / np.hypot(*sz)
                    nvec = _side_normal(nodes, crds, ip, jp, axial, h_r_dt, h_r2_dt)
                    if side != 2:
                        nvec = -nvec
                    if not fluid_elem[ir, it]:
                        nvec = -nvec
                    p = gid(ir, it, ip, jp)
                    sfn_acc[p] = nvec * 0.5 if sfn_acc[p] is None else sfn_acc[p] + nvec * 0.5
            if ocean and ir == n_r - 1 and not fluid_elem[ir, it]:  # outer side 2 (Quad.cpp:367-373)
                h_r_dt, h_r2_dt = 0.5 * r1 * abs(t1 - t0), 0.5 * r1 * r1 * abs(t1 - t0)
                for ip in range(5):
                    p = gid(ir, it, ip, 4)
                    nvec = _side_normal(nodes, crds, ip, 4, axial, h_r_dt, h_r2_dt)
                    surf_acc[p] = nvec if surf_acc[p] is None else surf_acc[p] + nvec
    # points
    mslen, ms, mflen, mf, sflen, sfn, sfni = [], [], [], [], [], [], []
    for p in range(npt):
        if has_s[p]:
            m = ms_acc[p]
            if len(m) == 1 or np.allclose(m, m[0], rtol=1e-12):  # XMath::equalRows -> Mass1D
                mslen.append(1)
                ms.append([1 / m[0]])
            else:
                mslen.append(nr_pt[p])
                ms.append(1 / m)
        else:
            mslen.append(0)
        if has_f[p]:
            m = mf_acc[p]
            if len(m) == 1 or np.allclose(m, m[0], rtol=1e-12):
                mflen.append(1)
                mf.append([1 / m[0]])
            else:
                mflen.append(nr_pt[p])
                mf.append(1 / m)
        else:
            mflen.append(0)
        if kind[p] == POINT_SOLID_FLUID:
            n = sfn_acc[p]
            mfl = mf_acc[p]
            if couple3d:
                ang = 2 * np.pi * np.arange(nr_pt[p]) / nr_pt[p]
                tilt = 1 + 0.02 * np.cos(ang)
                nn = np.outer(tilt, n)
                nn[:, 1] = 0.01 * np.sin(ang) * np.linalg.norm(n)
                mfv = np.full(nr_pt[p], mfl[0]) if len(mfl) == 1 else mfl
                sflen.append(nr_pt[p])
                sfn.append(nn)
                sfni.append(nn / mfv[:, None])
            else:
                sflen.append(1)
                sfn.append(n[None, :])
                sfni.append(n[None, :] / mfl[0])
        else:
            sflen.append(0)
    ea = B.element_arrays()
    # source on the axis (element it = 0 in the top solid layer) with orders 0..2
    sources = []
    if source:
        ir_s = max(i for i in range(n_r) if not fluid_elem[i, 0])
        e_s = ir_s * n_theta + 0
        force = (rng.normal(size=(25, 3, 3)) + 1j * rng.normal(size=(25, 3, 3))).astype(np.complex64) * 1e10
        force[:, 0, :] = force[:, 0, :].real
        sources.append((e_s, force))
    stf = np.exp(-((np.arange(stf_len) - stf_len / 4) / (stf_len / 10)) ** 2).astype(np.float32)
    # receivers in solid elements of the top layer
    solid_e = [ir * n_theta + it for ir in range(n_r) for it in range(n_theta) if not fluid_elem[ir, it]]
    r_elem = np.array(rng.choice(solid_e, n_receivers), np.int32) if n_receivers else np.zeros(0, np.int32)
    r_phi = rng.uniform(0, 2 * np.pi, len(r_elem)).astype(np.float32)
    r_w = rng.dirichlet(np.ones(25), len(r_elem)).astype(np.float32) if n_receivers else np.zeros((0, 25), np.float32)
    spec = DomainSpec(
        dt=dt, p_nr=nr_pt.astype(np.int32), p_kind=kind, p_axial=axial_pt.astype(np.uint8),
        p_fsurf=fsurf.astype(np.uint8), p_mslen=np.array(mslen, np.int32),
        p_ms=np.concatenate(ms).astype(np.float32) if ms else np.zeros(0, np.float32),
        p_mflen=np.array(mflen, np.int32),
        p_mf=np.concatenate(mf).astype(np.float32) if mf else np.zeros(0, np.float32),
        p_sflen=np.array(sflen, np.int32),
        p_sfn=np.concatenate(sfn).astype(np.float32) if sfn else np.zeros((0, 3), np.float32),
        p_sfni=np.concatenate(sfni).astype(np.float32) if sfni else np.zeros((0, 3), np.float32),
        nsls=nsls if att != ATT_NONE else 0, att_alpha=alpha, att_beta=beta, att_gamma=gamma,
        att_do_kappa=True, sources=sources, stf=stf, r_elem=r_elem, r_phi=r_phi, r_w=r_w,
        kahan=kahan, stability_interval=stability_interval, **ea)
    spec.p_crds = crds_pt
    if prt is not None:
        enr = spec.element_nr()
        lens = np.where(spec.e_in3d.astype(bool), enr, 1).astype(np.int32)
        xs = []
        for e in range(spec.n_elements):
            L = int(lens[e])
            ang = 2 * np.pi * np.arange(L) / L
            base = rng.normal(size=(4, 1, 25)) * (1 + 0.5 * np.cos(ang + rng.uniform(0, 2 * np.pi)))[None, :, None]
            x = prt * base
            x[0] += 1.0
            x[3] += 1.0
            xs.append(x.ravel())
        spec.prt_elem = np.arange(spec.n_elements, dtype=np.int32)
        spec.prt_len = lens
        spec.prt_x = np.concatenate(xs).astype(np.float32)
    if dumps:
        spec.r_dump = np.array([(3, 1, 2, 0)[i % 4] for i in range(len(r_elem))], np.int32)
    if ocean:
        spec.oc_pt, spec.oc_len, spec.oc_vals = _ocean_rows(ocean, surf_acc, ms_acc, nr_pt, crds_pt, rng)
    if surface_interval > 0:
        top = n_r - 1
        spec.sf_elem = np.array([top * n_theta + it for it in range(n_theta) if not fluid_elem[top, it]], np.int32)
        spec.sf_side = np.full(len(spec.sf_elem), 2, np.int32)
        spec.sf_interval = int(surface_interval)
    return spec


def _side_normal(nodes, crds, ip, jp, axial, h_r_dt, h_r2_dt):
    """Quad::computeNormal (Quad.cpp:661-715) without relabelling, before the sign flip:
    (sin theta, 0, cos theta) times the side's quadrature area."""
    from .spectral import weights, xi_eta
    sz = crds[ip * 5 + jp]
    sint, cost = sz[0] / np.hypot(*sz), sz[1] / np.hypot(*sz)
    nvec = np.array([sint, 0.0, cost])
    wsf = weights(ip, jp, axial)[0]
    if axial:
        if ip == 0:
            J = GEO.jacobian(nodes, xi_eta(ip, jp, axial))
            return nvec * wsf * J[0, 0] * h_r_dt
        return nvec * wsf / (1 + xi_eta(ip, jp, axial)[0]) * sint * h_r2_dt
    return nvec * wsf * sint * h_r2_dt


WATER_DENSITY = 1027.0  # OceanLoad3D::mWaterDensity


def ocean_rows(points, normal, mass, nr, colat, depth):
    """Ocean-load rows of GLLPoint::release (GLLPoint.cpp:57-72) for solid points.

    normal[i]: summed surface normal, [3] or [nr][3]; mass[i]: solid mass, [1] or [nr];
    depth[i]: ocean depth (m), scalar or [nr]; colat[i]: colatitude of the point.  Rows
    whose mass, depth and normal do not vary with azimuth become MassOcean1D (four values),
    the others MassOcean3D (nr x four values)."""
    lens, vals = [], []
    for i, p in enumerate(points):
        n = np.atleast_2d(np.asarray(normal[i], np.float64))
        m = np.atleast_1d(np.asarray(mass[i], np.float64))
        d = np.atleast_1d(np.asarray(depth[i], np.float64))
        flat = all(len(x) == 1 or np.ptp(x, 0).max() == 0 for x in (m, d, n))
        if flat:
            area = np.linalg.norm(n[0])
            mo = WATER_DENSITY * d[0] * area
            lens.append(1)
            vals.append([1.0 / (m[0] + mo), 1.0 / m[0], np.sin(colat[i]), np.cos(colat[i])])
        else:
            k = int(nr[p])
            n = np.broadcast_to(n, (k, 3))
            m = np.broadcast_to(m, (k,))
            d = np.broadcast_to(d, (k,))
            area = np.linalg.norm(n, axis=1)
            mo = WATER_DENSITY * d * area
            scal = np.sqrt(mo / (m * (m + mo)))
            lens.append(k)
            vals.append(np.column_stack([1.0 / m, n / area[:, None] * scal[:, None]]).ravel())
    return (np.asarray(points, np.int32), np.asarray(lens, np.int32),
            np.concatenate([np.ravel(v) for v in vals]).astype(np.float32) if vals else np.zeros(0, np.float32))


def _ocean_rows(kind, surf_acc, ms_acc, nr_pt, crds_pt, rng):
    pts = [p for p in range(len(surf_acc)) if surf_acc[p] is not None]
    normal, mass, depth, colat = [], [], [], []
    for p in pts:
        colat.append(np.arctan2(crds_pt[p][0], crds_pt[p][1]))
        mass.append(ms_acc[p])
        if kind == "3d":
            ang = 2 * np.pi * np.arange(nr_pt[p]) / nr_pt[p]
            nn = np.outer(1 + 0.05 * np.cos(ang), surf_acc[p])
            nn[:, 1] = 0.1 * np.sin(ang + rng.uniform(0, 2 * np.pi)) * np.linalg.norm(surf_acc[p])
            normal.append(nn)
            depth.append(3000.0 * (1 + 0.5 * np.cos(ang + rng.uniform(0, 2 * np.pi))))
        else:
            normal.append(surf_acc[p])
            depth.append(3000.0)
    return ocean_rows(pts, normal, mass, nr_pt, colat, depth)


def random_fields(spec: DomainSpec, seed=1, scale=1e-3, decay=1.5):
    """Random displacement with Fourier coefficients ~ N(0,1) * alpha^-decay (order 0 real)."""
    rng = np.random.default_rng(seed)
    ns, nf = spec.field_sizes()
    so, fo = spec.point_offsets()

    def make(n, offsets, ncomp):
        v = np.zeros(n, np.complex128)
        for p in range(spec.n_points):
            if offsets[p] < 0:
                continue
            na = spec.p_nr[p] // 2 + 1
            a = np.arange(na)
            amp = np.where(a == 0, 1.0, np.maximum(a, 1.0) ** -decay)
            blk = (rng.normal(size=(na, ncomp)) + 1j * rng.normal(size=(na, ncomp))) * amp[:, None] * scale
            blk[0] = blk[0].real
            v[offsets[p]:offsets[p] + na * ncomp] = blk.ravel()
        return v
    return make(ns, so, 3), make(nf, fo, 1)
