"""CPU tests: oracle against golden tables and invariants, host precompute, C-ABI exports."""
import ctypes
import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from axisem3d_gb300 import geometry as GEO
from axisem3d_gb300 import spectral as S
from axisem3d_gb300 import synth
from axisem3d_gb300.spec import ATT_CG4, ATT_FULL, MAT_ANISO, MAT_TISO

ROOT = Path(__file__).resolve().parents[1]
GOLD = json.loads((ROOT / "tests/golden/spectral_npol4.json").read_text())


def test_spectral_constants_match_reference_table():
    x, w, G = S.gll()
    xj, wj, Gj = S.glj()
    np.testing.assert_allclose(x, GOLD["pgll_4"], atol=1e-11)
    np.testing.assert_allclose(w, GOLD["wgll_4"], atol=1e-11)
    np.testing.assert_allclose(G.ravel(), GOLD["Ggll_4"], atol=1e-11)
    np.testing.assert_allclose(xj, GOLD["pglj_4"], atol=1e-11)
    np.testing.assert_allclose(wj, GOLD["wglj_4"], atol=1e-11)
    np.testing.assert_allclose(Gj.ravel(), GOLD["Gglj_4"], atol=1e-11)


def test_geometry_integral_factor_is_volume():
    """sum(ifact) over a spherical element = its meridional 'volume' int s ds dz."""
    r0, r1, t0, t1 = 5000e3, 5200e3, 0.1, 0.15
    nodes = np.array([[r0 * np.sin(t0), r0 * np.sin(t1), r1 * np.sin(t1), r1 * np.sin(t0)],
                      [r0 * np.cos(t0), r0 * np.cos(t1), r1 * np.cos(t1), r1 * np.cos(t0)]])
    _, ifact, _, _ = GEO.element_geometry(nodes, axial=False)
    exact = (r1 ** 3 - r0 ** 3) / 3 * (np.cos(t0) - np.cos(t1))  # int r^2 sin t dr dt
    assert abs(ifact.sum() - exact) / exact < 1e-6


def _oracle():
    from oracle.oracle_py import OracleDomain
    return OracleDomain


def _stiffness_matrix(spec, double=True):
    """Element stiffness matrix by unit impulses (SolidElement::test, SolidElement.cpp:96-187)."""
    OD = _oracle()
    d = OD(spec, double=double)
    n = d.nsolid
    so, _ = spec.point_offsets()
    cols = []
    idx = []
    for p in range(spec.n_points):
        na = spec.p_nr[p] // 2 + 1
        for a in range(na):
            for c in range(3):
                if spec.p_axial[p] and ((a == 0 and c != 2) or (a == 1 and c == 2) or a >= 2):
                    continue
                idx.append(so[p] + a * 3 + c)
    K = np.zeros((len(idx), len(idx)))
    for j, col in enumerate(idx):
        u = np.zeros(n, complex)
        u[col] = 2.0 if (col - so[np.searchsorted(so, col, side='right') - 1]) // 3 == 0 else 1.0
        d.set("displ", "solid", u)
        d.set("stiff", "solid", np.zeros(n, complex))
        d.compute_stiff()
        s = -d.get("stiff", "solid")
        K[:, j] = s[idx].real
    return K


@pytest.mark.parametrize("kw", [dict(nu=1), dict(nu=2, mat=MAT_TISO), dict(nu=1, mat=MAT_ANISO)])
def test_oracle_stiffness_positive_and_symmetric(kw):
    """The reference's own self-test: K positive diagonal and self-adjoint."""
    spec = synth.annulus_domain(n_theta=1, n_r=1, source=False, n_receivers=0, **kw)
    K = _stiffness_matrix(spec)
    assert (np.diag(K) > 0).all()
    scale = np.abs(K).max()
    assert np.abs(K - K.T).max() <= 1e-8 * scale


def test_oracle_float_vs_double():
    OD = _oracle()
    for kw in (dict(), dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=3), dict(fluid_layers=(0,), att=ATT_FULL)):
        spec = synth.annulus_domain(stf_len=16, **kw)
        a, b = OD(spec), OD(spec, double=True)
        a.step(16)
        b.step(16)
        ua, ub = a.get("displ"), b.get("displ")
        assert np.linalg.norm(ua - ub) <= 1e-5 * np.linalg.norm(ub)


def test_oracle_dft_conventions():
    """C2R/R2C follow FFTW: C2R unnormalised ignoring Im(X0), R2C scaled by 1/nr."""
    from oracle.oracle_py import load_oracle
    load_oracle()
    rng = np.random.default_rng(0)
    for nr in (1, 2, 5, 8, 17):
        x = rng.normal(size=nr)
        X = np.fft.rfft(x) / nr
        back = np.fft.irfft(X * nr, nr)
        np.testing.assert_allclose(back, x, atol=1e-12)


def test_header_declares_every_export():
    decl = re.findall(r"^(?:int|int64_t|int32_t|size_t)\s+(ax3d_\w+)\(", (ROOT / "include/ax3d.h").read_text(), re.M)
    assert len(decl) >= 20
    lib = ROOT / "axisem3d_gb300/libax3d.so"
    if not lib.exists():
        from axisem3d_gb300 import build
        build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ax3d_\w+)", out))
    assert set(decl) <= exported, set(decl) - exported
    ctypes.CDLL(str(lib))  # loads without a GPU


def test_capi_rejects_bad_input_without_gpu():
    """Argument checks happen before any device work."""
    from axisem3d_gb300 import capi
    lib = capi.load_library()
    cfg = capi.Config()
    cfg.npol = 5
    h = ctypes.c_void_p()
    assert lib.ax3d_create(ctypes.byref(cfg), ctypes.byref(h)) == 6
    buf = ctypes.create_string_buffer(256)
    lib.ax3d_last_error(buf, 256)
    assert b"nPol" in buf.value


def test_oracle_wisdom_labels():
    """Nu wisdom: a field with energy only in orders <= 3 learns Nu <= 3 everywhere."""
    OD = _oracle()
    spec = synth.annulus_domain(nu=8, source=False, n_receivers=0)
    d = OD(spec)
    rng = np.random.default_rng(0)
    so, _ = spec.point_offsets()
    u = np.zeros(d.nsolid, complex)
    for p in range(spec.n_points):
        na = spec.p_nr[p] // 2 + 1
        blk = np.zeros((na, 3), complex)
        blk[:4] = rng.normal(size=(4, 3)) + 1j * rng.normal(size=(4, 3))
        u[so[p]:so[p] + 3 * na] = blk.ravel()
    d.set("displ", "solid", u)
    d.learn_wisdom(1e-3)
    w = d.get_wisdom()
    assert w.max() <= 3 and w.min() >= 0 and (w == 3).mean() > 0.5


def test_oracle_surface_record_is_side_displacement():
    """The whole-surface record holds every side point's own Fourier rows (orders above a
    point's Nu zero), [component][point on the side][order] (SolidElement::feedDispOnSide)."""
    from axisem3d_gb300 import synth
    from oracle.oracle_py import OracleDomain
    spec = synth.annulus_domain(n_theta=3, n_r=2, nu_random=True, nu_max=6, stf_len=6, surface_interval=2)
    o = OracleDomain(spec)
    su, _ = synth.random_fields(spec, seed=21)
    o.set("displ", "solid", su)
    o.record(0)
    o.record(1)  # not a multiple of the interval: no record
    o.record(2)
    rec = o.surface(0, 2)
    so, _ = spec.point_offsets()
    enr = spec.element_nr()
    for k, e in enumerate(spec.sf_elem):
        na = enr[e] // 2 + 1
        for q in range(5):
            pt = spec.e_pts[e, q * 5 + 4]  # side 2: jpol = 4
            nu = spec.p_nr[pt] // 2
            for c in range(3):
                want = np.zeros(na, complex)
                want[:nu + 1] = su[so[pt] + 3 * np.arange(nu + 1) + c]
                np.testing.assert_allclose(rec[k][0, c, q], want, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(rec[0][0], rec[0][1])  # the field did not change between the records


@pytest.mark.parametrize("ocean", ["1d", "3d"])
def test_oracle_ocean_load_accel(ocean):
    """MassOcean1D / MassOcean3D: the oracle's acceleration on ocean points equals a numpy
    restatement (radial over m + m_ocean, tangential over m; per sample f/m - (f.n')n')."""
    from oracle.oracle_py import OracleDomain
    spec = synth.annulus_domain(seed=4, n_theta=3, n_r=2, nu=3, nu_random=True, nu_max=6, source=False,
                                n_receivers=0, ocean=ocean)
    assert (spec.oc_len > 1).any() == (ocean == "3d")
    o = OracleDomain(spec, double=True)
    so, _ = spec.point_offsets()
    rng = np.random.default_rng(5)
    f = np.zeros(o.nsolid, complex)
    for p in range(spec.n_points):
        if so[p] < 0:
            continue
        nr = spec.p_nr[p]
        blk = rng.normal(size=(nr // 2 + 1, 3)) + 1j * rng.normal(size=(nr // 2 + 1, 3))
        blk[0] = blk[0].real
        if nr % 2 == 0:
            blk[-1] = 0
        f[so[p]:so[p] + blk.size] = blk.ravel()
    o.set("stiff", "solid", f)
    o.update_newmark()
    acc = o.get("accel", "solid")
    ofs = 0
    for p, ln in zip(spec.oc_pt, spec.oc_len):
        v = spec.oc_vals[ofs:ofs + 4 * ln].astype(np.float64).reshape(ln, 4)
        ofs += 4 * ln
        if spec.p_axial[p]:
            continue
        nr = spec.p_nr[p]
        na = nr // 2 + 1
        F = f[so[p]:so[p] + 3 * na].reshape(na, 3)
        if ln == 1:
            imz, imr, st, ct = v[0]
            z = (F[:, 0] * st + F[:, 2] * ct) * imz
            r = (F[:, 0] * ct - F[:, 2] * st) * imr
            want = np.stack([z * st + r * ct, F[:, 1] * imr, z * ct - r * st], 1)
        else:
            x = np.stack([np.real(np.fft.ifft(_herm(F[:, c], nr)) * nr) for c in range(3)], 1)
            fn = (x * v[:, 1:]).sum(1)
            y = x * v[:, :1] - fn[:, None] * v[:, 1:]
            want = np.fft.rfft(y, axis=0)[:na] / nr
            want[0] = want[0].real
            if nr % 2 == 0:
                want[-1] = 0
        got = acc[so[p]:so[p] + 3 * na].reshape(na, 3)
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())


def _herm(X, nr):
    """Full spectrum of a real length-nr signal from orders 0..nr/2 (Hermitian)."""
    full = np.zeros(nr, complex)
    na = len(X)
    full[:na] = X
    for a in range(1, na):
        if nr - a != a:
            full[nr - a] = np.conj(X[a])
    full[0] = X[0].real
    return full


@pytest.mark.parametrize("field", ["translation", "rotation", "expansion"])
def test_oracle_strain_curl_of_analytic_fields(field):
    """Receivers flagged dump_strain / dump_curl (SolidElement::computeStrain/computeCurl):
    a rigid translation has no strain and no curl; a rigid rotation about z (u_phi = w s)
    has no strain and curl 2w z = (-2w sin t, 0, 2w cos t) in (theta, phi, r); u_s = w s
    has strain w (cos^2 t, 1, sin^2 t, 0, 2 sin t cos t, 0) (shear doubled), curl 0."""
    spec = synth.annulus_domain(seed=3, n_theta=6, n_r=4, nu=3, n_receivers=8, dumps=True, source=False,
                                stf_len=4, theta_max=1.0)
    o = _oracle()(spec, double=True)
    so, _ = spec.point_offsets()
    w = 1e-3
    u = np.zeros(o.nsolid, complex)
    for p in range(spec.n_points):
        na = spec.p_nr[p] // 2 + 1
        blk = np.zeros((na, 3), complex)
        s_ = spec.p_crds[p][0]
        if field == "translation":
            blk[0, 2], blk[1, 0], blk[1, 1] = 0.7 * w, (1 + 0.5j) * w / 2, (-0.5 + 1j) * w / 2
        elif field == "rotation":
            blk[0, 1] = w * s_
        else:
            blk[0, 0] = w * s_
        u[so[p]:so[p] + 3 * na] = blk.ravel()
    o.set("displ", "solid", u)
    o.record(0)
    st, cu = o.strain_curl("strain", 0, 1)[0], o.strain_curl("curl", 0, 1)[0]
    th = np.arctan2(spec.p_crds[:, 0], spec.p_crds[:, 1])
    i_s = i_c = 0
    for r in range(len(spec.r_elem)):
        wts = spec.r_w[r].astype(np.float64)
        t = th[spec.e_pts[spec.r_elem[r]]]
        want_s, want_c = np.zeros(6), np.zeros(3)
        if field == "rotation":
            want_c = 2 * w * np.array([-(wts * np.sin(t)).sum(), 0.0, (wts * np.cos(t)).sum()])
        if field == "expansion":
            want_s = w * np.array([(wts * np.cos(t) ** 2).sum(), wts.sum(), (wts * np.sin(t) ** 2).sum(), 0.0,
                                   (wts * np.sin(2 * t)).sum(), 0.0])
        if spec.r_dump[r] & 1:
            np.testing.assert_allclose(st[i_s], want_s, atol=2e-3 * w)
            i_s += 1
        if spec.r_dump[r] & 2:
            np.testing.assert_allclose(cu[i_c], want_c, atol=2e-3 * w)
            i_c += 1
    assert i_s == 4 and i_c == 4


@pytest.mark.parametrize("kw", [dict(), dict(mat=MAT_TISO, att=ATT_FULL, nu=3),
                                dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=4),
                                dict(in3d=True, mat=MAT_ANISO, att=ATT_FULL, nu=3),
                                dict(fluid_layers=(0,), nu_random=True, nu_max=5),
                                dict(fluid_layers=(1,), in3d=True, fluid3d=True, nu=4)],
                         ids=["iso1d", "ti1d_full", "ti3d_cg4", "aniso3d_full", "fluid1d", "fluid3d"])
def test_oracle_identity_relabelling_is_no_relabelling(kw):
    """PRT with X = (1, 0, 0, 1) maps the nine-component gradient onto the ordinary strain and
    the stress back onto the symmetric divergence: the stiffness (and, through two passes,
    the memory variables) equal the run without relabelling.  Isotropic elements go through
    the RTZ rotation only with relabelling, so they agree to the float theta tables."""
    out = []
    for prt in (None, 0.0):
        spec = synth.annulus_domain(prt=prt, **kw)
        o = _oracle()(spec, double=True)
        su, fu = synth.random_fields(spec, seed=3)
        o.set("displ", "solid", su)
        if o.nfluid:
            o.set("displ", "fluid", fu)
        o.compute_stiff()
        o.compute_stiff()
        out.append([o.get("stiff", "solid")] + ([o.get("stiff", "fluid")] if o.nfluid else []))
    for a, b in zip(*out):
        assert np.linalg.norm(a - b) <= 1e-7 * np.linalg.norm(b)


def test_oracle_relabelling_changes_the_stiffness():
    """A non-trivial X changes the stiffness (the relabelled path is not bypassed)."""
    res = []
    for prt in (0.0, 0.05):
        spec = synth.annulus_domain(prt=prt, in3d=True, nu=3)
        o = _oracle()(spec, double=True)
        o.set("displ", "solid", synth.random_fields(spec, seed=3)[0])
        o.compute_stiff()
        res.append(o.get("stiff", "solid"))
    assert np.linalg.norm(res[1] - res[0]) > 1e-3 * np.linalg.norm(res[0])


def test_oracle_queued_inputs_apply_at_the_next_step():
    """The oracle's asynchronous field calls mirror the library's: each step() starts from
    the oldest queued input; a third queued input is refused."""
    spec = synth.annulus_domain(nu=3, stf_len=6)
    a, b = _oracle()(spec), _oracle()(spec)
    x0, x1 = (synth.random_fields(spec, seed=s, scale=1e-6)[0] for s in (1, 2))
    a.set("displ", "solid", x0)
    a.step(1)
    r0 = a.get("displ", "solid")
    a.set("displ", "solid", x1)
    a.step(1)
    r1 = a.get("displ", "solid")
    b.set_async("displ", "solid", x0.astype(np.complex128))
    b.set_async("displ", "solid", x1.astype(np.complex128))
    with pytest.raises(Exception):
        b.set_async("displ", "solid", x1.astype(np.complex128))
    b.step(1)
    np.testing.assert_array_equal(b.get("displ", "solid"), r0)
    b.step(1)
    np.testing.assert_array_equal(b.get("displ", "solid"), r1)


def test_oracle_rejects_inconsistent_relabelling_ocean_and_dumps():
    """The reference's checks, mirrored by the oracle and the library: a PRT whose space does
    not match the element's (SolidElement::SolidElement), an ocean load on a fluid point or
    of the wrong length (MassOcean3D::checkCompatibility), strain / curl receivers in
    relabelled elements (not built)."""
    from axisem3d_gb300.capi import Ax3dError
    spec = synth.annulus_domain(prt=0.0, nu=3)
    spec.prt_len = spec.prt_len.copy()
    spec.prt_len[0] = 7  # a 1-D element given a 3-D relabelling
    spec.prt_x = np.ones(int(4 * 25 * spec.prt_len.sum()), np.float32)
    with pytest.raises(Ax3dError, match="different spaces"):
        _oracle()(spec)
    spec = synth.annulus_domain(fluid_layers=(0,), nu=3, ocean="1d")
    fluid_pt = int(np.flatnonzero(spec.p_kind == 1)[0])
    spec.oc_pt = np.concatenate([spec.oc_pt, [fluid_pt]]).astype(np.int32)
    spec.oc_len = np.concatenate([spec.oc_len, [1]]).astype(np.int32)
    spec.oc_vals = np.concatenate([spec.oc_vals, np.ones(4, np.float32)])
    with pytest.raises(Ax3dError, match="Fluid point with ocean load"):
        _oracle()(spec)
    spec = synth.annulus_domain(nu=3, ocean="1d")
    spec.oc_len = spec.oc_len.copy()
    spec.oc_len[0] = 2
    spec.oc_vals = np.ones(int(4 * spec.oc_len.sum()), np.float32)
    with pytest.raises(Ax3dError, match="Incompatible size"):
        _oracle()(spec)
    spec = synth.annulus_domain(prt=0.02, nu=3, n_receivers=4, dumps=True)
    with pytest.raises(Ax3dError, match="relabelled elements are not supported"):
        _oracle()(spec)


def _as_3d(spec):
    """The same domain with every element in physical space: moduli, attenuation moduli
    and relabelling X repeated over the element's samples."""
    import copy
    s3 = copy.deepcopy(spec)
    enr = spec.element_nr()
    km_of = {0: 2, 1: 5, 2: 21, 3: 1}
    mods, atts, mofs, aofs, xs = [], [], [], [], []
    xo = 0
    for e in range(spec.n_elements):
        nr = int(enr[e])
        km = km_of[int(spec.e_mat[e])]
        md = spec.e_mod[spec.e_mofs[e]:spec.e_mofs[e] + km * 25].reshape(km, 1, 25)
        mofs.append(sum(m.size for m in mods))
        mods.append(np.repeat(md, nr, 1).ravel())
        att = int(spec.e_att[e])
        npa = 4 if att == ATT_CG4 else 25
        aofs.append(sum(a.size for a in atts))
        if att:
            am = spec.e_attm[spec.e_aofs[e]:spec.e_aofs[e] + 2 * npa].reshape(2, 1, npa)
            atts.append(np.repeat(am, nr, 1).ravel())
        x = spec.prt_x[xo:xo + 100].reshape(4, 1, 25)
        xo += 100
        xs.append(np.repeat(x, nr, 1).ravel())
    s3.e_in3d = np.ones(spec.n_elements, np.uint8)
    s3.e_mod = np.concatenate(mods).astype(np.float32)
    s3.e_mofs = np.array(mofs, np.int64)
    s3.e_attm = (np.concatenate(atts) if atts else np.zeros(0)).astype(np.float32)
    s3.e_aofs = np.array(aofs, np.int64)
    s3.prt_len = enr.astype(np.int32)
    s3.prt_x = np.concatenate(xs).astype(np.float32)
    return s3


@pytest.mark.parametrize("kw", [dict(mat=MAT_TISO, att=ATT_CG4, nu=3), dict(mat=MAT_ANISO, att=ATT_FULL, nu=2),
                                dict(fluid_layers=(1,), nu=3)], ids=["ti_cg4", "aniso_full", "fluid"])
def test_oracle_prt1d_equals_prt3d_with_repeated_x(kw):
    """The Fourier-space relabelling (PRT_1D) and the per-sample one (PRT_3D) agree when the
    3-D element repeats the 1-D moduli and X over its samples (FP64 oracle, two passes so the
    memory variables take part)."""
    s1 = synth.annulus_domain(prt=0.05, **kw)
    s3 = _as_3d(s1)
    out = []
    for sp in (s1, s3):
        o = _oracle()(sp, double=True)
        su, fu = synth.random_fields(sp, seed=11)
        o.set("displ", "solid", su)
        if o.nfluid:
            o.set("displ", "fluid", fu)
        o.compute_stiff()
        o.compute_stiff()
        out.append([o.get("stiff", "solid")] + ([o.get("stiff", "fluid")] if o.nfluid else []))
    for a, b in zip(*out):
        assert np.linalg.norm(a - b) <= 1e-11 * np.linalg.norm(a)


def test_oracle_ocean3d_with_constant_rows_equals_ocean1d():
    """MassOcean3D with mass, depth and normal independent of azimuth (unit normal
    (sin t, 0, cos t)) gives MassOcean1D's acceleration: radial over m + m_ocean,
    tangential over m."""
    import copy
    spec = synth.annulus_domain(seed=4, n_theta=3, n_r=2, nu=3, nu_random=True, nu_max=6, source=False,
                                n_receivers=0, ocean="1d")
    s3 = copy.deepcopy(spec)
    lens, vals = [], []
    for i, p in enumerate(spec.oc_pt):
        imz, imr, st, ct = spec.oc_vals[4 * i:4 * i + 4].astype(np.float64)
        nr = int(spec.p_nr[p])
        if nr == 1:  # one sample: length 1 is the 1-D form (GLLPoint.cpp:58 never sees rows differ)
            lens.append(1)
            vals.append(spec.oc_vals[4 * i:4 * i + 4].astype(np.float64))
            continue
        m, mo = 1.0 / imr, 1.0 / imz - 1.0 / imr
        scal = np.sqrt(mo / (m * (m + mo)))
        lens.append(nr)
        vals.append(np.tile([1.0 / m, st * scal, 0.0, ct * scal], nr))
    s3.oc_len = np.array(lens, np.int32)
    s3.oc_vals = np.concatenate(vals).astype(np.float32)
    acc = []
    for sp in (spec, s3):
        o = _oracle()(sp, double=True)
        o.set("stiff", "solid", synth.random_fields(sp, seed=5)[0])
        o.update_newmark()
        acc.append(o.get("accel", "solid"))
    so, _ = spec.point_offsets()
    rows = np.concatenate([np.arange(so[p], so[p] + 3 * (spec.p_nr[p] // 2 + 1)) for p in spec.oc_pt])
    a, b = acc[0][rows], acc[1][rows]
    assert np.linalg.norm(a) > 0 and np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(a)


def test_header_compiles_as_c99(tmp_path):
    """include/ax3d.h is a C header: a C99 translation unit that takes the address of every
    declared entry point compiles warning-free with gcc (no C++ in the signatures)."""
    import shutil
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    decl = re.findall(r"^(?:int|int64_t|int32_t|size_t)\s+(ax3d_\w+)\(", (ROOT / "include/ax3d.h").read_text(), re.M)
    src = tmp_path / "t.c"
    src.write_text('#include "ax3d.h"\n#include <stdio.h>\ntypedef void (*fn)(void);\nstatic const fn table[] = {\n'
                   + "".join(f"    (fn)&{f},\n" for f in decl)
                   + '};\nint main(void) {\n    printf("%d\\n", (int)(sizeof table / sizeof table[0]));\n'
                   + "    return 0;\n}\n")
    res = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-c", str(src),
                          "-I", str(ROOT / "include"), "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.parametrize("kw", [dict(nu=1, prt=0.1), dict(nu=2, mat=MAT_TISO, prt=0.1),
                                dict(nu=1, mat=MAT_ANISO, prt=0.1), dict(nu=2, in3d=True, prt=0.1)],
                         ids=["iso_prt1d", "ti_prt1d", "aniso_prt1d", "iso_prt3d"])
def test_oracle_relabelled_stiffness_positive_and_symmetric(kw):
    """The reference's self-test on relabelled elements: the back-map of the stress is the
    adjoint of the strain map, so K stays self-adjoint with a positive diagonal (a
    transcription error in either map breaks the symmetry)."""
    spec = synth.annulus_domain(n_theta=1, n_r=1, source=False, n_receivers=0, **kw)
    assert len(spec.prt_elem) == 1
    K = _stiffness_matrix(spec)
    assert (np.diag(K) > 0).all()
    scale = np.abs(K).max()
    assert np.abs(K - K.T).max() <= 1e-8 * scale


def test_oracle_elastic_energy_is_conserved():
    """A source-free, non-attenuating elastic run (Newmark::solve on the FP64 oracle) keeps
    its energy 1/2 v^T M v + 1/2 u^T K u bounded, without drift: the mass, the stiffness
    and the update agree with one another (the Fourier inner product weighs order 0 once and
    the others twice)."""
    spec = synth.annulus_domain(seed=8, n_theta=3, n_r=2, nu=3, nu_random=True, nu_max=5, mat=MAT_TISO,
                                source=False, n_receivers=0, stf_len=400, dt=0.05)
    o = _oracle()(spec, double=True)
    su, _ = synth.random_fields(spec, seed=9, scale=1e-6, decay=2.0)
    o.set("displ", "solid", su)
    so, _ = spec.point_offsets()
    w = np.zeros(o.nsolid)
    m = np.zeros(o.nsolid)
    for p in range(spec.n_points):
        na = spec.p_nr[p] // 2 + 1
        ww = np.where(np.arange(na) == 0, 1.0, 2.0)
        w[so[p]:so[p] + 3 * na] = np.repeat(ww, 3)
        m[so[p]:so[p] + 3 * na] = 1.0 / float(spec.p_ms[spec.p_mslen[:p].sum()])
    energies = []
    for k in range(300):
        o.step(1)
        u, v = o.get("displ", "solid"), o.get("veloc", "solid")
        o.set("stiff", "solid", np.zeros(o.nsolid, complex))
        o.compute_stiff()
        ku = -o.get("stiff", "solid")
        kin = 0.5 * np.sum(w * m * np.abs(v) ** 2)
        pot = 0.5 * np.sum(w * np.real(np.conj(u) * ku))
        energies.append(kin + pot)
    e = np.array(energies[20:])
    assert e.min() > 0
    assert (e.max() - e.min()) / e.mean() < 0.05
    assert abs(e[-50:].mean() - e[:50].mean()) / e.mean() < 0.02


def test_oracle_empty_domain_steps():
    """Edge case: a domain without points or elements is accepted and steps (the step
    counter advances, no fields)."""
    from axisem3d_gb300.spec import DomainSpec
    z = lambda *s, dt=np.float32: np.zeros(s, dt)
    spec = DomainSpec(dt=0.1, p_nr=z(0, dt=np.int32), p_kind=z(0, dt=np.int8), p_axial=z(0, dt=np.uint8),
                      p_fsurf=z(0, dt=np.uint8), p_mslen=z(0, dt=np.int32), p_ms=z(0), p_mflen=z(0, dt=np.int32),
                      p_mf=z(0), p_sflen=z(0, dt=np.int32), p_sfn=z(0, 3), p_sfni=z(0, 3), e_pts=z(0, 25, dt=np.int32),
                      e_mat=z(0, dt=np.int8), e_axial=z(0, dt=np.uint8), e_in3d=z(0, dt=np.uint8), e_geo=z(0, 5, 25),
                      e_trig=z(0, 4, 25), e_mofs=z(0, dt=np.int64), e_mod=z(0), e_att=z(0, dt=np.int8),
                      e_aofs=z(0, dt=np.int64), e_attm=z(0), nsls=0, att_alpha=np.zeros(0), att_beta=np.zeros(0),
                      att_gamma=np.zeros(0), att_do_kappa=True, stf=np.ones(5, np.float32))
    o = _oracle()(spec)
    o.step(3)
    assert o.nsolid == 0 and o.nfluid == 0 and o.current_step == 4


@pytest.mark.parametrize("kw", [dict(nu=1), dict(nu=2), dict(nu=2, prt=0.1)], ids=["nu1", "nu2", "nu2_prt1d"])
def test_oracle_fluid_stiffness_positive_and_symmetric(kw):
    """FluidElement::test (FluidElement.cpp:94-161) on the oracle: unit impulses of the
    potential (2 for order 0) give a fluid stiffness with positive diagonal, self-adjoint."""
    spec = synth.annulus_domain(n_theta=1, n_r=1, fluid_layers=(0,), source=False, n_receivers=0, **kw)
    d = _oracle()(spec, double=True)
    _, fo = spec.point_offsets()
    idx = []
    for p in range(spec.n_points):
        na = spec.p_nr[p] // 2 + 1
        for a in range(na):
            if spec.p_axial[p] and a > 0:
                continue
            if spec.p_nr[p] % 2 == 0 and a == na - 1:
                continue
            idx.append((fo[p] + a, a))
    n = d.nfluid
    K = np.zeros((len(idx), len(idx)))
    for j, (col, a) in enumerate(idx):
        u = np.zeros(n, complex)
        u[col] = 2.0 if a == 0 else 1.0
        d.set("displ", "fluid", u)
        d.set("stiff", "fluid", np.zeros(n, complex))
        d.compute_stiff()
        K[:, j] = -d.get("stiff", "fluid")[[c for c, _ in idx]].real
    assert (np.diag(K) > 0).all()
    assert np.abs(K - K.T).max() <= 1e-8 * np.abs(K).max()


@pytest.mark.parametrize("kw,phase", [(dict(fluid_layers=(1,), in3d=True, fluid3d=True, mass3d=True), "fluid"),
                                      (dict(ocean="1d"), "solid"), (dict(ocean="3d"), "solid")],
                         ids=["fluid_mass3d", "ocean1d", "ocean3d"])
def test_oracle_mass_positive_and_symmetric(kw, phase):
    """SolidPoint::test / FluidPoint::test (SolidPoint.cpp:98-161, FluidPoint.cpp:104-155) on
    the oracle, point by point: unit stiffness impulses (2 for order 0) through one Newmark
    update give the inverse-mass matrix, with positive diagonal and self-adjoint -- for a
    phi-dependent (Mass3D) fluid mass and both ocean-load forms."""
    spec = synth.annulus_domain(seed=5, n_theta=2, n_r=2, nu=3, nu_random=True, nu_max=6, source=False,
                                n_receivers=0, **kw)
    so, fo = spec.point_offsets()
    ofs, nc = (so, 3) if phase == "solid" else (fo, 1)
    if phase == "solid":
        special = sorted(p for p in spec.oc_pt.tolist() if spec.p_kind[p] == 0)
    else:
        special = [int(p) for p in np.flatnonzero((spec.p_mflen > 1) & (spec.p_kind == 1))]
    assert special
    for p in special[:10]:
        d = _oracle()(spec, double=True)
        n = d.nsolid if phase == "solid" else d.nfluid
        nr = int(spec.p_nr[p])
        na = nr // 2 + 1
        rows = []
        for a in range(na):
            if nr % 2 == 0 and a == na - 1:
                continue
            for c in range(nc):
                if spec.p_axial[p] and ((nc == 3 and ((a == 0 and c != 2) or (a == 1 and c == 2) or a >= 2))
                                        or (nc == 1 and a > 0)):
                    continue
                rows.append((a, c))
        M = np.zeros((len(rows), len(rows)))
        for j, (a, c) in enumerate(rows):
            st = np.zeros(n, complex)
            st[ofs[p] + nc * a + c] = 2.0 if a == 0 else 1.0
            for which in ("displ", "veloc", "accel"):
                d.set(which, phase, np.zeros(n, complex))
            d.set("stiff", phase, st)
            d.update_newmark()
            acc = d.get("accel", phase)
            M[:, j] = [acc[ofs[p] + nc * a1 + c1].real for a1, c1 in rows]
        assert (np.diag(M) > 0).all(), p
        assert np.abs(M - M.T).max() <= 1e-9 * np.abs(M).max(), p


def test_cpp_host_interface_compiles(tmp_path):
    """include/ax3d.hpp (the C++ mirror of the reference's Domain over the C-ABI) compiles as
    C++17 with warnings as errors, and a program using every loop body links against
    libax3d.so (no GPU needed to compile and link)."""
    import shutil
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    lib = ROOT / "axisem3d_gb300/libax3d.so"
    if not lib.exists():
        from axisem3d_gb300 import build
        build.build()
    src = tmp_path / "host.cpp"
    src.write_text("""#include "ax3d.hpp"
#include <cstdio>
int main(int argc, char **) {
    if (argc < 2) return 0;  // compiled and linked only
    ax3d_config cfg{};
    cfg.npol = 4;
    try {
        ax3d::Domain dom(cfg);
        dom.finalize();
        dom.updateNewmark();
        dom.applySource(0);
        dom.computeStiff();
        dom.coupleSolidFluid();
        dom.record(0);
        dom.solve(1);
        std::printf("%d\\n", dom.currentStep());
    } catch (const ax3d::Error &e) {
        std::printf("%d %s\\n", e.code(), e.what());
    }
    return 0;
}
""")
    res = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", str(src), "-I", str(ROOT / "include"),
                          "-L", str(lib.parent), "-lax3d", f"-Wl,-rpath,{lib.parent}", "-o", str(tmp_path / "host")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(tmp_path / "host")], capture_output=True, text=True)
    assert run.returncode == 0


# ring sizes nr = 2 Nu + 1 of the GPU ring-size sweep, plus every length the benchmark's
# Nu range 8-256 can produce and a few even ones
RING_NR = sorted({2 * nu + 1 for nu in (8, 11, 18, 35, 65, 70, 100, 128, 150, 195, 254)}
                 | set(range(17, 514, 2)) | {16, 50, 64, 144, 260, 512})


def test_cpu_fft_baseline_transforms_match_exact_dft():
    """The CPU baseline's O(nr log nr) FP32 transforms (mixed-radix Stockham, Bluestein for
    large prime factors, two real columns per complex transform) against the exact DFT in
    double with FFTW's conventions, relative L2 <= 1e-6 per column, both directions."""
    from oracle.oracle_py import fft_pair, ifft_pair
    rng = np.random.default_rng(5)
    for nr in RING_NR:
        n = nr // 2 + 1
        X = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
        x1, x2 = fft_pair(nr, X[0], X[1])
        for got, spec in ((x1, X[0]), (x2, X[1])):
            want = np.fft.irfft(spec.astype(np.complex128), nr) * nr  # reads Re of orders 0 and nr/2 only
            assert np.linalg.norm(got - want) <= 1e-6 * np.linalg.norm(want), nr
        r = rng.standard_normal((2, nr)).astype(np.float32)
        Y1, Y2 = ifft_pair(r[0], r[1])
        for got, x in ((Y1, r[0]), (Y2, r[1])):
            want = np.fft.rfft(x.astype(np.float64)) / nr
            assert np.linalg.norm(got - want) <= 1e-6 * np.linalg.norm(want), nr


@pytest.mark.parametrize("att", [ATT_CG4, ATT_FULL])
def test_cpu_fft_baseline_loop_matches_oracle(att):
    """The timed CPU baseline (the oracle's loop with the FFT transforms) against the
    checker on the element benchmark's domain, Nu 8-256: element stiffness and two steps."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300 import workloads as W
    spec = W.element_benchmark(n_elem=20, seed=9, att=att)
    u0 = W.benchmark_displacement(spec, seed=8)
    out = []
    for fft in (False, True):
        d = OracleDomain(spec, fft=fft)
        d.set("displ", "solid", u0)
        d.compute_stiff()
        s = d.get("stiff", "solid")
        d.step(2)
        out.append((s, d.get("accel", "solid")))
    for a, b in zip(out[0], out[1]):
        assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(a)
