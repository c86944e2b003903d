"""GPU parity: the CUDA path through the C-ABI against the CPU oracle.

Tolerance: relative L2 <= 1e-5 against the FP32 oracle (the reference's default Real),
the parity bar for the floating-point path; the FP64 oracle error is reported too.
"""
import numpy as np
import pytest

from axisem3d_gb300 import synth
from axisem3d_gb300.spec import ATT_CG4, ATT_FULL, MAT_ANISO, MAT_TISO

pytestmark = pytest.mark.gpu

TOL = 1e-5

CASES = {
    "iso1d": dict(),
    "iso1d_fluid_mixednu": dict(fluid_layers=(0,), nu_random=True, nu_max=5),
    "ti1d_full": dict(mat=MAT_TISO, att=ATT_FULL, nu=3),
    "aniso1d_cg4": dict(mat=MAT_ANISO, att=ATT_CG4, nu=2),
    "iso3d": dict(in3d=True, nu=4),
    "ti3d_cg4": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=6),
    "ti3d_full_mixednu": dict(in3d=True, mat=MAT_TISO, att=ATT_FULL, nu_random=True, nu_max=9),
    "aniso3d_full": dict(in3d=True, mat=MAT_ANISO, att=ATT_FULL, nu=5),
    "fluid3d_mass3d_couple3d": dict(fluid_layers=(1,), in3d=True, fluid3d=True, mass3d=True,
                                    couple3d=True, nu=4, mat=MAT_TISO),
    "fluid_surface": dict(fluid_layers=(2,), nu=3),
    # FFT-friendly ring sizes: the mixed-radix transform (radices 2, 3, 4, 5, 7, 11, 13)
    "ti3d_cg4_fft25": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=12),
    "iso3d_full_fft_lucky_mixed": dict(in3d=True, att=ATT_FULL, nu_random=True, nu_max=40, lucky=True),
    "aniso3d_fft_even50": dict(in3d=True, mat=MAT_ANISO, nu=24, lucky=True),
    "iso3d_fft44": dict(in3d=True, nu=21, lucky=True),
    "fluid3d_fft36": dict(fluid_layers=(1,), in3d=True, fluid3d=True, nu=16, lucky=True, mat=MAT_TISO),
    "ti3d_fft260_chunked": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=128, lucky=True),
    # ring sizes with a prime factor above 13: direct prime passes and Bluestein
    "ti3d_cg4_direct131": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=65, n_theta=2, n_r=2),
    "iso3d_full_direct391": dict(in3d=True, att=ATT_FULL, nu=195, n_theta=2, n_r=2),
    "ti3d_cg4_bluestein509": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=254, n_theta=2, n_r=2),
    "fluid3d_bluestein257": dict(fluid_layers=(1,), in3d=True, fluid3d=True, nu=128, mat=MAT_TISO, n_theta=2,
                                 n_r=2),
    # ocean load on the outer surface points (MassOcean1D, MassOcean3D)
    "iso1d_ocean1d_mixednu": dict(ocean="1d", nu_random=True, nu_max=6),
    "ti3d_ocean3d_mass3d": dict(in3d=True, mat=MAT_TISO, mass3d=True, ocean="3d", nu_random=True, nu_max=7),
    # particle relabelling: PRT_1D (Fourier space) and PRT_3D (per sample), solid and fluid
    "iso1d_prt1d_mixednu": dict(prt=0.05, nu_random=True, nu_max=5),
    "ti1d_full_prt1d": dict(mat=MAT_TISO, att=ATT_FULL, nu=3, prt=0.05),
    "fluid1d_prt1d": dict(fluid_layers=(1,), nu=3, prt=0.05),
    "ti3d_cg4_prt3d": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=6, prt=0.05),
    "aniso3d_full_prt3d_mixednu": dict(in3d=True, mat=MAT_ANISO, att=ATT_FULL, nu_random=True, nu_max=7, prt=0.05),
    "fluid3d_prt3d": dict(fluid_layers=(1,), in3d=True, fluid3d=True, nu=5, prt=0.05),
    # PRT_3D on every transform kind: mixed radix (lucky sizes), a direct prime pass, Bluestein
    "aniso3d_full_prt3d_fft_lucky": dict(in3d=True, mat=MAT_ANISO, att=ATT_FULL, nu_random=True, nu_max=40,
                                         lucky=True, prt=0.05),
    "fluid3d_prt3d_direct131": dict(fluid_layers=(1,), in3d=True, fluid3d=True, nu=65, mat=MAT_TISO, n_theta=2,
                                    n_r=2, prt=0.05),
    "ti3d_cg4_prt3d_bluestein509": dict(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=254, n_theta=2, n_r=2, prt=0.05),
}
# time-loop steps for the cases whose O(nr^2) FP64 oracle transform is slow
STEPS = {"ti3d_fft260_chunked": 6, "ti3d_cg4_direct131": 10, "iso3d_full_direct391": 4,
         "ti3d_cg4_bluestein509": 4, "fluid3d_bluestein257": 6, "fluid3d_prt3d_direct131": 10,
         "ti3d_cg4_prt3d_bluestein509": 4}

# Every transform path of the physical-space kernel: each direct-pass shape (prime
# factors 17, 23, 37, 71, 131 and 47 x 3, 43 x 7, 17 x 23), Bluestein (257, 509) and
# smooth sizes, with transversely isotropic moduli and CG4 attenuation.
RING_NU = [8, 11, 18, 35, 65, 70, 100, 128, 150, 195, 254]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _pair(name, **extra):
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    spec = synth.annulus_domain(**{**CASES[name], **extra})
    return spec, Ax3dDomain(spec), OracleDomain(spec), OracleDomain(spec, double=True)


@pytest.mark.parametrize("name", list(CASES))
def test_compute_stiff_matches_oracle(ax3d_lib, name):
    spec, g, o, od = _pair(name)
    su, fu = synth.random_fields(spec, seed=3)
    for d in (g, o, od):
        d.set("displ", "solid", su)
        if d.nfluid:
            d.set("displ", "fluid", fu)
        d.compute_stiff()
    for phase in ("solid", "fluid"):
        if phase == "fluid" and not g.nfluid:
            continue
        a, b, c = g.get("stiff", phase), o.get("stiff", phase), od.get("stiff", phase)
        assert rel(a, b) <= TOL, (phase, rel(a, b), rel(a, c))


@pytest.mark.parametrize("nu", RING_NU)
def test_compute_stiff_ring_sizes(ax3d_lib, nu):
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    spec = synth.annulus_domain(n_theta=2, n_r=2, in3d=True, mat=MAT_TISO, att=ATT_CG4, nu=nu, seed=nu)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    su, _ = synth.random_fields(spec, seed=nu + 1)
    for d in (g, o):
        d.set("displ", "solid", su)
        d.compute_stiff()
        d.compute_stiff()  # second pass: the memory variables were updated by the first
    assert rel(g.get("stiff", "solid"), o.get("stiff", "solid")) <= TOL


@pytest.mark.parametrize("name", list(CASES))
def test_time_loop_matches_oracle(ax3d_lib, name):
    n = STEPS.get(name, 40)
    spec, g, o, _ = _pair(name, stf_len=n, stability_interval=min(10, n))
    su, fu = synth.random_fields(spec, seed=5, scale=1e-6)
    for d in (g, o):
        d.set("displ", "solid", su)
        if d.nfluid:
            d.set("displ", "fluid", fu)
        d.step(n)
    for which in ("displ", "veloc", "accel"):
        a, b = g.get(which, "solid"), o.get(which, "solid")
        assert rel(a, b) <= TOL, (which, rel(a, b))
        if g.nfluid:
            a, b = g.get(which, "fluid"), o.get(which, "fluid")
            assert rel(a, b) <= TOL, (which, "fluid", rel(a, b))
    sa, sb = g.seismograms(0, n), o.seismograms(0, n)
    assert rel(sa, sb) <= TOL, rel(sa, sb)
    assert g.current_step == o.current_step == n + 1


@pytest.mark.parametrize("name", ["iso1d", "ti3d_cg4", "fluid3d_mass3d_couple3d"])
def test_fine_grained_loop_bodies(ax3d_lib, name):
    """Domain's loop bodies one at a time (update, source, stiff, couple, record)."""
    spec, g, o, _ = _pair(name, stf_len=8)
    su, fu = synth.random_fields(spec, seed=9, scale=1e-5)
    for d in (g, o):
        d.set("displ", "solid", su)
        if d.nfluid:
            d.set("displ", "fluid", fu)
        for t in range(3):
            d.update_newmark()
            d.apply_source(t)
            d.compute_stiff()
            d.couple_solid_fluid()
            d.record(t)
    for which in ("displ", "veloc", "accel", "stiff"):
        assert rel(g.get(which, "solid"), o.get(which, "solid")) <= TOL, which


def test_kahan_closer_to_fp64(ax3d_lib):
    """Compensated Newmark: over 2,000 steps the compensated FP32 run ends strictly closer to
    the FP64 oracle than the plain FP32 run (displacement and seismograms), both within 1e-5."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    n = 2000
    od = OracleDomain(synth.annulus_domain(nu=2, stf_len=n), double=True)
    od.step(n)
    ref_u, ref_s = od.get("displ"), od.seismograms(0, n)
    err = {}
    for kahan in (False, True):
        g = Ax3dDomain(synth.annulus_domain(nu=2, stf_len=n, kahan=kahan))
        g.step(n)
        err[kahan] = (rel(g.get("displ"), ref_u), rel(g.seismograms(0, n), ref_s))
        g.close()
    for k in (0, 1):
        assert err[True][k] < err[False][k], err
        assert err[False][k] <= TOL, err


def test_unstable_is_reported(ax3d_lib):
    from axisem3d_gb300.capi import Ax3dDomain, Ax3dError
    spec = synth.annulus_domain(nu=1, stf_len=8, stability_interval=2)
    g = Ax3dDomain(spec)
    su, _ = synth.random_fields(spec)
    su[0] = np.nan
    g.set("displ", "solid", su)
    with pytest.raises(Ax3dError) as ei:
        g.step(4)
    assert ei.value.code == 4


def test_wisdom_learning_matches_oracle(ax3d_lib):
    """Nu wisdom learned during the time loop (every 5 steps), GPU vs oracle."""
    spec, g, o, _ = _pair("ti3d_cg4", stf_len=30)
    su, _ = synth.random_fields(spec, seed=13, scale=1e-6, decay=2.5)
    for d in (g, o):
        d.set("displ", "solid", su)
        d.set_wisdom_learning(5, 1e-2)
        d.step(30)
    wg, wo = g.get_wisdom(), o.get_wisdom()
    assert wg.shape == wo.shape == (spec.n_points,)
    assert (np.abs(wg - wo) <= 1).all() and (wg != wo).mean() <= 0.01


@pytest.mark.parametrize("att,in3d", [(ATT_CG4, True), (ATT_FULL, True), (ATT_CG4, False), (ATT_FULL, False)])
def test_element_benchmark_matches_oracle(ax3d_lib, att, in3d):
    """The element-stiffness benchmark's domain over its whole Nu range 8-256 (elements that
    own their points, so they assemble directly into the point stiffness): ten of the 20
    elements have rings above nr 186, which run on thread-block clusters, the rest on single
    CTAs.  compute_stiff (read-modify-write of the point stiffness), then three steps (the
    write-only stiffness rows of ax3d_step), TI moduli, CG4 or full-grid SLS; with 3-D
    material (physical-space path) and with 1-D material (Fourier-space path)."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300 import workloads as W
    from axisem3d_gb300.capi import Ax3dDomain
    spec = W.element_benchmark(n_elem=20, seed=9, att=att, nu_min=8, nu_max=256, in3d=in3d)
    nr = spec.element_nr()
    assert (nr > 186).sum() >= 6 and nr.max() > 450 and nr.min() < 32
    u0 = W.benchmark_displacement(spec, seed=8)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    for d in (g, o):
        d.set("displ", "solid", u0)
        d.compute_stiff()
    assert rel(g.get("stiff", "solid"), o.get("stiff", "solid")) <= TOL
    for d in (g, o):
        d.step(3)
    for which in ("displ", "veloc", "accel"):
        assert rel(g.get(which, "solid"), o.get(which, "solid")) <= TOL, which
    # element by element, so that no small ring hides behind the large ones
    so, _ = spec.point_offsets()
    a, b = g.get("accel", "solid"), o.get("accel", "solid")
    for e in range(spec.n_elements):
        p0, p1 = spec.e_pts[e, 0], spec.e_pts[e, 24]
        lo, hi = so[p0], so[p1] + 3 * (int(spec.p_nr[p1]) // 2 + 1)
        assert rel(a[lo:hi], b[lo:hi]) <= TOL, (e, int(nr[e]))


def test_surface_recorder_matches_oracle(ax3d_lib):
    """Whole-surface recording every 3 steps of a time loop (SurfaceRecorder), GPU vs oracle."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    spec = synth.annulus_domain(in3d=True, mat=MAT_TISO, att=ATT_CG4, nu_random=True, nu_max=9, stf_len=13,
                                surface_interval=3)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    su, _ = synth.random_fields(spec, seed=17, scale=1e-6)
    for d in (g, o):
        d.set("displ", "solid", su)
        d.step(13)
    for a, b in zip(g.surface(0, 5), o.surface(0, 5)):
        assert rel(a, b) <= TOL


@pytest.mark.parametrize("ocean", ["1d", "3d"])
def test_ocean_load_newmark_matches_oracle(ax3d_lib, ocean):
    """One Newmark update from a random stiffness: ocean points take MassOcean1D (row-local)
    or MassOcean3D (per-sample normal projection) on the GPU as in the oracle."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    spec = synth.annulus_domain(seed=6, n_theta=3, n_r=2, nu_random=True, nu_max=9, source=False,
                                n_receivers=0, ocean=ocean)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    su, _ = synth.random_fields(spec, seed=8)
    for d in (g, o):
        d.set("stiff", "solid", su)
        d.update_newmark()
    a, b = g.get("accel", "solid"), o.get("accel", "solid")
    assert rel(a, b) <= TOL, rel(a, b)
    so, _ = spec.point_offsets()
    rows = np.concatenate([np.arange(so[p], so[p] + 3 * (spec.p_nr[p] // 2 + 1)) for p in spec.oc_pt])
    assert rel(a[rows], b[rows]) <= TOL


@pytest.mark.parametrize("name", ["iso1d_fluid_mixednu", "ti3d_cg4", "aniso3d_full"])
def test_strain_curl_receivers_match_oracle(ax3d_lib, name):
    """dump_strain / dump_curl receivers (SolidElement::computeStrain / computeCurl,
    PointwiseRecorder) recorded every step of a time loop, GPU vs oracle."""
    n = 12
    spec, g, o, _ = _pair(name, stf_len=n, n_receivers=9, dumps=True)
    su, fu = synth.random_fields(spec, seed=9, scale=1e-6)
    for d in (g, o):
        d.set("displ", "solid", su)
        if d.nfluid:
            d.set("displ", "fluid", fu)
        d.step(n)
    for which in ("strain", "curl"):
        a, b = g.strain_curl(which, 0, n), o.strain_curl(which, 0, n)
        assert a.shape == b.shape and a.shape[1] > 0
        assert rel(a, b) <= TOL, (which, rel(a, b))


def test_streamed_field_transfers_match_synchronous(ax3d_lib):
    """ax3d_set_field_async / ax3d_get_field_async / ax3d_sync_fields: a loop that queues the
    next input and reads the last result back while steps run gives, step for step, the
    results of synchronous set / step / get calls."""
    from axisem3d_gb300.capi import Ax3dDomain
    spec = synth.annulus_domain(**CASES["ti3d_cg4"], stf_len=8)
    a, b = Ax3dDomain(spec), Ax3dDomain(spec)
    ins = [synth.random_fields(spec, seed=40 + k, scale=1e-6)[0].astype(np.complex64) for k in range(5)]
    want = []
    for x in ins:
        a.set("displ", "solid", x)
        a.step(1)
        want.append(a.get("displ", "solid").copy())
    outs = [np.zeros(b.nsolid, np.complex64) for _ in ins]
    b.set_async("displ", "solid", ins[0])
    for k in range(len(ins)):
        if k + 1 < len(ins):
            b.set_async("displ", "solid", ins[k + 1])
        b.step(1)
        b.get_async("displ", "solid", outs[k])
    b.sync_fields()
    for k in range(len(ins)):
        np.testing.assert_array_equal(outs[k], want[k])
    # the live displacement buffer switched with every queued input: plain calls and plain
    # steps continue from the last result
    np.testing.assert_array_equal(b.get("displ", "solid"), want[-1])
    a.step(2)
    b.step(2)
    for which in ("displ", "veloc", "accel"):
        np.testing.assert_array_equal(b.get(which, "solid"), a.get(which, "solid"))
    b.reset()
    a.reset()
    a.step(1)
    b.step(1)
    np.testing.assert_array_equal(b.get("displ", "solid"), a.get("displ", "solid"))
    # other fields go through the staging buffers
    v = synth.random_fields(spec, seed=77, scale=1e-6)[0].astype(np.complex64)
    a.set("veloc", "solid", v)
    a.step(1)
    b.set_async("veloc", "solid", v)
    b.step(1)
    got = np.zeros(b.nsolid, np.complex64)
    b.get_async("veloc", "solid", got)
    b.sync_fields()
    np.testing.assert_array_equal(got, a.get("veloc", "solid"))


def test_autotuned_schedule_keeps_results(ax3d_lib):
    """ax3d_autotune times bucket schedules on the domain's own elements, leaves the fields as
    they were, and the chosen schedule gives the oracle's results; a second domain of the
    same shape takes the cached choice."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300 import workloads as W
    from axisem3d_gb300.capi import Ax3dDomain
    spec = W.element_benchmark(n_elem=20, seed=9, att=ATT_CG4)
    u0 = W.benchmark_displacement(spec, seed=8)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    for d in (g, o):
        d.set("displ", "solid", u0)
        d.compute_stiff()
    before = {w: g.get(w, "solid").copy() for w in ("displ", "stiff")}
    rep = g.autotune(1)
    assert rep.startswith("chose ratio"), rep
    for w in ("displ", "stiff"):
        np.testing.assert_array_equal(g.get(w, "solid"), before[w])
    for d in (g, o):
        d.step(3)
    for which in ("displ", "veloc", "accel"):
        assert rel(g.get(which, "solid"), o.get(which, "solid")) <= TOL, which
    g2 = Ax3dDomain(spec)
    assert g2.autotune(1).startswith("cached")


@pytest.mark.parametrize("policy,merge", [(1, False), (2, False), (0, True), (2, True), (3, False), (3, True),
                                          (4, False), (4, True)])
def test_schedule_policies_match_oracle(ax3d_lib, policy, merge):
    """The benchmark's domain (Nu 8-256) under the other bucket schedules: policy 1 (256-thread
    CTAs with an SM's whole shared memory), policy 2 (512-thread CTAs above the rings that
    fit two CTAs per SM, clusters of 512-thread CTAs for the largest), policy 3 (as 2, with
    128-thread CTAs four per SM for the short rings) and policy 4 (as 3, with 64-thread CTAs
    eight per SM for the shortest), each also with the buckets of one launch shape merged
    into one launch; compute_stiff and three steps against the oracle."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300 import workloads as W
    from axisem3d_gb300.capi import Ax3dDomain
    spec = W.element_benchmark(n_elem=20, seed=9, att=ATT_CG4)
    u0 = W.benchmark_displacement(spec, seed=8)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    g.set_schedule(1.12, policy, 2, merge)
    for d in (g, o):
        d.set("displ", "solid", u0)
        d.compute_stiff()
    assert rel(g.get("stiff", "solid"), o.get("stiff", "solid")) <= TOL
    for d in (g, o):
        d.step(3)
    for which in ("displ", "veloc", "accel"):
        assert rel(g.get(which, "solid"), o.get(which, "solid")) <= TOL, which
