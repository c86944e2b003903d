"""Inputs/outputs boundary: parfiles, Exodus (NetCDF classic) mesh, CMTSOLUTION, STATIONS,
station NetCDF output, and the full time loop GPU vs oracle on a generated mesh."""
import numpy as np
import pytest

from axisem3d_gb300 import netcdf as NC
from axisem3d_gb300 import solver

SMALL_MESH = dict(n_theta=16, h_mantle=600e3, h_core=700e3, r_c=1500e3)


@pytest.fixture(scope="module")
def small_inputs(tmp_path_factory):
    d = tmp_path_factory.mktemp("c0") / "input"
    return solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=200, hdur=20.0, n_stations=6, seed=3)


def test_netcdf_roundtrip(tmp_path):
    ds = NC.Dataset()
    ds.add_dim("n", 4)
    ds.add_dim("m", 3)
    a = np.arange(12, dtype=np.float32).reshape(4, 3)
    ds.add_var("a", ("n", "m"), a, attrs={"latitude": 12.5, "units": "m"})
    ds.add_var("i", ("n",), np.array([1, 2, 3, 4]), dtype=np.int32)
    ds.add_strings("names", "num_names", "len_string", ["t0", "solid_fluid_boundary"])
    NC.write(tmp_path / "x.nc", ds)
    back = NC.read(tmp_path / "x.nc")
    np.testing.assert_array_equal(back["a"], a)
    np.testing.assert_array_equal(back["i"], [1, 2, 3, 4])
    assert back.strings("names") == ["t0", "solid_fluid_boundary"]
    assert float(back.variables["a"].attrs["latitude"][0]) == 12.5
    assert (tmp_path / "x.nc").read_bytes()[:4] == b"CDF\x02"


def test_netcdf_bad_hdf5_raises(tmp_path):
    """NetCDF-4 / HDF5 files go to the HDF5 reader, which names what it cannot read."""
    (tmp_path / "h.e").write_bytes(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    with pytest.raises(ValueError, match="HDF5"):
        NC.read(tmp_path / "h.e")
    (tmp_path / "g.e").write_bytes(b"\x89HDF\r\n\x1a\n\x02" + b"\0" * 64)
    with pytest.raises(ValueError, match="superblock version 2"):
        NC.read(tmp_path / "g.e")


def _spec_arrays_equal(a, b):
    return [k for k, v in vars(a).items() if isinstance(v, np.ndarray)
            and (v.shape != getattr(b, k).shape or not np.array_equal(v, getattr(b, k)))]


def test_rotated_axial_elements_read_back(tmp_path):
    """A mesh whose axial elements store the axis on side 0, 1 or 2 (ExodusModel::
    formAuxiliary rotates them to side 3, with their side sets and nodal values) gives the
    same domain as the mesh written with the axis on side 3."""
    specs = []
    for i, rot in enumerate((False, True)):
        d = solver.write_inputs(tmp_path / f"r{i}", mesh_kw=dict(SMALL_MESH, rotate_axis=rot), steps=10, nu=3,
                                attenuation=True)
        specs.append(solver.Simulation(d).build())
    ds = NC.read(tmp_path / "r1" / "mesh.e")
    axis = np.asarray(ds["side_ss1"]) - 1
    assert set(axis.tolist()) == {0, 1, 2}
    assert _spec_arrays_equal(specs[0], specs[1]) == []


def test_element_orientation_invariance(tmp_path):
    """The same Earth with every element stored in another node order (curved sides 0, 1, 2
    and 3, axial elements with the axis on sides 0-2): the mapping, Jacobians, integral
    factors and normals follow the orientation (Quad::Quad's curved-side search,
    SphericalMapping / SemiSphericalMapping) and the FP64 oracle's seismograms agree to
    rounding."""
    from oracle.oracle_py import OracleDomain
    seis, cos = [], []
    for i, kw in enumerate(({}, dict(rotate_all=True, rotate_axis=True))):
        d = solver.write_inputs(tmp_path / f"o{i}", mesh_kw=dict(SMALL_MESH, **kw), steps=100, hdur=20.0,
                                n_stations=6, seed=3, nu=3, attenuation=True)
        sim = solver.Simulation(d)
        spec = sim.build()
        cos.append(set(np.unique(sim.co).tolist()))
        o = OracleDomain(spec, double=True)
        o.step(100)
        seis.append(o.seismograms(0, 100))
    assert cos[1] == {-1, 0, 1, 2, 3} and 1 not in cos[0]
    assert np.linalg.norm(seis[1] - seis[0]) <= 1e-12 * np.linalg.norm(seis[0])


def test_transversely_isotropic_mesh(tmp_path):
    """A mesh with VPV / VPH / VSV / VSH / ETA (Material::Material, Material::createElastic):
    TransverselyIsotropic1D moduli A = rho vph^2, C = rho vpv^2, L = rho vsv^2, N = rho vsh^2
    (times iFact), F = eta (A - 2 L) where the mesh is anisotropic, Isotropic1D elsewhere with
    the moduli of the isotropic mesh; 3-D models on it are refused."""
    from axisem3d_gb300.spec import MAT_ISO, MAT_TISO
    specs, sims = [], []
    for i, ti in enumerate((False, True)):
        d = solver.write_inputs(tmp_path / f"t{i}", mesh_kw=dict(SMALL_MESH, ti=ti), steps=10, nu=3)
        sims.append(solver.Simulation(d))
        specs.append(sims[-1].build())
    a, b = specs
    assert (b.e_mat == MAT_TISO).sum() > 0 and (a.e_mat == MAT_TISO).sum() == 0
    ends = lambda sp: np.append(sp.e_mofs[1:], len(sp.e_mod))
    m = sims[1]._gll_material(sims[1].ex, sims[1].axial_e)
    for e in range(b.n_elements):
        mb = b.e_mod[b.e_mofs[e]:ends(b)[e]]
        if b.e_mat[e] == MAT_TISO:
            rho, vpv, vph, vsv, vsh, eta = (m[k][e] for k in ("RHO", "VPV", "VPH", "VSV", "VSH", "ETA"))
            A, C, L, N = rho * vph ** 2, rho * vpv ** 2, rho * vsv ** 2, rho * vsh ** 2
            ratio = mb.reshape(5, 25) / np.stack([A, C, eta * (A - 2 * L), L, N])  # = iFact at every point
            np.testing.assert_allclose(ratio, np.broadcast_to(ratio[3], (5, 25)), rtol=1e-5)
            assert (eta < 1).any() and not np.allclose(vph, vpv)
        else:
            np.testing.assert_array_equal(mb, a.e_mod[a.e_mofs[e]:ends(a)[e]])
    d = solver.write_inputs(tmp_path / "t3", mesh_kw=dict(SMALL_MESH, ti=True), steps=10, nu=3,
                            models3d=("gaussian_random$VS$Ref1D$0.04$500$200$7",))
    with pytest.raises(NotImplementedError, match="transversely"):
        solver.Simulation(d).build()


def test_hdf5_mesh_of_the_reference():
    """The reference's own template mesh (NetCDF-4 / HDF5, PREM anisotropic with one crust,
    50 s) and template inputs, when AX3D_REFERENCE_INPUT names a copy of that input folder:
    the mesh reads (chunked, compressed datasets), and the case builds as it is: TI upper
    mantle, attenuation, rotated axial elements, geographic ellipticity (flattened station
    and source latitudes), the reference's time step, and 40 stable oracle steps."""
    import os
    import shutil
    src = os.environ.get("AX3D_REFERENCE_INPUT")
    if not src:
        pytest.skip("AX3D_REFERENCE_INPUT is not set")
    from pathlib import Path
    from axisem3d_gb300.spec import MAT_TISO
    ds = NC.read(Path(src) / "AxiSEM_prem_ani_one_crust_50.e")
    assert ds["connect1"].shape == (2016, 4) and ds["coordx"].shape == (2115,)
    assert ds.strings("name_glo_var")[6] == "radius" and float(ds["vals_glo_var"][0, 6]) == 6371e3
    assert "crdsys = spherical" in ds.strings("info_records")
    names = ds.strings("name_elem_var")
    vpv = ds[f"vals_elem_var{names.index('VPV_0') + 1}eb1"]
    assert abs(float(vpv.max()) - 13716.622269026377) < 1e-6
    import tempfile
    d = Path(tempfile.mkdtemp()) / "input"
    shutil.copytree(src, d)
    for f in d.iterdir():
        f.chmod(0o644)
    sim = solver.Simulation(d)
    spec = sim.build()
    assert spec.n_elements == 2016 and (spec.e_mat == MAT_TISO).sum() == 256
    assert np.isfinite(spec.e_geo).all() and set(np.unique(sim.co).tolist()) == {-1, 0, 2, 3}
    assert sim.ellipticity_mode() == "geographic" and sim.geo_.flattening(6371e3) == 1 / 299.8
    # Quad::getDeltaT: the mesh's dt (courant x shortest side / vp, 2.524 s in the crust)
    # scaled by the closest GLL distance over the shortest side
    assert abs(spec.dt - 0.43585) < 1e-4 and abs(float(sim.ex.dt.min()) - 2.52414) < 1e-4
    from oracle.oracle_py import OracleDomain
    o = OracleDomain(spec)
    o.step(40)
    u = o.get("displ", "solid")
    assert np.isfinite(u).all() and 1e-4 < np.abs(u).max() < 1.0


def test_parameters_parsing(small_inputs):
    par = solver.Parameters(small_inputs)
    assert par.get("NU_CONST", int) == 2
    assert par.get("ATTENUATION", bool) is False
    assert par.get("SOURCE_TIME_FUNCTION") == "gauss"
    with pytest.raises(KeyError):
        par.get("NU_EMP_REF")


def test_missing_parfile_raises(tmp_path):
    with pytest.raises(FileNotFoundError, match="inparam"):
        solver.Parameters(tmp_path)


def test_mesh_and_domain_build(small_inputs):
    sim = solver.Simulation(small_inputs)
    spec = sim.build()
    ex = sim.ex
    # every axial element has its axis on side 3, fluid core, CMB coupling points exist
    assert (ex.side["t0"][ex.side["t0"] >= 0] == 3).all()
    assert ex.fluid.any() and (~ex.fluid).any()
    assert (spec.p_kind == 2).sum() > 0
    # 2 pi sum of integral factors = volume of the Earth (ifact carries s ds dz)
    assert spec.stf.size == 200 and len(spec.r_elem) == 6
    assert spec.sources and spec.sources[0][1].shape == (25, 3, 3)


def test_oracle_run_and_netcdf_output(small_inputs, tmp_path):
    from oracle.oracle_py import OracleDomain
    sim = solver.Simulation(small_inputs, output_dir=tmp_path)
    spec = sim.build()
    o = OracleDomain(spec)
    o.step(200)
    rtz = sim.rotate(o.seismograms(0, 200))
    assert np.isfinite(rtz).all() and np.abs(rtz).max() > 0
    p = sim.write_netcdf(rtz)
    ds = NC.read(p)
    assert ds["time_points"].shape == (200,)
    np.testing.assert_allclose(ds["SY.S001.RTZ"], rtz[:, 1], rtol=1e-6, atol=1e-30)


@pytest.mark.gpu
def test_full_solver_gpu_matches_oracle(small_inputs, ax3d_lib):
    """Seismograms of the whole loop (source, fluid core, solid-fluid coupling, axis, receivers)."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    sim = solver.Simulation(small_inputs)
    spec = sim.build()
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    g.step(200)
    o.step(200)
    a, b = g.seismograms(0, 200), o.seismograms(0, 200)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    for which in ("displ", "veloc"):
        x, y = g.get(which, "solid"), o.get(which, "solid")
        assert np.linalg.norm(x - y) <= 1e-5 * np.linalg.norm(y)


@pytest.mark.gpu
def test_transversely_isotropic_mesh_gpu_matches_oracle(tmp_path_factory, ax3d_lib):
    """A transversely isotropic mesh (TI top 220 km of the mantle) with its axial elements
    stored rotated, attenuation (CG4) on and Nu = 3: the GPU pre-loop's moduli equal the
    numpy pre-loop's, 200 steps of GPU seismograms match the FP32 oracle within 1e-5, and
    the GPU fields are as close to the FP64 oracle's as the FP32 oracle's are (the two FP32
    runs differ in operation order, ~1e-5 of the field after 200 attenuated TI steps)."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    from axisem3d_gb300.spec import MAT_TISO
    d = tmp_path_factory.mktemp("ti") / "input"
    solver.write_inputs(d, mesh_kw=dict(SMALL_MESH, ti=True, rotate_axis=True), steps=200, hdur=20.0,
                        n_stations=6, seed=3, nu=3, attenuation=True)
    host = solver.Simulation(d).build(preloop="host")
    spec = solver.Simulation(d).build(preloop="gpu")
    assert (spec.e_mat == MAT_TISO).sum() > 0
    np.testing.assert_array_equal(spec.e_mofs, host.e_mofs)
    np.testing.assert_allclose(spec.e_mod, host.e_mod, rtol=2e-6, atol=0)
    np.testing.assert_allclose(spec.e_attm, host.e_attm, rtol=2e-6, atol=1e-30)
    g, o, od = Ax3dDomain(spec), OracleDomain(spec), OracleDomain(spec, double=True)
    for dom in (g, o, od):
        dom.step(200)
    a, b = g.seismograms(0, 200), o.seismograms(0, 200)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
    for which in ("displ", "veloc"):
        x, y, z = g.get(which, "solid"), o.get(which, "solid"), od.get(which, "solid")
        assert rel(x, y) <= 3e-5, which
        assert rel(x, z) <= 2 * rel(y, z) + 1e-6, which


@pytest.mark.gpu
def test_rotated_elements_gpu_preloop_and_run(tmp_path_factory, ax3d_lib):
    """Every element stored in another node order (curved sides 0-3): the GPU geometry and
    mass pre-loop equals the numpy one, and 100 GPU steps match the oracle."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    d = tmp_path_factory.mktemp("rot") / "input"
    solver.write_inputs(d, mesh_kw=dict(SMALL_MESH, rotate_all=True, rotate_axis=True), steps=100, hdur=20.0,
                        n_stations=6, seed=3, nu=3, attenuation=True)
    host = solver.Simulation(d).build(preloop="host")
    spec = solver.Simulation(d).build(preloop="gpu")
    np.testing.assert_allclose(spec.e_geo, host.e_geo, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(spec.p_ms, host.p_ms, rtol=1e-6)
    np.testing.assert_allclose(spec.e_mod, host.e_mod, rtol=2e-6, atol=0)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    g.step(100)
    o.step(100)
    a, b = g.seismograms(0, 100), o.seismograms(0, 100)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)


@pytest.mark.gpu
def test_config0_at_size_gpu_matches_oracle(tmp_path_factory, ax3d_lib, capsys):
    """The small configuration at its full size: the default seeded half disk (5,856 quads,
    Nu = 2, fluid core), a moment tensor at 100 km, Gaussian STF of 50 s half duration, 2,000
    steps at the CFL dt, 20 stations.  GPU seismograms against the FP32 oracle (relative L2
    <= 1e-5, over all and per energetic trace); every energetic trace's error against the
    FP64 oracle is stated and bounded; the compensated (Kahan) Newmark run is closer to FP64
    than the plain FP32 run.  (Within 2,000 steps = 560 s the waves reach only the nearest
    stations; traces below 1e-3 of the largest are numerical noise around zero, so their
    relative error says nothing and they are left out of the per-trace figures.)"""
    import multiprocessing as mp
    from oracle.oracle_py import seismograms_of_inputs
    from axisem3d_gb300.capi import Ax3dDomain
    n = 2000
    d = tmp_path_factory.mktemp("cfg0") / "input"
    solver.write_inputs(d)  # the defaults are the configuration
    sim = solver.Simulation(d)
    spec = sim.build()
    assert spec.n_elements == 5856 and len(spec.r_elem) == 20 and sim.nsteps == n
    with mp.get_context("spawn").Pool(2) as pool:
        jobs = [pool.apply_async(seismograms_of_inputs, (str(d), n, dbl)) for dbl in (False, True)]
        g = Ax3dDomain(spec)
        g.step(n)
        sg = g.seismograms(0, n)
        g.close()
        gk = Ax3dDomain(sim.build(kahan=True))
        gk.step(n)
        sk = gk.seismograms(0, n)
        gk.close()
        s32, s64 = (j.get(timeout=1800) for j in jobs)
    nrm = lambda x: np.linalg.norm(x, axis=0)
    big = nrm(s64) > 1e-3 * nrm(s64).max()
    assert big.sum() >= 6
    rel = lambda a, b: np.where(big, nrm(a - b) / np.where(big, nrm(b), 1.0), 0.0)
    rel32 = rel(sg, s32)
    assert np.linalg.norm(sg - s32) <= 1e-5 * np.linalg.norm(s32)
    assert rel32[big].max() <= 1e-5, rel32[big].max()
    rel64, relk = rel(sg, s64), rel(sk, s64)
    tot, totk = (np.linalg.norm(x - s64) / np.linalg.norm(s64) for x in (sg, sk))
    with capsys.disabled():
        print(f"\nconfig 0, {n} steps: GPU vs FP64 oracle, relative L2 over all traces {tot:.3e} "
              f"(compensated {totk:.3e}); per energetic trace [receiver, component]:")
        for (r, c) in zip(*np.nonzero(big)):
            print(f"  rec {r:2d} comp {c}: plain {rel64[r, c]:.3e}  compensated {relk[r, c]:.3e}")
    assert rel64[big].max() <= 1e-5 and relk[big].max() <= 1e-5
    assert totk < tot, (totk, tot)


def _two_members(tmp_path_factory):
    specs = []
    for i, (depth, seed) in enumerate(((100.0, 3), (400.0, 5))):
        d = tmp_path_factory.mktemp(f"ens{i}") / "input"
        solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=120, hdur=20.0, n_stations=4, seed=seed, depth_km=depth)
        sim = solver.Simulation(d)
        specs.append(sim.build())
    dt = min(s.dt for s in specs)
    for s in specs:  # one dt and one STF for the ensemble
        s.dt = dt
        s.stf = specs[0].stf
    return specs


def test_ensemble_members_match_separate_runs(tmp_path_factory):
    """Concatenated members evolve exactly as they do alone (oracle)."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300 import ensemble
    specs = _two_members(tmp_path_factory)
    spec, info = ensemble.concat(specs)
    o = OracleDomain(spec)
    o.step(60)
    parts = ensemble.split_seismograms(o.seismograms(0, 60), info)
    for s, part in zip(specs, parts):
        a = OracleDomain(s)
        a.step(60)
        np.testing.assert_array_equal(part, a.seismograms(0, 60))


@pytest.mark.gpu
def test_ensemble_gpu_graph_matches_oracle(tmp_path_factory, ax3d_lib):
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300 import ensemble
    from axisem3d_gb300.capi import Ax3dDomain
    specs = _two_members(tmp_path_factory)
    spec, info = ensemble.concat(specs)
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    g.step(50)  # CUDA-graph path, in two calls
    g.step(70)
    o.step(120)
    a, b = g.seismograms(0, 120), o.seismograms(0, 120)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)


MODELS_3D = ("bubble$RHO$Ref1D$0.05$500$2891$20$40$true$true",   # straddles the CMB
             "bubble$VP$Ref3D$-0.05$500$2891$20$40$true$true",
             "gaussian_random$VS$Ref1D$0.04$500$200$7")


@pytest.fixture(scope="module")
def inputs_3d(tmp_path_factory):
    d = tmp_path_factory.mktemp("c3d") / "input"
    return solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=120, hdur=20.0, n_stations=6, seed=3, nu=4,
                               models3d=MODELS_3D)


def test_volumetric_3d_build(inputs_3d):
    """3-D elements, Mass3D points (solid and fluid) and 3-D solid-fluid coupling appear; a
    gaussian_random model acts on solid elements only (no fluid flag)."""
    sim = solver.Simulation(inputs_3d)
    spec = sim.build()
    assert spec.e_in3d[~sim.fluid].all()
    assert spec.e_in3d[sim.fluid].any() and not spec.e_in3d[sim.fluid].all()
    assert (spec.p_mslen > 1).any() and (spec.p_mflen > 1).any() and (spec.p_sflen > 1).any()
    nr = spec.element_nr()
    sizes = np.diff(np.append(spec.e_mofs, len(spec.e_mod)))
    # moduli rows: [2][nr][25] solid isotropic, [nr][25] fluid (3-D) or [25] (1-D)
    want = np.where(sim.fluid, np.where(spec.e_in3d > 0, nr, 1) * 25, 2 * nr * 25)
    assert (sizes == want).all()


def test_volumetric_3d_models_unit():
    from axisem3d_gb300 import model3d as M3D
    R = 6371e3
    b = M3D.Bubble("VS Ref1D 0.1 100 500 30 60 true".split(), (0.0, 0.0), R)
    v, inr = b.evaluate(b.center[None, :])
    assert inr[0] and v[0] == pytest.approx(0.1)
    far = b.center * 0.5
    assert not b.evaluate(far[None, :])[1][0]
    g = M3D.GaussianRandom("VP Ref1D 0.04 500 200 1".split(), R)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((20000, 3))
    x = x / np.linalg.norm(x, axis=1, keepdims=True) * rng.uniform(3.5e6, 6.3e6, (20000, 1))
    val = g.evaluate(x)[0]
    assert abs(val.mean()) < 0.01 and 0.02 < val.std() < 0.06
    with pytest.raises(ValueError):
        M3D.Bubble("VQ Ref1D 0.1 100 500 30 60".split(), (0.0, 0.0), R)
    ring = np.array([1.0, 2.0, 3.0])
    np.testing.assert_allclose(M3D.linear_resampling(6, ring), [1.0, 1.5, 2.0, 2.5, 3.0, 2.0])


class _FieldModel:
    """A volumetric model for apply_models: a perturbation and a range that are functions of
    the point (so any chunking of the points sees the same values)."""

    def __init__(self, prop, ref, fluid, frac, seed):
        self.prop, self.ref, self.fluid, self.frac, self.seed = prop, ref, fluid, frac, seed

    def evaluate(self, xyz):
        x, y, z = xyz[..., 0], xyz[..., 1], xyz[..., 2]
        val = 0.05 * np.sin(1e-6 * (x + 2 * y + 3 * z) + self.seed) + (3000.0 if self.ref == 0 else 0.0)
        inr = 0.5 * (np.sin(1e-5 * (1.3 * x + 0.7 * y - z) + 2 * self.seed) + 1) < self.frac
        return val, inr


def _apply_models_dense(models, props1d, crds, nr, fluid):
    """Material::addVolumetric3D on dense (n, nr, 25) float64 copies of every property, model
    after model (Volumetric3D reference kinds: absolute, Ref1D, Ref3D, reference difference)."""
    n = len(crds)
    phi = 2 * np.pi * np.arange(nr) / nr
    s, z = crds[..., 0], crds[..., 1]
    xyz = np.stack([s[:, None, :] * np.cos(phi)[None, :, None], s[:, None, :] * np.sin(phi)[None, :, None],
                    np.broadcast_to(z[:, None, :], (n, nr, 25))], -1)
    cur = {k: np.repeat(v[:, None, :], nr, 1).astype(float) for k, v in props1d.items()}
    touched = np.zeros(n, bool)
    for m in models:
        val, inr = m.evaluate(xyz)
        if not m.fluid:
            inr = inr & ~fluid[:, None, None]
        touched |= inr.any((1, 2))
        x1, x = props1d[m.prop][:, None, :], cur[m.prop]
        new = {0: np.broadcast_to(val, x.shape), 1: x1 * (1.0 + val), 2: x * (1.0 + val),
               3: (x - x1) * (1.0 + val) + x1}[m.ref]
        cur[m.prop] = np.where(inr, new, x)
    return {k: v.astype(np.float32) for k, v in cur.items()}, touched


@pytest.mark.parametrize("n,nr", [(7, 5), (31, 13), (4000, 30)])
def test_apply_models_matches_dense_restatement(n, nr):
    """model3d.apply_models keeps a property no model changes as its 1-D row (a read-only
    broadcast view), applies perturbations in place and works in chunks of ~2M samples; its
    values equal, bit for bit, the dense restatement above for every reference kind, models
    with and without fluid, partial ranges and (at n = 4000, nr = 30) chunks."""
    from axisem3d_gb300 import model3d as M3D
    rng = np.random.default_rng(n)
    props = {k: rng.uniform(1000.0, 9000.0, (n, 25)) for k in ("VP", "VS", "RHO")}
    crds = rng.uniform(0.0, 6e6, (n, 25, 2))
    fluid = rng.random(n) < 0.3
    for trial in range(8):
        models = [_FieldModel(str(rng.choice(["VP", "VS", "RHO"])), int(rng.integers(0, 4)), bool(rng.random() < 0.5),
                              float(rng.choice([0.0, 0.3, 1.0])), 10 * trial + i) for i in range(int(rng.integers(1, 4)))]
        got, t_got = M3D.apply_models(models, props, crds, nr, fluid)
        want, t_want = _apply_models_dense(models, props, crds, nr, fluid)
        np.testing.assert_array_equal(t_got, t_want)
        for k in want:
            assert got[k].shape == want[k].shape and got[k].dtype == np.float32
            np.testing.assert_array_equal(got[k], want[k])
            if not any(m.prop == k for m in models):
                assert got[k].strides[1] == 0  # left as the broadcast 1-D row
        assert solver._varies(got["RHO"]).tolist() == (want["RHO"].max(1) != want["RHO"].min(1)).any(1).tolist()


def test_point_numbering_matches_unique_rows(small_inputs):
    """The unique-point numbering of the build (one lexsort of the rounded coordinates)
    equals np.unique's row order, so the points keep their numbers."""
    sim = solver.Simulation(small_inputs)
    sim.build()
    key = np.round(sim.crds.reshape(-1, 2) / 1e-3).astype(np.int64)
    _, inv = np.unique(key, axis=0, return_inverse=True)
    np.testing.assert_array_equal(sim.e_pts.ravel(), inv.ravel())


def _normal_pointwise(nodes, crds, jac0, axial, co, e, side):
    """Quad::computeNormal (Quad.cpp:661-715) point by point: (local index, normal) of the
    five points on side `side` of element e."""
    from axisem3d_gb300 import spectral as S
    wg, wjw, xj = S.gll()[1], S.glj()[1], S.glj()[0]
    n0, n1 = nodes[e][:, side], nodes[e][:, (side + 1) % 4]
    r0, t0 = np.hypot(*n0), solver._colat(*n0)
    r1, t1 = np.hypot(*n1), solver._colat(*n1)
    rsf = 0.5 * (r0 + r1)
    h_r_dt, h_r2_dt = 0.5 * rsf * abs(t1 - t0), 0.5 * rsf * rsf * abs(t1 - t0)
    out = []
    for ip in range(5):
        for jp in range(5):
            if not ((side == 0 and jp == 0) or (side == 1 and ip == 4) or (side == 2 and jp == 4) or
                    (side == 3 and ip == 0)):
                continue
            k = ip * 5 + jp
            rr = np.hypot(*crds[e, k])
            sint, cost = crds[e, k, 0] / rr, crds[e, k, 1] / rr
            nvec = np.array([sint, 0.0, cost])
            wsf = (wjw if axial[e] else wg)[ip] if side in (0, 2) else wg[jp]
            if axial[e]:
                nvec *= wsf * jac0[e, ip, jp] * h_r_dt if ip == 0 else wsf / (1 + xj[ip]) * sint * h_r2_dt
            else:
                nvec *= wsf * sint * h_r2_dt
            out.append((k, -nvec if side != co[e] else nvec))
    return out


def test_boundary_normals_match_pointwise(small_inputs):
    """solver.boundary_normals (all boundary sides at once) equals the point-by-point
    Quad::computeNormal on the solid-fluid and the surface sides of the coarse mesh, bit for
    bit, axial elements included."""
    sim = solver.Simulation(small_inputs)
    sim.build()
    ex = sim.ex
    checked = 0
    for name in ("solid_fluid_boundary", "r1"):
        sides = ex.side.get(name)
        if sides is None:
            continue
        es = np.nonzero(sides >= 0)[0]
        ks, nvs = solver.boundary_normals(sim.nodes4, sim.crds, sim.jac[0], sim.axial_e, sim.co, es, sides[es])
        for i, e in enumerate(es):
            want = _normal_pointwise(sim.nodes4, sim.crds, sim.jac[0], sim.axial_e, sim.co, e, sides[e])
            assert ks[i].tolist() == [k for k, _ in want]
            np.testing.assert_array_equal(nvs[i], np.array([v for _, v in want]))
            checked += 1
    assert checked > 0 and sim.axial_e[np.nonzero(ex.side["r1"] >= 0)[0]].any()


def test_closest_gll_distance_is_the_smallest_pair():
    """solver.closest_gll_distance (squared distances, hypot on the near-minimal pairs only)
    equals the smallest hypot over all 300 pairs of each element's GLL points."""
    rng = np.random.default_rng(4)
    base = np.stack(np.meshgrid(np.linspace(0, 1, 5), np.linspace(0, 1, 5), indexing="ij"), -1).reshape(25, 2)
    crds = base[None] * rng.uniform(1e4, 1e5, (200, 1, 1)) + rng.normal(0, 3e3, (200, 25, 2)) + rng.uniform(0, 6e6, (200, 1, 2))
    crds[:5] = crds[:5, :1]  # coincident points: distance 0
    crds[5:10, 7] = crds[5:10, 3]
    pa, pb = np.triu_indices(25, 1)
    want = np.hypot(crds[:, pa, 0] - crds[:, pb, 0], crds[:, pa, 1] - crds[:, pb, 1]).min(1)
    np.testing.assert_array_equal(solver.closest_gll_distance(crds), want)


def test_unknown_volumetric_model_raises(tmp_path):
    d = solver.write_inputs(tmp_path / "input", mesh_kw=SMALL_MESH, steps=10, models3d=("s20rts",))
    with pytest.raises(NotImplementedError):
        solver.Simulation(d).build()


def test_per_element_nu_field(small_inputs):
    """A per-element Nu field sets each point's Nr = 2 max(Nu of its elements) + 1 (capped
    by the point's circumference and odd near the axis)."""
    sim = solver.Simulation(small_inputs)
    spec0 = sim.build()
    E = len(spec0.e_pts)
    nu = np.where(np.arange(E) % 2 == 0, 1, 3)
    spec = sim.build(nu_elem=nu)
    pnu = np.zeros(spec.n_points, int)
    np.maximum.at(pnu, spec.e_pts.ravel(), np.repeat(nu, 25))
    assert (spec.p_nr <= 2 * pnu + 2).all() and (spec.p_nr != spec0.p_nr).any()


@pytest.mark.gpu
def test_full_solver_3d_gpu_matches_oracle(inputs_3d, ax3d_lib):
    """3-D model: 3-D solid/fluid elements, Mass3D points and 3-D coupling through the loop."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    sim = solver.Simulation(inputs_3d)
    spec = sim.build()
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    g.step(120)
    o.step(120)
    a, b = g.seismograms(0, 120), o.seismograms(0, 120)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    x, y = g.get("displ", "fluid"), o.get("displ", "fluid")
    assert np.linalg.norm(x - y) <= 1e-5 * np.linalg.norm(y)


def test_whole_surface_edges_and_netcdf(tmp_path_factory):
    """OUT_STATIONS_WHOLE_SURFACE: every solid element touching the outer radius gives its
    outer side, tags follow the smallest colatitude, records land in axisem3d_surface.nc."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("sf") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=30, hdur=20.0, n_stations=2, seed=4,
                        whole_surface="true 6371.0 0 90")
    sim = solver.Simulation(d, output_dir=d.parent / "output")
    spec = sim.build()
    edges = sim.surface_edges
    assert len(edges) > 0 and len(spec.sf_elem) == len(edges)
    th = np.array([min(x[3], x[4]) for x in edges])
    assert (np.diff(th) >= 0).all() and th.min() >= 0 and th.max() < np.pi / 2
    sides = {0: (0, 20), 1: (20, 24), 2: (4, 24), 3: (0, 4)}
    for _, e, k, t0, t1 in edges:
        c = sim.crds[e].reshape(25, 2)
        q0, q1 = sides[k]
        np.testing.assert_allclose(np.hypot(*c[[q0, q1]].T), sim.R, rtol=1e-9)
        assert not sim.fluid[e]
    # the same window from below the surface is empty; a bad option size raises
    par = solver.Parameters(d)
    par.values["OUT_STATIONS_WHOLE_SURFACE"] = ["true", "6371.0", "0", "90", "true"]
    sim.par = par
    sim._surface(spec)
    assert sim.surface_edges == []
    par.values["OUT_STATIONS_WHOLE_SURFACE"] = ["true", "6371.0", "0"]
    with pytest.raises(ValueError, match="WHOLE_SURFACE"):
        sim._surface(spec)
    sim = solver.Simulation(d, output_dir=d.parent / "output")
    spec = sim.build()
    o = OracleDomain(spec)
    o.step(30)
    recs = sim.surface_records(o, 30)
    assert len(recs) == len(edges) and recs[0].shape == (30, 3, 5, 3)
    assert max(np.abs(r).max() for r in recs) > 0
    path = sim.write_surface_netcdf(recs)
    ds = NC.read(path)
    assert path.name == "axisem3d_surface.nc"
    assert ds["time_points"].shape == (30,) and ds["theta"].shape == (len(edges), 2)
    np.testing.assert_allclose(ds["theta"][:, 0], [x[3] for x in edges])
    w = 15 * 3
    for tag in (0, len(edges) - 1):
        np.testing.assert_allclose(ds[f"edge_{tag}r"], recs[tag].real.reshape(30, w).astype(np.float32))
        np.testing.assert_allclose(ds[f"edge_{tag}i"], recs[tag].imag.reshape(30, w).astype(np.float32))
    assert float(ds.attrs["radius"][0]) == sim.R


def test_ocean_load_constant(tmp_path_factory):
    """MODEL_3D_OCEAN_LOAD constant$4.0: every solid surface point gets a MassOcean1D row
    (1-D model), the ocean adds mass to the radial direction only, and the oracle's
    seismograms change; unknown names raise."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("oc") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=60, hdur=20.0, n_stations=3, seed=4, ocean="constant$4.0")
    sim = solver.Simulation(d)
    spec = sim.build()
    surf = set()
    for e in np.nonzero((sim.ex.side["r1"] >= 0) & ~sim.fluid)[0]:
        c = sim.crds[e].reshape(25, 2)
        surf |= {int(sim.e_pts[e, k]) for k in range(25) if abs(np.hypot(*c[k]) - sim.R) < 1.0}
    assert set(spec.oc_pt.tolist()) == surf and (spec.oc_len == 1).all()
    v = spec.oc_vals.reshape(-1, 4).astype(np.float64)
    assert (v[:, 0] < v[:, 1]).all()                        # 1/(m + m_ocean) < 1/m
    np.testing.assert_allclose(v[:, 2] ** 2 + v[:, 3] ** 2, 1.0, rtol=1e-6)
    o1 = OracleDomain(spec)
    o1.step(60)
    spec.oc_pt = spec.oc_pt[:0]
    o0 = OracleDomain(spec)
    o0.step(60)
    a, b = o1.seismograms(0, 60), o0.seismograms(0, 60)
    assert np.abs(a - b).max() > 1e-6 * np.abs(b).max()
    (d / "inparam.model").write_text((d / "inparam.model").read_text().replace("constant$4.0", "marsocean"))
    with pytest.raises(ValueError, match="Unknown ocean-load model"):
        solver.Simulation(d).build()


def test_station_strain_curl_and_enz(tmp_path_factory):
    """STATIONS keywords dump_strain / dump_curl (ReceiverCollection.cpp:58-72) flag the
    receivers; their strain (RTZ) and curl land in the synthetics file as NET.NAME.RTZ.strain
    and .RTZ.curl; ENZ rotates displacement by the back azimuth (PointwiseRecorder.cpp:80-88)."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("sc") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=40, hdur=20.0, n_stations=6, seed=4,
                        station_extra=("dump_strain", "dump_curl", "dump_strain dump_curl", "", "bogus"),
                        components="ENZ")
    (d / "STATIONS").write_text((d / "STATIONS").read_text() + "BAD LINE\nX1 SY notanumber 0 0 0\n")
    sim = solver.Simulation(d, output_dir=d.parent / "output")
    spec = sim.build()
    assert spec.r_dump.tolist() == [1, 2, 3, 0, 0, 1] and len(spec.r_elem) == 6
    assert all(0.0 <= b < 2 * np.pi for b in sim.baz)
    o = OracleDomain(spec)
    o.step(40)
    seis = o.seismograms(0, 40)
    enz = sim.rotate(seis)
    sim.components = "RTZ"
    rtz = sim.rotate(seis)
    sim.components = "ENZ"
    # ENZ is a rotation of (T, phi) about the vertical: horizontal norm and Z unchanged
    np.testing.assert_allclose(np.hypot(enz[..., 0], enz[..., 1]), np.hypot(rtz[..., 0], rtz[..., 1]), rtol=1e-9,
                               atol=1e-30)
    np.testing.assert_allclose(enz[..., 2], rtz[..., 2])
    st, cu = o.strain_curl("strain", 0, 40), o.strain_curl("curl", 0, 40)
    assert st.shape == (40, 3, 6) and cu.shape == (40, 2, 3) and np.abs(st).max() > 0
    p = sim.write_netcdf(enz, strain=st, curl=sim.rotate_curl(cu))
    ds = NC.read(p)
    np.testing.assert_allclose(ds["SY.S000.RTZ.strain"], st[:, 0].astype(np.float32))
    np.testing.assert_allclose(ds["SY.S005.RTZ.strain"], st[:, 2].astype(np.float32))
    assert ds["SY.S002.RTZ.curl"].shape == (40, 3) and "SY.S003.RTZ.curl" not in ds.variables


def test_wisdom_file_roundtrip_and_lookup(tmp_path):
    """NuWisdom::writeToFile / readFromFile (three- or four-column variable) and getNu
    (inverse-distance mean of the four nearest points, exact hits returned as stored)."""
    from axisem3d_gb300 import wisdom as W
    s = np.array([0.0, 1.0, 0.0, 1.0, 5.0])
    z = np.array([0.0, 0.0, 1.0, 1.0, 5.0])
    W.write_wisdom(tmp_path / "w.nc", s, z, [2, 4, 6, 8, 100], [10, 10, 10, 10, 10])
    data = W.read_wisdom(tmp_path / "w.nc")
    assert data.shape == (5, 4) and W.compression_ratio(data) == pytest.approx(120 / 50)
    assert W.wisdom_nu(data, [1.0], [0.0])[0] == 4                   # exact hit
    assert W.wisdom_nu(data, [0.5], [0.5])[0] == 5                   # centre of the square: mean 5
    ds = NC.Dataset()
    ds.add_dim("a", 2)
    ds.add_dim("b", 3)
    ds.add_var("axisem3d_wisdom", ("a", "b"), np.array([[0.0, 0.0, 3.0], [1.0, 0.0, 5.0]]))
    NC.write(tmp_path / "w3.nc", ds)
    np.testing.assert_array_equal(W.read_wisdom(tmp_path / "w3.nc")[:, 3], [3, 5])
    ds.variables.clear()
    ds.add_dim("c", 2)
    ds.add_var("axisem3d_wisdom", ("a", "c"), np.zeros((2, 2)))
    NC.write(tmp_path / "w2.nc", ds)
    with pytest.raises(ValueError, match="3 or 4 columns"):
        W.read_wisdom(tmp_path / "w2.nc")


def test_empirical_nr_field():
    """EmpNrField::getNrAtPoint: axis, epicentral-distance and surface scaling, minimum."""
    from axisem3d_gb300 import wisdom as W
    vals = {"NU_EMP_REF": "20", "NU_EMP_MIN": "3", "NU_EMP_SCALE_AXIS": "true", "NU_EMP_POW_AXIS": "0.5",
            "NU_EMP_SCALE_THETA": "true", "NU_EMP_FACTOR_PI": "2.0", "NU_EMP_THETA_START": "90",
            "NU_EMP_POW_THETA": "1.0", "NU_EMP_SCALE_DEPTH": "true", "NU_EMP_FACTOR_SURF": "3.0",
            "NU_EMP_DEPTH_START": "100", "NU_EMP_DEPTH_END": "300"}
    par = solver.Parameters.__new__(solver.Parameters)
    par.values = {k: [v] for k, v in vals.items()}
    R = 6371e3
    r = np.array([R, R - 200e3, R - 1000e3, R - 1000e3, 100.0])
    th = np.radians([45.0, 45.0, 45.0, 135.0, 45.0])
    nr = W.empirical_nr(par, r * np.sin(th), r * np.cos(th), R)
    def want(r_, t_):
        nu = 20 * np.sqrt(r_ * np.sin(t_) / R)
        if t_ > np.pi / 2:
            nu *= 1 + (t_ - np.pi / 2) / (np.pi / 2)
        d = R - r_
        if d <= 300e3:
            nu *= 3.0 if d <= 100e3 else 1 + 2.0 / (100e3 - 300e3) * (d - 300e3)
        return 2 * max(3, int(np.ceil(nu))) + 1
    assert nr.tolist() == [want(a, b) for a, b in zip(r, th)]


def test_wisdom_learn_then_reuse(tmp_path_factory):
    """NU_WISDOM_LEARN writes (s, z, learned Nu, Nu) of every point after the loop; a second
    run with NU_TYPE wisdom reads it back and takes each point's learned Nu."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("wl") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, nu=6, steps=60, hdur=20.0, n_stations=2, seed=5)
    (d / "inparam.nu").write_text("NU_TYPE constant\nNU_CONST 6\nNU_WISDOM_LEARN true\nNU_WISDOM_LEARN_EPSILON 1e-3\n"
                                  "NU_WISDOM_LEARN_INTERVAL 10\nNU_WISDOM_LEARN_OUTPUT wisdom.nc\n")
    out = d.parent / "output"
    sim = solver.Simulation(d, output_dir=out)
    spec = sim.build()
    sim.run(domain=OracleDomain(spec))
    from axisem3d_gb300 import wisdom as W
    data = W.read_wisdom(out / "wisdom.nc")
    assert data.shape == (spec.n_points, 4) and (data[:, 2] <= data[:, 3]).all() and data[:, 2].min() >= 0
    (d / "wisdom.nc").write_bytes((out / "wisdom.nc").read_bytes())
    (d / "inparam.nu").write_text("NU_TYPE wisdom\nNU_WISDOM_REUSE_INPUT wisdom.nc\nNU_WISDOM_REUSE_FACTOR 1.0\n"
                                  "NU_WISDOM_LEARN false\n")
    sim2 = solver.Simulation(d, output_dir=out)
    spec2 = sim2.build()
    learned = data[:, 2].astype(int)
    # exact hits: 2 Nu_learned + 1 under the same axis / spacing limit as the first run's Nr
    np.testing.assert_array_equal(spec2.p_nr, np.minimum(2 * learned + 1, spec.p_nr))
    assert spec2.p_nr.sum() < spec.p_nr.sum() and sim2.wisdom_ratio == pytest.approx(W.compression_ratio(data))


@pytest.mark.gpu
@pytest.mark.parametrize("attenuation", [False, True])
def test_gpu_preloop_moduli_match_host(tmp_path_factory, ax3d_lib, attenuation):
    """ax3d_precompute_elastic (FP64 on the GPU) gives the solver's moduli and attenuation
    moduli (1-D and 3-D elements, CG4) as the numpy pre-loop does, to float rounding."""
    d = tmp_path_factory.mktemp("pre") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=20, hdur=20.0, n_stations=2, seed=3, nu=4,
                        models3d=MODELS_3D, attenuation=attenuation)
    a = solver.Simulation(d).build(preloop="host")
    b = solver.Simulation(d).build(preloop="gpu")
    assert a.e_in3d.any() and (a.e_in3d == 0).any()
    np.testing.assert_allclose(b.e_mod, a.e_mod, rtol=2e-6, atol=0)
    assert len(a.e_attm) == len(b.e_attm) and (len(a.e_attm) > 0) == attenuation
    np.testing.assert_allclose(b.e_attm, a.e_attm, rtol=2e-6, atol=1e-30)


def _ti_model(seed=2):
    rng = np.random.default_rng(seed)
    rows = np.array([1, 7, 1, 13, 5])
    ifact = rng.uniform(1e9, 5e9, (len(rows), 25))
    model = {k: [rng.uniform(lo, hi, (r, 25)).astype(np.float32) for r in rows] for k, lo, hi in
             (("vpv", 8e3, 9e3), ("vph", 8e3, 9.5e3), ("vsv", 4e3, 5e3), ("vsh", 4e3, 5.2e3), ("eta", 0.9, 1.0),
              ("rho", 3e3, 4e3), ("qkappa", 1e4, 6e4), ("qmu", 80, 600))}
    return rows, ifact, model


NAMES8 = ("vpv", "vph", "vsv", "vsh", "eta", "rho", "qkappa", "qmu")


def test_oracle_preloop_elastic_matches_numpy():
    """The oracle's FP64 Material::createElastic + AttBuilder + AttAxiSEM restatement and the
    numpy pre-loop agree (TI and isotropic, no / full / CG4 attenuation)."""
    from axisem3d_gb300 import attenuation as ATT
    from axisem3d_gb300 import preloop as PL
    from axisem3d_gb300.spec import ATT_CG4, ATT_FULL, ATT_NONE
    from oracle.oracle_py import pre_elastic
    rows, ifact, model = _ti_model()
    w, y = ATT.fit_sls(3, 1 / 200, 1 / 10)
    sls = PL.SLSFit(w, y, 1 / 200, 1 / 10, 1.0)
    per_elem = [np.stack([model[k][e] for k in NAMES8]) for e in range(len(rows))]
    for att in (ATT_NONE, ATT_FULL, ATT_CG4):
        for iso in (False, True):
            m = dict(model) if att != ATT_NONE else {k: v for k, v in model.items() if k not in ("qkappa", "qmu")}
            h_mod, h_att = PL.moduli_host(rows, ifact, m, isotropic=iso, att=att, sls=sls)
            o_mod, o_att = pre_elastic(rows, ifact, per_elem, iso, att, (w, y, 1 / 200, 1 / 10, 1.0, True))
            np.testing.assert_allclose(o_mod.astype(np.float32), h_mod, rtol=1e-6)
            np.testing.assert_allclose(o_att.astype(np.float32), h_att, rtol=1e-6, atol=1e-30)


def _mesh_elements(tmp_path_factory, name, **kw):
    d = tmp_path_factory.mktemp(name) / "input"
    solver.write_inputs(d, steps=10, n_stations=2, seed=3, **kw)
    sim = solver.Simulation(d)
    spec = sim.build()
    return sim, spec


def test_oracle_preloop_geometry_matches_numpy(tmp_path_factory):
    """The oracle's FP64 Quad::createGraident / formIntegralFactor restatement and the numpy
    pre-loop agree on every element of the default half disk (spherical, linear and
    semi-spherical mappings, axial elements)."""
    from axisem3d_gb300 import geometry as GEO
    from axisem3d_gb300 import preloop as PL
    from oracle.oracle_py import pre_geometry
    sim, _ = _mesh_elements(tmp_path_factory, "geo")
    et = sim.ex.etype
    assert len(np.unique(et)) >= 2 and sim.axial_e.any()
    geo, ifact, crds, _, _ = GEO.batch_geometry(sim.nodes4, et, sim.co, sim.axial_e)
    og, oi, oc = pre_geometry(sim.nodes4, et, sim.co, sim.axial_e, PL.spectral_table())
    for a, b in ((og, geo), (oi, ifact), (oc, crds)):
        scale = np.abs(b).max(axis=tuple(range(1, b.ndim)), keepdims=True)
        assert (np.abs(a - b) <= 1e-11 * scale).all()


@pytest.mark.gpu
def test_gpu_preloop_geometry_and_mass_match_oracle(tmp_path_factory, ax3d_lib):
    """ax3d_precompute_geometry and ax3d_precompute_mass (FP64 on the GPU) against the oracle's
    FP64 restatement on every element of the default half disk (fluid core included), and the
    domain built with the GPU pre-loop against the host pre-loop."""
    from axisem3d_gb300 import preloop as PL
    from oracle.oracle_py import pre_geometry, pre_mass
    sim, spec_h = _mesh_elements(tmp_path_factory, "geog")
    et = sim.ex.etype
    og, oi, oc = pre_geometry(sim.nodes4, et, sim.co, sim.axial_e, PL.spectral_table())
    gg, gi, gc = PL.geometry_gpu(sim.nodes4, et, sim.co, sim.axial_e)
    for a, b in ((gg, og), (gi, oi), (gc, oc)):
        scale = np.abs(b).max(axis=tuple(range(1, b.ndim)), keepdims=True)
        assert (np.abs(a - b) <= 1e-12 * scale).all()
    E = len(et)
    rng = np.random.default_rng(4)
    rows = rng.integers(1, 6, E)
    rho = rng.uniform(2.6e3, 13e3, int(rows.sum()) * 25).astype(np.float32)
    vp = rng.uniform(5.8e3, 13.7e3, int(rows.sum()) * 25).astype(np.float32)
    fl = sim.fluid.astype(np.uint8)
    assert fl.any() and (fl == 0).any()
    gm = PL.mass_gpu(rows, oi, rho, vp, fl)
    om = pre_mass(rows, oi, rho.astype(np.float64), vp.astype(np.float64), fl)
    np.testing.assert_allclose(gm, om, rtol=1e-14)
    spec_g = solver.Simulation(sim.input_dir).build(preloop="gpu")
    np.testing.assert_allclose(spec_g.e_geo, spec_h.e_geo, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(spec_g.p_ms, spec_h.p_ms, rtol=1e-6)
    np.testing.assert_allclose(spec_g.p_mf, spec_h.p_mf, rtol=1e-6)


@pytest.mark.gpu
def test_gpu_preloop_transversely_isotropic(ax3d_lib):
    """ax3d_precompute_elastic: TI and isotropic moduli with no, full and CG4 attenuation,
    random model values, GPU (FP64, rounded to FP32) against the oracle's FP64 restatement of
    Material::createElastic + AttBuilder + AttAxiSEM."""
    from axisem3d_gb300 import preloop as PL
    from axisem3d_gb300 import attenuation as ATT
    from axisem3d_gb300.spec import ATT_CG4, ATT_FULL, ATT_NONE
    from oracle.oracle_py import pre_elastic
    rows, ifact, model = _ti_model()
    w, y = ATT.fit_sls(3, 1 / 200, 1 / 10)
    sls = PL.SLSFit(w, y, 1 / 200, 1 / 10, 1.0)
    per_elem = [np.stack([model[k][e] for k in NAMES8]) for e in range(len(rows))]
    for att in (ATT_NONE, ATT_FULL, ATT_CG4):
        for iso in (False, True):
            m = dict(model) if att != ATT_NONE else {k: v for k, v in model.items() if k not in ("qkappa", "qmu")}
            g_mod, g_att = PL.moduli_gpu(rows, ifact, m, isotropic=iso, att=att, sls=sls)
            o_mod, o_att = pre_elastic(rows, ifact, per_elem, iso, att, (w, y, 1 / 200, 1 / 10, 1.0, True))
            np.testing.assert_allclose(g_mod, o_mod.astype(np.float32), rtol=1e-6)
            np.testing.assert_allclose(g_att, o_att.astype(np.float32), rtol=1e-6, atol=1e-30)


def test_point_force_source(tmp_path_factory):
    """SOURCE_TYPE point_force (PointForce::computeSourceFourier): orders 0 and 1 on the axis
    column.  A vertical force excites order 0 only: no transverse motion anywhere.  A force
    along theta at the pole (x) radiates SH as sin(azimuth) and P-SV as cos(azimuth): no T at
    azimuth 0, no R or Z at azimuth 90.  An unknown source type raises."""
    from oracle.oracle_py import OracleDomain
    out = {}
    for name, force in (("vertical", (0.0, 0.0, 1e16)), ("horizontal", (1e16, 0.0, 0.0))):
        d = tmp_path_factory.mktemp("pf" + name) / "input"
        solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=250, hdur=20.0, n_stations=4, seed=6, force=force)
        (d / "STATIONS").write_text("".join(f"A{i}  SY  10.0  {az:.1f}  0.0  0.0\n"
                                            for i, az in enumerate((0.0, 30.0, 60.0, 90.0))))
        sim = solver.Simulation(d)
        spec = sim.build()
        elem, f = spec.sources[0]
        assert f.shape == (25, 2, 3) and np.abs(f[5:]).max() == 0  # axis column only (ipol = 0)
        o = OracleDomain(spec, double=True)
        o.step(250)
        out[name] = sim.rotate(o.seismograms(0, 250))  # [t][station][R, T, Z]
    v, h = out["vertical"], out["horizontal"]
    peak = np.abs(v).max()
    assert peak > 0 and np.abs(v[..., 1]).max() <= 1e-12 * peak
    hp = np.abs(h).max()
    assert np.abs(h[:, 0, 1]).max() <= 1e-10 * hp                        # T at azimuth 0
    assert np.abs(h[:, 3, [0, 2]]).max() <= 1e-6 * np.abs(h[:, 3, 1]).max()  # R, Z at azimuth 90
    assert np.abs(h[:, 3, 1]).max() > 1e-2 * hp
    d = tmp_path_factory.mktemp("pfbad") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=10, n_stations=2, seed=6)
    (d / "inparam.time_src_recv").write_text((d / "inparam.time_src_recv").read_text().replace(
        "SOURCE_TYPE earthquake", "SOURCE_TYPE explosion"))
    with pytest.raises(ValueError, match="Unknown source type"):
        solver.Simulation(d).build()


def test_ascii_output_and_duplicated_stations(tmp_path_factory):
    """OUT_STATIONS_FORMAT ascii netcdf: one text file per station (time + R, T, Z; strain and
    curl files for flagged receivers) beside the NetCDF file; OUT_STATIONS_DUPLICATED rename
    appends __DUPLICATED<k> to a repeated NET.NAME, error refuses it."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("asc") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=30, hdur=20.0, n_stations=3, seed=4,
                        station_extra=("dump_strain dump_curl", "", ""))
    st = (d / "STATIONS").read_text().splitlines()
    (d / "STATIONS").write_text("\n".join(st + [st[1]]) + "\n")  # S001 twice
    tsr = (d / "inparam.time_src_recv").read_text().replace("OUT_STATIONS_FORMAT netcdf", "OUT_STATIONS_FORMAT ascii netcdf")
    (d / "inparam.time_src_recv").write_text(tsr)
    out = d.parent / "output"
    sim = solver.Simulation(d, output_dir=out)
    spec = sim.build()
    assert [r[0] for r in sim.receivers] == ["S000", "S001", "S002", "S001__DUPLICATED1"]
    o = OracleDomain(spec)
    o.step(30)
    rtz = sim.rotate(o.seismograms(0, 30))
    st_, cu = o.strain_curl("strain", 0, 30), o.strain_curl("curl", 0, 30)
    paths = sim.write_outputs(rtz, strain=st_, curl=cu)
    names = sorted(p.name for p in paths)
    assert "SY.S001__DUPLICATED1.RTZ.ascii" in names and "axisem3d_synthetics.nc" in names
    a = np.loadtxt(out / "stations" / "SY.S002.RTZ.ascii")
    assert a.shape == (30, 4)
    np.testing.assert_allclose(a[:, 0], -sim.shift + np.arange(30) * sim.dt)
    np.testing.assert_allclose(a[:, 1:], rtz[:, 2].astype(np.float32), rtol=1e-6, atol=1e-37)
    s0 = np.loadtxt(out / "stations" / "SY.S000.RTZ.strain.ascii")
    assert s0.shape == (30, 7)
    np.testing.assert_allclose(s0[:, 1:], st_[:, 0].astype(np.float32), rtol=1e-6, atol=1e-37)
    assert np.loadtxt(out / "stations" / "SY.S000.RTZ.curl.ascii").shape == (30, 4)
    (d / "inparam.time_src_recv").write_text(tsr.replace("OUT_STATIONS_DUPLICATED rename", "OUT_STATIONS_DUPLICATED error"))
    with pytest.raises(ValueError, match="Duplicated station keys"):
        solver.Simulation(d).build()
    (d / "inparam.time_src_recv").write_text(tsr.replace("OUT_STATIONS_DUPLICATED rename", "OUT_STATIONS_DUPLICATED maybe"))
    with pytest.raises(ValueError, match="OUT_STATIONS_DUPLICATED"):
        solver.Simulation(d).build()


def test_2d_mode_and_null_source(tmp_path_factory):
    """MODEL_2D_MODE source-centered: the 3-D models are sampled at one azimuth, so every
    element stays 1-D but takes the model's values there (two azimuths through and beside
    a bubble differ); DEVELOP_NON_SOURCE_MODE gives no source term and a quiet field."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("m2d") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=20, hdur=20.0, n_stations=2, seed=3, nu=4,
                        models3d=MODELS_3D)
    full = solver.Simulation(d).build()
    assert full.e_in3d.any()
    mods = []
    for az in (0.0, 180.0):
        txt = (d / "inparam.model").read_text().replace("MODEL_2D_MODE off",
                                                         f"MODEL_2D_MODE source-centered\nMODEL_2D_AZIMUTH {az}")
        (d / "inparam.model").write_text(txt)
        spec = solver.Simulation(d).build()
        assert not spec.e_in3d.any()
        mods.append(spec.e_mod.copy())
        (d / "inparam.model").write_text(txt.replace(f"MODEL_2D_MODE source-centered\nMODEL_2D_AZIMUTH {az}",
                                                     "MODEL_2D_MODE off"))
    assert mods[0].shape == mods[1].shape and np.abs(mods[0] - mods[1]).max() > 0
    (d / "inparam.model").write_text((d / "inparam.model").read_text().replace("MODEL_2D_MODE off",
                                                                               "MODEL_2D_MODE sideways"))
    with pytest.raises(ValueError, match="MODEL_2D_MODE"):
        solver.Simulation(d).build()
    d2 = tmp_path_factory.mktemp("null") / "input"
    solver.write_inputs(d2, mesh_kw=SMALL_MESH, steps=20, hdur=20.0, n_stations=2, seed=3)
    adv = (d2 / "inparam.advanced").read_text().replace("DEVELOP_NON_SOURCE_MODE false", "DEVELOP_NON_SOURCE_MODE true")
    (d2 / "inparam.advanced").write_text(adv)
    sim = solver.Simulation(d2)
    spec = sim.build()
    assert spec.sources == [] and sim.src_lat == 90.0
    o = OracleDomain(spec)
    o.step(20)
    assert np.abs(o.seismograms(0, 20)).max() == 0


def test_record_interval_subsamples_station_output(tmp_path_factory):
    """OUT_STATIONS_RECORD_INTERVAL 3: the station files keep steps 0, 3, 6, ... with their
    times (PointwiseRecorder::record)."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("riv") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=20, hdur=20.0, n_stations=2, seed=4)
    t = (d / "inparam.time_src_recv").read_text()
    (d / "inparam.time_src_recv").write_text(t.replace("OUT_STATIONS_RECORD_INTERVAL 1", "OUT_STATIONS_RECORD_INTERVAL 3")
                                             .replace("OUT_STATIONS_FORMAT netcdf", "OUT_STATIONS_FORMAT netcdf ascii"))
    sim = solver.Simulation(d, output_dir=d.parent / "out")
    spec = sim.build()
    o = OracleDomain(spec)
    o.step(20)
    rtz = sim.rotate(o.seismograms(0, 20))
    sim.write_outputs(rtz)
    ds = NC.read(d.parent / "out" / "stations" / "axisem3d_synthetics.nc")
    np.testing.assert_allclose(ds["time_points"], -sim.shift + np.arange(0, 20, 3) * sim.dt)
    np.testing.assert_allclose(ds["SY.S001.RTZ"], rtz[::3, 1].astype(np.float32))
    a = np.loadtxt(d.parent / "out" / "stations" / "SY.S000.RTZ.ascii")
    assert a.shape == (7, 4)


def test_user_nr_field_and_refused_options(tmp_path_factory):
    """NU_TYPE user-defined (UserNrField as shipped: Nu linear in depth through the
    (depth, nu) pairs); data-driven geometric models and ellipticity, not built, are refused."""
    from axisem3d_gb300 import wisdom as W
    nr = W.user_nr(["0", "8", "1000e3", "2", "3000e3", "2"], [0.0, 0.0, 0.0, 0.0],
                   [6371e3, 6371e3 - 500e3, 6371e3 - 1000e3, 100.0], 6371e3)
    assert nr.tolist() == [17, 11, 5, 5]
    with pytest.raises(ValueError, match="even and positive"):
        W.user_nr(["0", "8", "1"], [0.0], [6371e3], 6371e3)
    d = tmp_path_factory.mktemp("unr") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=10, n_stations=2, seed=3)
    (d / "inparam.nu").write_text("NU_TYPE user-defined\nNU_USER_PARAMETER_LIST 0 6 2000e3 2\nNU_WISDOM_LEARN false\n")
    spec = solver.Simulation(d).build()
    assert spec.p_nr.max() <= 13 and spec.p_nr.min() >= 1 and len(np.unique(spec.p_nr)) > 2
    m = (d / "inparam.model").read_text()
    (d / "inparam.model").write_text(m.replace("MODEL_3D_GEOMETRIC_NUM 0", "MODEL_3D_GEOMETRIC_NUM 1\nMODEL_3D_GEOMETRIC_LIST crust1"))
    with pytest.raises(NotImplementedError, match="not shipped"):
        solver.Simulation(d).build()
    (d / "inparam.model").write_text(m + "MODEL_3D_ELLIPTICITY_MODE full\nMODEL_3D_ELLIPTICITY_INVF 298.3\n")
    with pytest.raises(ValueError, match="ELLIPTICITY"):
        solver.Simulation(d).build()


def test_legacy_attenuation_refused_and_slice_plots_warned(tmp_path_factory):
    """ATTENUATION_SPECFEM_LEGACY (a different SLS fit, not built) stops the build; slice plots
    (output only) give a warning."""
    d = tmp_path_factory.mktemp("leg") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=10, n_stations=2, seed=3, attenuation=True)
    adv = (d / "inparam.advanced").read_text()
    (d / "inparam.advanced").write_text(adv.replace("ATTENUATION_SPECFEM_LEGACY false", "ATTENUATION_SPECFEM_LEGACY true"))
    with pytest.raises(ValueError, match="SPECFEM"):
        solver.Simulation(d).build()
    (d / "inparam.advanced").write_text(adv)
    m = (d / "inparam.model").read_text()
    (d / "inparam.model").write_text(m.replace("MODEL_PLOT_SLICES_NUM 0", "MODEL_PLOT_SLICES_NUM 1"))
    with pytest.warns(UserWarning, match="slice plots"):
        solver.Simulation(d).build()


def test_loop_info_reports_in_chunks(tmp_path_factory):
    """OPTION_LOOP_INFO_INTERVAL: Simulation.run steps in chunks and reports each (the
    Newmark::solve screen info); the result equals one uninterrupted run."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("loop") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=25, hdur=20.0, n_stations=2, seed=3)
    adv = (d / "inparam.advanced").read_text().replace("OPTION_LOOP_INFO_INTERVAL 1000", "OPTION_LOOP_INFO_INTERVAL 10")
    (d / "inparam.advanced").write_text(adv)
    sim = solver.Simulation(d)
    spec = sim.build()
    lines = []
    rtz, dom = sim.run(domain=OracleDomain(spec), log=lines.append)
    assert len(lines) == 3 and "25 / 25 (100%)" in lines[-1] and "10 / 25 (40%)" in lines[0]
    ref, _ = sim.run(domain=OracleDomain(spec))
    np.testing.assert_array_equal(rtz, ref)


def test_randomized_initial_displacement_with_null_source(tmp_path_factory):
    """DEVELOP_RANDOMIZE_DISP0 with DEVELOP_NON_SOURCE_MODE (the reference's scaling-test
    backends): a tiny random initial field, orders 0-2 only, makes a source-free run move."""
    from oracle.oracle_py import OracleDomain
    d = tmp_path_factory.mktemp("rnd") / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=20, hdur=20.0, n_stations=2, seed=3, nu=4)
    adv = (d / "inparam.advanced").read_text().replace("DEVELOP_NON_SOURCE_MODE false", "DEVELOP_NON_SOURCE_MODE true")
    (d / "inparam.advanced").write_text(adv + "DEVELOP_RANDOMIZE_DISP0 true\n")
    sim = solver.Simulation(d)
    spec = sim.build()
    dom = OracleDomain(spec)
    sim.randomize_displacement(dom)
    u = dom.get("displ", "solid")
    so, _ = spec.point_offsets()
    p = int(np.flatnonzero((spec.p_nr >= 9) & (spec.p_kind == 0))[0])
    blk = u[so[p]:so[p] + 3 * (spec.p_nr[p] // 2 + 1)].reshape(-1, 3)
    assert np.abs(blk[:3]).max() > 0 and np.abs(blk[3:]).max() == 0 and np.abs(blk).max() <= 2e-30
    rtz, _ = sim.run(domain=OracleDomain(spec))
    assert 0 < np.abs(rtz).max() < 1e-25


def test_reference_template_parfiles_parse(tmp_path):
    """The parameter entries of the reference's own template/input/inparam.* (fixture made by
    tests/golden/make_inparam_golden.py) written out in the parfile layout -- keys padded to a
    column, comment lines and blank lines between them -- parse back entry for entry: every
    key is registered, every value list is kept, and the typed getters read them."""
    import json
    from pathlib import Path
    fx = json.loads((Path(__file__).parent / "golden" / "inparam_template.json").read_text())
    for name in solver.PARFILES:
        lines = [f"# {name}: reference template entries", ""]
        for key, vals in fx[name]:
            lines += [f"# {key.lower()}", f"{key:<44}{'   '.join(vals)}  ", ""]
        (tmp_path / name).write_text("\n".join(lines))
    par = solver.Parameters(tmp_path)
    for name in solver.PARFILES:
        for key, vals in fx[name]:
            assert key in solver.REGISTRY, key
            assert par.values[key][:len(vals)] == vals, key
    assert par.get("NU_CONST", int) == 2 and par.get("NU_WISDOM_LEARN", bool) is False
    assert par.get("NU_WISDOM_LEARN_EPSILON", float) == 1e-3
    assert par.get("ATTENUATION_CG4", bool) is True
    assert par.get("MODEL_3D_VOLUMETRIC_LIST", str, 1) == "crust1"


def _bump_inputs(tmp_path_factory, name, latlon, **kw):
    from pathlib import Path
    d = tmp_path_factory.mktemp(name) / "input"
    solver.write_inputs(d, mesh_kw=SMALL_MESH, steps=60, hdur=20.0, n_stations=3, seed=3, nu=4, **kw)
    pm = Path(d) / "inparam.model"
    pm.write_text(pm.read_text().replace(
        "MODEL_3D_GEOMETRIC_NUM 0", f"MODEL_3D_GEOMETRIC_NUM 1\nMODEL_3D_GEOMETRIC_LIST bump$6371${latlon}$20$15$400"))
    return d


class _Const:
    """A geometric model with a constant radial shift."""

    def __init__(self, c):
        self.c = c

    def delta_r(self, xyz, r_center):
        return np.full(xyz.shape[:-1], self.c)


class _Linear:
    """deltaR = k (r - r0)."""

    def __init__(self, k, r0):
        self.k, self.r0 = k, r0

    def delta_r(self, xyz, r_center):
        return self.k * (np.linalg.norm(xyz, axis=-1) - self.r0)


def test_relabelling_of_analytic_undulations(small_inputs):
    """Relabelling.cpp restated on fields with known answers: no undulation is no relabelling; a
    constant radial shift c has no gradient, so X = (1 / (1 + c/Z), 0, 0, 1) and the Jacobian is
    (1 + c/Z)^2; deltaR = k (r - r0) is linear in eta on a spherical element, so its radial
    derivative is k to rounding, its other derivatives vanish, X3 = 1 / (1 + k)."""
    from axisem3d_gb300 import relabelling as RL
    sim = solver.Simulation(small_inputs)
    spec = sim.build()
    E = spec.n_elements
    e = next(i for i in range(E) if not sim.axial_e[i] and not sim.fluid[i] and sim.ex.etype[i] == 0)
    pn = spec.p_nr[spec.e_pts[e]]
    nr = int(pn.max())
    args = (spec.e_geo[e].astype(np.float64), sim.crds[e], nr, pn, False, 0.0)
    assert RL.Relabelled([_Const(0.0)], *args).zero
    geo = None
    from axisem3d_gb300 import geometry as GEO
    geo, _, _, _, _ = GEO.batch_geometry(sim.nodes4[e:e + 1], sim.ex.etype[e:e + 1], sim.co[e:e + 1], sim.axial_e[e:e + 1])
    args = (geo[0], sim.crds[e], nr, pn, False, 0.0)
    Z = np.hypot(sim.crds[e, :, 0], sim.crds[e, :, 1])
    r_ = RL.Relabelled([_Const(1500.0)], *args)
    assert not r_.zero and r_.par1d()
    X = r_.stiff_x()
    np.testing.assert_allclose(X[0], np.broadcast_to(1 / (1 + 1500.0 / Z), X[0].shape), rtol=1e-9)
    assert np.abs(X[1]).max() < 1e-9 and np.abs(X[2]).max() < 1e-9
    np.testing.assert_allclose(X[3], 1.0, atol=1e-9)
    np.testing.assert_allclose(r_.stiff_jacobian(), np.broadcast_to((1 + 1500.0 / Z) ** 2, (nr, 25)), rtol=1e-9)
    r_ = RL.Relabelled([_Linear(0.01, 3.0e6)], *args)
    np.testing.assert_allclose(r_.dZdZ, 0.01, atol=1e-9)
    assert np.abs(r_.dZdR).max() < 1e-9 and np.abs(r_.dZdT).max() < 1e-9
    np.testing.assert_allclose(r_.stiff_x()[3], 1 / 1.01, rtol=1e-9)


def test_geometric_bump_builds_relabelled_elements(tmp_path_factory):
    """MODEL_3D_GEOMETRIC_LIST bump: an undulation centred on the source axis keeps the
    relabelled elements 1-D (PRT_1D), one off the axis makes them 3-D (PRT_3D) with per-slice
    moduli; the time loop runs on the oracle; an unknown model is refused."""
    from oracle.oracle_py import OracleDomain
    s1 = solver.Simulation(_bump_inputs(tmp_path_factory, "bump1", "0$0"))
    a = s1.build()
    assert len(s1.relab) > 0 and set(a.prt_len.tolist()) == {1} and not s1.e3d.any()
    s2 = solver.Simulation(_bump_inputs(tmp_path_factory, "bump2", "30$40"))
    b = s2.build()
    assert len(s2.relab) > 0 and (b.prt_len > 1).all() and s2.e3d[b.prt_elem].all()
    o = OracleDomain(b)
    o.step(60)
    seis = o.seismograms(0, 60)
    assert np.isfinite(seis).all() and np.abs(seis).max() > 0
    d = _bump_inputs(tmp_path_factory, "bump3", "0$0")
    from pathlib import Path
    pm = Path(d) / "inparam.model"
    pm.write_text(pm.read_text().replace("bump$", "crust1$"))
    with pytest.raises(NotImplementedError, match="crust1"):
        solver.Simulation(d).build()


@pytest.mark.gpu
def test_geometric_bump_gpu_matches_oracle(tmp_path_factory, ax3d_lib):
    """The full solver on a mesh relabelled by an off-axis bump of the surface (PRT_3D
    elements, per-slice moduli and masses from the relabelling Jacobians), GPU vs oracle."""
    from oracle.oracle_py import OracleDomain
    from axisem3d_gb300.capi import Ax3dDomain
    spec = solver.Simulation(_bump_inputs(tmp_path_factory, "bumpg", "30$40")).build()
    g, o = Ax3dDomain(spec), OracleDomain(spec)
    g.step(60)
    o.step(60)
    a, b = g.seismograms(0, 60), o.seismograms(0, 60)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    for which in ("displ", "veloc"):
        x, y = g.get(which, "solid"), o.get(which, "solid")
        assert np.linalg.norm(x - y) <= 1e-5 * np.linalg.norm(y)


@pytest.mark.gpu
def test_gpu_gaussian_random_sampling_matches_host(ax3d_lib):
    """ax3d_sample_gaussian_random (FP64 on the GPU) against the host evaluation of the same
    Gaussian-random model (FP32 phases, FP64 sum) on the rings of random GLL points, full 3-D
    and 2-D mode."""
    from axisem3d_gb300 import model3d as M3D
    m = M3D.GaussianRandom(["VS", "ref1d", "0.04", "500", "200", "7"], 6371e3)
    rng = np.random.default_rng(3)
    n, nr = 40, 37
    r = rng.uniform(3500e3, 6371e3, (n, 25))
    t = rng.uniform(0.0, np.pi, (n, 25))
    crds = np.stack([r * np.sin(t), r * np.cos(t)], -1)
    for phi2d in (None, 0.7):
        g = m.evaluate_rings_gpu(crds, nr, phi2d)
        phi = 2 * np.pi * np.arange(nr) / nr if phi2d is None else np.full(nr, phi2d)
        s, z = crds[..., 0], crds[..., 1]
        xyz = np.stack([s[:, None, :] * np.cos(phi)[None, :, None], s[:, None, :] * np.sin(phi)[None, :, None],
                        np.broadcast_to(z[:, None, :], (n, nr, 25))], -1)
        h, _ = m.evaluate(xyz)
        assert np.abs(g - h).max() <= 1e-5 * np.abs(h).max()
    # one call over elements of different slice counts (the solver's batched sampling)
    rows = rng.integers(1, 9, n)
    flat = m.evaluate_rows_gpu(crds, rows)
    ofs = np.concatenate([[0], np.cumsum(rows * 25)])
    assert len(flat) == ofs[-1]
    for e in range(n):
        np.testing.assert_array_equal(flat[ofs[e]:ofs[e + 1]].reshape(rows[e], 25),
                                      m.evaluate_rings_gpu(crds[e:e + 1], int(rows[e]))[0])


def test_hdf5_reader_on_a_written_file(tmp_path):
    """The HDF5 reader on a file written by the test's own minimal HDF5 writer: contiguous
    int32 / float64 / one-byte-string datasets, a compact dataset and chunked datasets with
    edge chunks through deflate, shuffle + deflate and shuffle + deflate + Fletcher-32 come
    back exact through netcdf.read."""
    from tests import _hdf5_writer as W
    rng = np.random.default_rng(5)
    conn = rng.integers(1, 2000, (37, 4)).astype("<i4")
    crd = rng.normal(size=101).astype("<f8")
    vals = rng.normal(size=(3, 29)).astype("<f8")
    names = np.zeros((3, 33), "S1")
    for i, s in enumerate(("r1", "solid_fluid_boundary", "t0")):
        names[i, :len(s)] = np.frombuffer(s.encode(), "S1")
    small = rng.integers(-5, 5, 7).astype("<i4")
    W.write(tmp_path / "m.e", {"connect1": (conn, (16, 4)), "coordx": crd, "ss_names": names,
                               "vals": (vals, (2, 8)), "coordy": (crd[::-1].copy(), (32,), ("shuffle", "deflate")),
                               "coordz": (crd * 2, (40,), ("shuffle", "deflate", "fletcher32")),
                               "eb_prop1": (small, "compact")})
    ds = NC.read(tmp_path / "m.e")
    np.testing.assert_array_equal(ds["connect1"], conn)
    np.testing.assert_array_equal(ds["coordx"], crd)
    np.testing.assert_array_equal(ds["coordy"], crd[::-1])
    np.testing.assert_array_equal(ds["coordz"], crd * 2)
    np.testing.assert_array_equal(ds["eb_prop1"], small)
    np.testing.assert_array_equal(ds["vals"], vals)
    assert ds.strings("ss_names") == ["r1", "solid_fluid_boundary", "t0"]
    assert ds.attrs["unread_datasets"] == []
    # two-level chunk B-trees (3 chunks per leaf) and object headers in two blocks
    big = rng.normal(size=(50, 7)).astype("<f8")
    W.write(tmp_path / "m2.e", {"vals": (big, (4, 3), ("shuffle", "deflate")), "connect1": (conn, (5, 4)),
                                "coordx": crd}, fanout=3, continuation=True)
    ds = NC.read(tmp_path / "m2.e")
    np.testing.assert_array_equal(ds["vals"], big)
    np.testing.assert_array_equal(ds["connect1"], conn)
    np.testing.assert_array_equal(ds["coordx"], crd)


def test_geographic_ellipticity_mode(tmp_path):
    """MODEL_3D_ELLIPTICITY_MODE geographic (ExodusModel.cpp:557-572, Geodesy.cpp:64-117,
    176-199): station and source latitudes become geocentric colatitudes with the flattening
    1 / MODEL_3D_ELLIPTICITY_INVF scaled by the mesh's ellipticity profile; off leaves them
    spherical; full (the ellipsoidal deformation of the mesh) is refused."""
    import math
    g = solver.Geodesy(6371e3, 1 / 299.8, [0.0, 0.5, 1.0], [0.7, 0.8, 1.0])
    assert g.flattening(6371e3) == pytest.approx(1 / 299.8)
    assert g.flattening(0.75 * 6371e3) == pytest.approx(0.9 / 299.8)
    t = g.lat2theta(45.0, 0.0)
    assert t == pytest.approx(math.pi / 2 - math.atan((1 - 1 / 299.8) ** 2))
    for lat in (-89.0, -30.0, 0.0, 12.5, 60.0):
        assert g.theta2lat(g.lat2theta(lat, 2e5), 2e5) == pytest.approx(lat, abs=1e-12)
    assert solver.Geodesy(6371e3).lat2theta(30.0, 0.0) == pytest.approx(math.radians(60.0))
    thetas = {}
    for mode in ("off", "geographic"):
        d = solver.write_inputs(tmp_path / mode, mesh_kw=SMALL_MESH, steps=10, nu=2, n_stations=6,
                                system="geographic")
        (d / "STATIONS").write_text("".join(f"S{i} XX {la:.3f} {lo:.3f} 0.0 0.0\n" for i, (la, lo) in
                                            enumerate([(45.0, 10.0), (-30.0, 60.0), (60.0, -120.0), (10.0, 170.0)])))
        p = d / "inparam.model"
        p.write_text(p.read_text() + f"MODEL_3D_ELLIPTICITY_MODE {mode}\nMODEL_3D_ELLIPTICITY_INVF 299.8\n")
        sim = solver.Simulation(d)
        sim.build()
        thetas[mode] = np.array([r[5] for r in sim.receivers])
        # the outputs name the geographic coordinates back (Receiver.cpp:38-39)
        np.testing.assert_allclose([r[2] for r in sim.receivers], [45.0, -30.0, 60.0, 10.0], atol=1e-9)
        np.testing.assert_allclose([r[3] for r in sim.receivers], [10.0, 60.0, -120.0, 170.0], atol=1e-9)
    diff = np.abs(thetas["geographic"] - thetas["off"])
    assert diff.max() > 1e-4 and diff.max() < 0.01  # at most ~1/300 rad of latitude shift
    d = solver.write_inputs(tmp_path / "full", mesh_kw=SMALL_MESH, steps=10, nu=2)
    p = d / "inparam.model"
    p.write_text(p.read_text() + "MODEL_3D_ELLIPTICITY_MODE full\nMODEL_3D_ELLIPTICITY_INVF 299.8\n")
    with pytest.raises(ValueError, match="full"):
        solver.Simulation(d).build()
