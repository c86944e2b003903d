"""The entry point that allocates nothing, against the domain path.

Callers that cannot allocate device memory (their own pre-sized pool, or no allocation
once a run has started) call ax3d_compute_stiff_iso1d_noalloc with their own buffers.
This test gives it buffers made by torch, makes the start-up call (nelem = 0) that loads
the scratch and the kernels, runs it twice in a row on different displacements and
compares each result with ax3d_compute_stiff on the same mesh and with the CPU oracle, at
the tolerance of the other parity tests (relative L2 <= 1e-5); the device's free memory
and torch's allocated bytes must not move across the second call.
"""
import ctypes as C

import numpy as np
import pytest

from axisem3d_gb300 import synth
from axisem3d_gb300.spec import ATT_NONE, MAT_ISO, g_matrices

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_stiffness_matches_domain_path():
    import torch
    from axisem3d_gb300 import build, capi
    build.build()
    lib = capi.load_library()
    fn = lib.ax3d_compute_stiff_iso1d_noalloc
    fn.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                   C.POINTER(C.c_double), C.c_void_p]

    nu = 3
    spec = synth.annulus_domain(seed=4, n_theta=5, n_r=3, nu=nu, mat=MAT_ISO, att=ATT_NONE, source=False,
                                n_receivers=0)
    ne, npt = spec.n_elements, spec.n_points
    dom = capi.Ax3dDomain(spec)

    # caller-owned device buffers
    dev = torch.device("cuda:0")
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    pts = t(spec.e_pts, torch.int32)
    axial = t(spec.e_axial, torch.uint8)
    geo = t(spec.e_geo, torch.float32)
    lm = t(spec.e_mod.reshape(ne, 2, 25), torch.float32)
    refs = [[] for _ in range(npt)]
    for e in range(ne):
        for l in range(25):
            refs[spec.e_pts[e, l]].append(e * 25 + l)
    gptr = t(np.concatenate([[0], np.cumsum([len(r) for r in refs])]), torch.int32)
    gref = t(np.concatenate([np.array(r, np.int64) for r in refs]), torch.int32)
    gll, glj = g_matrices()
    pg = gll.ctypes.data_as(C.POINTER(C.c_double))
    pj = glj.ctypes.data_as(C.POINTER(C.c_double))

    from oracle.oracle_py import OracleDomain
    orc = OracleDomain(spec)

    # start-up call: loads the scratch and the kernels on this device, launches nothing
    assert fn(0, nu, None, None, None, None, 0, None, None, None, None, pg, pj, None) == 0

    for k, seed in enumerate((21, 22)):  # two calls in a row share (and overwrite) the static scratch
        u, _ = synth.random_fields(spec, seed=seed)
        dom.set("displ", "solid", u)
        dom.set("stiff", "solid", np.zeros_like(u))
        dom.compute_stiff()
        ref = dom.get("stiff")
        orc.set("displ", "solid", u)
        orc.set("stiff", "solid", np.zeros_like(u))
        orc.compute_stiff()
        du = t(u.astype(np.complex64).view(np.float32), torch.float32)
        st = torch.zeros(2 * u.size, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        free0, alloc0 = torch.cuda.mem_get_info(dev)[0], torch.cuda.memory_allocated(dev)
        rc = fn(ne, nu, pts.data_ptr(), axial.data_ptr(), geo.data_ptr(), lm.data_ptr(), npt, gptr.data_ptr(),
                gref.data_ptr(), du.data_ptr(), st.data_ptr(), pg, pj, None)
        assert rc == 0, rc
        torch.cuda.synchronize()
        if k == 1:  # after the first real call nothing on the device may grow
            assert torch.cuda.mem_get_info(dev)[0] == free0
            assert torch.cuda.memory_allocated(dev) == alloc0
        got = st.cpu().numpy().view(np.complex64)
        assert _rel(got, ref) <= TOL, _rel(got, ref)
        want = orc.get("stiff", "solid")
        assert _rel(got, want) <= TOL, _rel(got, want)


def test_noalloc_rejects_oversized_batch():
    from axisem3d_gb300 import capi
    lib = capi.load_library()
    fn = lib.ax3d_compute_stiff_iso1d_noalloc
    fn.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 4 + [C.c_int32] + [C.c_void_p] * 4 + \
        [C.POINTER(C.c_double)] * 2 + [C.c_void_p]
    gll, glj = g_matrices()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = fn(1_000_000, 256, dummy, dummy, dummy, dummy, 10, dummy, dummy, dummy, dummy,
            gll.ctypes.data_as(C.POINTER(C.c_double)), glj.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == 1
    buf = C.create_string_buffer(512)
    lib.ax3d_last_error(buf, 512)
    assert b"static scratch" in buf.value
    odd = C.c_void_p(20)  # not 8-byte aligned: refused before any launch
    rc = fn(1, 1, dummy, dummy, dummy, dummy, 10, dummy, dummy, odd, dummy,
            gll.ctypes.data_as(C.POINTER(C.c_double)), glj.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == 1
    lib.ax3d_last_error(buf, 512)
    assert b"aligned" in buf.value
