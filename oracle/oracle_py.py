"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded only by tests/, __graft_entry__.smoke() and the CPU legs of bench.py.
OracleDomain drives oracle/_build/libax3d_oracle.so (the checker: exact DFT) through the
same Domain API as axisem3d_gb300.capi.Ax3dDomain, in FP32 (the reference's default Real)
or FP64; with fft=True it drives oracle/_build/libax3d_cpufft.so instead, the same loop
with O(nr log nr) FP32 transforms, which bench.py times as the CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from axisem3d_gb300.capi import _DomainBase, bind

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libax3d_oracle.so"
LIB_FFT = HERE / "_build" / "libax3d_cpufft.so"
_libs = {}


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-j2", "-C", str(HERE)], check=True)
    return LIB


def load_oracle(fft: bool = False) -> C.CDLL:
    if fft not in _libs:
        path = LIB_FFT if fft else LIB
        srcs = [HERE / n for n in ("ax3d_oracle.hpp", "ax3d_oracle_capi.cpp", "ax3d_fft.hpp", "ax3d_oracle_preloop.hpp")]
        if not path.exists() or any(s.stat().st_mtime > path.stat().st_mtime for s in srcs):
            build_oracle()
        lib = C.CDLL(str(path))
        bind(lib, "axo_", C.POINTER(C.c_double), extra_double_io=True)
        bind(lib, "axod_", C.POINTER(C.c_double), extra_double_io=True)
        lib.axo_last_error.argtypes = [C.c_char_p, C.c_size_t]
        lib.axo_last_error.restype = C.c_size_t
        if fft:
            for n in ("axf_c2r_pair", "axf_r2c_pair"):
                getattr(lib, n).argtypes = [C.c_int32] + [C.POINTER(C.c_float)] * 4
        _libs[fft] = lib
    return _libs[fft]


def fft_pair(nr: int, X1: np.ndarray, X2: np.ndarray):
    """The CPU baseline's C2R of two Hermitian columns (orders 0..nr/2) -> two real columns."""
    lib = load_oracle(fft=True)
    a = np.ascontiguousarray(X1, np.complex64)
    b = np.ascontiguousarray(X2, np.complex64)
    x1, x2 = np.zeros(nr, np.float32), np.zeros(nr, np.float32)
    f = lambda v: v.ctypes.data_as(C.POINTER(C.c_float))
    lib.axf_c2r_pair(nr, f(a.view(np.float32)), f(b.view(np.float32)), f(x1), f(x2))
    return x1, x2


def ifft_pair(x1: np.ndarray, x2: np.ndarray):
    """The CPU baseline's R2C (x 1/nr) of two real columns -> orders 0..nr/2 of each."""
    lib = load_oracle(fft=True)
    nr = len(x1)
    a = np.ascontiguousarray(x1, np.float32)
    b = np.ascontiguousarray(x2, np.float32)
    X1, X2 = np.zeros(nr // 2 + 1, np.complex64), np.zeros(nr // 2 + 1, np.complex64)
    f = lambda v: v.ctypes.data_as(C.POINTER(C.c_float))
    lib.axf_r2c_pair(nr, f(a), f(b), f(X1.view(np.float32)), f(X2.view(np.float32)))
    return X1, X2


class OracleDomain(_DomainBase):
    """The oracle's Domain: Real = float (default) or double."""

    err_name = "axo_last_error"
    field_dtype = np.float64
    field_ctype = C.c_double

    def __init__(self, spec, double: bool = False, fft: bool = False):
        if double and fft:
            raise ValueError("the FFT CPU baseline is FP32 only")
        self.prefix = "axod_" if double else "axo_"
        self.lib = load_oracle(fft=fft)
        self._build(spec, 0, with_first=False)


def seismograms_of_inputs(input_dir, nsteps: int, double: bool = False, kahan: bool = False) -> np.ndarray:
    """Build the domain of a parfile directory and run the oracle for nsteps; returns the
    seismograms [step][receiver][component].  A module-level function, so that tests can
    run it in spawned worker processes beside the GPU run."""
    from axisem3d_gb300 import solver
    spec = solver.Simulation(input_dir).build(kahan=kahan)
    o = OracleDomain(spec, double=double)
    o.step(nsteps)
    return o.seismograms(0, nsteps)


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def pre_geometry(nodes, etype, co, axial, spectral):
    """FP64 Quad::createGraident + formIntegralFactor: geo [n,5,25], ifact [n,25], crds [n,25,2]."""
    lib = load_oracle()
    n = len(etype)
    nodes = np.ascontiguousarray(nodes, np.float64)
    et = np.ascontiguousarray(etype, np.int8)
    cc = np.ascontiguousarray(co, np.int8)
    ax = np.ascontiguousarray(axial, np.uint8)
    sp = np.ascontiguousarray(spectral, np.float64)
    geo, ifact, crds = np.zeros((n, 5, 25)), np.zeros((n, 25)), np.zeros((n, 25, 2))
    lib.axo_pre_geometry(C.c_int32(n), _pd(nodes), et.ctypes.data_as(C.c_void_p), cc.ctypes.data_as(C.c_void_p),
                         ax.ctypes.data_as(C.c_void_p), _pd(sp), _pd(geo), _pd(ifact), _pd(crds))
    return geo, ifact, crds


def pre_mass(rows, ifact, rho, vp, fluid):
    """FP64 Material::computeElementalMass; rho, vp flat [sum rows * 25]."""
    lib = load_oracle()
    rows = np.ascontiguousarray(rows, np.int32)
    ifact = np.ascontiguousarray(ifact, np.float64)
    rho = np.ascontiguousarray(rho, np.float64)
    vp = np.ascontiguousarray(vp if vp is not None else np.ones_like(rho), np.float64)
    fl = np.ascontiguousarray(fluid, np.uint8)
    mass = np.zeros(int(rows.sum()) * 25)
    lib.axo_pre_mass(C.c_int32(len(rows)), rows.ctypes.data_as(C.c_void_p), _pd(ifact), _pd(rho), _pd(vp),
                     fl.ctypes.data_as(C.c_void_p), _pd(mass))
    return mass


def pre_elastic(rows, ifact, model, iso, att, fit=None):
    """FP64 Material::createElastic (+ AttBuilder, AttAxiSEM).  model: list over elements of
    [8][rows][25] arrays (vpv, vph, vsv, vsh, eta, rho, qkappa, qmu).  fit: (w, y, f_min,
    f_max, f_ref, do_kappa).  Returns flat moduli and attenuation moduli."""
    lib = load_oracle()
    rows = np.ascontiguousarray(rows, np.int32)
    ifact = np.ascontiguousarray(ifact, np.float64)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(m, np.float64).reshape(-1) for m in model]))
    km, npa = (2 if iso else 5), (4 if att == 2 else 25)
    mod = np.zeros(int(rows.sum()) * 25 * km)
    attm = np.zeros(max(1, int(rows.sum()) * 2 * npa if att else 1))
    w, y, fmin, fmax, fref, dk = fit if fit is not None else (np.zeros(1), np.zeros(1), 1.0, 1.0, 1.0, True)
    w = np.ascontiguousarray(w, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    lib.axo_pre_elastic(C.c_int32(len(rows)), rows.ctypes.data_as(C.c_void_p), _pd(ifact), _pd(flat),
                        C.c_int32(int(iso)), C.c_int32(att), C.c_int32(len(w)), _pd(w), _pd(y), C.c_double(fmin),
                        C.c_double(fmax), C.c_double(fref), C.c_int32(int(dk)), _pd(mod), _pd(attm))
    return mod, attm[: int(rows.sum()) * 2 * npa] if att else np.zeros(0)
