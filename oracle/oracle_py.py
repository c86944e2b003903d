"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded only by tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py.
OracleDomain drives oracle/_build/libax3d_oracle.so through the same Domain API as
axisem3d_gb300.capi.Ax3dDomain, in FP32 (the reference's default Real) or FP64.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from axisem3d_gb300.capi import _DomainBase, bind

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libax3d_oracle.so"
_lib = None


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load_oracle() -> C.CDLL:
    global _lib
    if _lib is None:
        srcs = [HERE / "ax3d_oracle.hpp", HERE / "ax3d_oracle_capi.cpp"]
        if not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
            build_oracle()
        lib = C.CDLL(str(LIB))
        bind(lib, "axo_", C.POINTER(C.c_double), extra_double_io=True)
        bind(lib, "axod_", C.POINTER(C.c_double), extra_double_io=True)
        lib.axo_last_error.argtypes = [C.c_char_p, C.c_size_t]
        lib.axo_last_error.restype = C.c_size_t
        _lib = lib
    return _lib


class OracleDomain(_DomainBase):
    """The oracle's Domain: Real = float (default) or double."""

    err_name = "axo_last_error"
    field_dtype = np.float64
    field_ctype = C.c_double

    def __init__(self, spec, double: bool = False):
        self.prefix = "axod_" if double else "axo_"
        self.lib = load_oracle()
        self._build(spec, 0, with_first=False)
