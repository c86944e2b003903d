"""ctypes binding of the GB300 C-ABI (include/ax3d.h) and a Domain object on top of it.

`Ax3dDomain` is the Python face of the reference's Domain (SOLVER/src/core/domain/Domain.h):
`update_newmark`, `apply_source`, `compute_stiff`, `couple_solid_fluid`, `record` map
one-to-one onto Domain's loop bodies, `step(n)` runs Newmark::solve's loop body n times.
Errors raise Ax3dError with the library's message, like the reference's
std::runtime_error("Class::method || msg").  There is no fallback: if libax3d.so is
missing or no GPU is present the constructor raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from .spec import DomainSpec, g_matrices

LIB_PATH = Path(__file__).resolve().parent / "libax3d.so"

AX3D_OK = 0
ERRORS = {1: "ARG", 2: "STATE", 3: "CUDA", 4: "UNSTABLE", 5: "NOMEM", 6: "UNSUPPORTED", 7: "TIMEOUT"}
FIELD = {"displ": 0, "veloc": 1, "accel": 2, "stiff": 3}
PHASE = {"solid": 0, "fluid": 1}


class Ax3dError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("npol", C.c_int32), ("dt", C.c_double),
                ("g_gll", C.POINTER(C.c_double)), ("g_glj", C.POINTER(C.c_double)),
                ("nsls", C.c_int32), ("att_alpha", C.POINTER(C.c_double)),
                ("att_beta", C.POINTER(C.c_double)), ("att_gamma", C.POINTER(C.c_double)),
                ("att_do_kappa", C.c_int32), ("kahan", C.c_int32),
                ("stability_interval", C.c_int32), ("device", C.c_int32)]


def _p(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


P_I32, P_I64, P_F32, P_F64, P_I8, P_U8 = (C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_float),
                                          C.POINTER(C.c_double), C.POINTER(C.c_int8), C.POINTER(C.c_uint8))


def bind(lib: C.CDLL, prefix: str, field_ctype, extra_double_io: bool = False):
    """Declare the C signatures of one implementation of the ax3d API."""
    f = lambda n: getattr(lib, prefix + n)
    f("create").argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    f("add_points").argtypes = [C.c_void_p, C.c_int32, P_I32, P_I8, P_U8, P_U8, P_I32, P_F32, P_I32, P_F32,
                                P_I32, P_F32, P_F32] + ([] if extra_double_io else [P_I32])
    f("add_elements").argtypes = [C.c_void_p, C.c_int32, P_I32, P_I8, P_U8, P_U8, P_F32, P_F32, P_I64, P_F32,
                                  P_I8, P_I64, P_F32] + ([] if extra_double_io else [P_I32])
    f("add_source").argtypes = [C.c_void_p, C.c_int32, C.c_int32, P_F32]
    f("set_stf").argtypes = [C.c_void_p, C.c_int32, P_F32]
    f("add_receivers").argtypes = [C.c_void_p, C.c_int32, P_I32, P_F32, P_F32]
    f("finalize").argtypes = [C.c_void_p]
    f("field_size").argtypes = [C.c_void_p, C.c_int32]
    f("field_size").restype = C.c_int64
    f("get_field").argtypes = [C.c_void_p, C.c_int32, C.c_int32, field_ctype]
    f("set_field").argtypes = [C.c_void_p, C.c_int32, C.c_int32, field_ctype]
    for n in ("update_newmark", "compute_stiff", "couple_solid_fluid", "reset", "destroy"):
        f(n).argtypes = [C.c_void_p]
    for n in ("apply_source", "record", "step"):
        f(n).argtypes = [C.c_void_p, C.c_int32]
    f("read_seismograms").argtypes = [C.c_void_p, C.c_int32, C.c_int32, field_ctype]
    f("current_step").argtypes = [C.c_void_p]
    f("current_step").restype = C.c_int32
    f("set_wisdom_learning").argtypes = [C.c_void_p, C.c_int32, C.c_float]
    f("learn_wisdom").argtypes = [C.c_void_p, C.c_float]
    f("get_wisdom").argtypes = [C.c_void_p, P_I32]
    f("add_surface").argtypes = [C.c_void_p, C.c_int32, P_I32, P_I32, C.c_int32]
    f("set_field_async").argtypes = [C.c_void_p, C.c_int32, C.c_int32, field_ctype]
    f("get_field_async").argtypes = [C.c_void_p, C.c_int32, C.c_int32, field_ctype]
    f("sync_fields").argtypes = [C.c_void_p]
    f("set_prt").argtypes = [C.c_void_p, C.c_int32, P_I32, P_I32, C.POINTER(C.c_float)]
    f("set_receiver_dumps").argtypes = [C.c_void_p, C.c_int32, P_I32]
    f("read_strain_curl").argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, field_ctype]
    f("add_ocean_load").argtypes = [C.c_void_p, C.c_int32, P_I32, P_I32, C.POINTER(C.c_float)]
    f("surface_record_size").argtypes = [C.c_void_p]
    f("surface_record_size").restype = C.c_int64
    f("read_surface").argtypes = [C.c_void_p, C.c_int32, C.c_int32, field_ctype]


_LIB = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libax3d.so (built by axisem3d_gb300.build); raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise Ax3dError(6, f"{p} is missing: run `python -m axisem3d_gb300.build` (needs nvcc)")
    lib = C.CDLL(str(p))
    bind(lib, "ax3d_", P_F32)
    lib.ax3d_last_error.argtypes = [C.c_char_p, C.c_size_t]
    lib.ax3d_last_error.restype = C.c_size_t
    lib.ax3d_enable_timers.argtypes = [C.c_void_p, C.c_int32]
    lib.ax3d_autotune.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_size_t]
    lib.ax3d_set_schedule.argtypes = [C.c_void_p, C.c_double, C.c_int32, C.c_int32, C.c_int32]
    lib.ax3d_read_timers.argtypes = [C.c_void_p, P_F64, P_I64]
    if path is None:
        _LIB = lib
    return lib


class _DomainBase:
    """Shared driver of one ax3d-API implementation (prefix + element type)."""

    prefix = "ax3d_"
    err_name = "ax3d_last_error"
    field_dtype = np.float32
    field_ctype = C.c_float

    def _err(self) -> str:
        buf = C.create_string_buffer(1024)
        getattr(self.lib, self.err_name)(buf, 1024)
        return buf.value.decode(errors="replace")

    def _ck(self, rc: int):
        if rc != AX3D_OK:
            raise Ax3dError(rc, self._err())

    def _call(self, name, *args):
        return getattr(self.lib, self.prefix + name)(*args)

    def _build(self, spec: DomainSpec, device: int, with_first: bool):
        self.spec = spec
        gll, glj = g_matrices()
        self._keep = [gll, glj]
        a = np.ascontiguousarray(spec.att_alpha, np.float64)
        b = np.ascontiguousarray(spec.att_beta, np.float64)
        g = np.ascontiguousarray(spec.att_gamma, np.float64)
        self._keep += [a, b, g]
        cfg = Config(4, float(spec.dt), _p(gll, C.c_double), _p(glj, C.c_double), int(spec.nsls),
                     _p(a, C.c_double), _p(b, C.c_double), _p(g, C.c_double), int(bool(spec.att_do_kappa)),
                     int(bool(spec.kahan)), int(spec.stability_interval), int(device))
        h = C.c_void_p()
        self._ck(self._call("create", C.byref(cfg), C.byref(h)))
        self.h = h
        c = np.ascontiguousarray
        first = C.c_int32()
        extra = [C.byref(first)] if with_first else []
        self._ck(self._call(
            "add_points", h, spec.n_points, _p(c(spec.p_nr, np.int32), C.c_int32),
            _p(c(spec.p_kind, np.int8), C.c_int8), _p(c(spec.p_axial, np.uint8), C.c_uint8),
            _p(c(spec.p_fsurf, np.uint8), C.c_uint8), _p(c(spec.p_mslen, np.int32), C.c_int32),
            _p(c(spec.p_ms, np.float32), C.c_float), _p(c(spec.p_mflen, np.int32), C.c_int32),
            _p(c(spec.p_mf, np.float32), C.c_float), _p(c(spec.p_sflen, np.int32), C.c_int32),
            _p(c(spec.p_sfn, np.float32), C.c_float), _p(c(spec.p_sfni, np.float32), C.c_float), *extra))
        self._ck(self._call(
            "add_elements", h, spec.n_elements, _p(c(spec.e_pts, np.int32), C.c_int32),
            _p(c(spec.e_mat, np.int8), C.c_int8), _p(c(spec.e_axial, np.uint8), C.c_uint8),
            _p(c(spec.e_in3d, np.uint8), C.c_uint8), _p(c(spec.e_geo, np.float32), C.c_float),
            _p(c(spec.e_trig, np.float32), C.c_float), _p(c(spec.e_mofs, np.int64), C.c_int64),
            _p(c(spec.e_mod, np.float32), C.c_float), _p(c(spec.e_att, np.int8), C.c_int8),
            _p(c(spec.e_aofs, np.int64), C.c_int64), _p(c(spec.e_attm, np.float32), C.c_float), *extra))
        for elem, force in spec.sources:
            f = c(np.asarray(force, np.complex64).view(np.float32))
            self._ck(self._call("add_source", h, int(elem), int(force.shape[1]), _p(f, C.c_float)))
        stf = c(spec.stf, np.float32)
        self._ck(self._call("set_stf", h, len(stf), _p(stf, C.c_float)))
        if len(spec.r_elem):
            self._ck(self._call("add_receivers", h, len(spec.r_elem), _p(c(spec.r_elem, np.int32), C.c_int32),
                                _p(c(spec.r_phi, np.float32), C.c_float), _p(c(spec.r_w, np.float32), C.c_float)))
        if len(spec.prt_elem):
            self._ck(self._call("set_prt", h, len(spec.prt_elem), _p(c(spec.prt_elem, np.int32), C.c_int32),
                                _p(c(spec.prt_len, np.int32), C.c_int32), _p(c(spec.prt_x, np.float32), C.c_float)))
        if len(spec.r_dump) and np.any(spec.r_dump):
            self._ck(self._call("set_receiver_dumps", h, len(spec.r_dump), _p(c(spec.r_dump, np.int32), C.c_int32)))
        if len(spec.oc_pt):
            self._ck(self._call("add_ocean_load", h, len(spec.oc_pt), _p(c(spec.oc_pt, np.int32), C.c_int32),
                                _p(c(spec.oc_len, np.int32), C.c_int32), _p(c(spec.oc_vals, np.float32), C.c_float)))
        if len(spec.sf_elem):
            self._ck(self._call("add_surface", h, len(spec.sf_elem), _p(c(spec.sf_elem, np.int32), C.c_int32),
                                _p(c(spec.sf_side, np.int32), C.c_int32), int(spec.sf_interval)))
        self._ck(self._call("finalize", h))
        self.nsolid = int(self._call("field_size", h, 0))
        self.nfluid = int(self._call("field_size", h, 1))

    # ---- Domain API ----
    def step(self, n: int = 1):
        self._ck(self._call("step", self.h, int(n)))

    def update_newmark(self):
        self._ck(self._call("update_newmark", self.h))

    def apply_source(self, tstep: int):
        self._ck(self._call("apply_source", self.h, int(tstep)))

    def compute_stiff(self):
        self._ck(self._call("compute_stiff", self.h))

    def couple_solid_fluid(self):
        self._ck(self._call("couple_solid_fluid", self.h))

    def record(self, tstep: int):
        self._ck(self._call("record", self.h, int(tstep)))

    def reset(self):
        self._ck(self._call("reset", self.h))

    @property
    def current_step(self) -> int:
        return int(self._call("current_step", self.h))

    def set_wisdom_learning(self, interval: int, cutoff: float):
        """Domain::learnWisdom every `interval` steps during step() (NU_WISDOM_LEARN_INTERVAL/_EPSILON)."""
        self._ck(self._call("set_wisdom_learning", self.h, int(interval), float(cutoff)))

    def learn_wisdom(self, cutoff: float):
        self._ck(self._call("learn_wisdom", self.h, float(cutoff)))

    def get_wisdom(self) -> np.ndarray:
        """Per point Nu wisdom (SolidPoint::getNuWisdom)."""
        out = np.zeros(max(self.spec.n_points, 1), np.int32)
        self._ck(self._call("get_wisdom", self.h, _p(out, C.c_int32)))
        return out[:self.spec.n_points]

    @property
    def complex_dtype(self):
        return np.complex64 if self.field_dtype == np.float32 else np.complex128

    def get(self, which: str = "displ", phase: str = "solid", out: np.ndarray | None = None) -> np.ndarray:
        """Copy a field to the host as complex64 (GPU) / complex128 (FP64 oracle) values."""
        n = self.nsolid if phase == "solid" else self.nfluid
        if out is None:
            out = np.zeros(max(n, 1), self.complex_dtype)
        buf = out.view(self.field_dtype)
        self._ck(self._call("get_field", self.h, FIELD[which], PHASE[phase], _p(buf, self.field_ctype)))
        return out[:n]

    def set(self, which: str, phase: str, values: np.ndarray):
        n = self.nsolid if phase == "solid" else self.nfluid
        v = np.ascontiguousarray(values, self.complex_dtype)
        if v.size != n:
            raise ValueError(f"field size {v.size} != {n}")
        buf = v.view(self.field_dtype)
        self._ck(self._call("set_field", self.h, FIELD[which], PHASE[phase], _p(buf, self.field_ctype)))

    def set_async(self, which: str, phase: str, values: np.ndarray):
        """Queue `values` (keep it alive and unchanged, ideally pinned, until sync_fields) as
        the field the next step() starts from; at most two queued."""
        n = self.nsolid if phase == "solid" else self.nfluid
        if values.dtype != self.complex_dtype or not values.flags.c_contiguous or values.size != n:
            raise ValueError("set_async needs a contiguous array of the field's dtype and size")
        self._ck(self._call("set_field_async", self.h, FIELD[which], PHASE[phase],
                            _p(values.view(self.field_dtype), self.field_ctype)))

    def get_async(self, which: str, phase: str, out: np.ndarray):
        """Snapshot the field after the steps enqueued so far into `out` (complete after
        sync_fields)."""
        n = self.nsolid if phase == "solid" else self.nfluid
        if out.dtype != self.complex_dtype or not out.flags.c_contiguous or out.size < n:
            raise ValueError("get_async needs a contiguous array of the field's dtype and size")
        self._ck(self._call("get_field_async", self.h, FIELD[which], PHASE[phase],
                            _p(out.view(self.field_dtype), self.field_ctype)))

    def sync_fields(self):
        self._ck(self._call("sync_fields", self.h))

    def strain_curl(self, which: str, first: int, n: int) -> np.ndarray:
        """Strain ([n][strain receivers][6], RTZ) or curl ([n][curl receivers][3]) of steps
        first..first+n-1 for the receivers flagged dump_strain / dump_curl."""
        bit, k = (1, 6) if which == "strain" else (2, 3)
        nrec = int(np.count_nonzero(np.asarray(self.spec.r_dump, np.int32) & bit)) if len(self.spec.r_dump) else 0
        out = np.zeros(max(n * nrec * k, 1), self.field_dtype)
        self._ck(self._call("read_strain_curl", self.h, 0 if bit == 1 else 1, int(first), int(n),
                            _p(out, self.field_ctype)))
        return out[:n * nrec * k].astype(np.float64).reshape(n, nrec, k)

    def seismograms(self, first: int, n: int) -> np.ndarray:
        nrec = len(self.spec.r_elem)
        out = np.zeros(max(n * nrec * 3, 1), self.field_dtype)
        self._ck(self._call("read_seismograms", self.h, int(first), int(n), _p(out, self.field_ctype)))
        return out[:n * nrec * 3].astype(np.float64).reshape(n, nrec, 3)

    def surface(self, first: int, n: int) -> list[np.ndarray]:
        """Whole-surface records first..first+n-1 (SurfaceRecorder): one complex array per
        edge, shaped [n][3][5][Nu_e + 1] ([component][point on the side][order])."""
        row = int(self._call("surface_record_size", self.h))
        out = np.zeros(max(n * row, 1), self.complex_dtype)
        self._ck(self._call("read_surface", self.h, int(first), int(n), _p(out.view(self.field_dtype),
                                                                             self.field_ctype)))
        out = out[:n * row].reshape(n, row)
        edges, ofs = [], 0
        for e in self.spec.sf_elem:
            na = int(self.spec.element_nr()[e]) // 2 + 1
            edges.append(out[:, ofs:ofs + 15 * na].reshape(n, 3, 5, na))
            ofs += 15 * na
        return edges

    def close(self):
        if getattr(self, "h", None):
            self._call("destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


TIMERS = ("step", "elements", "points", "assemble", "couple", "source", "record", "other")


class Ax3dDomain(_DomainBase):
    """A domain resident on one GB300, driven through libax3d.so."""

    def __init__(self, spec: DomainSpec, device: int = 0, lib: C.CDLL | None = None):
        self.lib = lib or load_library()
        self._build(spec, device, with_first=True)

    def autotune(self, trials: int = 2) -> str:
        """ax3d_autotune: the physical-space bucket schedule from timed element passes on this
        domain (cached per process by shape); returns the library's report."""
        buf = C.create_string_buffer(4096)
        self._ck(self.lib.ax3d_autotune(self.h, int(trials), buf, 4096))
        return buf.value.decode()

    def set_schedule(self, ratio: float = 1.12, policy: int = 0, nside: int = 3, merge: bool = False):
        """ax3d_set_schedule: the physical-space bucket schedule, by hand."""
        self._ck(self.lib.ax3d_set_schedule(self.h, float(ratio), int(policy), int(nside), int(merge)))

    def enable_timers(self, on: bool = True):
        self._ck(self.lib.ax3d_enable_timers(self.h, int(on)))

    def read_timers(self) -> dict:
        """{phase: (device ms, kernel launches)} accumulated since the last read."""
        ms = np.zeros(len(TIMERS))
        n = np.zeros(len(TIMERS), np.int64)
        self._ck(self.lib.ax3d_read_timers(self.h, _p(ms, C.c_double), _p(n, C.c_int64)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(TIMERS)}
