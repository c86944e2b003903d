"""Volumetric 3-D models: the MODEL_3D_VOLUMETRIC_LIST entries of inparam.model.

Each entry is "name$param1$param2...", split on '$' (Volumetric3D::buildInparam,
SOLVER/src/3d_model/3d_volumetric/Volumetric3D.cpp:23-95).  A model returns, for points
given in the source-centred Cartesian frame, a value and an in-range mask; the caller
applies it to one material property with one of the four reference types
(Material::addVolumetric3D, SOLVER/src/preloop/physics/material/Material.cpp:125-212):

    Absolute          X = value (SI)
    Reference1D       X = X1D * (1 + value)
    Reference3D       X = X * (1 + value)
    ReferencePerturb  X = (X - X1D) * (1 + value) + X1D

Built models:
  bubble           SOLVER/src/3d_model/3d_volumetric/simple_shapes/Volumetric3D_bubble.cpp:11-137
                   bubble$PROP$REF$value$radius_km$depth_km$lat$lon[$src_centred$fluid$hwhm_km]
  gaussian_random  a seeded stationary Gaussian random field (a synthetic stand-in for
                   tomography models whose data files are not shipped):
                   gaussian_random$PROP$REF$rms$lateral_corr_km$radial_corr_km$seed[$fluid]
PROP is VP, VS or RHO (VP/VS act on both the vertical and horizontal velocities).
"""
from __future__ import annotations

import math
import os

import numpy as np

PROPS = ("VP", "VS", "RHO")
REFS = {"absolute": 0, "abs": 0, "reference1d": 1, "ref1d": 1, "reference3d": 2, "ref3d": 2,
        "referenceperturb": 3, "refptb": 3}
ABS_SI = {"VP": 1e3, "VS": 1e3, "RHO": 1e3}   # km/s, g/cm^3 -> SI (MaterialPropertyAbsSI)


def _truthy(s):
    return s.strip().lower() in ("true", "1", "yes", "on")


def _rotation(theta, phi):
    ct, st, cp, sp = math.cos(theta), math.sin(theta), math.cos(phi), math.sin(phi)
    return np.array([[ct * cp, -sp, st * cp], [ct * sp, cp, st * sp], [-st, 0.0, ct]])


class Model3D:
    prop = "VP"
    ref = 1
    fluid = False

    def _head(self, params, name, nmin):
        if len(params) < nmin:
            raise ValueError(f"Volumetric3D_{name}::initialize || need at least {nmin} parameters")
        prop = params[0].strip().upper()
        if prop not in PROPS:
            raise ValueError(f"Volumetric3D_{name}::initialize || Unknown material property, name = {params[0]}")
        ref = params[1].strip().lower()
        if ref not in REFS:
            raise ValueError(f"Volumetric3D_{name}::initialize || Unknown material reference type, type = {params[1]}")
        self.prop, self.ref = prop, REFS[ref]

    def evaluate(self, xyz):
        """xyz: (..., 3) source-frame Cartesian [m] -> (value, in_range), both shaped (...)."""
        raise NotImplementedError


def _spherical_colat(lat_deg, depth):
    return math.radians(90.0 - lat_deg)


class Bubble(Model3D):
    def __init__(self, params, src, R, lat2theta=None):
        """src = (latitude, longitude[, depth m]); lat2theta(lat, depth) the geodesy's
        geographic latitude -> geocentric colatitude (spherical when None)."""
        self._head(params, "bubble", 7)
        value, radius, depth, lat, lon = (float(p) for p in params[2:7])
        self.value, self.radius = value, radius * 1e3
        src_centred = _truthy(params[7]) if len(params) > 7 else False
        self.fluid = _truthy(params[8]) if len(params) > 8 else False
        hwhm = float(params[9]) * 1e3 if len(params) > 9 else -1.0
        r = R - depth * 1e3
        if src_centred:
            t, p = math.radians(lat), math.radians(lon)
            self.center = r * np.array([math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t)])
        else:
            l2t = lat2theta or _spherical_colat
            t, p = l2t(lat, depth * 1e3), math.radians(lon % 360)
            xg = r * np.array([math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t)])
            slat, slon = src[0], src[1]
            sdep = src[2] if len(src) > 2 else 0.0
            self.center = _rotation(l2t(slat, sdep), math.radians(slon % 360)).T @ xg
        self.hwhm = self.radius * 0.2 if hwhm < 0 else hwhm
        if self.ref == 0:
            self.hwhm = 0.0
            self.value *= ABS_SI[self.prop]

    def evaluate(self, xyz):
        d = np.linalg.norm(xyz - self.center, axis=-1) - self.radius
        d = np.maximum(d, 0.0)
        inr = d <= 4.0 * self.hwhm
        if self.hwhm > 0:
            sd = self.hwhm / math.sqrt(2.0 * math.log(2.0))
            val = self.value * np.exp(-d * d / (2.0 * sd * sd))
        else:
            val = np.full(d.shape, self.value)
        return np.where(inr, val, 0.0), inr


class GaussianRandom(Model3D):
    """delta(x) = rms sqrt(2/M) sum_j cos(kr_j r + kl_j . (R n) + phase_j), r = |x|, n = x/r,
    kr_j ~ N(0, 1/Lr^2), kl_j ~ N(0, I/Ll^2): a stationary field with RMS `rms` and
    covariance rms^2 exp(-dr^2/(2Lr^2) - R^2|dn|^2/(2Ll^2))."""
    modes = 64

    def __init__(self, params, R):
        self._head(params, "gaussian_random", 6)
        self.rms = float(params[2])
        ll, lr = float(params[3]) * 1e3, float(params[4]) * 1e3
        seed = int(params[5])
        self.fluid = _truthy(params[6]) if len(params) > 6 else False
        rng = np.random.default_rng(seed)
        self.kr = rng.standard_normal(self.modes) / lr
        self.kl = rng.standard_normal((self.modes, 3)) / ll
        self.ph = rng.uniform(0.0, 2 * math.pi, self.modes)
        self.R = R
        self._kr = self.kr.astype(np.float32)
        self._klR = (R * self.kl.T).astype(np.float32)
        self._ph = self.ph.astype(np.float32)
        if self.ref == 0:
            raise ValueError("Volumetric3D_gaussian_random::initialize || reference type must be relative")

    def _eval_flat(self, x):
        # phases and cosines in FP32 (|phase| < ~200 rad: error < 1e-5 rad, i.e. < 1e-6 in
        # the perturbation), the sum over modes in FP64
        r = np.linalg.norm(x, axis=-1)
        n = (x / np.maximum(r, 1e-9)[:, None]).astype(np.float32)
        arg = n @ self._klR
        arg += r.astype(np.float32)[:, None] * self._kr
        arg += self._ph
        return self.rms * math.sqrt(2.0 / self.modes) * np.cos(arg, out=arg).sum(-1, dtype=np.float64)

    def evaluate_rings_gpu(self, crds, nr, phi2d=None, device=0):
        """The field on the nr slices of every GLL point, crds (n, 25, 2) = (s, z), computed by
        ax3d_sample_gaussian_random (FP64 on the GPU); (n, nr, 25)."""
        return self.evaluate_rows_gpu(crds, np.full(len(crds), int(nr), np.int32), phi2d, device).reshape(
            len(crds), int(nr), 25)

    def evaluate_rows_gpu(self, crds, rows, phi2d=None, device=0):
        """The field on rows[e] slices of every GLL point of element e, crds (n, 25, 2), in
        one sampler call; flat, element e's (rows[e], 25) block after those of elements < e."""
        import ctypes as C
        from .capi import load_library
        lib = load_library()
        f = lib.ax3d_sample_gaussian_random
        P_D = C.POINTER(C.c_double)
        f.argtypes = [C.c_int32, C.c_int32, C.c_void_p, P_D, C.c_int32, P_D, P_D, P_D, C.c_double, C.c_int32,
                      C.c_double, P_D]
        n = len(crds)
        rows = np.ascontiguousarray(rows, np.int32)
        c = np.ascontiguousarray(crds, np.float64)
        kr = np.ascontiguousarray(self.kr, np.float64)
        klR = np.ascontiguousarray(self.R * self.kl.T, np.float64)
        ph = np.ascontiguousarray(self.ph, np.float64)
        out = np.empty(int(rows.astype(np.int64).sum()) * 25)
        d = lambda a: a.ctypes.data_as(P_D)
        rc = f(int(device), n, rows.ctypes.data_as(C.c_void_p), d(c), self.modes, d(kr), d(klR), d(ph), self.rms,
               int(phi2d is not None), float(phi2d or 0.0), d(out))
        if rc != 0:
            buf = C.create_string_buffer(512)
            lib.ax3d_precompute_last_error(buf, 512)
            raise RuntimeError(buf.value.decode())
        return out

    def evaluate(self, xyz):
        shape = xyz.shape[:-1]
        flat = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.empty(len(flat))
        chunk = 1 << 15
        spans = [(i, min(i + chunk, len(flat))) for i in range(0, len(flat), chunk)]

        def work(span):
            out[span[0]:span[1]] = self._eval_flat(flat[span[0]:span[1]])

        if len(spans) > 4:   # numpy's cos releases the GIL: threads share the cores
            from concurrent.futures import ThreadPoolExecutor
            with ThreadPoolExecutor(min(16, os.cpu_count() or 1)) as ex:
                list(ex.map(work, spans))
        else:
            for sp in spans:
                work(sp)
        return out.reshape(shape), np.ones(shape, bool)


def volumetric_models(par, src_latlon, R, lat2theta=None):
    """Volumetric3D::buildInparam: the MODEL_3D_VOLUMETRIC_NUM models of the list."""
    n = par.get("MODEL_3D_VOLUMETRIC_NUM", int)
    out = []
    for i in range(n):
        try:
            entry = par.get("MODEL_3D_VOLUMETRIC_LIST", str, i)
        except (KeyError, IndexError):
            raise ValueError("Volumetric3D::buildInparam || Not enough model names provided in "
                             f"MODEL_3D_VOLUMETRIC_LIST, MODEL_3D_VOLUMETRIC_NUM = {n}")
        strs = entry.split("$")
        name, params = strs[0].lower(), strs[1:]
        if name == "bubble":
            out.append(Bubble(params, src_latlon, R, lat2theta))
        elif name == "gaussian_random":
            out.append(GaussianRandom(params, R))
        else:
            raise NotImplementedError(f"Volumetric3D::buildInparam || volumetric model {strs[0]} is not built "
                                      "(its data files are not shipped)")
    return out


def apply_models(models, props1d, crds, nr, fluid, phi2d=None, gpu=False, presampled=None):
    """3-D properties of a group of elements sharing one Nr.

    props1d: {"VP","VS","RHO": (n, 25)} 1-D values at the GLL points; crds (n, 25, 2) = (s, z);
    fluid (n,) bool.  Slice alpha sits at phi = 2 pi alpha / nr, or every slice at phi2d in
    2-D mode (Quad::computeGeocentricGlobal with phi2D).  Returns ({prop: (n, nr, 25)
    float32}, touched (n,) bool): elements with any point inside any model's range; a property
    no model changes is its 1-D row broadcast over the slices (a read-only view).  gpu: sample the
    Gaussian-random models on the GPU (ax3d_sample_gaussian_random); presampled: {model
    index: (n, nr, 25)} values already sampled for this group."""
    phi = 2 * math.pi * np.arange(nr) / nr if phi2d is None else np.full(nr, float(phi2d))
    n = len(crds)
    out = {}
    touched = np.zeros(n, bool)
    on_gpu = dict(presampled or {})
    on_gpu.update({i: m.evaluate_rings_gpu(crds, nr, phi2d) for i, m in enumerate(models)
                   if gpu and isinstance(m, GaussianRandom) and i not in on_gpu})
    host = len(on_gpu) < len(models)
    step = max(1, (1 << 21) // (nr * 25))   # ~2M samples per chunk
    for a in range(0, n, step):
        b = min(n, a + step)
        if host:
            s, z = crds[a:b, :, 0], crds[a:b, :, 1]
            xyz = np.stack([s[:, None, :] * np.cos(phi)[None, :, None], s[:, None, :] * np.sin(phi)[None, :, None],
                            np.broadcast_to(z[:, None, :], (b - a, nr, 25))], -1)
        # the properties a model has changed, (n, nr, 25); the others stay the 1-D row, which
        # broadcasts over the slices
        cur = {}
        for i, m in enumerate(models):
            if i in on_gpu:
                val = on_gpu[i][a:b]
                inr = np.ones((b - a, 1, 1), bool)  # the sampler covers every point
            else:
                val, inr = m.evaluate(xyz)
            if not m.fluid:
                inr = inr & ~fluid[a:b, None, None]
            if not inr.any():
                continue
            touched[a:b] |= inr.any((1, 2))
            x1 = props1d[m.prop][a:b, None, :].astype(float)
            x = cur.get(m.prop, x1)
            if m.ref == 0:
                cur[m.prop] = np.where(inr, val, x)
                continue
            new = 1.0 + val  # a new array: the perturbation applied in place
            if m.ref == 1:
                new *= x1
            elif m.ref == 2:
                new *= x
            else:
                new *= x - x1
                new += x1
            if not inr.all():
                np.copyto(new, x, where=~inr)
            cur[m.prop] = new
        for k in cur:
            if k not in out:  # first change of k: the chunks before hold its 1-D row
                out[k] = np.empty((n, nr, 25), np.float32)
                out[k][:a] = props1d[k][:a, None, :]
        for k in out:
            out[k][a:b] = cur[k] if k in cur else props1d[k][a:b, None, :]
    for k, v in props1d.items():
        if k not in out:  # no model changes k: its 1-D row, broadcast over the slices (read-only)
            out[k] = np.broadcast_to(v.astype(np.float32)[:, None, :], (n, nr, 25))
    return {k: out[k] for k in props1d}, touched


def linear_resampling(new_size, original):
    """XMath::linearResampling (SOLVER/src/preloop/utilities/XMath.cpp:161-186): slice values of a
    ring of len(original) samples, resampled onto new_size equally spaced slices."""
    n = len(original)
    if new_size == n:
        return np.asarray(original, float)
    if np.all(original == original[0]):
        return np.full(new_size, float(original[0]))
    dphi, dphi0 = 2 * math.pi / new_size, 2 * math.pi / n
    out = np.empty(new_size)
    for i in range(new_size):
        p = i * dphi
        l0 = int(p / dphi0)
        l1 = 0 if l0 + 1 == n else l0 + 1
        out[i] = (original[l1] - original[l0]) / dphi0 * (p - l0 * dphi0) + original[l0]
    return out
