"""Pre-loop precompute of many elements at once: geometry, elemental mass, elastic and
attenuation moduli.

geometry_gpu runs ax3d_precompute_geometry (Quad::createGraident + formIntegralFactor,
Quad.cpp:509-547, FP64 on the GPU) and mass_gpu ax3d_precompute_mass
(Material::computeElementalMass, Material.cpp:233-255).

moduli_gpu runs ax3d_precompute_elastic (FP64 on the GPU); moduli_host is the same
computation in numpy (FP64) with the functions the solver uses one element at a time
(Material::createElastic, Material.cpp:280-379; AttBuilder, AttBuilder.cpp:17-129;
AttAxiSEM::computeAttFactors, AttAxiSEM.cpp:14-57).  Inputs per element: rows = 1 (1-D) or
nr (3-D), the integral factors [25], and the model values vpv, vph, vsv, vsh, eta, rho
(and qkappa, qmu with attenuation) as [rows][25].  Outputs: the moduli [k][rows][25]
(k = 2: lambda, mu for isotropic elements; 5: A, C, F, L, N) and the attenuation moduli
[2][rows][npa], each concatenated over the elements.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import attenuation as ATT
from .spec import ATT_CG4, ATT_NONE


@dataclass
class SLSFit:
    w: np.ndarray
    y: np.ndarray
    f_min: float
    f_max: float
    f_ref: float
    do_kappa: bool = True


def _flat(a):
    """One contiguous float32 vector of an array, or of a list of per-element arrays."""
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, np.float32).reshape(-1)
    return np.ascontiguousarray(np.concatenate([np.asarray(x, np.float32).reshape(-1) for x in a]))


def moduli_gpu(rows, ifact, model: dict, isotropic=False, att=ATT_NONE, sls: SLSFit | None = None, device=0):
    """ax3d_precompute_elastic.  model: name -> list over elements of [rows][25] arrays, or
    their concatenation (vpv, vph, vsv, vsh, eta, rho[, qkappa, qmu])."""
    from .capi import load_library
    lib = load_library()
    f = lib.ax3d_precompute_elastic
    P_F = C.POINTER(C.c_float)
    P_D = C.POINTER(C.c_double)
    f.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int32), P_D] + [P_F] * 8 + \
        [C.c_int32, C.c_int32, C.c_int32, P_D, P_D, C.c_double, C.c_double, C.c_double, C.c_int32, P_F, P_F]
    rows = np.ascontiguousarray(rows, np.int32)
    ifact = np.ascontiguousarray(ifact, np.float64)
    n = len(rows)
    km = 2 if isotropic else 5
    npa = 4 if att == ATT_CG4 else 25
    mod = np.zeros(max(int(km * 25 * rows.sum()), 1), np.float32)
    attm = np.zeros(max(int(2 * npa * rows.sum()) if att != ATT_NONE else 1, 1), np.float32)
    names = ["vpv", "vph", "vsv", "vsh", "eta", "rho"] + (["qkappa", "qmu"] if att != ATT_NONE else [])
    arrs = [_flat(model[k]) for k in names] + [None] * (8 - len(names))
    ptr = lambda a, t: a.ctypes.data_as(t) if a is not None else None
    w = np.ascontiguousarray(sls.w if sls else np.zeros(1), np.float64)
    y = np.ascontiguousarray(sls.y if sls else np.zeros(1), np.float64)
    rc = f(int(device), n, ptr(rows, C.POINTER(C.c_int32)), ptr(ifact, P_D), *[ptr(a, P_F) for a in arrs],
           int(bool(isotropic)), int(att), len(w) if sls else 0, ptr(w, P_D), ptr(y, P_D),
           float(sls.f_min if sls else 0), float(sls.f_max if sls else 0), float(sls.f_ref if sls else 0),
           int(sls.do_kappa if sls else 1), ptr(mod, P_F), ptr(attm, P_F))
    if rc != 0:
        buf = C.create_string_buffer(512)
        lib.ax3d_precompute_last_error(buf, 512)
        raise RuntimeError(buf.value.decode())
    return mod[:int(km * 25 * rows.sum())], attm[:int(2 * npa * rows.sum()) if att != ATT_NONE else 0]


def moduli_host(rows, ifact, model: dict, isotropic=False, att=ATT_NONE, sls: SLSFit | None = None):
    """The same in numpy (FP64), element after element."""
    mods, atts = [], []
    for e, nr in enumerate(rows):
        g = {k: np.asarray(v[e], np.float32).astype(np.float64).reshape(nr, 25) for k, v in model.items()}
        f = np.asarray(ifact[e], np.float64)[None, :]
        A = g["rho"] * g["vph"] ** 2 * f
        Cc = g["rho"] * g["vpv"] ** 2 * f
        L = g["rho"] * g["vsv"] ** 2 * f
        N = g["rho"] * g["vsh"] ** 2 * f
        F = g["eta"] * (A - 2 * L)
        if att != ATT_NONE:
            kappa, mu = ATT.voigt_ti(A, Cc, F, L, N)
            A, Cc, F, L, N = A - (kappa + 4 / 3 * mu), Cc - (kappa + 4 / 3 * mu), F - (kappa - 2 / 3 * mu), L - mu, N - mu
            fac = ATT.att_factors(sls.w, sls.y, sls.f_min, sls.f_max, sls.f_ref, 1.0, g["qkappa"], g["qmu"],
                                  sls.do_kappa)
            kappa, mu, dk, dm = ATT.apply_attenuation(kappa, mu, g["qkappa"], g["qmu"], ifact[e], att == ATT_CG4,
                                                      (fac[3], fac[4]))
            A, Cc, F, L, N = A + (kappa + 4 / 3 * mu), Cc + (kappa + 4 / 3 * mu), F + (kappa - 2 / 3 * mu), L + mu, N + mu
            atts.append(np.concatenate([dk.ravel(), dm.ravel()]))
        mods.append((np.stack([F, L]) if isotropic else np.stack([A, Cc, F, L, N])).ravel())
    return (np.concatenate(mods).astype(np.float32),
            np.concatenate(atts).astype(np.float32) if atts else np.zeros(0, np.float32))


def _check(lib, rc):
    if rc != 0:
        buf = C.create_string_buffer(512)
        lib.ax3d_precompute_last_error(buf, 512)
        raise RuntimeError(buf.value.decode())


def spectral_table():
    """GLL nodes, GLL weights, GLJ(0,1) nodes, GLJ weights (nPol = 4) as one [20] FP64 array."""
    from . import spectral as S
    return np.ascontiguousarray(np.concatenate([S.gll()[0], S.gll()[1], S.glj()[0], S.glj()[1]]), np.float64)


def geometry_gpu(nodes, etype, co, axial, device=0):
    """ax3d_precompute_geometry: nodes [E,2,4] -> geo [E,5,25], ifact [E,25], crds [E,25,2] (FP64)."""
    from .capi import load_library
    lib = load_library()
    f = lib.ax3d_precompute_geometry
    P_D = C.POINTER(C.c_double)
    f.argtypes = [C.c_int32, C.c_int32, P_D, C.c_void_p, C.c_void_p, C.c_void_p, P_D, P_D, P_D, P_D]
    nodes = np.ascontiguousarray(nodes, np.float64)
    E = nodes.shape[0]
    et = np.ascontiguousarray(etype, np.int8)
    cc = np.ascontiguousarray(co, np.int8)
    ax = np.ascontiguousarray(axial, np.uint8)
    sp = spectral_table()
    geo, ifact, crds = np.zeros((E, 5, 25)), np.zeros((E, 25)), np.zeros((E, 25, 2))
    d = lambda a: a.ctypes.data_as(P_D)
    _check(lib, f(int(device), E, d(nodes), et.ctypes.data_as(C.c_void_p), cc.ctypes.data_as(C.c_void_p),
                  ax.ctypes.data_as(C.c_void_p), d(sp), d(geo), d(ifact), d(crds)))
    return geo, ifact, crds


def mass_gpu(rows, ifact, rho, vp, fluid, device=0):
    """ax3d_precompute_mass: element masses [sum rows * 25] (FP64) from rho (and vp for fluids)
    given per element as [rows][25] back to back."""
    from .capi import load_library
    lib = load_library()
    f = lib.ax3d_precompute_mass
    P_D = C.POINTER(C.c_double)
    f.argtypes = [C.c_int32, C.c_int32, C.c_void_p, P_D, C.c_void_p, C.c_void_p, C.c_void_p, P_D]
    rows = np.ascontiguousarray(rows, np.int32)
    ifact = np.ascontiguousarray(ifact, np.float64)
    rho = np.ascontiguousarray(rho, np.float32)
    vp = np.ascontiguousarray(vp, np.float32) if vp is not None else None
    fl = np.ascontiguousarray(fluid, np.uint8)
    mass = np.zeros(int(rows.sum()) * 25)
    _check(lib, f(int(device), len(rows), rows.ctypes.data_as(C.c_void_p), ifact.ctypes.data_as(P_D),
                  rho.ctypes.data_as(C.c_void_p), vp.ctypes.data_as(C.c_void_p) if vp is not None else None,
                  fl.ctypes.data_as(C.c_void_p), mass.ctypes.data_as(P_D)))
    return mass


def jacobian_from_geometry(geo):
    """(J00, J01, J10, J11, det) [E,5,5] from the createGraident operators: dsdxii dzdeta -
    dsdeta dzdxii = 1 / detJ, then J00 = dsdxii detJ, J01 = -dsdeta detJ, J10 = -dzdxii detJ,
    J11 = dzdeta detJ."""
    E = geo.shape[0]
    g = geo.reshape(E, 5, 5, 5)
    det = 1.0 / (g[:, 0] * g[:, 3] - g[:, 1] * g[:, 2])
    return g[:, 0] * det, -g[:, 1] * det, -g[:, 2] * det, g[:, 3] * det, det
