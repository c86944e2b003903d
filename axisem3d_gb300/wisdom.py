"""Nu wisdom files and the Nr fields that read them.

NuWisdom (preloop/nrfield/wisdom/NuWisdom.cpp:13-127) stores, per GLL point, (s, z, Nu
learned, Nu of the run) and writes them as one NetCDF variable "axisem3d_wisdom" [n][4]
(double); files with three columns are read with the learned Nu repeated.  A later run
with NU_TYPE wisdom (WisdomNrField.cpp:10-24) takes, at every GLL point, the inverse-
distance mean of the learned Nu of the four nearest stored points (the stored value itself
at distance below 1e-10), times NU_WISDOM_REUSE_FACTOR, rounded.  NU_TYPE empirical is
EmpNrField::getNrAtPoint (EmpNrField.cpp:26-62); NU_TYPE user-defined is the shipped
UserNrField (UserNrField.cpp:20-80): Nu linear in depth through NU_USER_PARAMETER_LIST
(depth0 nu0 depth1 nu1 ..., metres).
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from . import netcdf as NC

VAR = "axisem3d_wisdom"
NUM_INTERP = 4  # WisdomNrField::mNumInterpPoints


def _round(x):
    """std::round: halves away from zero."""
    x = np.asarray(x, np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def write_wisdom(path, s, z, nu_learn, nu_orig) -> Path:
    """NuWisdom::writeToFile: rows (s, z, Nu learned, Nu of the run)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    data = np.column_stack([np.asarray(s, np.float64), np.asarray(z, np.float64),
                            np.asarray(nu_learn, np.float64), np.asarray(nu_orig, np.float64)])
    ds = NC.Dataset()
    ds.add_dim("dim_0", data.shape[0])
    ds.add_dim("dim_1", 4)
    ds.add_var(VAR, ("dim_0", "dim_1"), data)
    NC.write(path, ds)
    return path


def read_wisdom(path) -> np.ndarray:
    """NuWisdom::readFromFile: [n][4]; a three-column file repeats column 2 as column 3."""
    data = np.asarray(NC.read(path)[VAR], np.float64)
    if data.ndim != 2 or data.shape[1] not in (3, 4):
        raise ValueError("NuWisdom::readFromFile || Inconsistent dimensions for wisdom data, must be a matrix "
                         f"of 3 or 4 columns || File = {path}")
    if data.shape[1] == 3:
        data = np.column_stack([data, data[:, 2]])
    return np.column_stack([data[:, :2], _round(data[:, 2:])])


def wisdom_nu(data: np.ndarray, s, z, k: int = NUM_INTERP) -> np.ndarray:
    """NuWisdom::getNu at every (s, z): inverse-distance mean over the k nearest points."""
    if len(data) == 0:
        raise ValueError("NuWisdom::getNu || Wisdom is empty.")
    from scipy.spatial import cKDTree
    q = np.column_stack([np.ravel(s), np.ravel(z)])
    k = min(k, len(data))
    dist, idx = cKDTree(data[:, :2]).query(q, k=k)
    dist, idx = dist.reshape(len(q), k), idx.reshape(len(q), k)
    nu = data[:, 2][idx]
    out = np.empty(len(q))
    for i in range(len(q)):
        hit = np.flatnonzero(dist[i] < 1e-10)
        if hit.size:
            out[i] = nu[i, hit[0]]
        else:
            w = 1.0 / dist[i]
            out[i] = _round((nu[i] * w).sum() / w.sum())
    return out.astype(np.int64)


def compression_ratio(data: np.ndarray) -> float:
    """NuWisdom::getCompressionRatio: sum of learned Nu over sum of run Nu."""
    return float(data[:, 2].sum() / data[:, 3].sum())


def empirical_nr(par, s, z, r_outer) -> np.ndarray:
    """EmpNrField::getNrAtPoint for every point (NU_EMP_* keywords)."""
    nu_ref = par.get("NU_EMP_REF", int)
    nu_min = par.get("NU_EMP_MIN", int)
    scale_s, scale_t, scale_d = (par.get(k, bool) for k in ("NU_EMP_SCALE_AXIS", "NU_EMP_SCALE_THETA",
                                                             "NU_EMP_SCALE_DEPTH"))
    pow_s = par.get("NU_EMP_POW_AXIS", float)
    fact_pi = par.get("NU_EMP_FACTOR_PI", float)
    start_t = math.radians(par.get("NU_EMP_THETA_START", float))
    pow_t = par.get("NU_EMP_POW_THETA", float)
    fact_d0 = par.get("NU_EMP_FACTOR_SURF", float)
    start_d = par.get("NU_EMP_DEPTH_START", float) * 1e3
    end_d = par.get("NU_EMP_DEPTH_END", float) * 1e3
    s = np.asarray(s, np.float64)
    z = np.asarray(z, np.float64)
    r = np.hypot(s, z)
    theta = np.where(r < 1e-10, 0.0, np.arccos(np.clip(z / np.where(r < 1e-10, 1.0, r), -1.0, 1.0)))
    d = r_outer - r
    nu = np.full(s.shape, float(nu_ref))
    if scale_s:
        nu = nu * (s / r_outer) ** pow_s
    if scale_t:
        nu = np.where(theta > start_t,
                      nu * (1.0 + (fact_pi - 1.0) * ((theta - start_t) / (math.pi - start_t)) ** pow_t), nu)
    if scale_d:
        ramp = 1.0 + (fact_d0 - 1.0) / (start_d - end_d) * (d - end_d) if start_d != end_d else fact_d0
        nu = np.where(d <= end_d, np.where(d <= start_d, nu * fact_d0, nu * ramp), nu)
    nr = 2 * np.maximum(nu_min, np.ceil(nu).astype(np.int64)) + 1
    if (nr <= 0).any():
        raise ValueError("EmpNrField::getNrAtPoint || Non-positive Nr.")
    return nr


def user_nr(params, s, z, r_outer) -> np.ndarray:
    """UserNrField::getNrAtPoint as shipped: Nu interpolated linearly in depth between the
    (depth, nu) pairs of NU_USER_PARAMETER_LIST, held constant outside them; nr = 2 nu + 1
    truncated to an integer."""
    params = [float(v) for v in params]
    nd = len(params) // 2
    if nd == 0 or len(params) % 2 == 1:
        raise ValueError("UserNrField::getNrAtPoint || Using the default UserNrField.cpp, the number of the "
                         "user-defined parameters must be even and positive.")
    d = r_outer - np.hypot(np.asarray(s, np.float64), np.asarray(z, np.float64))
    depths = np.array(params[0::2])
    nus = np.array(params[1::2])
    nu = np.interp(d, depths, nus)  # constant beyond the first and last depth
    nr = (2 * nu + 1).astype(np.int64)
    if (nr <= 0).any():
        raise ValueError("UserNrField::getNrAtPoint || Non-positive Nr.")
    return nr
