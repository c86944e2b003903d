"""Host driver mirroring axisem_main (SOLVER/src/axisem.cpp:12-207) for the GB300 path.

Reads the reference's inputs -- the four inparam.* parfiles, an Exodus meridian mesh
(NetCDF classic), CMTSOLUTION and STATIONS -- builds the packed domain (the counterpart
of Mesh::release), runs Newmark::solve's loop on the GPU through the C-ABI, and writes
the station seismograms as NetCDF with the reference's variable names
(SOLVER/src/core/output/pointwise/PointwiseIONetCDF.cpp:63-195).
Pre-computation is FP64 (geometry, materials, masses, normals, source, receivers).
"""
from __future__ import annotations

import functools
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import attenuation as ATT
from . import model3d as M3D
from . import geometry as GEO
from . import netcdf as NC
from . import relabelling as RL
from . import spectral as S
from .spec import (ATT_CG4, ATT_FULL, ATT_NONE, MAT_ACOUSTIC, MAT_ISO, MAT_TISO, POINT_FLUID, POINT_SOLID,
                   POINT_SOLID_FLUID, DomainSpec)

# the parameter registry (Parameters::registerAll, Parameters.cpp:23-100)
REGISTRY = """MODEL_1D_EXODUS_MESH_FILE MODEL_3D_VOLUMETRIC_NUM MODEL_3D_VOLUMETRIC_LIST MODEL_3D_GEOMETRIC_NUM
MODEL_3D_GEOMETRIC_LIST MODEL_3D_ELLIPTICITY_MODE MODEL_3D_ELLIPTICITY_INVF MODEL_3D_OCEAN_LOAD MODEL_2D_MODE
MODEL_2D_LATITUDE MODEL_2D_LONGITUDE MODEL_2D_AZIMUTH MODEL_PLOT_SLICES_NUM MODEL_PLOT_SLICES_LIST ATTENUATION
NU_TYPE NU_CONST NU_EMP_REF NU_EMP_MIN NU_EMP_SCALE_AXIS NU_EMP_POW_AXIS NU_EMP_SCALE_THETA NU_EMP_POW_THETA
NU_EMP_FACTOR_PI NU_EMP_THETA_START NU_EMP_SCALE_DEPTH NU_EMP_FACTOR_SURF NU_EMP_DEPTH_START NU_EMP_DEPTH_END
NU_WISDOM_LEARN NU_WISDOM_LEARN_EPSILON NU_WISDOM_LEARN_INTERVAL NU_WISDOM_LEARN_OUTPUT NU_WISDOM_REUSE_INPUT
NU_WISDOM_REUSE_FACTOR NU_USER_PARAMETER_LIST TIME_DELTA_T TIME_DELTA_T_FACTOR TIME_RECORD_LENGTH SOURCE_TYPE
SOURCE_FILE SOURCE_TIME_FUNCTION SOURCE_STF_HALF_DURATION OUT_STATIONS_FILE OUT_STATIONS_DUPLICATED
OUT_STATIONS_SYSTEM OUT_STATIONS_FORMAT OUT_STATIONS_COMPONENTS OUT_STATIONS_RECORD_INTERVAL
OUT_STATIONS_DUMP_INTERVAL OUT_STATIONS_WHOLE_SURFACE OUT_STATIONS_DEPTH_REF ATTENUATION_CG4
ATTENUATION_SPECFEM_LEGACY ATTENUATION_QKAPPA DD_PROC_INTERVAL DD_NCUTS_PER_PROC OPTION_VERBOSE_LEVEL
OPTION_STABILITY_INTERVAL OPTION_LOOP_INFO_INTERVAL DEVELOP_MAX_TIME_STEPS DEVELOP_NON_SOURCE_MODE
DEVELOP_DIAGNOSE_PRELOOP DEVELOP_MEASURED_COSTS DEVELOP_RANDOMIZE_DISP0 FFTW_LUCKY_NUMBER FFTW_DISABLE_WISDOM""".split()

PARFILES = ("inparam.model", "inparam.nu", "inparam.time_src_recv", "inparam.advanced")


class Parameters:
    """Parameters::readParFile / parseLine / getValue (Parameters.cpp:15-137, Parameters.h:25-49):
    whitespace-separated KEY value... lines, '#' comments, registered keys only."""

    def __init__(self, input_dir):
        self.values = {k: [] for k in REGISTRY}
        for f in PARFILES:
            p = Path(input_dir) / f
            if not p.exists():
                raise FileNotFoundError(f"Parameters::readParFile || Error opening parameter file: || {p}")
            for line in p.read_text().splitlines():
                strs = line.strip().split()
                if not strs or strs[0].startswith("#"):
                    continue
                if strs[0] in self.values:
                    self.values[strs[0]].extend(strs[1:])

    def get(self, key, typ=str, index=0):
        v = self.values.get(key)
        if not v or index >= len(v):
            raise KeyError(f"Parameters::getValue || Parameter {key} not found or incomplete")
        s = v[index]
        if typ is bool:
            if s.lower() in ("true", "yes", "on", "1"):
                return True
            if s.lower() in ("false", "no", "off", "0"):
                return False
            raise ValueError(f"Parameters::getValue || bad bool for {key}: {s}")
        return typ(s)


@dataclass
class Exodus:
    """The quantities ExodusModel::buildInparam exposes (ExodusModel.cpp:53-247, 519-573)."""
    nodes: np.ndarray       # [N, 2] (s, z)
    conn: np.ndarray        # [E, 4] 0-based
    etype: np.ndarray       # [E]
    fluid: np.ndarray       # [E] bool
    dt: np.ndarray          # [E]
    nodal: dict             # name -> [E, 4]
    side: dict              # side-set name -> [E] side (-1 none)
    glob: dict              # global variables
    isotropic: bool = True  # VP_0 / VS_0 (isotropic) or VPV_0 ... ETA_0 (TI) variables
    ellip: np.ndarray = None  # [2, n] ellipticity knots (r / R) and coefficients

    @staticmethod
    def read(path):
        d = NC.read(path)
        names = d.strings("name_glo_var")
        glob = dict(zip(names, np.asarray(d["vals_glo_var"], float).ravel()))
        conn = np.asarray(d["connect1"], np.int64) - 1
        E = len(conn)
        ss = d.strings("ss_names")
        side = {}
        for i, nm in enumerate(ss):
            v = np.full(E, -1)
            v[np.asarray(d[f"elem_ss{i + 1}"]) - 1] = np.asarray(d[f"side_ss{i + 1}"]) - 1
            side[nm] = v
        enames = d.strings("name_elem_var")
        ev = {nm: np.asarray(d[f"vals_elem_var{i + 1}eb1"], float).ravel() for i, nm in enumerate(enames)}
        nodal = {}
        for base in ("VP", "VS", "VPV", "VPH", "VSV", "VSH", "ETA", "RHO", "QMU", "QKAPPA"):
            if f"{base}_0" in ev:
                nodal[base] = np.stack([ev[f"{base}_{k}"] for k in range(4)], 1)
        # ExodusModel::isIsotropic (ExodusModel.cpp:575-578) and Material::Material
        # (Material.cpp:36-50): isotropic meshes give vpv = vph = VP, vsv = vsh = VS, eta = 1;
        # "vp" / "vs" of a TI mesh are vpv / vsv (Material::getProperty)
        iso = "VP" in nodal
        if iso:
            nodal["VPV"] = nodal["VPH"] = nodal["VP"]
            nodal["VSV"] = nodal["VSH"] = nodal["VS"]
            nodal["ETA"] = np.ones_like(nodal["VP"])
        else:
            nodal["VP"], nodal["VS"] = nodal["VPV"], nodal["VSV"]
        # ExodusModel::formAuxiliary (ExodusModel.cpp:378-404): the nodes of an axial element
        # are rotated so that side 3 lies on the axis (side set "t1" names the axis when present)
        axis = side.get("t1", side.get("t0"))
        if axis is not None:
            for e in np.nonzero((axis >= 0) & (axis != 3))[0]:
                a = int(axis[e])
                perm = [(j + a - 3) % 4 for j in range(4)]
                conn[e] = conn[e][perm]
                for v in {id(v): v for v in nodal.values()}.values():  # aliases rotate once
                    v[e] = v[e][perm]
                for v in side.values():
                    if v[e] != -1:
                        v[e] = (v[e] - a + 3) % 4
            if "t1" in side:
                side["t0"] = side["t1"]
        info = d.strings("info_records")
        if not any("spherical" in s for s in info):
            raise ValueError("Exodus || only crdsys = spherical meshes are supported")
        return Exodus(np.stack([d["coordx"], d["coordy"]], 1).astype(float), conn,
                      ev["element_type"].astype(int), ev["fluid"] > 0.5, ev.get("dt", np.zeros(E)), nodal, side, glob,
                      iso, np.asarray(d["ellipticity"], float) if "ellipticity" in d else None)


def _int_or(par, key, default):
    try:
        return par.get(key, int)
    except KeyError:
        return default


def _flag(par, key):
    try:
        return par.get(key, bool)
    except KeyError:
        return False


def is_lucky(n: int, force_odd: bool) -> bool:
    """PreloopFFTW::isLuckyNumber (PreloopFFTW.cpp:59-99): FFT-friendly ring sizes, with
    prime factors <= 13, at most one factor 11 or 13, odd when forced, even above 10."""
    if force_odd and n % 2 == 0:
        return False
    if not force_odd and n % 2 and n > 10:
        return False
    m = n
    for p in (2, 3, 5, 7, 11, 13):
        while m % p == 0:
            m //= p
    if m != 1:
        return False
    e = f = 0
    m = n
    while m % 11 == 0:
        m //= 11
        e += 1
    m = n
    while m % 13 == 0:
        m //= 13
        f += 1
    return e + f <= 1


def next_lucky(n: int, force_odd: bool) -> int:
    """PreloopFFTW::nextLuckyNumber (PreloopFFTW.cpp:101-109)."""
    while not is_lucky(n, force_odd):
        n += 1
    return n


def _lagrange(x, nodes):
    """XMath::interpLagrange: basis values of the Lagrange polynomials on nodes at x."""
    out = np.ones(len(nodes))
    for i in range(len(nodes)):
        for j in range(len(nodes)):
            if i != j:
                out[i] *= (x - nodes[j]) / (nodes[i] - nodes[j])
    return out


def _rot(theta, phi):
    """Geodesy::rotationMatrix (Geodesy.cpp:56-68)."""
    ct, st, cp, sp = math.cos(theta), math.sin(theta), math.cos(phi), math.sin(phi)
    return np.array([[ct * cp, -sp, st * cp], [ct * sp, cp, st * sp], [-st, 0.0, ct]])


def _parse_keys(text, keys):
    """Source::parseLine / checkValue (Source.cpp:104-119): a line whose first token contains
    the key (case-insensitive) gives the value that follows; every key must be found."""
    out = {}
    for line in text.splitlines():
        toks = line.split()
        if len(toks) < 2:
            continue
        for k in keys:
            if k.lower() in toks[0].lower():
                try:
                    out[k] = float(toks[1])
                except ValueError:
                    pass
    for k in keys:
        if k not in out:
            raise ValueError(f"Source::checkValue || Error reading {k}.")
    return out


def _varies(a):
    """Per element of a (n, nr, 25) property: whether any point's value changes over the
    slices (none for a 1-D row broadcast over them)."""
    if a.strides[1] == 0:
        return np.zeros(len(a), bool)
    return (a.max(1) != a.min(1)).any(1)


def closest_gll_distance(crds):
    """XMath::findClosestDist over each element's 25 GLL points, crds (E, 25, 2): the
    smallest distance between two of them.  Every pair once, point-major for contiguous
    gathers; the distance (hypot) is taken only for the pairs whose squared distance is within
    1e-9 of the element's smallest, which always holds the closest pair."""
    pa, pb = np.triu_indices(25, 1)
    T = np.ascontiguousarray(np.asarray(crds, float).transpose(1, 2, 0))
    D = T[pa] - T[pb]
    d2 = D[:, 0] * D[:, 0] + D[:, 1] * D[:, 1]
    pr, pe = np.nonzero(d2 <= d2.min(0) * (1 + 1e-9))
    out = np.full(T.shape[2], np.inf)
    np.minimum.at(out, pe, np.hypot(D[pr, 0, pe], D[pr, 1, pe]))
    return out


def boundary_normals(nodes, crds, jac0, axial_e, co, es, sides):
    """Quad::computeNormal (Quad.cpp:661-715) without relabelling, for the five points of side
    sides[i] of element es[i]: local indices (n, 5) and normals (n, 5, 3).  nodes (E, 2, 4),
    crds (E, 25, 2), jac0 the (E, 5, 5) first Jacobian entry, co the curved side per element."""
    wg, wjw, xj = S.gll()[1], S.glj()[1], S.glj()[0]
    es, sides = np.asarray(es, np.int64), np.asarray(sides, np.int64)
    n0, n1 = nodes[es, :, sides], nodes[es, :, (sides + 1) % 4]
    r0, r1 = np.hypot(n0[:, 0], n0[:, 1]), np.hypot(n1[:, 0], n1[:, 1])
    dth = np.abs(np.array([_colat(*b) - _colat(*a) for a, b in zip(n0, n1)]))
    rsf = 0.5 * (r0 + r1)
    h_r_dt, h_r2_dt = (0.5 * rsf * dth)[:, None], (0.5 * rsf * rsf * dth)[:, None]
    ip, jp = _SIDE_IP[sides], _SIDE_JP[sides]
    k = ip * 5 + jp
    sz = crds[es[:, None], k]
    rr = np.hypot(sz[..., 0], sz[..., 1])
    sint, cost = sz[..., 0] / rr, sz[..., 1] / rr
    ax = np.asarray(axial_e, bool)[es][:, None]
    wsf = np.where(np.isin(sides, (0, 2))[:, None], np.where(ax, wjw[ip], wg[ip]), wg[jp])
    with np.errstate(divide="ignore", invalid="ignore"):
        fac = np.where(~ax, wsf * sint * h_r2_dt,
                       np.where(ip == 0, wsf * jac0[es[:, None], ip, jp] * h_r_dt, wsf / (1 + xj[ip]) * sint * h_r2_dt))
    nv = np.stack([sint, np.zeros_like(sint), cost], -1) * fac[..., None]
    return k, np.where((sides != np.asarray(co)[es])[:, None, None], -nv, nv)


# the five points of each element side in GLL index order: (ip, jp) with jp = 0 (side 0),
# ip = 4 (side 1), jp = 4 (side 2) and ip = 0 (side 3), local index ip * 5 + jp
_SIDE_IP = np.array([[0, 1, 2, 3, 4], [4] * 5, [0, 1, 2, 3, 4], [0] * 5])
_SIDE_JP = np.array([[0] * 5, [0, 1, 2, 3, 4], [4] * 5, [0, 1, 2, 3, 4]])


def _colat(s, z):
    """Geodesy::rtheta (Geodesy.cpp:13-16): colatitude of (s, z), 0 at the centre."""
    r = math.hypot(s, z)
    return 0.0 if r < 1e-300 else math.acos(max(-1.0, min(1.0, z / r)))


def src_to_glob(theta_s, phi_s, src_theta, src_phi):
    """Geodesy::rotateSrc2Glob on the unit sphere (no ellipticity)."""
    x = np.array([math.sin(theta_s) * math.cos(phi_s), math.sin(theta_s) * math.sin(phi_s), math.cos(theta_s)])
    xg = _rot(src_theta, src_phi) @ x
    t = math.acos(max(-1.0, min(1.0, xg[2])))
    p = math.atan2(xg[1], xg[0]) if math.hypot(xg[0], xg[1]) > 1e-300 else phi_s
    return t, (p + 2 * math.pi) % (2 * math.pi)


def back_azimuth(src_theta, src_phi, rec_theta, rec_phi):
    """Geodesy::backAzimuth (Geodesy.cpp:149-174) with atan4 (Geodesy.cpp:24-38): geocentric
    colatitudes and longitudes in radians, spherical Earth."""
    d, e, f, c = math.sin(src_phi), -math.cos(src_phi), -math.sin(src_theta), math.cos(src_theta)
    a, b = f * e, -f * d
    d1, e1, f1, c1 = math.sin(rec_phi), -math.cos(rec_phi), -math.sin(rec_theta), math.cos(rec_theta)
    g1, h1 = -c1 * e1, c1 * d1
    ss = (a - d1) ** 2 + (b - e1) ** 2 + c * c - 2.0
    sc = (a - g1) ** 2 + (b - h1) ** 2 + (c - f1) ** 2 - 2.0
    if math.hypot(ss, sc) < 1e-300:
        return 0.0
    t = math.atan2(ss, sc)
    if t < 0.0:
        t += math.pi
    if ss < 0.0:
        t += math.pi
    return t


class Geodesy:
    """Geodesy::setup / getFlattening / lat2Theta_r / theta2Lat_r (Geodesy.cpp:64-117,
    176-199): the flattening at radius r is the global flattening 1 / MODEL_3D_ELLIPTICITY_INVF
    times the mesh's ellipticity profile (linear between knots of r / R, 1 beyond the last),
    zero with MODEL_3D_ELLIPTICITY_MODE off; geographic latitudes become geocentric
    colatitudes through tan(lat_c) = (1 - f)^2 tan(lat)."""

    def __init__(self, r_outer=6371e3, flattening=0.0, knots=(), coeffs=()):
        self.R, self.f0 = float(r_outer), float(flattening)
        self.knots, self.coeffs = np.asarray(knots, float), np.asarray(coeffs, float)

    def flattening(self, r):
        f, rr = 1.0, r / self.R
        for i in range(1, len(self.knots)):
            if rr <= self.knots[i]:
                k0, k1, c0, c1 = self.knots[i - 1], self.knots[i], self.coeffs[i - 1], self.coeffs[i]
                f = (c1 - c0) / (k1 - k0) * (rr - k0) + c0
                break
        return f * self.f0

    @staticmethod
    def _clamp(lat, limit_round, limit_bound, what):
        if abs(lat) > limit_bound:
            raise ValueError(f"Geodesy::{what} || Latitude out of range [-90, 90]")
        return max(-limit_round, min(limit_round, lat))

    def lat2theta(self, lat_deg, depth):
        """Geocentric colatitude (rad) of a geographic latitude (deg) at the given depth (m)."""
        f = self.flattening(self.R - depth)
        lat = self._clamp(lat_deg, 90.0 - 1e-10, 90.1, "lat2Theta")
        if f == 0.0:
            return math.pi / 2 - math.radians(lat)
        return math.pi / 2 - math.atan((1 - f) ** 2 * math.tan(math.radians(lat)))

    def theta2lat(self, theta, depth):
        """Geographic latitude (deg) of a geocentric colatitude (rad) at the given depth (m)."""
        f = self.flattening(self.R - depth)
        lat = self._clamp(math.pi / 2 - theta, math.radians(90.0 - 1e-10), math.radians(90.1), "theta2Lat")
        if f == 0.0:
            return math.degrees(lat)
        return math.degrees(math.atan(math.tan(lat) / (1 - f) ** 2))


def glob_to_src(theta_g, phi_g, src_theta, src_phi):
    """Geodesy::rotateGlob2Src on the unit sphere (no ellipticity)."""
    x = np.array([math.sin(theta_g) * math.cos(phi_g), math.sin(theta_g) * math.sin(phi_g), math.cos(theta_g)])
    xs = _rot(src_theta, src_phi).T @ x
    t = math.acos(max(-1.0, min(1.0, xs[2])))
    p = math.atan2(xs[1], xs[0])
    return t, (p + 2 * math.pi) % (2 * math.pi)


class Simulation:
    def __init__(self, input_dir, output_dir=None):
        self.input_dir = Path(input_dir)
        self.output_dir = Path(output_dir or self.input_dir.parent / "output")
        self.par = Parameters(self.input_dir)

    def _mesh_geometry(self, preloop):
        """The Exodus mesh and every element's GLL geometry (Quad::createGraident +
        formIntegralFactor; FP64 on the GPU when preloop = "gpu").  Nothing here depends on
        Nr, so a later build of the same simulation (another Nu field) reuses it (copies of
        the arrays)."""
        cache = getattr(self, "_geometry_cache", {})
        if preloop in cache:
            ex, E, axial_e, co, nodes, geo, ifact, crds, theta, jac = cache[preloop]
            self.ex, self.R = ex, float(ex.glob.get("radius", 6371e3))
            return (ex, E, axial_e.copy(), co.copy(), nodes.copy(), geo.copy(), ifact.copy(), crds.copy(),
                    theta.copy(), tuple(a.copy() for a in jac))
        res = self._mesh_geometry_compute(preloop)
        ex, E, axial_e, co, nodes, geo, ifact, crds, theta, jac = res
        self._geometry_cache = {preloop: (ex, E, axial_e.copy(), co.copy(), nodes.copy(), geo.copy(), ifact.copy(),
                                          crds.copy(), theta.copy(), tuple(a.copy() for a in jac))}
        return res

    def _mesh_geometry_compute(self, preloop):
        par = self.par
        ex = Exodus.read(self.input_dir / par.get("MODEL_1D_EXODUS_MESH_FILE"))
        self.ex = ex
        self.R = float(ex.glob.get("radius", 6371e3))
        E = len(ex.conn)
        axial_e = ex.side.get("t0", np.full(E, -1)) >= 0
        if (ex.side["t0"][axial_e] != 3).any():
            raise ValueError("Quad::Quad || Axial side must be 3.")
        # the curved side of each spherical / semi-spherical element (Quad::Quad, Quad.cpp:51-87)
        # with the mesh's distance tolerance (shortest element side / 1000, ExodusModel.cpp:70-86)
        r = np.hypot(ex.nodes[ex.conn][..., 0], ex.nodes[ex.conn][..., 1])
        xy = ex.nodes[ex.conn]
        tol = float(np.hypot(*(xy - np.roll(xy, -1, axis=1)).transpose(2, 0, 1)).min()) / 1000.0
        r0, r1, r2, r3 = r[:, 0], r[:, 1], r[:, 2], r[:, 3]
        co = np.full(E, -1)
        sph, semi = ex.etype == 0, ex.etype == 2
        a02 = (np.abs(r0 - r1) < tol) & (np.abs(r2 - r3) < tol)
        a13 = (np.abs(r1 - r2) < tol) & (np.abs(r3 - r0) < tol)
        co = np.where(sph & a02, np.where(r2 > r0, 2, 0), co)
        co = np.where(sph & ~a02 & a13, np.where(r3 > r1, 3, 1), co)
        if (sph & ~a02 & ~a13).any():
            raise ValueError("Quad::Quad || Invalid spherical element shape.")
        c_semi = np.select([(np.abs(r0 - r1) < tol) & (r0 > r2), (np.abs(r1 - r2) < tol) & (r1 > r3),
                            (np.abs(r2 - r3) < tol) & (r2 > r0), (np.abs(r3 - r0) < tol) & (r3 > r1)], [0, 1, 2, 3], -1)
        co = np.where(semi, c_semi, co)
        if (semi & (c_semi < 0)).any():
            raise ValueError("Quad::Quad || Invalid semi-spherical element shape.")
        if (axial_e & (ex.etype != 1) & ((3 + co) % 2 == 0)).any():
            raise ValueError("Quad::Quad || Conflict in axial setting.")
        nodes = np.transpose(ex.nodes[ex.conn], (0, 2, 1))
        if preloop == "gpu":
            # Quad::createGraident + formIntegralFactor on the GPU (FP64)
            from . import preloop as PL
            geo, ifact, crds = PL.geometry_gpu(nodes, ex.etype, co, axial_e)
            rr = np.hypot(crds[..., 0], crds[..., 1])
            theta = np.where(rr < 1e-10, 0.0, np.arccos(np.clip(crds[..., 1] / np.where(rr < 1e-10, 1.0, rr), -1, 1)))
            jac = PL.jacobian_from_geometry(geo)
        else:
            geo, ifact, crds, theta, jac = GEO.batch_geometry(nodes, ex.etype, co, axial_e)
        return ex, E, axial_e, co, nodes, geo, ifact, crds, theta, jac

    @staticmethod
    def _gll_material(ex, axial_e):
        """1-D material at the GLL points: bilinear in (xi, eta) of the element's nodal values."""
        E = len(ex.conn)
        xg = S.gll()[0]
        xj = S.glj()[0]
        XI = np.where(axial_e[:, None, None], xj[None, :, None], xg[None, :, None]) * np.ones((1, 1, 5))
        ETA = np.broadcast_to(xg[None, None, :], (E, 5, 5))
        shp = np.stack([(1 - XI) * (1 - ETA), (1 + XI) * (1 - ETA), (1 + XI) * (1 + ETA), (1 - XI) * (1 + ETA)], -1) / 4
        return {k: np.einsum("epqk,ek->epq", shp, v).reshape(E, 25) for k, v in ex.nodal.items()}

    def feature_pass(self, preloop="host"):
        """What the learned-Nu element features need before any Nr is chosen, without the
        rest of the pre-loop: the element GLL coordinates, the 1-D Vp and Vs per element, the
        3-D models and the source depth."""
        ex, E, axial_e, co, nodes, geo, ifact, crds, theta, jac = self._mesh_geometry(preloop)
        mat = self._gll_material(ex, axial_e)
        self.crds = crds
        self.vp_e, self.vs_e = mat["VP"].mean(1), mat["VS"].mean(1)
        self.geo_ = self.geodesy()
        self.models = M3D.volumetric_models(self.par, self._src_llz(), self.R, self.geo_.lat2theta)
        self.src_dep = self._source_depth()

    def ellipticity_mode(self):
        return (self.par.values.get("MODEL_3D_ELLIPTICITY_MODE") or ["off"])[0].lower()

    def geodesy(self):
        """Geodesy::setup as ExodusModel::buildInparam calls it (ExodusModel.cpp:557-572): no
        flattening with MODEL_3D_ELLIPTICITY_MODE off, else 1 / MODEL_3D_ELLIPTICITY_INVF
        with the mesh's ellipticity profile (the mesh read first)."""
        if self.ellipticity_mode() == "off":
            return Geodesy(self.R)
        inv_f = self.par.get("MODEL_3D_ELLIPTICITY_INVF", float)
        if inv_f <= 0.0:
            raise ValueError("ExodusModel::buildInparam || Invalid flattening.")
        ell = self.ex.ellip
        return Geodesy(self.R, 1.0 / inv_f, *((ell[0], ell[1]) if ell is not None else ((), ())))

    def _src_llz(self):
        """(latitude, longitude, depth m) of the source for the geodesy's rotations."""
        lat, lon = self._cmt_latlon()
        return lat, lon, self._source_depth()

    def _source_depth(self):
        """Source depth in m from SOURCE_FILE (0 in non-source mode)."""
        if _flag(self.par, "DEVELOP_NON_SOURCE_MODE"):
            return 0.0
        text = (self.input_dir / self.par.get("SOURCE_FILE")).read_text()
        if self.par.get("SOURCE_TYPE").lower() == "point_force":
            return _parse_keys(text, ("depth",))["depth"] * 1e3
        for line in text.splitlines()[1:]:
            if ":" in line and line.split(":", 1)[0].strip() == "depth":
                return float(line.split(":", 1)[1]) * 1e3
        raise ValueError("Source::buildInparam || no depth in SOURCE_FILE")

    # ------------------------------------------------------------------ build
    def build(self, kahan=False, nu_elem=None, preloop="host") -> DomainSpec:
        """Pack the domain.  nu_elem: optional per-element Fourier order (a learned or user
        Nu field) replacing NU_CONST; each point takes the maximum over its elements.
        preloop = "gpu" computes the element geometry (ax3d_precompute_geometry), the
        Gaussian-random 3-D model samples (ax3d_sample_gaussian_random), the 1-D elemental
        masses (ax3d_precompute_mass) and the solid elements' moduli (ax3d_precompute_elastic)
        in FP64 on the GPU instead of numpy."""
        par = self.par
        ex, E, axial_e, co, nodes, geo, ifact, crds, theta, jac = self._mesh_geometry(preloop)
        self.nodes4, self.co, self.axial_e = nodes, co, axial_e
        # unique GLL points by coordinates (Connectivity::formElemToGLL)
        tol = 1e-3
        key = np.round(crds.reshape(-1, 2) / tol).astype(np.int64)
        # rows numbered in lexicographic (s, z) key order, as np.unique(axis=0) would, by one
        # lexsort instead of a sort of structured rows
        order = np.lexsort((key[:, 1], key[:, 0]))
        ks = key[order]
        first = np.ones(len(ks), bool)
        first[1:] = (ks[1:] != ks[:-1]).any(1)
        inv = np.empty(len(ks), np.int64)
        inv[order] = np.cumsum(first) - 1
        e_pts = inv.reshape(E, 25).astype(np.int32)
        P = int(e_pts.max()) + 1
        pcrd = np.zeros((P, 2))
        pcrd[e_pts.ravel()] = crds.reshape(-1, 2)
        pcrd[np.abs(pcrd[:, 0]) < 1e-6, 0] = 0.0
        mat = self._gll_material(ex, axial_e)
        vp, vs, rho = mat["VP"], mat["VS"], mat["RHO"]
        fl = ex.fluid
        # Nr field (NrField::buildInparam, NrField.cpp:20-64) with Quad::formNrField's limits;
        # point coordinates rounded as formNrField does (offset = min(1e-5, distTol / 1e3))
        nr0 = self._nr_field(pcrd, nodes)
        if nu_elem is not None:
            # a per-element Nu field (learned or user): point Nu = max over its elements
            pnu = np.zeros(P, np.int64)
            np.maximum.at(pnu, e_pts.ravel(), np.repeat(np.asarray(nu_elem, np.int64), 25))
            nr0 = 2 * pnu + 1
        size_e = np.sqrt(np.abs(ifact.sum(1) / np.maximum(crds[..., 0].mean(1), 1.0)))  # ~ element edge
        spacing = np.full(P, np.inf)
        np.minimum.at(spacing, e_pts.ravel(), np.repeat(size_e / 4.0, 25))
        upper = np.maximum(3, (2 * np.pi * pcrd[:, 0] / spacing).astype(int))
        p_nr = np.minimum(nr0, upper)
        p_axial = np.abs(pcrd[:, 0]) < 1e-6
        near_axis = np.zeros(P, bool)
        near_axis[e_pts[axial_e].ravel()] = True
        force_odd = (p_nr % 2 == 0) & near_axis
        p_nr = np.where(force_odd, p_nr + 1, p_nr)
        if _flag(par, "FFTW_LUCKY_NUMBER"):
            key = 2 * p_nr.astype(np.int64) + force_odd
            uk, inv = np.unique(key, return_inverse=True)
            p_nr = np.array([next_lucky(int(k // 2), bool(k % 2)) for k in uk])[inv.ravel()]
        # volumetric 3-D models (Material::addVolumetric3D) on each element's Nr slices
        e_nr = p_nr[e_pts].max(1)
        self.geo_ = self.geodesy()
        models = M3D.volumetric_models(par, self._src_llz(), self.R, self.geo_.lat2theta)
        self.phi2d = self._phi2d()
        # options that would change the physics but are not built here: refuse them rather
        # than run without them (Geometric3D::buildInparam, ExodusModel.cpp:557-572)
        if self.ellipticity_mode() == "full":
            raise ValueError("Geometric3D::buildInparam || MODEL_3D_ELLIPTICITY_MODE full (the ellipsoidal "
                             "deformation of the mesh) is not built; use off or geographic.")
        if _flag(par, "ATTENUATION") and _flag(par, "ATTENUATION_SPECFEM_LEGACY"):
            raise ValueError("AttBuilder::buildInparam || ATTENUATION_SPECFEM_LEGACY: the SPECFEM SLS fit is "
                             "not built; set it false.")
        if _int_or(par, "MODEL_PLOT_SLICES_NUM", 0) > 0:
            import warnings
            warnings.warn("MODEL_PLOT_SLICES_NUM > 0: slice plots (SlicePlot) are not written by this solver")
        e3d = np.zeros(E, bool)
        props3 = {}
        rho_var, vp_var = np.zeros(E, bool), np.zeros(E, bool)
        rho_first, vp_first, vp_max3 = rho.copy(), vp.copy(), vp.max(1)
        if models:
            # GPU: each Gaussian-random model sampled on every element's slices in one call,
            # elements ordered by Nr so that each group's block is contiguous
            groups = np.unique(e_nr)
            pre = {}
            if preloop == "gpu":
                order = np.argsort(e_nr, kind="stable")
                bounds = np.concatenate([[0], np.cumsum([int(nr) * 25 * int((e_nr == nr).sum()) for nr in groups])])
                for i, m in enumerate(models):
                    if isinstance(m, M3D.GaussianRandom):
                        pre[i] = m.evaluate_rows_gpu(crds[order], e_nr[order], self.phi2d)
            for gi, nr in enumerate(groups):
                sel = np.nonzero(e_nr == nr)[0]
                cur, touched = M3D.apply_models(models, {"VP": vp[sel], "VS": vs[sel], "RHO": rho[sel]},
                                                crds[sel], int(nr), fl[sel], phi2d=self.phi2d,
                                                gpu=preloop == "gpu",
                                                presampled={i: v[bounds[gi]:bounds[gi + 1]].reshape(len(sel), int(nr), 25)
                                                            for i, v in pre.items()})
                tj = np.nonzero(touched)[0]
                if self.phi2d is not None:
                    # 2-D mode: every slice sees the model at phi2D, so the element stays
                    # 1-D with the first row (isSolidPar1D, XMath::structuredUseFirstRow)
                    vp[sel[tj]], vs[sel[tj]], rho[sel[tj]] = cur["VP"][tj, 0], cur["VS"][tj, 0], cur["RHO"][tj, 0]
                    continue
                e3d[sel[tj]] = True
                # per element, for the mass and the time step below: whether rho (vp) varies
                # over the slices, the first slice, and the largest Vp of the element
                g3 = cur if len(tj) == len(sel) else {k: v[tj] for k, v in cur.items()}
                rho_var[sel[tj]] = _varies(g3["RHO"])
                vp_var[sel[tj]] = _varies(g3["VP"])
                rho_first[sel[tj]], vp_first[sel[tj]] = g3["RHO"][:, 0], g3["VP"][:, 0]
                vp_max3[sel[tj]] = g3["VP"].max((1, 2))
                for jj, j in enumerate(tj):
                    props3[sel[j]] = {k: v[jj] for k, v in g3.items()}
        # particle relabelling from the geometric models (Quad::addGeometric3D, Quad.cpp:249-255;
        # Relabelling::addUndulation): the elements with a nonzero undulation
        gmodels = RL.geometric_models(par, self._cmt_latlon(), self.R)
        ti_mesh = not ex.isotropic
        if ti_mesh and (models or gmodels):
            raise NotImplementedError("Material::addVolumetric3D / Relabelling || 3-D models on a transversely "
                                      "isotropic mesh are not built here; use no 3-D models or an isotropic mesh")
        relab = {}
        if gmodels:
            # element centre radius (Quad::computeCenterRadius: mapping at xi = eta = 0)
            rcen = np.zeros(E)
            zero = np.zeros((1, 1))
            for e in range(E):
                sc, zc, *_ = GEO._batch_map_jac(nodes[e:e + 1], zero, zero, int(ex.etype[e]), int(max(co[e], 0)))
                rcen[e] = float(np.hypot(sc[0, 0], zc[0, 0]))
            for e in range(E):
                r_ = RL.Relabelled(gmodels, geo[e], crds[e], int(e_nr[e]), p_nr[e_pts[e]], bool(axial_e[e]),
                                   rcen[e], phi2d=self.phi2d)
                if not r_.zero:
                    relab[e] = r_
            for e, r_ in relab.items():
                if not r_.par1d() and not e3d[e]:
                    # elem1D = elem1D && isPar1D (Quad.cpp:388-389, 406-407): the element turns 3-D
                    n = int(e_nr[e])
                    e3d[e] = True
                    props3[e] = {"VP": np.repeat(vp[e][None, :], n, 0), "VS": np.repeat(vs[e][None, :], n, 0),
                                 "RHO": np.repeat(rho[e][None, :], n, 0)}
        self.relab = relab
        # stiffness Jacobian of each relabelled element, on its rows (1 for a 1-D element)
        jstiff = {e: (r_.stiff_jacobian() if e3d[e] else r_.stiff_jacobian()[:1]) for e, r_ in relab.items()}
        self.e3d, self.models = e3d, models
        self.vp_e, self.vs_e = vp.mean(1), vs.mean(1)
        # point phases, masses (Material::computeElementalMass), coupling normals
        has_s = np.zeros(P, bool)
        has_f = np.zeros(P, bool)
        has_s[e_pts[~fl].ravel()] = True
        has_f[e_pts[fl].ravel()] = True
        kind = np.where(has_s & has_f, POINT_SOLID_FLUID, np.where(has_f, POINT_FLUID, POINT_SOLID)).astype(np.int8)
        # elements whose mass varies with phi (3-D rho, or 3-D vp in a fluid); the others
        # add a constant; 3-D masses are resampled onto each point's own Nr
        # (Material.cpp:215-224, XMath::linearResampling)
        not_relab = np.ones(E, bool)
        not_relab[list(relab)] = False
        rho_first[~e3d], vp_first[~e3d] = rho[~e3d], vp[~e3d]  # 1-D elements (2-D mode: the model at phi2D)
        m3e = np.nonzero(e3d & not_relab & (rho_var | (fl & vp_var)))[0].tolist()
        m1 = np.ones(E, bool)
        m1[m3e] = False
        m1[list(relab)] = False
        ms = np.zeros(P)
        mf = np.zeros(P)
        rho0, vp0 = rho_first, vp_first
        sm, fm = m1 & ~fl, m1 & fl
        if preloop == "gpu":  # Material::computeElementalMass on the GPU (FP64), then assembled
            from . import preloop as PL
            em = PL.mass_gpu(np.ones(int(m1.sum())), ifact[m1], rho0[m1], vp0[m1], fl[m1]).reshape(-1, 25)
            sel = np.nonzero(m1)[0]
            np.add.at(ms, e_pts[sel[~fl[sel]]].ravel(), em[~fl[sel]].ravel())
            np.add.at(mf, e_pts[sel[fl[sel]]].ravel(), em[fl[sel]].ravel())
        else:
            np.add.at(ms, e_pts[sm].ravel(), (rho0[sm] * ifact[sm]).ravel())
            np.add.at(mf, e_pts[fm].ravel(), (ifact[fm] / (rho0[fm] * vp0[fm] ** 2)).ravel())
        ms3, mf3 = {}, {}
        for e in m3e:
            for k in range(25):
                p = int(e_pts[e, k])
                rr = M3D.linear_resampling(int(p_nr[p]), props3[e]["RHO"][:, k])
                if fl[e]:
                    vv = M3D.linear_resampling(int(p_nr[p]), props3[e]["VP"][:, k])
                    mf3[p] = mf3.get(p, 0.0) + ifact[e, k] / (rr * vv ** 2)
                else:
                    ms3[p] = ms3.get(p, 0.0) + rr * ifact[e, k]
        for e, r_ in relab.items():
            # Material::computeElementalMass with the relabelling's mass Jacobian (Material.cpp:233-255)
            for k in range(25):
                p = int(e_pts[e, k])
                n = int(p_nr[p])
                rr = (M3D.linear_resampling(n, props3[e]["RHO"][:, k]) if e3d[e] else np.full(n, rho[e, k]))
                jm = r_.mass_jacobian(k)
                if fl[e]:
                    vv = (M3D.linear_resampling(n, props3[e]["VP"][:, k]) if e3d[e] else np.full(n, vp[e, k]))
                    mf3[p] = mf3.get(p, 0.0) + ifact[e, k] / (rr * vv ** 2) * jm
                else:
                    ms3[p] = ms3.get(p, 0.0) + rr * ifact[e, k] * jm
        sfn = np.zeros((P, 3))
        sfn3 = {}  # undulated boundary: normals per slice (Quad::computeNormal with getSFNormalRTZ)
        sfside = ex.side.get("solid_fluid_boundary", np.full(E, -1))
        side_normals = functools.partial(boundary_normals, nodes, crds, jac[0], axial_e, co)

        sf_e = np.nonzero(sfside >= 0)[0]
        sf_k, sf_nv = side_normals(sf_e, sfside[sf_e])
        plain = ~np.isin(sf_e, list(relab))
        # GLLPoint::addSFNormal, element by element
        np.add.at(sfn, e_pts[sf_e[plain, None], sf_k[plain]].ravel(),
                  (0.5 * np.where(fl[sf_e[plain]][:, None, None], sf_nv[plain], -sf_nv[plain])).reshape(-1, 3))
        for i in np.nonzero(~plain)[0]:
            e = sf_e[i]
            for k, nvec in zip(sf_k[i], sf_nv[i]):
                pk = e_pts[e, k]
                # normal_RTZ per slice rotated to (s, phi, z), times the same area factor
                sint, cost = crds[e, k, 0] / np.hypot(*crds[e, k]), crds[e, k, 1] / np.hypot(*crds[e, k])
                Q = np.array([[cost, 0.0, sint], [0.0, 1.0, 0.0], [-sint, 0.0, cost]])
                nv = relab[e].sf_normal_rtz(k) @ Q.T * float(nvec @ np.array([sint, 0.0, cost]))
                sfn3[pk] = sfn3.get(pk, 0.0) + 0.5 * (nv if fl[e] else -nv)
        # moduli (Material::createElastic / createAcoustic, isotropic)
        att_on = par.get("ATTENUATION", bool)
        cg4 = par.get("ATTENUATION_CG4", bool)
        dokappa = par.get("ATTENUATION_QKAPPA", bool)
        # time step (Mesh::getDeltaT x TIME_DELTA_T_FACTOR, or TIME_DELTA_T)
        dt_user = par.get("TIME_DELTA_T", float)
        # Quad::getDeltaT (Quad.cpp:291-305): dt on slices = courant hmin / vmax with the mesh's
        # courant = dt_ref vmax_ref / hmin_ref, hmin from the deformed element (relabelling)
        # and vmax = the largest P velocity of each slice after the 3-D models
        # (Material::getVMax, Material.cpp:521-537); the element's dt is the smallest
        # Quad::getCourant (Quad.cpp:617-628): courant = the mesh's dt x vmax_ref / the shortest
        # element side, vmax_ref = max(vpv, vph) over the element's nodes (Material::getVMaxRef);
        # hmin = the closest two GLL points (XMath::findClosestDist), per slice when relabelled
        xy4 = ex.nodes[ex.conn]
        hmin_edge = np.hypot(*(xy4 - np.roll(xy4, -1, axis=1)).transpose(2, 0, 1)).min(1)
        vmax_ref = np.maximum(ex.nodal["VPV"], ex.nodal["VPH"]).max(1)
        courant = ex.dt.astype(float) * vmax_ref / hmin_edge
        hmin_gll = closest_gll_distance(crds)
        vmax_1d = np.maximum(mat["VPV"], mat["VPH"]).max(1)
        vmax_e = np.where(e3d, vp_max3, vmax_1d)  # the slice maximum: 3-D elements' largest slice
        dt_e = courant * hmin_gll / vmax_e
        for e in relab:
            vm = props3[e]["VP"].max(1) if e3d[e] else np.full(int(e_nr[e]), vmax_1d[e])
            dt_e[e] = float((courant[e] * relab[e].hmin_slices() / vm).min())
        dt = dt_user if dt_user > 0 else float(dt_e.min()) * par.get("TIME_DELTA_T_FACTOR", float)
        self.dt = dt
        attk = ATT_NONE
        alpha = beta = gamma = np.zeros(0)
        nsls = 0
        if att_on and "nr_lin_solids" in ex.glob:
            nsls = int(ex.glob["nr_lin_solids"])
            w = np.array([ex.glob[f"w_{i}"] for i in range(nsls)])
            y = np.array([ex.glob[f"y_{i}"] for i in range(nsls)])
            fmin, fmax, fref = ex.glob["f_min"], ex.glob["f_max"], ex.glob["f_ref"]
            alpha, beta, gamma, _, _ = ATT.att_factors(w, y, fmin, fmax, fref, dt, np.ones(1), np.ones(1), dokappa)
            attk = ATT_CG4 if cg4 else ATT_FULL
        e_mod, e_attm, e_mat, e_att = [], [], [], []
        fit = (w, y, fmin, fmax, fref) if attk != ATT_NONE else None
        ti_mod = self._moduli_ti(fl, mat, ifact, attk, fit, dokappa, cg4, dt, preloop) if ti_mesh else None
        gpu_mod = self._moduli_gpu(E, fl, e3d, props3, vp, vs, rho, ifact, mat, attk, fit,
                                   dokappa, jstiff) if preloop == "gpu" and not ti_mesh else None
        for e in range(E):
            f = ifact[e]
            # (nr, 25) for 3-D elements, (1, 25) for 1-D ones
            vp_e, vs_e, rho_e = ((props3[e]["VP"], props3[e]["VS"], props3[e]["RHO"]) if e3d[e]
                                 else (vp[e][None, :], vs[e][None, :], rho[e][None, :]))
            if fl[e]:  # Material::createAcoustic: K = iFact / rho, times the stiffness Jacobian
                # stored as float32 here, so that with the GPU's float32 solid moduli the
                # concatenation below needs no float64 copy
                e_mod.append((f / rho_e * jstiff.get(e, 1.0)).ravel().astype(np.float32))
                e_attm.append(np.zeros(0, np.float32))
                e_mat.append(MAT_ACOUSTIC)
                e_att.append(ATT_NONE)
                continue
            if ti_mod is not None:
                mod_e, attm_e, iso_e = ti_mod[e]
                e_mod.append(mod_e)
                e_attm.append(attm_e)
                e_mat.append(MAT_ISO if iso_e else MAT_TISO)
                e_att.append(attk)
                continue
            if gpu_mod is not None:
                e_mod.append(gpu_mod[e][0])
                e_attm.append(gpu_mod[e][1])
                e_mat.append(MAT_ISO)
                e_att.append(attk)
                continue
            # relabelling multiplies the moduli by the stiffness Jacobian before the attenuation split
            lam = rho_e * (vp_e ** 2 - 2 * vs_e ** 2) * f * jstiff.get(e, 1.0)
            mu = rho_e * vs_e ** 2 * f * jstiff.get(e, 1.0)
            attm = np.zeros(0)
            if attk != ATT_NONE:
                A = C = lam + 2 * mu
                F, L, N = lam, mu, mu
                kappa, mu_v = ATT.voigt_ti(A, C, F, L, N)
                qk = np.broadcast_to(mat["QKAPPA"][e][None, :], lam.shape)
                qm = np.broadcast_to(mat["QMU"][e][None, :], lam.shape)
                fac = ATT.att_factors(w, y, fmin, fmax, fref, dt, qk, qm, dokappa)
                lam, mu, dk, dm = ATT.apply_attenuation(kappa, mu_v, qk, qm, f, cg4, (fac[3], fac[4]))
                lam = lam - 2.0 / 3.0 * mu
                attm = np.concatenate([dk.ravel(), dm.ravel()])
            e_mod.append(np.stack([lam, mu]).ravel())
            e_attm.append(attm)
            e_mat.append(MAT_ISO)
            e_att.append(attk)
        mofs = np.concatenate([[0], np.cumsum([len(m) for m in e_mod])[:-1]]).astype(np.int64)
        aofs = np.concatenate([[0], np.cumsum([len(m) for m in e_attm])[:-1]]).astype(np.int64)
        # fluid points on the free surface (FluidPoint mFluidSurf)
        fsurf = np.zeros(P, bool)
        surf = ex.side.get("r1", np.full(E, -1))
        for e in np.nonzero((surf >= 0) & fl)[0]:
            s_ = surf[e]
            for ip in range(5):
                for jp in range(5):
                    if (s_ == 0 and jp == 0) or (s_ == 1 and ip == 4) or (s_ == 2 and jp == 4) or (s_ == 3 and ip == 0):
                        fsurf[e_pts[e, ip * 5 + jp]] = True
        def pack_mass(has, m1d, m3d):
            """Point mass rows: 1 value (Mass1D) or Nr values when they vary (Mass3D)."""
            full = {p: m1d[p] + v for p, v in m3d.items() if np.ptp(m1d[p] + v) > 0}
            lens = has.astype(np.int64)
            for p in full:
                lens[p] = len(full[p])
            ofs = np.concatenate([[0], np.cumsum(lens)[:-1]])
            vals = np.zeros(int(lens.sum()))
            one = has & (lens == 1)
            tot = m1d.copy()
            for p, v in m3d.items():
                if p not in full:
                    tot[p] += v[0]
            vals[ofs[one]] = 1.0 / tot[one]
            for p, v in full.items():
                vals[ofs[p]:ofs[p] + lens[p]] = 1.0 / v
            return lens.astype(np.int32), vals.astype(np.float32)
        p_mslen, p_ms = pack_mass(has_s, ms, ms3)
        oc_pt, oc_len, oc_vals = self._ocean_load(ex, fl, e_pts, crds, side_normals, ms, ms3, p_nr)
        p_mflen, p_mf = pack_mass(has_f, mf, mf3)
        # coupling rows (SolidFluidCoupling1D / 3D when the fluid mass varies with phi)
        sflen = np.where(kind == POINT_SOLID_FLUID, 1, 0).astype(np.int32)
        sfrows, sfirows = [], []
        for p in np.nonzero(kind == POINT_SOLID_FLUID)[0]:
            mfp = mf[p] + mf3.get(p, 0.0)
            if p in sfn3:  # undulated boundary: SFCoupling3D with per-slice normals
                n = int(p_nr[p])
                rows = sfn[p][None, :] + sfn3[p]
                mfr = np.broadcast_to(np.ravel(mfp), (n,)) if np.size(mfp) in (1, n) else mfp
                sflen[p] = n
                sfrows.append(rows)
                sfirows.append(rows / np.asarray(mfr, float)[:, None])
            elif np.ndim(mfp) and np.ptp(mfp) > 0:
                sflen[p] = len(mfp)
                rows = np.repeat(sfn[p][None, :], len(mfp), 0)
                sfrows.append(rows)
                sfirows.append(rows / mfp[:, None])
            else:
                sfrows.append(sfn[p][None, :])
                sfirows.append(sfn[p][None, :] / float(np.ravel(mfp)[0]))
        sfrows = np.concatenate(sfrows) if sfrows else np.zeros((0, 3))
        sfirows = np.concatenate(sfirows) if sfirows else np.zeros((0, 3))
        spec = DomainSpec(
            dt=dt, p_nr=p_nr.astype(np.int32), p_kind=kind, p_axial=p_axial.astype(np.uint8),
            p_fsurf=fsurf.astype(np.uint8),
            p_mslen=p_mslen, p_ms=p_ms, p_mflen=p_mflen, p_mf=p_mf,
            p_sflen=sflen, p_sfn=sfrows.astype(np.float32), p_sfni=sfirows.astype(np.float32),
            e_pts=e_pts, e_mat=np.array(e_mat, np.int8), e_axial=axial_e.astype(np.uint8),
            e_in3d=e3d.astype(np.uint8), e_geo=geo.astype(np.float32),
            e_trig=GEO.trig_tables(theta).transpose(1, 0, 2).astype(np.float32),
            e_mofs=mofs, e_mod=np.concatenate(e_mod).astype(np.float32, copy=False), e_att=np.array(e_att, np.int8),
            e_aofs=aofs, e_attm=(np.concatenate(e_attm) if e_attm else np.zeros(0)).astype(np.float32, copy=False),
            nsls=nsls, att_alpha=alpha, att_beta=beta, att_gamma=gamma, att_do_kappa=dokappa,
            kahan=kahan, stability_interval=par.get("OPTION_STABILITY_INTERVAL", int),
            oc_pt=oc_pt, oc_len=oc_len, oc_vals=oc_vals, p_crds=pcrd)
        if relab:
            # the PRT of each relabelled element (Relabelling::createPRT): X [4][25] on a 1-D
            # element (PRT_1D), [4][Nr][25] on a 3-D one (PRT_3D)
            pe, pl, px = [], [], []
            for e in sorted(relab):
                X = relab[e].stiff_x()
                pe.append(e)
                pl.append(X.shape[1] if e3d[e] else 1)
                px.append((X if e3d[e] else X[:, :1, :]).ravel())
            spec.prt_elem = np.array(pe, np.int32)
            spec.prt_len = np.array(pl, np.int32)
            spec.prt_x = np.concatenate(px).astype(np.float32)
            if len(oc_pt) and any(e in relab for e in np.nonzero(fl == 0)[0] if (ex.side.get("r1", np.full(E, -1))[e] >= 0)):
                raise ValueError("Quad::setOceanLoad3D || ocean load on an undulated surface is not built; "
                                 "use MODEL_3D_OCEAN_LOAD none with geometric models there.")
        self.e_pts, self.crds, self.jac, self.fluid = e_pts, crds, jac, fl
        self._source(spec)
        self._stf(spec)
        self._receivers(spec)
        self._surface(spec)
        self.spec = spec
        return spec

    # ------------------------------------------------------------------ source
    @staticmethod
    def _moduli_ti(fl, mat, ifact, attk, fit, dokappa, cg4, dt, preloop):
        """Material::createElastic (Material.cpp:280-379) for the 1-D solid elements of a
        transversely isotropic mesh: A = rho vph^2, C = rho vpv^2, L = rho vsv^2, N = rho vsh^2
        (times iFact), F = eta (A - 2 L), the attenuation split on their Voigt average; an
        element with vpv = vph, vsv = vsh and eta = 1 (Material::isIsotropic, tolerance
        tinyDouble = 1e-10) keeps F, L as Isotropic1D.  FP64 on the GPU (preloop = "gpu",
        ax3d_precompute_elastic) or numpy.  {element: (moduli, attenuation moduli, isotropic)}."""
        solid = np.nonzero(~fl)[0]
        g = {k: mat[k][solid] for k in ("VPV", "VPH", "VSV", "VSH", "ETA", "RHO")}
        nrm = lambda a: np.sqrt((a * a).sum(1))
        iso = ((nrm(g["VPV"] - g["VPH"]) < 1e-10 * nrm(g["VPV"])) & (nrm(g["VSV"] - g["VSH"]) < 1e-10 * nrm(g["VSV"]))
               & (nrm(g["ETA"] - 1.0) < 1e-10))
        npa = 4 if attk == ATT_CG4 else 25
        f = ifact[solid]
        if preloop == "gpu":
            from . import preloop as PL
            model = {k.lower(): [v[i][None, :] for i in range(len(solid))] for k, v in g.items()}
            if attk != ATT_NONE:
                model["qkappa"] = [mat["QKAPPA"][e][None, :] for e in solid]
                model["qmu"] = [mat["QMU"][e][None, :] for e in solid]
            sls = PL.SLSFit(*fit, do_kappa=dokappa) if fit else None
            mod, att = PL.moduli_gpu(np.ones(len(solid), np.int32), f, model, isotropic=False, att=attk, sls=sls)
            mod = mod.reshape(len(solid), 5, 25)
            att = att.reshape(len(solid), -1) if attk != ATT_NONE else np.zeros((len(solid), 0), np.float32)
        else:
            A = g["RHO"] * g["VPH"] ** 2 * f
            C = g["RHO"] * g["VPV"] ** 2 * f
            L = g["RHO"] * g["VSV"] ** 2 * f
            N = g["RHO"] * g["VSH"] ** 2 * f
            F = g["ETA"] * (A - 2 * L)
            att = np.zeros((len(solid), 2 * npa if attk != ATT_NONE else 0))
            if attk != ATT_NONE:
                w, y, fmin, fmax, fref = fit
                kappa, mu = ATT.voigt_ti(A, C, F, L, N)
                for i, e in enumerate(solid):
                    qk, qm = mat["QKAPPA"][e][None, :], mat["QMU"][e][None, :]
                    fac = ATT.att_factors(w, y, fmin, fmax, fref, dt, qk, qm, dokappa)
                    k2, m2, dk, dm = ATT.apply_attenuation(kappa[i][None, :], mu[i][None, :], qk, qm, f[i], cg4,
                                                           (fac[3], fac[4]))
                    dkap, dmu = k2[0] - kappa[i], m2[0] - mu[i]
                    A[i] += dkap + 4.0 / 3.0 * dmu
                    C[i] += dkap + 4.0 / 3.0 * dmu
                    F[i] += dkap - 2.0 / 3.0 * dmu
                    L[i] += dmu
                    N[i] += dmu
                    att[i] = np.concatenate([dk.ravel(), dm.ravel()])
            mod = np.stack([A, C, F, L, N], 1).astype(np.float32)
            att = att.astype(np.float32)
        out = {}
        for i, e in enumerate(solid):
            out[e] = ((mod[i, 2:4] if iso[i] else mod[i]).ravel(), att[i], bool(iso[i]))
        return out

    def _moduli_gpu(self, E, fl, e3d, props3, vp, vs, rho, ifact, mat, attk, fit, dokappa, jstiff=None):
        """Isotropic solid moduli of every solid element in one ax3d_precompute_elastic call;
        returns {element: (moduli [2][rows][25], attenuation moduli)}.  jstiff: relabelled
        elements' stiffness Jacobians, applied through rho (every modulus is linear in it)."""
        from . import preloop as PL
        solid = np.nonzero(~fl)[0]
        jstiff = jstiff or {}
        rows = np.array([props3[e]["VP"].shape[0] if e3d[e] else 1 for e in solid], np.int64)

        def stacked(key, base, scale):
            """[rows][25] of every solid element (3-D rows, or the 1-D row) times its scale,
            concatenated."""
            return np.concatenate([(props3[e][key] if e3d[e] else base[e][None, :]) *
                                   (scale[e] if e in scale else 1) for e in solid] if scale else
                                  [props3[e][key] if e3d[e] else base[e][None, :] for e in solid])
        vp_s, vs_s = stacked("VP", vp, {}), stacked("VS", vs, {})
        model = {"vpv": vp_s, "vph": vp_s, "vsv": vs_s, "vsh": vs_s,
                 "eta": np.ones((int(rows.sum()), 25), np.float32), "rho": stacked("RHO", rho, jstiff)}
        if attk != ATT_NONE:
            model["qkappa"] = np.repeat(mat["QKAPPA"][solid], rows, axis=0)
            model["qmu"] = np.repeat(mat["QMU"][solid], rows, axis=0)
        sls = PL.SLSFit(*fit, do_kappa=dokappa) if fit else None
        mod, att = PL.moduli_gpu(np.array(rows), ifact[solid], model, isotropic=True, att=attk, sls=sls)
        npa = 4 if attk == ATT_CG4 else 25
        out, mo, ao = {}, 0, 0
        for e, nr in zip(solid.tolist(), rows.tolist()):
            na = 2 * nr * npa if attk != ATT_NONE else 0
            out[e] = (mod[mo:mo + 2 * nr * 25], att[ao:ao + na])
            mo += 2 * nr * 25
            ao += na
        return out

    def _phi2d(self):
        """MODEL_2D_MODE (Mesh.cpp:44-70): off, source-centered (MODEL_2D_AZIMUTH, degrees) or
        geographic (MODEL_2D_LATITUDE / _LONGITUDE rotated to the source frame): the azimuth
        at which 3-D models are sampled for every slice, None when off."""
        par = self.par
        mode = (par.values.get("MODEL_2D_MODE") or ["off"])[0].lower()
        if mode == "off":
            return None
        if mode == "source-centered":
            return math.radians(par.get("MODEL_2D_AZIMUTH", float)) % (2 * math.pi)
        if mode == "geographic":
            lat, lon, dep = self._src_llz()
            _, ph = glob_to_src(self.geo_.lat2theta(par.get("MODEL_2D_LATITUDE", float), 0.0),
                                math.radians(par.get("MODEL_2D_LONGITUDE", float) % 360),
                                self.geo_.lat2theta(lat, dep), math.radians(lon % 360))
            return ph
        raise ValueError("Mesh::Mesh || Invalid input for MODEL_2D_MODE.")

    def _nr_field(self, pcrd, nodes):
        """NU_TYPE constant (ConstNrField), empirical (EmpNrField) or wisdom (WisdomNrField,
        reading NU_WISDOM_REUSE_INPUT from the input directory)."""
        from . import wisdom as W
        par = self.par
        nutype = par.get("NU_TYPE").lower()
        dn = nodes - np.roll(nodes, -1, axis=2)
        dist_tol = float(np.hypot(dn[:, 0], dn[:, 1]).min()) / 1000.0
        off = min(1e-5, dist_tol / 1e3)
        sz = np.round(pcrd / off) * off
        self.wisdom_ratio = None
        if nutype == "constant":
            return 2 * par.get("NU_CONST", int) + 1
        if nutype == "empirical":
            return W.empirical_nr(par, sz[:, 0], sz[:, 1], self.R)
        if nutype == "user-defined":
            return W.user_nr(par.values.get("NU_USER_PARAMETER_LIST", []), sz[:, 0], sz[:, 1], self.R)
        if nutype == "wisdom":
            data = W.read_wisdom(self.input_dir / par.get("NU_WISDOM_REUSE_INPUT"))
            factor = par.get("NU_WISDOM_REUSE_FACTOR", float)
            factor = 1.0 if factor <= 1e-10 else factor
            self.wisdom_ratio = W.compression_ratio(data)
            return 2 * W._round(W.wisdom_nu(data, sz[:, 0], sz[:, 1]) * factor).astype(np.int64) + 1
        raise ValueError("NrField::build || Invalid parameter, keyword = NU_TYPE.")

    def learn_parameters(self):
        """LearnParameters (NuWisdom.cpp:134-150): (interval, cutoff, output path) when
        NU_WISDOM_LEARN is on, else None."""
        par = self.par
        if not _flag(par, "NU_WISDOM_LEARN"):
            return None
        eps = min(max(par.get("NU_WISDOM_LEARN_EPSILON", float), 1e-5), 0.1)
        interval = par.get("NU_WISDOM_LEARN_INTERVAL", int)
        interval = 5 if interval <= 0 else interval
        return interval, eps, self.output_dir / par.get("NU_WISDOM_LEARN_OUTPUT")

    def dump_wisdom(self, dom, path=None):
        """Domain::dumpWisdom (Domain.cpp:404-438): (s, z, learned Nu, Nu) of every point."""
        from . import wisdom as W
        lp = self.learn_parameters()
        path = path or (lp[2] if lp else self.output_dir / "wisdom.nc")
        nu = dom.get_wisdom()
        return W.write_wisdom(path, self.spec.p_crds[:, 0], self.spec.p_crds[:, 1], nu, self.spec.p_nr // 2)

    def _ocean_load(self, ex, fl, e_pts, crds, side_normals, ms, ms3, p_nr):
        """MODEL_3D_OCEAN_LOAD (OceanLoad3D::buildInparam, OceanLoad3D.cpp:20-52): 'none' or
        'constant$<depth km>' (OceanLoad3D_const, 3 km by default).  Solid elements on the
        surface side set give their outer points the summed side normal and the ocean depth
        (Quad::setOceanLoad3D, Quad.cpp:254-282, and Quad.cpp:367-373); GLLPoint::release
        (GLLPoint.cpp:57-72) turns each into MassOcean1D or MassOcean3D rows."""
        from .synth import ocean_rows
        name, *params = self.par.get("MODEL_3D_OCEAN_LOAD").split("$")
        self.ocean_depth = 0.0
        none = (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
        if name.lower() == "none":
            return none
        if name.lower() == "crust1":
            raise ValueError("OceanLoad3D_crust1::initialize || the crust1.0 tables are not part of this "
                             "package; use constant$<depth km>.")
        if name.lower() != "constant":
            raise ValueError(f"OceanLoad3D::buildInparam || Unknown ocean-load model name {name}.")
        depth = float(params[0]) * 1e3 if params else 3000.0
        self.ocean_depth = depth
        surf = ex.side.get("r1", np.full(len(fl), -1))
        normal = {}
        es = np.nonzero((surf >= 0) & ~fl)[0]
        ks, nvs = side_normals(es, surf[es])
        for p, nvec in zip(e_pts[es[:, None], ks].ravel().tolist(), nvs.reshape(-1, 3)):
            normal[p] = normal.get(p, 0.0) + nvec  # GLLPoint::addSurfNormal
        pts = sorted(normal)
        if depth == 0.0 or not pts:
            return none
        _, first = np.unique(e_pts.ravel(), return_index=True)  # one element slot per point
        coords = crds.reshape(-1, 2)[first[np.array(pts)]]
        mass = [ms[p] + ms3.get(p, 0.0) for p in pts]
        return ocean_rows(pts, [normal[p] for p in pts], mass, p_nr,
                          [_colat(*c) for c in coords], [depth] * len(pts))

    def _cmt_latlon(self):
        """Source latitude/longitude of the CMTSOLUTION (Source.cpp:121-140), needed before
        the source itself is built to place geographic 3-D anomalies."""
        if _flag(self.par, "DEVELOP_NON_SOURCE_MODE"):
            return 90.0, 0.0
        if self.par.get("SOURCE_TYPE").lower() == "point_force":
            v = _parse_keys((self.input_dir / self.par.get("SOURCE_FILE")).read_text(), ("latitude", "longitude"))
            return v["latitude"], v["longitude"]
        vals = {}
        for line in (self.input_dir / self.par.get("SOURCE_FILE")).read_text().splitlines()[1:]:
            if ":" in line:
                k, v = line.split(":", 1)
                vals[k.strip()] = v.strip()
        return float(vals["latitude"]), float(vals["longitude"])

    def _source(self, spec):
        """CMTSOLUTION (Source.cpp:121-234) -> Earthquake::computeSourceFourier (Earthquake.cpp:20-88);
        SOURCE_TYPE point_force -> PointForce::computeSourceFourier (PointForce.cpp)."""
        par = self.par
        if _flag(par, "DEVELOP_NON_SOURCE_MODE"):
            # NullSource (Source.cpp:126-132, NullSource.h): no source term; Source() sits at
            # the north pole on the surface (Source.h:18)
            self.src_lat, self.src_lon, self.src_dep = 90.0, 0.0, 0.0
            self.half_duration = 0.0
            spec.sources = []
            self.src_elem = -1
            return
        stype = par.get("SOURCE_TYPE").lower()
        if stype == "point_force":
            return self._point_force(spec)
        if stype != "earthquake":
            raise ValueError(f"Source::buildInparam || Unknown source type: {par.get('SOURCE_TYPE')}")
        vals = {}
        for line in (self.input_dir / par.get("SOURCE_FILE")).read_text().splitlines()[1:]:
            if ":" in line:
                k, v = line.split(":", 1)
                vals[k.strip()] = v.strip()
        self.src_lat, self.src_lon = float(vals["latitude"]), float(vals["longitude"])
        self.src_dep = float(vals["depth"]) * 1e3
        M = {k: float(vals[k]) * 1e-7 for k in ("Mrr", "Mtt", "Mpp", "Mrt", "Mrp", "Mtp")}  # dyn*cm -> N*m
        self.half_duration = float(vals.get("half duration", 0.0))
        host, eta = self._locate_source(self.R - self.src_dep)
        fz = _lagrange(eta, S.gll()[0])
        Ggll, Gglj = S.gll()[2], S.glj()[2]
        J00, J01, J10, J11, det = (a[host] for a in self.jac)
        Mxx, Myy, Mzz, Mxy, Mxz, Myz = M["Mtt"], M["Mpp"], M["Mrr"], M["Mtp"], M["Mrt"], M["Mrp"]
        f = np.zeros((25, 3, 3), complex)
        for ip in range(5):
            for jp in range(5):
                for js in range(5):
                    fact = fz[js]
                    a00, a01, a10, a11 = (J00[0, js] / det[0, js], J01[0, js] / det[0, js],
                                          J10[0, js] / det[0, js], J11[0, js] / det[0, js])
                    GU = Gglj[ip, 0] * (1.0 if js == jp else 0.0)  # (G^T w)(0, js)
                    UG = (Ggll[jp, js] if ip == 0 else 0.0)          # (w G)(0, js)
                    dwds = a11 * GU - a10 * UG
                    dwdz = a00 * UG - a01 * GU
                    k = ip * 5 + jp
                    f[k, 0, 0] += fact * dwds * (Mxx + Myy) / (2 * np.pi)
                    f[k, 0, 2] += fact * dwdz * Mzz / (2 * np.pi)
                    f[k, 1, 0] += fact * dwdz * (Mxz - 1j * Myz) / (4 * np.pi)
                    f[k, 1, 1] += fact * dwdz * (Mxz - 1j * Myz) / (4 * np.pi) * 1j
                    f[k, 1, 2] += fact * dwds * (Mxz - 1j * Myz) / (2 * np.pi)
                    f[k, 2, 0] += fact * dwds * ((Mxx - Myy) / 2 - 1j * Mxy) / (2 * np.pi)
                    f[k, 2, 1] += fact * dwds * ((Mxx - Myy) / 2 - 1j * Mxy) / (2 * np.pi) * 1j
        spec.sources = [(int(host), f.astype(np.complex64))]
        self.src_elem = int(host)

    def _point_force(self, spec):
        """SOURCE_TYPE point_force (Source.cpp:190-226): latitude, longitude, depth (km) and
        the force Ft, Fp, Fr (N) from SOURCE_FILE, each line's first token containing the key
        (Source::parseLine).  PointForce::computeSourceFourier: orders 0 (Fr / 2 pi, z) and 1
        ((Ft - i Fp) / 4 pi, (Fp + i Ft) / 4 pi on s, phi) on the axis column, weighted by
        the Lagrange factors of the source depth."""
        keys = _parse_keys((self.input_dir / self.par.get("SOURCE_FILE")).read_text(),
                           ("latitude", "longitude", "depth", "ft", "fp", "fr"))
        self.src_lat, self.src_lon = keys["latitude"], keys["longitude"]
        self.src_dep = keys["depth"] * 1e3
        self.half_duration = 0.0
        host, eta = self._locate_source(self.R - self.src_dep)
        fz = _lagrange(eta, S.gll()[0])
        ft, fp, fr = keys["ft"], keys["fp"], keys["fr"]
        f = np.zeros((25, 2, 3), complex)
        for jp in range(5):
            f[jp, 0, 2] = fz[jp] * fr / (2 * np.pi)
            f[jp, 1, 0] = fz[jp] * (ft - 1j * fp) / (4 * np.pi)
            f[jp, 1, 1] = fz[jp] * (fp + 1j * ft) / (4 * np.pi)
        spec.sources = [(int(host), f.astype(np.complex64))]
        self.src_elem = int(host)

    def _locate_source(self, zsrc):
        """Source::locate (Source.cpp:61-94): the axial solid element whose axis side spans
        z = zsrc, and eta there."""
        host, eta = None, None
        for e in np.nonzero(self.axial_e & ~self.fluid)[0]:
            z = self.crds[e].reshape(5, 5, 2)[0, :, 1]  # axis column, jpol = 0..4
            zmin, zmax = z.min(), z.max()
            if zmin - 1e-3 <= zsrc <= zmax + 1e-3 and z[0] > -1e-6 and z[4] > -1e-6:
                # eta from the linear radius on the axis (exact for spherical and linear mappings)
                eta = -1.0 + 2.0 * (zsrc - z[0]) / (z[4] - z[0])
                host = e
                break
        if host is None:
            raise RuntimeError("Source::release || Error locating source.")
        return host, eta

    # ------------------------------------------------------------------ STF
    def _stf(self, spec):
        """STF::buildInparam (STF.cpp:21-62) with Erf/Gauss/Ricker (ErfSTF.cpp, GaussSTF.cpp:10-21)."""
        par = self.par
        dt = self.dt
        hdur = par.get("SOURCE_STF_HALF_DURATION", float)
        if hdur < 5 * dt:
            hdur = 5 * dt
        decay = 1.628
        duration = par.get("TIME_RECORD_LENGTH", float)
        nb = math.ceil(2.5 * hdur / dt)
        na = math.ceil(duration / dt)
        shift = nb * dt
        t = -shift + np.arange(nb + na + 1) * dt
        kind = par.get("SOURCE_TIME_FUNCTION").lower()
        if kind == "erf":
            from scipy.special import erf
            stf = erf(decay / hdur * t) * 0.5 + 0.5
        elif kind == "gauss":
            stf = np.exp(-(decay / hdur * t) ** 2) * decay / (hdur * math.sqrt(math.pi))
        elif kind == "ricker":
            a = decay / hdur
            stf = 2 * a * a * np.exp(-(a * t) ** 2) * (2 * t * t * a * a - 1)
        else:
            raise ValueError(f"STF::buildInparam || Unknown stf type: {kind}")
        cap = par.get("DEVELOP_MAX_TIME_STEPS", int)
        if cap > 0:
            stf = stf[:cap]
        spec.stf = stf.astype(np.float32)
        self.shift = shift
        self.nsteps = len(stf)

    # ------------------------------------------------------------------ receivers
    def _receivers(self, spec):
        """STATIONS -> Receiver (Receiver.cpp:23-117): source-centred (theta, phi), element and
        Lagrange weights (GLJ along xi on axial elements), back azimuth, and the optional
        dump_strain / dump_curl keywords after the sixth column (ReceiverCollection.cpp:48-81;
        lines with fewer than six columns or bad numbers are skipped)."""
        par = self.par
        self.baz = []
        system = par.get("OUT_STATIONS_SYSTEM").lower()
        self.components = par.get("OUT_STATIONS_COMPONENTS").upper()
        lines = [l.split() for l in (self.input_dir / par.get("OUT_STATIONS_FILE")).read_text().splitlines() if l.strip()]
        src_t = self.geo_.lat2theta(self.src_lat, self.src_dep)  # Geodesy::lat2Theta_d
        src_p = math.radians(self.src_lon % 360)
        dup = par.get("OUT_STATIONS_DUPLICATED").lower()
        if dup not in ("ignore", "rename", "error"):
            raise ValueError("ReceiverCollection::buildInparam || Invalid parameter, keyword = OUT_STATIONS_DUPLICATED.")
        keys_seen = set()
        rec, dumps = [], []
        for toks in lines:
            if len(toks) < 6:
                continue
            name, net = toks[0], toks[1]
            try:
                la, lo, bur = float(toks[2]), float(toks[3]), float(toks[5])
            except ValueError:
                continue
            # duplicated NET.NAME keys (ReceiverCollection.cpp:98-117): renamed NAME__DUPLICATED<k>
            # or an error; "ignore" keeps them as they are
            if dup != "ignore" and f"{net}.{name}" in keys_seen:
                if dup == "error":
                    raise ValueError("ReceiverCollection::ReceiverCollection || Duplicated station keys "
                                     f"(network_name) found in station data file || Name = {name}; Network = {net}")
                base, k = name, 0
                while f"{net}.{name}" in keys_seen:
                    k += 1
                    name = f"{base}__DUPLICATED{k}"
            keys_seen.add(f"{net}.{name}")
            extra = {t.lower() for t in toks[6:]}
            dumps.append((1 if "dump_strain" in extra else 0) | (2 if "dump_curl" in extra else 0))
            if system == "geographic":
                th_g, ph_g = self.geo_.lat2theta(la, bur), math.radians(lo % 360)  # Receiver.cpp:27
                th, ph = glob_to_src(th_g, ph_g, src_t, src_p)
            else:
                th, ph = math.radians(la), math.radians(lo)
                th_g, ph_g = src_to_glob(th, ph, src_t, src_p)
            self.baz.append(back_azimuth(src_t, src_p, th_g, ph_g))
            # the station's geographic coordinates as the outputs name them (Receiver.cpp:38-39)
            lat_g = self.geo_.theta2lat(th_g, bur)
            lon_g = math.degrees(ph_g - 2 * math.pi if ph_g > math.pi else ph_g)
            r = self.R - bur
            e, xi, eta = self._locate(r * math.sin(th), r * math.cos(th))
            wxi = _lagrange(xi, S.glj()[0] if self.axial_e[e] else S.gll()[0])
            weta = _lagrange(eta, S.gll()[0])
            rec.append((name, net, lat_g, lon_g, bur, th, ph, e, np.outer(wxi, weta).ravel()))
        self.receivers = rec
        spec.r_dump = np.array(dumps, np.int32)
        spec.r_elem = np.array([r[7] for r in rec], np.int32)
        spec.r_phi = np.array([r[6] for r in rec], np.float32)
        spec.r_w = np.array([r[8] for r in rec], np.float32).reshape(len(rec), 25)

    def _surface(self, spec):
        """OUT_STATIONS_WHOLE_SURFACE (ReceiverCollection.cpp:186-220, 281-300): 'false', or
        'true [radius_km [dist_min_deg dist_max_deg [from_upper]]]'.  Every solid element
        whose centre lies inside the distance window and on the requested side of the radius
        contributes its edge at that radius (Quad::edgeAtRadius, Quad.cpp:747-770); edges are
        tagged by their smallest colatitude (SurfaceRecorder::initialize)."""
        par = self.par
        v = par.values.get("OUT_STATIONS_WHOLE_SURFACE") or ["false"]
        self.surface_edges = []
        if not par.get("OUT_STATIONS_WHOLE_SURFACE", bool):
            return
        if len(v) not in (1, 2, 4, 5):
            raise ValueError("ReceiverCollection::buildInparam || Invalid parameter, keyword = OUT_STATIONS_WHOLE_SURFACE.")
        r, dmin, dmax, upper = self.R, 0.0, 180.0, False
        if len(v) >= 2:
            r = float(v[1]) * 1e3
        if len(v) >= 4:
            dmin, dmax = float(v[2]), float(v[3])
        if len(v) == 5:
            upper = par.get("OUT_STATIONS_WHOLE_SURFACE", bool, 4)
        nodes = self.nodes4  # [E, 2, 4] (s, z) of the four corners
        rn = np.hypot(nodes[:, 0], nodes[:, 1])
        # ExodusModel::mDistTolerance: the shortest quad side / 1000 (ExodusModel.cpp:70-86)
        dn = nodes - np.roll(nodes, -1, axis=2)
        tol = float(np.hypot(dn[:, 0], dn[:, 1]).min()) / 1000.0
        edges = []
        for e in range(len(rn)):
            if self.fluid[e]:
                continue
            sc, zc = nodes[e, 0].mean(), nodes[e, 1].mean()
            dist = math.degrees(_colat(sc, zc))
            if dist < dmin or dist > dmax or upper != (rn[e].mean() > r):
                continue
            for k in range(4):
                if abs(rn[e, k] - r) < tol and abs(rn[e, (k + 1) % 4] - r) < tol:
                    # colatitudes of the side's first and last GLL points (SurfaceInfo.cpp:9-16,
                    # Element::getCoordsOnSide); point index ipol * 5 + jpol
                    q0, q1 = ((0, 20), (20, 24), (4, 24), (0, 4))[k]
                    c = self.crds[e].reshape(25, 2)
                    th0, th1 = _colat(*c[q0]), _colat(*c[q1])
                    edges.append((min(th0, th1), e, k, th0, th1))
                    break
        edges.sort()
        self.surface_edges = edges
        spec.sf_elem = np.array([x[1] for x in edges], np.int32)
        spec.sf_side = np.array([x[2] for x in edges], np.int32)
        spec.sf_interval = max(par.get("OUT_STATIONS_RECORD_INTERVAL", int), 1)

    def write_surface_netcdf(self, records, path=None):
        """output/stations/axisem3d_surface.nc (SurfaceIO.cpp:63-150): time_points, per edge
        edge_<tag>r / edge_<tag>i [steps][5 x 3 x (Nu + 1)] with the record's
        [component][point][order] layout, theta [edges][2], GLL, GLJ and the source
        attributes.  records: one [steps][3][5][Nu + 1] complex array per edge."""
        from . import spectral as S
        path = Path(path or self.output_dir / "stations" / "axisem3d_surface.nc")
        path.parent.mkdir(parents=True, exist_ok=True)
        n = records[0].shape[0] if records else 0
        iv = self.spec.sf_interval
        ds = NC.Dataset()
        ds.add_dim("ntime", n)
        ds.add_dim("nedge", len(records))
        ds.add_dim("two", 2)
        ds.add_dim("npol", 5)
        ds.add_var("time_points", ("ntime",), -self.shift + np.arange(n) * iv * self.dt)
        for tag, rec in enumerate(records):
            w = rec.shape[1] * rec.shape[2] * rec.shape[3]
            ds.add_dim(f"ncol_{tag}", w)
            flat = rec.reshape(n, w)
            ds.add_var(f"edge_{tag}r", ("ntime", f"ncol_{tag}"), flat.real.astype(np.float32))
            ds.add_var(f"edge_{tag}i", ("ntime", f"ncol_{tag}"), flat.imag.astype(np.float32))
        ds.add_var("theta", ("nedge", "two"), np.array([[x[3], x[4]] for x in self.surface_edges], np.float64))
        ds.add_var("GLL", ("npol",), S.gll()[0])
        ds.add_var("GLJ", ("npol",), S.glj()[0])
        # spherical geometry: both flattenings are zero
        ds.attrs.update({"source_latitude": float(self.src_lat), "source_longitude": float(self.src_lon),
                         "source_depth": float(self.src_dep), "source_flattening": 0.0,
                         "surface_flattening": 0.0, "radius": float(self.R)})
        NC.write(path, ds)
        return path

    def _locate(self, s, z):
        """Quad::invMapping by Newton iterations (Mapping.cpp:17-28) over candidate elements."""
        if getattr(self, "_cen_of", None) is not self.crds:  # element centres, once per mesh
            self._cen, self._cen_of = self.crds.mean(1), self.crds
        cen = self._cen
        order = np.argsort(np.hypot(cen[:, 0] - s, cen[:, 1] - z))
        for e in order[:64]:
            if self.fluid[e]:
                continue
            xe = np.zeros(2)
            n = self.nodes4[e:e + 1]
            for _ in range(12):
                ss, zz, J00, J01, J10, J11 = GEO._batch_map_jac(n, np.array([[xe[0]]]), np.array([[xe[1]]]),
                                                               int(self.ex.etype[e]), int(self.co[e]))
                d = np.array([s - ss[0, 0], z - zz[0, 0]])
                if np.hypot(*d) < 1e-7:
                    break
                J = np.array([[J00[0, 0], J01[0, 0]], [J10[0, 0], J11[0, 0]]])
                xe = xe + np.linalg.solve(J, d)
            if np.all(np.abs(xe) <= 1.000001):
                return int(e), float(np.clip(xe[0], -1, 1)), float(np.clip(xe[1], -1, 1))
        raise RuntimeError(f"Receiver::locate || station at (s, z) = ({s}, {z}) not found")

    # ------------------------------------------------------------------ output
    def rotate(self, seis):
        """PointwiseRecorder::record's SPZ -> RTZ / ENZ rotation (PointwiseRecorder.cpp:76-93)."""
        out = np.array(seis, np.float64)
        if self.components == "SPZ":
            return out
        for i, r in enumerate(self.receivers):
            th = r[5]
            s_, p_, z_ = seis[:, i, 0], seis[:, i, 1], seis[:, i, 2]
            ur = s_ * math.sin(th) + z_ * math.cos(th)
            ut = s_ * math.cos(th) - z_ * math.sin(th)
            if self.components == "ENZ":
                cb, sb = math.cos(self.baz[i]), math.sin(self.baz[i])
                out[:, i, 0], out[:, i, 1], out[:, i, 2] = -ut * sb + p_ * cb, -ut * cb - p_ * sb, ur
            else:
                out[:, i, 0], out[:, i, 1], out[:, i, 2] = ut, p_, ur
        return out

    def rotate_curl(self, curl):
        """Curl of the flagged receivers (theta, phi, r) -> ENZ when OUT_STATIONS_COMPONENTS is
        ENZ (PointwiseRecorder.cpp:116-129); strain stays in RTZ."""
        out = np.array(curl, np.float64)
        if self.components != "ENZ":
            return out
        idx = [i for i in range(len(self.receivers)) if self.spec.r_dump[i] & 2]
        for k, i in enumerate(idx):
            cb, sb = math.cos(self.baz[i]), math.sin(self.baz[i])
            ut, up, ur = curl[:, k, 0], curl[:, k, 1], curl[:, k, 2]
            out[:, k, 0], out[:, k, 1], out[:, k, 2] = -ut * sb + up * cb, -ut * cb - up * sb, ur
        return out

    def _recorded(self, arr):
        """Rows of the steps PointwiseRecorder::record keeps (tstep % OUT_STATIONS_RECORD_INTERVAL
        == 0, PointwiseRecorder.cpp:62-66; the library records every step) and their times."""
        iv = max(_int_or(self.par, "OUT_STATIONS_RECORD_INTERVAL", 1), 1)
        n = arr.shape[0] if arr is not None else 0
        return (arr[::iv] if arr is not None else None), -self.shift + np.arange(0, n, iv) * self.dt

    def write_netcdf(self, seis_rtz, path=None, strain=None, curl=None):
        """output/stations/axisem3d_synthetics.nc with time_points and NET.NAME.<comp>, plus
        NET.NAME.RTZ.strain [steps][6] and NET.NAME.RTZ.curl [steps][3] for the receivers
        flagged dump_strain / dump_curl (PointwiseIONetCDF.cpp:56-95), one row per recorded
        step."""
        path = Path(path or self.output_dir / "stations" / "axisem3d_synthetics.nc")
        path.parent.mkdir(parents=True, exist_ok=True)
        seis_rtz, t = self._recorded(seis_rtz)
        strain, _ = self._recorded(strain)
        curl, _ = self._recorded(curl)
        n = seis_rtz.shape[0]
        ds = NC.Dataset()
        ds.add_dim("ntime", n)
        ds.add_dim("ncomp", 3)
        ds.add_var("time_points", ("ntime",), t)
        for i, r in enumerate(self.receivers):
            ds.add_var(f"{r[1]}.{r[0]}.{self.components}", ("ntime", "ncomp"), seis_rtz[:, i].astype(np.float32),
                       attrs={"latitude": float(r[2]), "longitude": float(r[3]), "depth": float(r[4])})
        dump = np.asarray(self.spec.r_dump, np.int32) if len(self.spec.r_dump) else np.zeros(len(self.receivers), np.int32)
        for bit, arr, tag, k in ((1, strain, "strain", 6), (2, curl, "curl", 3)):
            if arr is None:
                continue
            if k == 6:
                ds.add_dim("nstrain", 6)
            for j, i in enumerate(np.flatnonzero(dump & bit)):
                r = self.receivers[i]
                ds.add_var(f"{r[1]}.{r[0]}.RTZ.{tag}", ("ntime", "nstrain" if k == 6 else "ncomp"),
                           arr[:, j].astype(np.float32))
        NC.write(path, ds)
        return path

    def write_ascii(self, seis_rtz, strain=None, curl=None, out_dir=None):
        """PointwiseIOAscii (PointwiseIOAscii.cpp): per station NET.NAME.<comp>.ascii with rows
        (time, 3 components), and NET.NAME.RTZ.strain.ascii (time, 6) /
        NET.NAME.RTZ.curl.ascii (time, 3) for the flagged receivers; full precision,
        space-separated."""
        out = Path(out_dir or self.output_dir / "stations")
        out.mkdir(parents=True, exist_ok=True)
        seis_rtz, t = self._recorded(seis_rtz)
        strain, _ = self._recorded(strain)
        curl, _ = self._recorded(curl)
        dump = np.asarray(self.spec.r_dump, np.int32) if len(self.spec.r_dump) else np.zeros(len(self.receivers), np.int32)

        def put(path, cols):
            rows = np.column_stack([t] + [np.asarray(c, np.float64) for c in cols])
            path.write_text("".join(" " + " ".join(repr(float(v)) for v in r) + "\n" for r in rows))

        paths = []
        for i, r in enumerate(self.receivers):
            base = f"{r[1]}.{r[0]}"
            p = out / f"{base}.{self.components}.ascii"
            put(p, [seis_rtz[:, i, k].astype(np.float32) for k in range(3)])
            paths.append(p)
        for bit, arr, tag, k in ((1, strain, "strain", 6), (2, curl, "curl", 3)):
            if arr is None:
                continue
            for j, i in enumerate(np.flatnonzero(dump & bit)):
                r = self.receivers[i]
                p = out / f"{r[1]}.{r[0]}.RTZ.{tag}.ascii"
                put(p, [arr[:, j, c].astype(np.float32) for c in range(k)])
                paths.append(p)
        return paths

    def write_outputs(self, seis_rtz, strain=None, curl=None):
        """OUT_STATIONS_FORMAT (ReceiverCollection.cpp:341-372), any of: ascii (one file per
        station), netcdf (axisem3d_synthetics.nc) and netcdf_no_assemble (one file per rank,
        here rank 0: axisem3d_synthetics.nc.rank0)."""
        fmts = {f.lower() for f in self.par.values.get("OUT_STATIONS_FORMAT", [])}
        if not fmts or not fmts <= {"ascii", "netcdf", "netcdf_no_assemble"}:
            raise ValueError("ReceiverCollection::buildInparam || Invalid parameter, keyword = OUT_STATIONS_FORMAT.")
        paths = []
        if "ascii" in fmts:
            paths += self.write_ascii(seis_rtz, strain=strain, curl=curl)
        if "netcdf" in fmts:
            paths.append(self.write_netcdf(seis_rtz, strain=strain, curl=curl))
        if "netcdf_no_assemble" in fmts:
            paths.append(self.write_netcdf(seis_rtz, path=self.output_dir / "stations" / "axisem3d_synthetics.nc.rank0",
                                           strain=strain, curl=curl))
        return paths

    # ------------------------------------------------------------------ run
    def run(self, domain=None, nsteps=None, log=None):
        """Newmark::solve through the library; with NU_WISDOM_LEARN on, learns the wisdom
        during the loop and writes it to NU_WISDOM_LEARN_OUTPUT afterwards.  With
        OPTION_LOOP_INFO_INTERVAL > 0 and a `log` callable, the steps run in chunks of that
        many and each chunk reports simulation time, steps done and wall time elapsed /
        remaining / total in hours, as Newmark.cpp:72-88 prints."""
        import time
        from .capi import Ax3dDomain
        dom = domain or Ax3dDomain(self.spec)
        n = nsteps or self.nsteps
        lp = self.learn_parameters()
        if lp:
            dom.set_wisdom_learning(lp[0], lp[1])
        if _flag(self.par, "DEVELOP_RANDOMIZE_DISP0"):
            self.randomize_displacement(dom)
        interval = _int_or(self.par, "OPTION_LOOP_INFO_INTERVAL", 0) if log else 0
        if interval <= 0:
            dom.step(n)
        else:
            t0 = time.perf_counter()
            done = 0
            while done < n:
                k = min(interval, n - done)
                dom.step(k)
                done += k
                elapsed = (time.perf_counter() - t0) / 3600.0
                total = elapsed / done * n
                log(f"  SIMULATION TIME / sec     =   {-self.shift + done * self.dt}\n"
                    f"  TIME STEP / TOTAL STEPS   =   {done} / {n} ({int(100.0 * done / n)}%)\n"
                    f"  WALLTIME ELAPSED  / h     =   {elapsed}\n"
                    f"  WALLTIME REMAINED / h     =   {total - elapsed}\n"
                    f"  WALLTIME TOTAL    / h     =   {total}\n")
        if lp:
            self.dump_wisdom(dom, lp[2])
        seis = dom.seismograms(0, n)
        return self.rotate(seis), dom

    def randomize_displacement(self, dom, seed=0):
        """DEVELOP_RANDOMIZE_DISP0 (Domain::initDisplTinyRandom, Domain.cpp:76-80;
        SolidPoint::randomDispl): orders 0..2 of every point's displacement uniform in
        [-1, 1] (real and imaginary) times 1e-30, masked like the points mask their fields
        (order 0 real; on the axis only the orders and components that survive there).  A
        seeded numpy generator replaces std::rand."""
        rng = np.random.default_rng(seed)
        spec = self.spec
        so, fo = spec.point_offsets()
        for phase, ofs, nc in (("solid", so, 3), ("fluid", fo, 1)):
            n = dom.nsolid if phase == "solid" else dom.nfluid
            if n == 0:
                continue
            u = np.zeros(n, complex)
            for p in np.flatnonzero(ofs >= 0):
                na = int(spec.p_nr[p]) // 2 + 1
                k = min(3, na)
                blk = (rng.uniform(-1, 1, (k, nc)) + 1j * rng.uniform(-1, 1, (k, nc))) * 1e-30
                blk[0] = blk[0].real
                if spec.p_nr[p] % 2 == 0 and k == na:
                    blk[-1] = 0.0  # Nyquist
                if spec.p_axial[p]:
                    if nc == 3:
                        blk[0, :2] = 0.0      # order 0: only z on the axis
                        if k > 1:
                            blk[1, 2] = 0.0   # order 1: no z; s and phi tied
                            blk[1, 1] = 1j * blk[1, 0]
                        blk[2:] = 0.0
                    else:
                        blk[1:] = 0.0
                u[ofs[p]:ofs[p] + k * nc] = blk.ravel()
            dom.set("displ", phase, u)

    def surface_records(self, dom, nsteps=None):
        """The whole-surface records of steps 0..nsteps-1 (one per OUT_STATIONS_RECORD_INTERVAL
        steps, ReceiverCollection.cpp:314-321), one complex array per edge in tag order."""
        n = nsteps or self.nsteps
        if not self.surface_edges:
            return []
        return dom.surface(0, -(-n // self.spec.sf_interval))


def write_inputs(input_dir, mesh_kw=None, nu=2, stf="gauss", hdur=50.0, steps=2000, record_length=None,
                 n_stations=20, depth_km=100.0, seed=0, attenuation=False, system="source_centered",
                 models3d=(), lucky=False, whole_surface="false", ocean="none", station_extra=(),
                 components="RTZ", force=None):
    """Seeded inputs of the small benchmark configuration: mesh, four parfiles, CMTSOLUTION
    (moment tensor ~ N(0, 1e20 N*m) written in dyn*cm) and STATIONS at uniform distance."""
    from . import mesher
    d = Path(input_dir)
    d.mkdir(parents=True, exist_ok=True)
    ds = mesher.write_half_disk(d / "mesh.e", seed=seed, **(mesh_kw or {}))
    dt = float(ds["vals_glo_var"][1])
    rl = record_length if record_length is not None else steps * dt
    vol = f"MODEL_3D_VOLUMETRIC_NUM {len(models3d)}\n" + \
        (f"MODEL_3D_VOLUMETRIC_LIST {' '.join(models3d)}\n" if models3d else "")
    (d / "inparam.model").write_text(f"MODEL_1D_EXODUS_MESH_FILE mesh.e\n{vol}"
                                     f"MODEL_3D_GEOMETRIC_NUM 0\nMODEL_3D_OCEAN_LOAD {ocean}\nMODEL_2D_MODE off\n"
                                     f"MODEL_PLOT_SLICES_NUM 0\nATTENUATION {'true' if attenuation else 'false'}\n")
    (d / "inparam.nu").write_text(f"NU_TYPE constant\nNU_CONST {nu}\nNU_WISDOM_LEARN false\n")
    (d / "inparam.time_src_recv").write_text(
        f"TIME_DELTA_T 0.0\nTIME_DELTA_T_FACTOR 1.0\nTIME_RECORD_LENGTH {rl}\nSOURCE_TYPE {'point_force' if force else 'earthquake'}\n"
        f"SOURCE_FILE {'POINTFORCE' if force else 'CMTSOLUTION'}\nSOURCE_TIME_FUNCTION {stf}\nSOURCE_STF_HALF_DURATION {hdur}\n"
        f"OUT_STATIONS_FILE STATIONS\nOUT_STATIONS_SYSTEM {system}\nOUT_STATIONS_DUPLICATED rename\n"
        f"OUT_STATIONS_FORMAT netcdf\nOUT_STATIONS_COMPONENTS {components}\nOUT_STATIONS_RECORD_INTERVAL 1\n"
        f"OUT_STATIONS_DUMP_INTERVAL 1000\nOUT_STATIONS_WHOLE_SURFACE {whole_surface}\nOUT_STATIONS_DEPTH_REF false\n")
    (d / "inparam.advanced").write_text(
        f"ATTENUATION_CG4 true\nATTENUATION_SPECFEM_LEGACY false\nATTENUATION_QKAPPA true\n"
        f"OPTION_VERBOSE_LEVEL essential\nOPTION_STABILITY_INTERVAL 100\nOPTION_LOOP_INFO_INTERVAL 1000\n"
        f"DEVELOP_MAX_TIME_STEPS {steps}\nDEVELOP_NON_SOURCE_MODE false\n"
        f"FFTW_LUCKY_NUMBER {'true' if lucky else 'false'}\n")
    rng = np.random.default_rng(seed)
    m = rng.normal(0.0, 1e20, 6) * 1e7  # N*m -> dyn*cm (Source.cpp:171-177)
    names = ["Mrr", "Mtt", "Mpp", "Mrt", "Mrp", "Mtp"]
    (d / "CMTSOLUTION").write_text(
        "PDE 2026 1 1 0 0 0.0 0.0 0.0 100.0 6.0 6.0 SYNTHETIC\nevent name:     synthetic\ntime shift:      0.00\n"
        f"half duration:   {hdur:.2f}\nlatitude:       0.0\nlongitude:      0.0\ndepth:          {depth_km:.4f}\n"
        + "".join(f"{k}:       {v:.6e}\n" for k, v in zip(names, m)))
    if force:  # point force (Ft, Fp, Fr) in N at the same place (PointForce, Source.cpp:190-226)
        (d / "POINTFORCE").write_text(f"latitude:  0.0\nlongitude: 0.0\ndepth:     {depth_km:.4f}\n"
                                      + "".join(f"{k}:  {v:.6e}\n" for k, v in zip(("Ft", "Fp", "Fr"), force)))
    dist = np.linspace(10.0, 170.0, n_stations)
    extra = [f"  {station_extra[i % len(station_extra)]}" if station_extra else "" for i in range(n_stations)]
    (d / "STATIONS").write_text("".join(f"S{i:03d}       SY       {t:.4f}     {(37.0 * i) % 360:.4f}    0.0    0.0"
                                        f"{extra[i]}\n" for i, t in enumerate(dist)))
    return d
