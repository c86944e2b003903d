"""Particle relabelling pre-loop: undulations of 3-D geometric models -> the quantities a
relabelled element and its points take (FP64, host).

Restates SOLVER/src/preloop/physics/relabelling/Relabelling.cpp:
  addUndulation (32-58)        deltaR of every model on the element's Nr slices, at the GLL
                               points rotated to geocentric coordinates
                               (Quad::computeGeocentricGlobal, Quad.cpp:468-481)
  getStiffJacobian (60-83)     J = (1 + dZ/Z)^2 (1 + dZ_Z), or (1 + dZ_Z)^3 at the centre
  getStiffX (85-109)           X0 = 1/J0, X1 = -J1/(J0 J3), X2 = -J2/(J0 J3), X3 = 1/J3
  getMassJacobian (111-132)    as the stiffness Jacobian on each point's own Nr
  getSFNormalRTZ (134-152)     (-J1 J0, -J2 J0, J0^2)
  isZero / isPar1D (154-160)
  checkHmin (182-206)          Gaussian smoothing of increasing order until the deformed
                               element's smallest GLL distance, resampled five times
                               denser, stays above 0.8 of its minimum over the slices
                               (Quad::getHminSlices, Quad.cpp:630-654)
  formGradientUndulation (208-268) the gradient of dZ by R2C, the element's scalar gradient
                               (PreloopGradient::gradScalar, PreloopGradient.cpp:17-47) and
                               C2R, rotated from (s, phi, z) to (R = theta, T = phi, Z = r)
  formMassUndulation (270-281) linear resampling to each point's Nr
with XMath::gaussianSmoothing, trigonResampling, linearResampling and findClosestDist
(SOLVER/src/preloop/utilities/XMath.cpp:18-31, 74-186).  Transforms follow FFTW's
conventions (R2C x 1/n, C2R unnormalised) as PreloopFFTW does (PreloopFFTW.cpp:47-57).

Geometric models (MODEL_3D_GEOMETRIC_LIST, Geometric3D::buildInparam, Geometric3D.cpp:19-70).
The reference's crust1 and EMC models read data tables that are not shipped; this project
provides one analytic model with the same interface (deltaR at a point, given in the
source-centred frame):
  bump$r_km$lat$lon$height_km$hwhm_deg$taper_km[$src_centred]
      an interface at radius r_km raised by height_km * exp(-d^2 / (2 sd^2)) at angular
      distance d from (lat, lon), sd = hwhm / sqrt(2 ln 2); the displacement tapers
      linearly to zero at r_km +- taper_km (above the surface it is cut), so the points of
      neighbouring elements agree.
"""
from __future__ import annotations

import math

import numpy as np

from . import spectral as S

TINY = 1e-10  # tinyDouble (SOLVER/src/global.h:9)


def _truthy(s):
    return s.strip().lower() in ("true", "1", "yes", "on")


def _rotation(theta, phi):
    ct, st, cp, sp = math.cos(theta), math.sin(theta), math.cos(phi), math.sin(phi)
    return np.array([[ct * cp, -sp, st * cp], [ct * sp, cp, st * sp], [-st, 0.0, ct]])


class Bump:
    """Gaussian undulation of a spherical interface (see the module docstring)."""

    def __init__(self, params, src_latlon, R):
        if len(params) < 6:
            raise ValueError("Geometric3D_bump::initialize || need r_km, lat, lon, height_km, hwhm_deg, taper_km")
        r_km, lat, lon, h_km, hwhm, taper = (float(p) for p in params[:6])
        src_centred = _truthy(params[6]) if len(params) > 6 else False
        self.rb, self.h, self.taper, self.R = r_km * 1e3, h_km * 1e3, taper * 1e3, R
        self.sd = math.radians(hwhm) / math.sqrt(2.0 * math.log(2.0))
        if src_centred:
            t, p = math.radians(lat), math.radians(lon)
            self.n0 = np.array([math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t)])
        else:
            t, p = math.radians(90.0 - lat), math.radians(lon)
            ng = np.array([math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t)])
            slat, slon = src_latlon
            self.n0 = _rotation(math.radians(90.0 - slat), math.radians(slon)).T @ ng

    def delta_r(self, xyz, r_center):
        """xyz (..., 3) source-frame Cartesian [m] -> deltaR (...)."""
        r = np.linalg.norm(xyz, axis=-1)
        cosd = np.clip((xyz @ self.n0) / np.where(r > 0, r, 1.0), -1.0, 1.0)
        d = np.arccos(cosd)
        w = np.clip(1.0 - np.abs(r - self.rb) / self.taper, 0.0, None)
        w = np.where(r > self.R * (1 + 1e-12), 0.0, w)
        return np.where(r > 0, self.h * np.exp(-d * d / (2 * self.sd * self.sd)) * w, 0.0)


def geometric_models(par, src_latlon, R):
    """Geometric3D::buildInparam: the MODEL_3D_GEOMETRIC_NUM models of the list."""
    try:
        n = par.get("MODEL_3D_GEOMETRIC_NUM", int)
    except KeyError:
        return []
    out = []
    for i in range(n):
        try:
            entry = par.get("MODEL_3D_GEOMETRIC_LIST", str, i)
        except (KeyError, IndexError):
            raise ValueError("Geometric3D::buildInparam || Not enough model names provided in "
                             f"MODEL_3D_GEOMETRIC_LIST, MODEL_3D_GEOMETRIC_NUM = {n}")
        strs = entry.split("$")
        name, params = strs[0].lower(), strs[1:]
        if name == "bump":
            out.append(Bump(params, src_latlon, R))
        else:
            raise NotImplementedError(f"Geometric3D::buildInparam || geometric model {strs[0]} is not built "
                                      "(its data files are not shipped); the analytic 'bump' model is")
    return out


# ------------------------------------------------------------------ XMath
def gaussian_smoothing(data, order, dev, period=True):
    """XMath::gaussianSmoothing (XMath.cpp:74-115) of a ring of values."""
    n = len(data)
    order = min(order, (n + 1) // 2 - 1)
    if n == 0 or order <= 0:
        return np.asarray(data, float).copy()
    dev = dev * order
    i = np.arange(order + 1)
    g = np.exp(-0.5 * i * i / (dev * dev))
    ker = np.concatenate([g[:0:-1], g])
    ker /= ker.sum()
    out = np.zeros(n)
    for j in range(-order, order + 1):
        k = np.arange(n) + j
        k = k % n if period else np.clip(k, 0, n - 1)
        out += ker[j + order] * np.asarray(data, float)[k]
    return out


def equal_rows(m, tol=TINY):
    """XMath::equalRows (XMath.h:68-74): every row within tol (relative) of the first."""
    m = np.asarray(m, float)
    if m.ndim == 1:
        m = m[:, None]
    n0 = np.linalg.norm(m[0])
    return bool(np.all(np.linalg.norm(m[1:] - m[0], axis=1) <= tol * n0))


def trigon_resampling(new_size, original):
    """XMath::trigonResampling (XMath.cpp:132-159): Fourier interpolation onto new_size slices."""
    x = np.asarray(original, float)
    n = len(x)
    if new_size == n:
        return x.copy()
    if equal_rows(x):
        return np.full(new_size, x[0])
    F = np.fft.rfft(x) / n
    a = np.arange(len(F))
    w = np.where((n % 2 == 0) & (a == len(F) - 1), 1.0, 2.0)
    w[0] = 1.0
    phi = 2 * math.pi * np.arange(new_size) / new_size
    F = F.copy()
    F[0] = F[0].real
    return np.real((w * F)[None, :] * np.exp(1j * np.outer(phi, a))).sum(1)


def linear_resampling(new_size, original):
    """XMath::linearResampling (XMath.cpp:161-186)."""
    x = np.asarray(original, float)
    n = len(x)
    if new_size == n:
        return x.copy()
    if equal_rows(x):
        return np.full(new_size, x[0])
    dphi, dphi0 = 2 * math.pi / new_size, 2 * math.pi / n
    p = np.arange(new_size) * dphi
    l0 = (p / dphi0).astype(int)
    l1 = np.where(l0 + 1 == n, 0, l0 + 1)
    return (x[l1] - x[l0]) / dphi0 * (p - l0 * dphi0) + x[l0]


def closest_dist(c):
    """XMath::findClosestDist (XMath.cpp:18-31) of points c (n, 2)."""
    d = np.linalg.norm(c[:, None, :] - c[None, :, :], axis=-1)
    d[np.diag_indices(len(c))] = np.inf
    return float(d.min())


# ------------------------------------------------------------------ transforms (FFTW conventions)
def r2c(x):
    """R2C x 1/n: orders 0..n/2 of a real ring."""
    return np.fft.rfft(np.asarray(x, float)) / len(x)


def c2r(X, n):
    """C2R, unnormalised, reading only Re of order 0 (and of the Nyquist order of an even n)."""
    X = np.array(X, complex)
    X[0] = X[0].real
    if n % 2 == 0:
        X[n // 2] = X[n // 2].real
    return np.fft.irfft(X, n) * n


# ------------------------------------------------------------------ one element
class Relabelled:
    """Relabelling of one element.  geo: [5, 25] operators (dsdxii, dsdeta, dzdxii, dzdeta,
    inv_s); crds: [25, 2] (s, z); nr: the element's Nr; point_nr: [25]; axial."""

    def __init__(self, models, geo, crds, nr, point_nr, axial, r_center, phi2d=None):
        self.geo, self.crds, self.nr, self.point_nr, self.axial = geo, crds, int(nr), np.asarray(point_nr), axial
        self.Z = np.hypot(crds[:, 0], crds[:, 1])
        self.theta = np.where(self.Z < 1e-10, 0.0, np.arccos(np.clip(crds[:, 1] / np.where(self.Z > 0, self.Z, 1), -1, 1)))
        # addUndulation: deltaR on the Nr slices of every GLL point
        phi = 2 * math.pi * np.arange(self.nr) / self.nr if phi2d is None else np.full(self.nr, float(phi2d))
        s, z = crds[:, 0], crds[:, 1]
        xyz = np.stack([s[None, :] * np.cos(phi)[:, None], s[None, :] * np.sin(phi)[:, None],
                        np.broadcast_to(z[None, :], (self.nr, 25))], -1)
        dz = np.zeros((self.nr, 25))
        for m in models:
            dz += m.delta_r(xyz, r_center)
        self.dZ = dz
        self.dZdR = np.zeros_like(dz)
        self.dZdT = np.zeros_like(dz)
        self.dZdZ = np.zeros_like(dz)
        self.zero = bool(np.abs(dz).max() < TINY)
        if not self.zero:
            self.check_hmin()
            self.form_gradient()

    # Quad::getHminSlices with the current undulation
    def hmin_slices(self):
        base = self.crds
        st, ct = np.sin(self.theta), np.cos(self.theta)
        return np.array([closest_dist(base + np.stack([self.dZ[k] * st, self.dZ[k] * ct], 1))
                         for k in range(self.nr)])

    def hmin_ref(self):
        return closest_dist(self.crds)

    def check_hmin(self):
        original = self.dZ.copy()
        max_order = (self.nr + 1) // 2 - 1
        for order in range(max_order + 1):
            self.dZ = np.stack([gaussian_smoothing(original[:, p], order, 100.0, True) for p in range(25)], 1)
            hmin = self.hmin_slices()
            if trigon_resampling(5 * self.nr, hmin).min() >= hmin.min() * 0.8:
                return
        raise RuntimeError("Relabelling::checkHmin || Program should not have reached here.")

    def form_gradient(self):
        nr, nu = self.nr, self.nr // 2
        if nr % 2 == 0:  # mask the Nyquist order first
            self.dZ = np.stack([trigon_resampling(nr, trigon_resampling(nr - 1, self.dZ[:, p])) for p in range(25)], 1)
        U = np.stack([r2c(self.dZ[:, p]) for p in range(25)], 1)  # [nu + 1][25]
        Gl = S.gll()[2]
        Gx = S.glj()[2] if self.axial else Gl
        dsdxii, dsdeta, dzdxii, dzdeta, inv_s = (self.geo[i].reshape(5, 5) for i in range(5))
        nyq = nr % 2 == 0
        grad = np.zeros((nu + 1, 3, 5, 5), complex)
        for a in range(nu + 1 - nyq):
            u = U[a].reshape(5, 5)
            GU = Gx.T @ u
            UG = u @ Gl
            grad[a, 0] = dzdeta * GU + dzdxii * UG
            grad[a, 1] = inv_s * (1j * a * u)
            grad[a, 2] = dsdeta * GU + dsdxii * UG
        if self.axial:  # PreloopGradient::gradScalar's axial masking
            grad[0, 0, 0] = 0
            grad[0, 1, 0] = 0
            if nu >= 1:
                grad[1, 1, 0] = 1j * grad[1, 0, 0]
                grad[1, 2, 0] = 0
            grad[2:, :, 0] = 0
        g = grad.reshape(nu + 1, 3, 25)
        drds = np.stack([c2r(g[:, 0, p], nr) for p in range(25)], 1)
        self.dZdT = np.stack([c2r(g[:, 1, p], nr) for p in range(25)], 1)
        drdz = np.stack([c2r(g[:, 2, p], nr) for p in range(25)], 1)
        st, ct = np.sin(self.theta), np.cos(self.theta)
        self.dZdZ = drdz * ct + drds * st
        self.dZdR = -drdz * st + drds * ct

    # ---- products ----
    def par1d(self):
        return equal_rows(self.dZ)

    def _j0(self, dz, dzdz):
        centre = self.Z < TINY
        return np.where(centre, 1.0 + dzdz, 1.0 + dz / np.where(centre, 1.0, self.Z))

    def stiff_jacobian(self):
        J0 = self._j0(self.dZ, self.dZdZ)
        J22 = 1.0 + self.dZdZ
        J = np.where(self.Z < TINY, J22 ** 3, J0 * J0 * J22)
        if J.min() <= 0:
            raise RuntimeError("Relabelling::getStiffJacobian || Negative Jacobian.")
        return J

    def stiff_x(self):
        """[4][Nr][25]."""
        J0 = self._j0(self.dZ, self.dZdZ)
        J3 = 1.0 + self.dZdZ
        return np.stack([1.0 / J0, -self.dZdR / (J0 * J3), -self.dZdT / (J0 * J3), 1.0 / J3])

    def mass_fields(self, p):
        """dZ, dZ_R, dZ_T, dZ_Z of point p resampled to its own Nr (formMassUndulation)."""
        n = int(self.point_nr[p])
        return [linear_resampling(n, f[:, p]) for f in (self.dZ, self.dZdR, self.dZdT, self.dZdZ)]

    def mass_jacobian(self, p):
        dz, _, _, dzdz = self.mass_fields(p)
        J22 = 1.0 + dzdz
        if self.Z[p] < TINY:
            J = J22 ** 3
        else:
            J00 = 1.0 + dz / self.Z[p]
            J = J00 * J00 * J22
        if J.min() <= 0:
            raise RuntimeError("Relabelling::getMassJacobian || Negative Jacobian.")
        return J

    def sf_normal_rtz(self, p):
        """[Nr_p][3] (R, T, Z) of the undulated boundary's normal (getSFNormalRTZ)."""
        dz, dzdr, dzdt, dzdz = self.mass_fields(p)
        J0 = 1.0 + dzdz if self.Z[p] < TINY else 1.0 + dz / self.Z[p]
        return np.stack([-dzdr * J0, -dzdt * J0, J0 * J0], 1)
