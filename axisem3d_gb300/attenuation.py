"""FP64 attenuation precompute: SLS fit and the AxiSEM attenuation factors.

* fit_sls: relaxation frequencies w_l (log-spaced over the band) and weights y_l fitted
  in FP64 by least squares so that Q^-1(omega) = sum_l y_l omega w_l / (omega^2 + w_l^2)
  is flat over [f_min, f_max] (the standard-linear-solid approximation of constant Q,
  Emmerich & Korn 1987).  The reference reads these from its mesher
  (SOLVER/src/preloop/exodus/ExodusModel.cpp:533-549); the mesher is not part of the
  reference repository, so this project fits its own.
* att_factors: AttAxiSEM::computeAttFactors (SOLVER/src/preloop/physics/attenuation/AttAxiSEM.cpp:14-57).
* apply_attenuation: AttBuilder::createAttenuation1D/3D
  (SOLVER/src/preloop/physics/attenuation/AttBuilder.cpp:17-129) with the Voigt split of
  Material::createElastic (SOLVER/src/preloop/physics/material/Material.cpp:336-355).
"""
from __future__ import annotations

import numpy as np

from .geometry import cg4_weights

CG4_POINTS = (6, 8, 16, 18)  # (1,1), (1,3), (3,1), (3,3)


def fit_sls(nsls: int, f_min: float, f_max: float, nfreq: int = 200):
    w = 2 * np.pi * np.logspace(np.log10(f_min), np.log10(f_max), nsls)
    om = 2 * np.pi * np.logspace(np.log10(f_min), np.log10(f_max), nfreq)
    A = om[:, None] * w[None, :] / (om[:, None] ** 2 + w[None, :] ** 2)
    y, *_ = np.linalg.lstsq(A, np.ones(nfreq), rcond=None)
    return w, y


def att_factors(w, y, f_min, f_max, f_ref, dt, qkappa, qmu, do_kappa):
    """AttAxiSEM::computeAttFactors -> alpha, beta, gamma, (dkp, kpAtt, kpNoAtt), (dmu, muAtt, muNoAtt)."""
    w = np.asarray(w, float)
    y = np.asarray(y, float)
    ysum = y.sum()
    yd = y / ysum
    w0 = f_ref * 2 * np.pi
    w1 = np.sqrt(f_min * f_max) * 2 * np.pi
    fact = float(np.sum(yd * w * w / (w1 * w1 + w * w)))
    alpha = np.exp(-w * dt)
    beta = ((1 - alpha) / (w * dt) - alpha) * yd
    gamma = ((alpha - 1) / (w * dt) + 1) * yd
    qkappa = np.asarray(qkappa, float)
    qmu = np.asarray(qmu, float)
    if do_kappa:
        kp_no = 1 + 2 * np.log(w1 / w0) / np.pi / qkappa
        dkp = kp_no / (qkappa / ysum + (1 - fact))
        kp_att = kp_no + dkp * fact
    else:
        dkp = np.zeros_like(qkappa)
        kp_att = np.ones_like(qkappa)
        kp_no = np.ones_like(qkappa)
    mu_no = 1 + 2 * np.log(w1 / w0) / np.pi / qmu
    dmu = mu_no / (qmu / ysum + (1 - fact))
    mu_att = mu_no + dmu * fact
    return alpha, beta, gamma, (dkp, kp_att, kp_no), (dmu, mu_att, mu_no)


def voigt_ti(A, C, F, L, N):
    """Voigt average of a TI tensor (Material.cpp:338-339)."""
    kappa = (4 * A + C + 4 * F - 4 * N) / 9
    mu = (A + C - 2 * F + 6 * L + 5 * N) / 15
    return kappa, mu


def apply_attenuation(kappa, mu, qkappa, qmu, ifact, cg4, factors):
    """AttBuilder: returns (kappa', mu', dkappa_att, dmu_att) for one element.

    kappa, mu, qkappa, qmu have shape (nr, 25) (nr = 1 for 1D elements).  dkappa_att
    / dmu_att have shape (nr, 4) for CG4 and (nr, 25) otherwise."""
    (dkf, kp_att, kp_no), (dmf, mu_att, mu_no) = factors
    kappa = np.array(kappa, float)
    mu = np.array(mu, float)
    if cg4:
        wcg = cg4_weights(ifact)
        idx = list(CG4_POINTS)
        dk = wcg[None, :] * dkf[:, idx] * kappa[:, idx]
        dm = wcg[None, :] * dmf[:, idx] * mu[:, idx]
        kappa = kappa * kp_no
        mu = mu * mu_no
        for i, p in enumerate(idx):
            kappa[:, p] *= 1 + wcg[i] * (kp_att[:, p] / kp_no[:, p] - 1)
            mu[:, p] *= 1 + wcg[i] * (mu_att[:, p] / mu_no[:, p] - 1)
    else:
        dk = dkf * kappa
        dm = dmf * mu
        kappa = kappa * kp_att
        mu = mu * mu_att
    return kappa, mu, dk, dm
