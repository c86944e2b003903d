"""Batched ensembles: many independent simulations in one domain.

The simulations share no points, so concatenating their packed descriptions gives one
domain whose every kernel launch per step (element buckets, assembly, Newmark) covers all
of them; with the step captured as a CUDA graph the whole ensemble advances with one graph
launch per step.  All members must share dt, the SLS coefficients and the source-time
function (one STF per domain, as in the reference's Domain::setSTF); sources, meshes,
materials and receivers differ freely.
"""
from __future__ import annotations

import numpy as np

from .spec import DomainSpec


def concat(specs: list[DomainSpec]):
    """Returns (spec, info) with info = per-member point, element and receiver ranges."""
    if not specs:
        raise ValueError("ensemble.concat || no members")
    s0 = specs[0]
    for s in specs[1:]:
        if abs(s.dt - s0.dt) > 1e-12 * s0.dt:
            raise ValueError("ensemble.concat || members must share dt")
        if s.nsls != s0.nsls or (s.nsls and not (np.allclose(s.att_alpha, s0.att_alpha)
                                                 and np.allclose(s.att_beta, s0.att_beta)
                                                 and np.allclose(s.att_gamma, s0.att_gamma))):
            raise ValueError("ensemble.concat || members must share the SLS coefficients")
        if len(s.stf) != len(s0.stf) or not np.array_equal(s.stf, s0.stf):
            raise ValueError("ensemble.concat || members must share the source-time function")
    cat = lambda name: np.concatenate([getattr(s, name) for s in specs])
    p_off = np.cumsum([0] + [s.n_points for s in specs])
    e_off = np.cumsum([0] + [s.n_elements for s in specs])
    m_off = np.cumsum([0] + [len(s.e_mod) for s in specs])
    a_off = np.cumsum([0] + [len(s.e_attm) for s in specs])
    r_off = np.cumsum([0] + [len(s.r_elem) for s in specs])
    sources = [(int(e) + int(e_off[i]), f) for i, s in enumerate(specs) for e, f in s.sources]
    spec = DomainSpec(
        dt=s0.dt, p_nr=cat("p_nr"), p_kind=cat("p_kind"), p_axial=cat("p_axial"), p_fsurf=cat("p_fsurf"),
        p_mslen=cat("p_mslen"), p_ms=cat("p_ms"), p_mflen=cat("p_mflen"), p_mf=cat("p_mf"),
        p_sflen=cat("p_sflen"), p_sfn=np.concatenate([s.p_sfn.reshape(-1, 3) for s in specs]),
        p_sfni=np.concatenate([s.p_sfni.reshape(-1, 3) for s in specs]),
        e_pts=np.concatenate([s.e_pts + p_off[i] for i, s in enumerate(specs)]).astype(np.int32),
        e_mat=cat("e_mat"), e_axial=cat("e_axial"), e_in3d=cat("e_in3d"), e_geo=cat("e_geo"),
        e_trig=cat("e_trig"),
        e_mofs=np.concatenate([s.e_mofs + m_off[i] for i, s in enumerate(specs)]).astype(np.int64),
        e_mod=cat("e_mod"), e_att=cat("e_att"),
        e_aofs=np.concatenate([s.e_aofs + a_off[i] for i, s in enumerate(specs)]).astype(np.int64),
        e_attm=cat("e_attm"), nsls=s0.nsls, att_alpha=s0.att_alpha, att_beta=s0.att_beta,
        att_gamma=s0.att_gamma, att_do_kappa=s0.att_do_kappa, sources=sources, stf=s0.stf,
        r_elem=np.concatenate([s.r_elem + e_off[i] for i, s in enumerate(specs)]).astype(np.int32),
        r_phi=cat("r_phi"), r_w=np.concatenate([s.r_w.reshape(-1, 25) for s in specs]),
        kahan=s0.kahan, stability_interval=s0.stability_interval)
    info = {"points": list(zip(p_off[:-1], p_off[1:])), "elements": list(zip(e_off[:-1], e_off[1:])),
            "receivers": list(zip(r_off[:-1], r_off[1:]))}
    return spec, info


def split_seismograms(seis, info):
    """[steps][all receivers][3] -> list of per-member [steps][receivers][3]."""
    return [seis[:, a:b] for a, b in info["receivers"]]
