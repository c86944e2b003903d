"""DomainSpec: the packed, structure-of-arrays description of a domain.

It is exactly what the C-ABI (include/ax3d.h) consumes: one record per GLL point and
per element, the source terms, the source-time function and the receivers.  Builders
(the mesher, the synthetic element benchmark, tests) produce a DomainSpec; the GB300
library (capi.Ax3dDomain) consumes it.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import spectral as S

MAT_ISO, MAT_TISO, MAT_ANISO, MAT_ACOUSTIC = 0, 1, 2, 3
ATT_NONE, ATT_FULL, ATT_CG4 = 0, 1, 2
POINT_SOLID, POINT_FLUID, POINT_SOLID_FLUID = 0, 1, 2
N_MODULI = {MAT_ISO: 2, MAT_TISO: 5, MAT_ANISO: 21, MAT_ACOUSTIC: 1}


@dataclass
class DomainSpec:
    dt: float
    # points
    p_nr: np.ndarray          # int32 [P]
    p_kind: np.ndarray        # int8  [P]
    p_axial: np.ndarray       # uint8 [P]
    p_fsurf: np.ndarray       # uint8 [P]
    p_mslen: np.ndarray       # int32 [P]
    p_ms: np.ndarray          # float32 concat
    p_mflen: np.ndarray       # int32 [P]
    p_mf: np.ndarray          # float32 concat
    p_sflen: np.ndarray       # int32 [P]
    p_sfn: np.ndarray         # float32 [sum len, 3]
    p_sfni: np.ndarray        # float32 [sum len, 3]
    # elements
    e_pts: np.ndarray         # int32 [E, 25]
    e_mat: np.ndarray         # int8  [E]
    e_axial: np.ndarray       # uint8 [E]
    e_in3d: np.ndarray        # uint8 [E]
    e_geo: np.ndarray         # float32 [E, 5, 25]
    e_trig: np.ndarray        # float32 [E, 4, 25]
    e_mofs: np.ndarray        # int64 [E]
    e_mod: np.ndarray         # float32 concat
    e_att: np.ndarray         # int8 [E]
    e_aofs: np.ndarray        # int64 [E]
    e_attm: np.ndarray        # float32 concat
    # attenuation (global SLS factors)
    nsls: int = 0
    att_alpha: np.ndarray = field(default_factory=lambda: np.zeros(0))
    att_beta: np.ndarray = field(default_factory=lambda: np.zeros(0))
    att_gamma: np.ndarray = field(default_factory=lambda: np.zeros(0))
    att_do_kappa: bool = False
    # sources: list of (element, force [25, norders, 3] complex64)
    sources: list = field(default_factory=list)
    stf: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    # receivers
    r_elem: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    r_phi: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    r_w: np.ndarray = field(default_factory=lambda: np.zeros((0, 25), np.float32))
    # (s, z) of every point; informational (tests, output), not passed to the library
    p_crds: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    # particle relabelling (PRT_1D / PRT_3D): elements, length 1 or nr, X [4][len][25] each
    prt_elem: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    prt_len: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    prt_x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    # per receiver: bit 0 dump_strain, bit 1 dump_curl (empty: none)
    r_dump: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    # whole-surface recorder: edges (element, side 0..3) recorded every sf_interval steps
    sf_elem: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    sf_side: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    sf_interval: int = 1
    # ocean load (MassOcean1D / MassOcean3D) on solid points: len 1 -> (1/(m + m_ocean), 1/m,
    # sin theta, cos theta), len nr -> nr x (1/m, scaled unit normal s, phi, z)
    oc_pt: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    oc_len: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    oc_vals: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    kahan: bool = False
    stability_interval: int = 0

    @property
    def n_points(self) -> int:
        return len(self.p_nr)

    @property
    def n_elements(self) -> int:
        return len(self.e_mat)

    def element_nr(self) -> np.ndarray:
        return self.p_nr[self.e_pts].max(axis=1)

    def field_sizes(self):
        na = self.p_nr // 2 + 1
        ns = int(3 * na[self.p_kind != POINT_FLUID].sum())
        nf = int(na[self.p_kind != POINT_SOLID].sum())
        return ns, nf

    def point_offsets(self):
        """Complex offsets of every point's solid and fluid blocks (-1 if absent)."""
        na = self.p_nr.astype(np.int64) // 2 + 1
        hs = self.p_kind != POINT_FLUID
        hf = self.p_kind != POINT_SOLID
        so = np.where(hs, np.cumsum(np.where(hs, 3 * na, 0)) - np.where(hs, 3 * na, 0), -1)
        fo = np.where(hf, np.cumsum(np.where(hf, na, 0)) - np.where(hf, na, 0), -1)
        return so, fo


def g_matrices():
    """G(i,j) = l_i'(xi_j) on GLL and GLJ(0,1) nodes, row-major [25] FP64."""
    return S.gll()[2].ravel().copy(), S.glj()[2].ravel().copy()
