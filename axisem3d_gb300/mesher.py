"""Seeded meridional half-disk mesher writing an Exodus-II file (NetCDF classic).

The reference meshes come from salvus_mesher_lite, which is not part of the reference
repository; this module writes the subset of the Exodus schema that the reference's
ExodusModel reads (SOLVER/src/preloop/exodus/ExodusModel.cpp:53-247, 519-573):
coordx/coordy, connect1 (1-based), name_glo_var/vals_glo_var (radius, dt, nr_lin_solids,
f_min, f_max, f_ref, w_i, y_i), info_records ("crdsys = spherical"), ss_names +
elem_ss#/side_ss# for the axis "t0", the surface "r1" and "solid_fluid_boundary",
ellipticity [2][n], name_elem_var + vals_elem_var#eb1 for element_type (0 spherical,
1 linear, 2 semi-spherical), fluid, dt and nodal VP_k, VS_k, RHO_k, QMU_k, QKAPPA_k
(k = element node 0..3).

Geometry (meridional half plane s >= 0): spherical shells between radius r_c and R with
n_theta elements in colatitude, a semi-spherical ring from the square's boundary to r_c,
and a central square [0, a] x [-a, a] of linear elements.  Elements touching the south
part of the axis are ordered with their curved side 0 so that the axis is side 3, as
Quad requires (Quad.cpp:93-104).  Layers: crust 0-35 km (Vp 5.8, Vs 3.2, rho 2.6), mantle
to 2891 km depth (linear in radius 8.0->13.7, 4.5->7.3, 3.4->5.5), fluid core (8.0->11.0,
Vs 0, 9.9->13.0), the three-layer Earth of the small benchmark configuration.
"""
from __future__ import annotations

import numpy as np

from . import attenuation as ATT
from . import netcdf as NC

R_EARTH = 6371e3
R_MOHO = R_EARTH - 35e3
R_CMB = R_EARTH - 2891e3


def three_layer(r):
    """(vp, vs, rho) in SI at radius r (array); `side` picks the layer at a discontinuity."""
    r = np.asarray(r, float)
    vp = np.empty_like(r)
    vs = np.empty_like(r)
    rho = np.empty_like(r)
    crust = r >= R_MOHO
    mantle = (r >= R_CMB) & ~crust
    core = r < R_CMB
    vp[crust], vs[crust], rho[crust] = 5.8e3, 3.2e3, 2.6e3
    x = (r[mantle] - R_CMB) / (R_MOHO - R_CMB)  # 0 at CMB, 1 at Moho
    vp[mantle] = (13.7 - 5.7 * x) * 1e3
    vs[mantle] = (7.3 - 2.8 * x) * 1e3
    rho[mantle] = (5.5 - 2.1 * x) * 1e3
    x = r[core] / R_CMB  # 0 at centre, 1 at CMB
    vp[core] = (11.0 - 3.0 * x) * 1e3
    vs[core] = 0.0
    rho[core] = (13.0 - 3.1 * x) * 1e3
    return vp, vs, rho


def _radii(r0, r1, h):
    n = max(1, int(np.ceil((r1 - r0) / h)))
    return np.linspace(r0, r1, n + 1)


def half_disk(n_theta=96, h_mantle=100e3, h_core=110e3, r_c=1500e3, seed=0, courant=0.6,
              nsls=3, f_min=1 / 200.0, f_max=1 / 10.0, f_ref=1.0, qmu=(600.0, 80.0), qkappa=57823.0,
              ti=False, rotate_axis=False, rotate_all=False):
    """Return a NetCDF Dataset with the Exodus schema.  n_theta must be a multiple of 4.
    ti: write the transversely isotropic variables (VPV, VPH, VSV, VSH, ETA) with radial
    anisotropy in the top 220 km of the mantle (vph = 1.03 vpv, vsh = 1.04 vsv, eta = 0.95),
    as PREM-like meshes do.  rotate_axis: store the axial elements with their nodes rotated so
    that the axis is side 0, 1 or 2 (in turn), as meshers may write them.  rotate_all: store
    every other element with its nodes rotated by e % 4 (its curved side then 0, 1, 2 or 3):
    the same Earth in other local orientations."""
    if n_theta % 4:
        raise ValueError("n_theta must be a multiple of 4")
    rng = np.random.default_rng(seed)
    nc = n_theta // 4
    a = 0.8 * r_c / np.sqrt(2.0)
    thetas = np.linspace(0.0, np.pi, n_theta + 1)
    # radial knots of the shells (layer boundaries are knots)
    rs = np.unique(np.concatenate([_radii(r_c, R_CMB, h_core), _radii(R_CMB, R_MOHO, h_mantle), [R_MOHO, R_EARTH]]))
    nodes_sz = []
    node_id = {}

    def nid(s, z):
        key = (round(s, 3), round(z, 3))
        if key not in node_id:
            node_id[key] = len(nodes_sz)
            nodes_sz.append((s, z))
        return node_id[key]

    quads, etype = [], []
    # central square [0, a] x [-a, a]: nc x 2nc linear elements
    sg = np.linspace(0.0, a, nc + 1)
    zg = np.linspace(-a, a, 2 * nc + 1)
    for i in range(nc):
        for j in range(2 * nc):
            quads.append([nid(sg[i], zg[j]), nid(sg[i + 1], zg[j]), nid(sg[i + 1], zg[j + 1]), nid(sg[i], zg[j + 1])])
            etype.append(1)
    # square boundary from (0, a) clockwise to (0, -a): 4 nc segments
    bnd = [(sg[i], a) for i in range(nc + 1)] + [(a, zg[2 * nc - j]) for j in range(1, 2 * nc + 1)] + \
          [(sg[nc - i], -a) for i in range(1, nc + 1)]
    circ = [(r_c * np.sin(t), r_c * np.cos(t)) for t in thetas]
    for k in range(n_theta):
        b0, b1, c0, c1 = bnd[k], bnd[k + 1], circ[k], circ[k + 1]
        if k == n_theta - 1:  # touches the south axis: curved side 0, axis side 3
            quads.append([nid(*c1), nid(*c0), nid(*b0), nid(*b1)])
        else:
            quads.append([nid(*b0), nid(*b1), nid(*c1), nid(*c0)])
        etype.append(2)
    # shells
    for ir in range(len(rs) - 1):
        r0, r1 = rs[ir], rs[ir + 1]
        for k in range(n_theta):
            t0, t1 = thetas[k], thetas[k + 1]
            n00 = (r0 * np.sin(t0), r0 * np.cos(t0))
            n01 = (r0 * np.sin(t1), r0 * np.cos(t1))
            n11 = (r1 * np.sin(t1), r1 * np.cos(t1))
            n10 = (r1 * np.sin(t0), r1 * np.cos(t0))
            if k == n_theta - 1:
                quads.append([nid(*n11), nid(*n10), nid(*n00), nid(*n01)])
            else:
                quads.append([nid(*n00), nid(*n01), nid(*n11), nid(*n10)])
            etype.append(0)
    xy = np.array(nodes_sz)
    xy[np.abs(xy[:, 0]) < 1e-6, 0] = 0.0
    conn = np.array(quads, np.int64)
    etype = np.array(etype)
    E = len(conn)
    # element centroids -> layer (fluid / solid), nodal material evaluated per element side
    cen = xy[conn].mean(1)
    rcen = np.hypot(cen[:, 0], cen[:, 1])
    fluid = rcen < R_CMB
    # nodal radii pulled slightly into the element so discontinuities take the element's side
    rn = np.hypot(xy[conn][..., 0], xy[conn][..., 1])
    rin = rn + 1e-3 * (rcen[:, None] - rn)
    vp, vs, rho = three_layer(rin)
    # side sets: axis (side 3 on s = 0), surface (r = R), solid-fluid boundary (r = R_CMB)
    ax_e, ax_s, sf_e, sf_s, su_e, su_s = [], [], [], [], [], []
    for e in range(E):
        for side in range(4):
            p0, p1 = xy[conn[e, side]], xy[conn[e, (side + 1) % 4]]
            if abs(p0[0]) < 1e-6 and abs(p1[0]) < 1e-6:
                ax_e.append(e)
                ax_s.append(side)
            r0, r1 = np.hypot(*p0), np.hypot(*p1)
            if abs(r0 - R_EARTH) < 1.0 and abs(r1 - R_EARTH) < 1.0:
                su_e.append(e)
                su_s.append(side)
            if abs(r0 - R_CMB) < 1.0 and abs(r1 - R_CMB) < 1.0:
                sf_e.append(e)
                sf_s.append(side)
    # the element's time step as AxiSEM's mesher writes it: courant * (shortest element side) /
    # vmax; the solver scales it by the closest GLL distance over that side (Quad::getDeltaT)
    xy4 = xy[conn]
    side = np.hypot(*(xy4 - np.roll(xy4, -1, axis=1)).transpose(2, 0, 1)).min(1)
    dt_e = courant * side / vp.max(1)
    # attenuation: SLS fit and Q per layer
    w, y = ATT.fit_sls(nsls, f_min, f_max)
    qm = np.where(fluid, 1e5, np.where(rcen > R_MOHO, qmu[1], qmu[0]))
    qm = qm * (1 + 0.0 * rng.random(E))

    ds = NC.Dataset()
    ds.add_dim("num_nodes", len(xy))
    ds.add_dim("num_elem", E)
    ds.add_dim("num_el_in_blk1", E)
    ds.add_dim("num_nod_per_el1", 4)
    ds.add_var("coordx", ("num_nodes",), xy[:, 0])
    ds.add_var("coordy", ("num_nodes",), xy[:, 1])
    ds.add_var("connect1", ("num_el_in_blk1", "num_nod_per_el1"), conn + 1, dtype=np.int32)
    gnames = ["radius", "dt", "nr_lin_solids", "f_min", "f_max", "f_ref"] + [f"w_{i}" for i in range(nsls)] + \
             [f"y_{i}" for i in range(nsls)]
    gvals = [R_EARTH, float(dt_e.min()), nsls, f_min, f_max, f_ref] + list(w) + list(y)
    ds.add_strings("name_glo_var", "num_glo_var", "len_string", gnames)
    ds.add_var("vals_glo_var", ("num_glo_var",), np.array(gvals, float))
    ds.add_strings("info_records", "num_info", "len_line", ["crdsys = spherical", f"seed = {seed}"], 81)
    sets = [("t0", ax_e, ax_s), ("r1", su_e, su_s), ("solid_fluid_boundary", sf_e, sf_s)]
    ds.add_strings("ss_names", "num_side_sets", "len_string", [s[0] for s in sets])
    for i, (_, ee, ss) in enumerate(sets):
        ds.add_dim(f"num_side_ss{i + 1}", len(ee))
        ds.add_var(f"elem_ss{i + 1}", (f"num_side_ss{i + 1}",), np.array(ee) + 1, dtype=np.int32)
        ds.add_var(f"side_ss{i + 1}", (f"num_side_ss{i + 1}",), np.array(ss) + 1, dtype=np.int32)
    ds.add_dim("two", 2)
    ds.add_dim("num_ellip", 2)
    # ellipticity profile as AxiSEM's mesher writes it: knots r / R and the flattening relative
    # to the surface's (a linear stand-in for the Clairaut profile, 0.7227 at the centre)
    ds.add_var("ellipticity", ("two", "num_ellip"), np.array([[0.0, 1.0], [0.7227, 1.0]]))
    enames, evals = ["element_type", "fluid", "dt"], [etype.astype(float), fluid.astype(float), dt_e]
    if ti:
        aniso = (rin > R_EARTH - 220e3) & ~fluid[:, None]
        mats = (("VPV", vp), ("VPH", np.where(aniso, 1.03 * vp, vp)), ("VSV", vs),
                ("VSH", np.where(aniso, 1.04 * vs, vs)), ("ETA", np.where(aniso, 0.95, 1.0)))
    else:
        mats = (("VP", vp), ("VS", vs))
    # stored node order: element e's node k is node (k + shift[e]) % 4 of the built element
    shift = {}
    if rotate_axis:  # the axis on side 0, 1 or 2; the reader rotates it back to side 3
        for i, e in enumerate(ax_e):
            shift[e] = (3 - i % 3) % 4
    if rotate_all:  # every other element's nodes rotated as well (curved sides 1 / 3 occur)
        axial_set = set(ax_e)
        for e in range(E):
            if e not in axial_set:
                shift[e] = e % 4
    mats = mats + (("RHO", rho), ("QMU", np.repeat(qm[:, None], 4, 1)), ("QKAPPA", np.full((E, 4), qkappa)))
    if shift:
        conn_w = conn.copy()
        for e, t in shift.items():
            conn_w[e] = conn[e][[(k + t) % 4 for k in range(4)]]
        mats = tuple((nm, _rotate_rows(np.asarray(v, float), shift)) for nm, v in mats)
        ds.variables["connect1"].data[...] = (conn_w + 1).astype(">i4")
        for i, (_, ee, ss) in enumerate(sets):
            ds.variables[f"side_ss{i + 1}"].data[...] = np.array(
                [(sd - shift.get(e, 0)) % 4 for e, sd in zip(ee, ss)], np.int64) + 1
    for nm, v in mats:
        for k in range(4):
            enames.append(f"{nm}_{k}")
            evals.append(v[:, k])
    ds.add_strings("name_elem_var", "num_elem_var", "len_string", enames)
    for i, v in enumerate(evals):
        ds.add_var(f"vals_elem_var{i + 1}eb1", ("num_el_in_blk1",), np.asarray(v, float))
    return ds


def _rotate_rows(v, shift):
    """Nodal values [E, 4] of the elements in shift stored in their rotated node order."""
    v = v.copy()
    for e, t in shift.items():
        v[e] = v[e][[(k + t) % 4 for k in range(4)]]
    return v


def write_half_disk(path, **kw):
    ds = half_disk(**kw)
    NC.write(path, ds)
    return ds
