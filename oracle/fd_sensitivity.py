"""Restatement of the reference's finite-difference shape sensitivities (test
infrastructure only): IWG::select_dRdp_FD_geometry_bulk / _double
(FEM/INT/src/IWG/cl_FEM_IWG.cpp:2997-3154) perturb one coordinate of one
IG vertex inside one cluster, re-evaluate that cluster's residual (and the
cluster measures of the Nitsche parameter, add_cluster_measure_dRdp_FD_
geometry, :3827-3924) and difference it:

  * step: relative, delta = |1e-6 * (max - min of the IP cell's coordinate)/3|
    clamped to [1e-12, (max - min)/3] (IWG::build_perturbation_size_relative,
    :2846-2872, mToleranceFD = 1e-12, finite_difference_perturbation_size 1e-6,
    PRM/src/fn_PRM_FEM_Parameters.hpp:297-319);
  * scheme: forward (POINT_1_FORWARD), backward where the perturbed point
    would leave the IP cell (check_ig_coordinates_inside_ip_element, :2900-2992);
  * the per-cluster derivatives are summed per vertex (the pdv assembly).

Contracted with the adjoint: g_(v,d) = d(Q - lambda^T R)/dx_(v,d), and with the
intersection-vertex direction: dF/dt_v = g_v . (x_p1 - x_p0).
"""
import numpy as np

from .oracle import OracleModel

CELL_HEX8, CELL_TRI3, SHAPE_RECT, MODEL_3D = 1, 2, 0, 2


def oracle_model(x, sets):
    """Oracle model of an XFEM set list (bulk, side and double-sided sets, in the
    oracle's set order bulk / side / double)."""
    o = OracleModel(3, CELL_HEX8, SHAPE_RECT, x["mesh"])
    for kind, a in sets:
        if kind == "bulk":
            o.add_bulk_set(a["ig_cell"], a["rule"], MODEL_3D, a["ip_cells"], a["E"], a["nu"], a.get("ig_offsets"),
                           a.get("ig_coords"), a.get("ig_param"))
    for kind, a in sets:
        if kind == "side":
            o.add_side_set(a["iwg"], a["rule"], MODEL_3D, a["ip_cells"], a["ordinals"], a["E"], a["nu"], a["alpha"],
                           a["value"])
    for kind, a in sets:
        if kind == "double":
            o.add_double_side_set(a["iwg"], a["facet_cell"], a["rule"], MODEL_3D, a["leader"], a["follower"],
                                  a["offsets"], a["coords"], a["leader_param"], a["follower_param"], a["EL"], a["EF"],
                                  a["nu"], a["alpha"])
    o.finalize()
    return o


def _cluster_index(sets, x):
    """Oracle set index of every cut set and the interface set, and for every
    IG vertex the clusters it appears in."""
    nb = sum(1 for k, _ in sets if k == "bulk")
    ns = sum(1 for k, _ in sets if k == "side")
    cut_sets = []  # (oracle set index, set dict)
    k_bulk = 0
    for k, a in sets:
        if k == "bulk":
            if a.get("ig_offsets") is not None:
                cut_sets.append((k_bulk, a))
            k_bulk += 1
    iface = None
    kd = 0
    for k, a in sets:
        if k == "double":
            if a["facet_cell"] == CELL_TRI3:  # TRI3 facets: the interface
                iface = (nb + ns + kd, a)
            kd += 1
    return cut_sets, iface


def fd_index(sets, x):
    """Lookups of the FD loop, built once (like the model): the cut sets and the
    interface set, the clusters of every background cell, the background cells
    whose clusters hold each IG vertex, and each background cell's bounds."""
    cut_sets, iface = _cluster_index(sets, x)
    bg = x["cell_background"]
    # background cell -> (cut set position, eq) per phase; interface eq per background cell
    cut_of_cell = {}
    for pos, (si, a) in enumerate(cut_sets):
        for e, cell in enumerate(a["ip_cells"]):
            cut_of_cell.setdefault(int(bg[cell]), []).append((pos, e))
    if_of_cell = {}
    if iface is not None:
        for e, cell in enumerate(iface[1]["leader"]):
            if_of_cell[int(bg[cell])] = e
    # (vertex, background cell) pairs of every integration cell and interface facet
    pv, pc = [], []
    for pos, (si, a) in enumerate(cut_sets):
        offs = np.asarray(a["ig_offsets"])
        e_of_row = np.repeat(np.arange(len(offs) - 1), np.diff(offs))
        cell_of_row = bg[np.asarray(a["ip_cells"])[e_of_row]]
        ids = np.asarray(a["ig_vertex_ids"]).reshape(len(e_of_row), -1)
        pv.append(ids.ravel())
        pc.append(np.repeat(cell_of_row, ids.shape[1]))
    if iface is not None:
        a = iface[1]
        offs = np.asarray(a["offsets"])
        e_of_row = np.repeat(np.arange(len(offs) - 1), np.diff(offs))
        cell_of_row = bg[np.asarray(a["leader"])[e_of_row]]
        ids = np.asarray(a["facet_vertex_ids"]).reshape(len(e_of_row), -1)
        pv.append(ids.ravel())
        pc.append(np.repeat(cell_of_row, ids.shape[1]))
    pairs = np.unique(np.stack([np.concatenate(pv), np.concatenate(pc)], axis=1), axis=0) if pv else \
        np.zeros((0, 2), dtype=np.int64)
    nv = len(x["vertices"]["kind"])
    vstart = np.searchsorted(pairs[:, 0], np.arange(nv + 1))
    # bounds of a background cell: the first IP cell on it
    cells_u, first = np.unique(bg, return_index=True)
    X = x["mesh"]["coords"][x["mesh"]["cells"][first]]
    bounds = {int(c): (X[k].min(axis=0), X[k].max(axis=0)) for k, c in enumerate(cells_u)}
    return dict(cut_sets=cut_sets, iface=iface, cut_of_cell=cut_of_cell, if_of_cell=if_of_cell,
                pair_cells=pairs[:, 1], vstart=vstart, bounds=bounds)


def reference_fd_dfdt(orc, sets, x, u, lam, vertices, rel=1e-6, tol=1e-12, index=None):
    """dF/dt_v for the given intersection vertices by the reference's FD scheme on
    the oracle's cluster residuals (F = Q - lambda^T R; Q the bulk strain energy).
    `index`: the lookups of fd_index (built here when not given)."""
    ix = fd_index(sets, x) if index is None else index
    cut_sets, iface = ix["cut_sets"], ix["iface"]
    cut_of_cell, if_of_cell = ix["cut_of_cell"], ix["if_of_cell"]
    V = x["vertices"]

    def cut_arrays(pos, e):
        si, a = cut_sets[pos]
        o0, o1 = a["ig_offsets"][e], a["ig_offsets"][e + 1]
        return (a["ig_coords"][o0 * 12:o1 * 12].reshape(-1, 4, 3).copy(),
                a["ig_param"][o0 * 12:o1 * 12].reshape(-1, 4, 3).copy(),
                a["ig_vertex_ids"][o0:o1])

    def facet_arrays(e):
        a = iface[1]
        o0, o1 = a["offsets"][e], a["offsets"][e + 1]
        return (a["coords"][o0 * 9:o1 * 9].reshape(-1, 3, 3).copy(),
                a["leader_param"][o0 * 9:o1 * 9].reshape(-1, 3, 3).copy(),
                a["follower_param"][o0 * 9:o1 * 9].reshape(-1, 3, 3).copy(),
                a["facet_vertex_ids"][o0:o1])

    def F_cluster(si, e, interface):
        ids = orc.element_topology(si, e)
        _, R = orc.element_matrices(si, e, u)
        if interface:
            return -float(lam[ids] @ R)
        return float((0.5 * u[ids] - lam[ids]) @ R)

    out = np.zeros(len(vertices))
    for iv, v in enumerate(vertices):
        p0, p1 = V["parents"][v, 0], V["parents"][v, 1]
        dxdt = V["coords"][p1] - V["coords"][p0]
        xv = V["coords"][v]
        # background cells whose clusters contain v
        cells = ix["pair_cells"][ix["vstart"][v]:ix["vstart"][v + 1]]
        g = np.zeros(3)
        for cell in cells:
            cell = int(cell)
            lo, hi = ix["bounds"][cell]
            members = cut_of_cell.get(cell, [])
            ie = if_of_cell.get(cell)
            base = {}
            for pos, e in members:
                base[(pos, e)] = cut_arrays(pos, e)
            fbase = facet_arrays(ie) if ie is not None else None
            for d in range(3):
                maxp = (hi[d] - lo[d]) / 3.0
                delta = max(min(abs(rel * maxp), maxp), min(maxp, tol))
                sign = -1.0 if xv[d] + delta >= hi[d] else 1.0  # backward at the upper bound

                def perturbed(arr_x, arr_p, vid, cell_lo, cell_hi, amount):
                    ax, ap = arr_x.copy(), arr_p.copy()
                    m = vid == v
                    ax[m, d] += amount
                    ap[m, d] = -1.0 + 2.0 * (ax[m, d] - cell_lo[d]) / (cell_hi[d] - cell_lo[d])
                    return ax, ap

                # cut clusters of this cell
                for pos, e in members:
                    si = cut_sets[pos][0]
                    cx, cp, cv = base[(pos, e)]
                    if not np.any(cv == v):
                        continue
                    f0 = F_cluster(si, e, False)
                    ax, ap = perturbed(cx, cp, cv, lo, hi, sign * delta)
                    orc.update_ig(si, e, ax.ravel(), ap.ravel())
                    f1 = F_cluster(si, e, False)
                    orc.update_ig(si, e, cx.ravel(), cp.ravel())
                    g[d] += (f1 - f0) / (sign * delta)
                # interface cluster of this cell: facets and the cluster volumes
                if ie is not None:
                    fx, fl, ff, fv = fbase
                    f0 = F_cluster(iface[0], ie, True)
                    ax, al = perturbed(fx, fl, fv, lo, hi, sign * delta)
                    _, af = perturbed(fx, ff, fv, lo, hi, sign * delta)
                    orc.update_facets(iface[0], ie, ax.ravel(), al.ravel(), af.ravel())
                    for pos, e in members:
                        cx, cp, cv = base[(pos, e)]
                        bx, bp = perturbed(cx, cp, cv, lo, hi, sign * delta)
                        orc.update_ig(cut_sets[pos][0], e, bx.ravel(), bp.ravel())
                    f1 = F_cluster(iface[0], ie, True)
                    orc.update_facets(iface[0], ie, fx.ravel(), fl.ravel(), ff.ravel())
                    for pos, e in members:
                        cx, cp, cv = base[(pos, e)]
                        orc.update_ig(cut_sets[pos][0], e, cx.ravel(), cp.ravel())
                    g[d] += (f1 - f0) / (sign * delta)
        out[iv] = float(g @ dxdt)
    return out
