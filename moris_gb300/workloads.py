"""Seeded input builders of the benchmark workloads (host side, over the C ABI).

Each builder returns a finalized FemModel plus the arrays a caller needs.  The
same seeds and arrays feed the oracle in the tests.

* plane_strain_cantilever -- 2D linear elasticity (E = 1, nu = 0.3, plane
  strain) on a uniform n x n QUAD4 mesh of the unit square with linear
  B-spline extraction, QUAD_2x2; clamped at x = 0 by the symmetric Nitsche
  Dirichlet IWG (alpha = 100, the reference's weak-clamp mechanism), traction
  (1e-3, 0) at x = 1 by the Neumann IWG, BAR_3 on the edges.
* simp_3d -- SIMP-like density problem: n^3 HEX8 mesh of the unit cube with
  linear B-splines, HEX_2x2x2, E(x) = rho(x)^3 with rho the nodal field
  smooth_density(n, seed) interpolated at the Gauss points, nu = 0.3; clamped
  at x = 0 (Nitsche, alpha = 100) and loaded by the traction (1e-3, 0, 0) at
  x = 1 (QUAD_2x2 facets; the facet's E is E0 times the cube of the mean
  density of its element's nodes).
* elasticity_3d -- 3D linear elasticity on an n^3 HEX8 mesh of the unit cube,
  quadratic B-spline extraction, HEX_3x3x3, E per element log-uniform in
  [1e-3, 1] (splitmix64), nu = 0.3.
"""
import numpy as np

from . import (CELL_HEX8, CELL_QUAD4, CELL_TET4, CELL_TRI3, FemModel, IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE,
               IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE, IWG_STRUC_LINEAR_NEUMANN, IWG_STRUC_LINEAR_VW_GHOST,
               MODEL_3D, MODEL_PLANE_STRAIN, RULE_BAR_3, RULE_HEX_3x3x3, RULE_QUAD_2x2, RULE_TET_4, RULE_TRI_7,
               SHAPE_RECTANGULAR, hmr_uniform_mesh)
from . import RULE_HEX_2x2x2, RULE_QUAD_2x2 as _RULE_QUAD_2x2
from .rng import uniform01

BASE_SEED = 20261203
NITSCHE_ALPHA = 100.0
TRACTION = 1e-3


def plane_strain_cantilever(n=128, finalize=True):
    mesh = hmr_uniform_mesh(2, (n, n), (1.0, 1.0), 1)
    nc = len(mesh["cells"])
    E = np.ones(nc)
    m = FemModel(2, mesh, SHAPE_RECTANGULAR)
    m.add_bulk_set(np.arange(nc, dtype=np.int32), E, 0.3, RULE_QUAD_2x2, MODEL_PLANE_STRAIN)
    left = np.arange(0, nc, n, dtype=np.int32)
    right = np.arange(n - 1, nc, n, dtype=np.int32)
    m.add_side_set(IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, left, np.full(len(left), 3), E[left], 0.3,
                   RULE_BAR_3, MODEL_PLANE_STRAIN, alpha=NITSCHE_ALPHA, value=(0.0, 0.0))
    m.add_side_set(IWG_STRUC_LINEAR_NEUMANN, right, np.full(len(right), 1), E[right], 0.3, RULE_BAR_3,
                   MODEL_PLANE_STRAIN, value=(TRACTION, 0.0))
    if finalize:
        m.finalize()
    return m, mesh, E


def elasticity_3d(n=64, seed=BASE_SEED + 2, finalize=True):
    mesh = hmr_uniform_mesh(3, (n, n, n), (1.0, 1.0, 1.0), 2)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 + 3.0 * uniform01(seed, nc))
    m = FemModel(3, mesh, SHAPE_RECTANGULAR)
    m.add_bulk_set(np.arange(nc, dtype=np.int32), E, 0.3, RULE_HEX_3x3x3, MODEL_3D)
    if finalize:
        m.finalize()
    return m, mesh, E


def sphere_field(n, seed, nspheres=40, rmin=0.03, rmax=0.12):
    """Level set min_k(|x - c_k| - r_k) at the (n+1)^3 nodes of the unit cube,
    centres uniform in the cube and radii uniform in [rmin, rmax] (splitmix64
    stream of `seed`: 3 nspheres centre coordinates, then nspheres radii)."""
    u = uniform01(seed, 4 * nspheres)
    cen = u[:3 * nspheres].reshape(nspheres, 3)
    rad = rmin + (rmax - rmin) * u[3 * nspheres:]
    g = np.arange(n + 1) / n
    # node (ix, iy, iz) at flat index (iz (n+1) + iy) (n+1) + ix; the squared
    # distance is separable, summed in the order x^2 + y^2, then + z^2
    phi = np.full((n + 1) ** 3, np.inf)
    for k in range(nspheres):
        dx, dy, dz = g - cen[k, 0], g - cen[k, 1], g - cen[k, 2]
        d2 = (dx * dx)[None, None, :] + (dy * dy)[None, :, None]
        d2 = d2 + (dz * dz)[:, None, None]
        np.minimum(phi, (np.sqrt(d2) - rad[k]).ravel(), out=phi)
    return phi


XFEM_E = (1.0, 0.1)
XFEM_NU = 0.3
XFEM_NITSCHE_ALPHA = 100.0
XFEM_GHOST_ALPHA = 0.01


def xfem_sets(x, E=XFEM_E, nu=XFEM_NU, tet_rule=RULE_TET_4, tri_rule=RULE_TRI_7, hex_rule=RULE_HEX_2x2x2,
              alpha_if=XFEM_NITSCHE_ALPHA, alpha_gh=XFEM_GHOST_ALPHA, ghost_iwg=IWG_STRUC_LINEAR_VW_GHOST,
              ghost_rule=None):
    """Set list of a decomposed XFEM mesh (phase-wise elasticity, Nitsche
    interface, ghost penalty: virtual work by default, or the normal-field
    ghost with ghost_iwg = IWG_GHOST_NORMAL_FIELD), in the order bulk sets,
    then double-sided sets: [(kind, args)], kind 'bulk' or 'double'.  Empty
    sets are left out."""
    sets = []
    for p in (0, 1):
        c = x["uncut%d" % p]
        if len(c):
            sets.append(("bulk", dict(ip_cells=c, E=np.full(len(c), E[p]), nu=nu, rule=hex_rule, ig_cell=CELL_HEX8)))
    for p in (0, 1):
        c = x["cut%d" % p]
        if len(c["cells"]):
            sets.append(("bulk", dict(ip_cells=c["cells"], E=np.full(len(c["cells"]), E[p]), nu=nu, rule=tet_rule,
                                      ig_cell=CELL_TET4, ig_offsets=c["ig_offsets"], ig_coords=c["ig_coords"],
                                      ig_param=c["ig_param"], ig_vertex_ids=c["ig_vertices"])))
    it = x["interface"]
    if len(it["leader"]):
        n = len(it["leader"])
        sets.append(("double", dict(iwg=IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE, leader=it["leader"],
                                    follower=it["follower"], offsets=it["offsets"], coords=it["coords"],
                                    leader_param=it["param"], follower_param=it["param"], EL=np.full(n, E[0]),
                                    EF=np.full(n, E[1]), nu=nu, rule=tri_rule, facet_cell=CELL_TRI3, alpha=alpha_if,
                                    facet_vertex_ids=it["vertices"])))
    for p in (0, 1):
        g = x["ghost%d" % p]
        n = len(g["leader"])
        if n:
            sets.append(("double", dict(iwg=ghost_iwg, leader=g["leader"], follower=g["follower"],
                                        offsets=g["offsets"], coords=g["coords"], leader_param=g["leader_param"],
                                        follower_param=g["follower_param"], EL=np.full(n, E[p]), EF=np.full(n, E[p]),
                                        nu=nu, rule=RULE_QUAD_2x2 if ghost_rule is None else ghost_rule,
                                        facet_cell=CELL_QUAD4, alpha=alpha_gh)))
    return sets


def add_xfem_sets(m, sets):
    for kind, a in sets:
        if kind == "bulk":
            m.add_bulk_set(a["ip_cells"], a["E"], a["nu"], a["rule"], MODEL_3D, ig_cell=a["ig_cell"],
                           ig_offsets=a.get("ig_offsets"), ig_coords=a.get("ig_coords"), ig_param=a.get("ig_param"),
                           ig_vertex_ids=a.get("ig_vertex_ids"))
        elif kind == "double":
            m.add_double_side_set(a["iwg"], a["leader"], a["follower"], a["offsets"], a["coords"], a["leader_param"],
                                  a["follower_param"], a["EL"], a["EF"], a["nu"], a["rule"], a["facet_cell"],
                                  a["alpha"], facet_vertex_ids=a.get("facet_vertex_ids"))
        else:
            m.add_side_set(a["iwg"], a["ip_cells"], a["ordinals"], a["E"], a["nu"], a["rule"], MODEL_3D,
                           alpha=a.get("alpha", 0.0), value=a["value"])


def xfem_spheres(n=96, seed=BASE_SEED + 3, nspheres=40, rmin=0.03, rmax=0.12, order=1, finalize=True, device=False,
                 **kw):
    """Two-phase XFEM workload: n^3 HEX8 background of the unit cube with
    B-splines of `order`, cut by the sphere level set; phase 0 (phi >= 0) E = 1,
    phase 1 (inside the spheres) E = 0.1, nu = 0.3; uncut cells HEX_2x2x2, cut
    clusters TET4 cells with TET_4, Nitsche interface (alpha 100, TRI_7),
    virtual-work ghost (alpha 0.01, QUAD_2x2).  device=True decomposes on the
    GPU (the same arrays).  Returns (model, decomposition, set list)."""
    from . import xtk
    phi = sphere_field(n, seed, nspheres, rmin, rmax)
    x = xtk.decompose((n, n, n), (1.0, 1.0, 1.0), order, phi, device=device)
    sets = xfem_sets(x, **kw)
    m = FemModel(3, x["mesh"], SHAPE_RECTANGULAR)
    add_xfem_sets(m, sets)
    if finalize:
        m.finalize()
    return m, x, sets


def smooth_density(n, seed, rho_min=1e-3, passes=3):
    """Seeded smoothed noise on the (n+1)^3 grid nodes mapped to [rho_min, 1]:
    uniform noise, `passes` sweeps of a 3x3x3 box filter (edge-replicated),
    then an affine min-max map."""
    m = n + 1
    f = uniform01(seed, m ** 3).reshape(m, m, m)
    for _ in range(passes):
        g = np.pad(f, 1, mode="edge")
        acc = np.zeros_like(f)
        for dz in range(3):
            for dy in range(3):
                for dx in range(3):
                    acc += g[dz:dz + m, dy:dy + m, dx:dx + m]
        f = acc / 27.0
    lo, hi = f.min(), f.max()
    return (rho_min + (1.0 - rho_min) * (f - lo) / (hi - lo)).ravel()


def simp_3d(n=128, seed=BASE_SEED + 5, finalize=True, beta=3.0):
    mesh = hmr_uniform_mesh(3, (n, n, n), (1.0, 1.0, 1.0), 1)
    nc = len(mesh["cells"])
    rho = smooth_density(n, seed)
    E0 = np.ones(nc)
    m = FemModel(3, mesh, SHAPE_RECTANGULAR)
    m.add_bulk_set(np.arange(nc, dtype=np.int32), E0, 0.3, RULE_HEX_2x2x2, MODEL_3D, node_density=rho,
                   density_exponent=beta)
    cells = np.arange(nc)
    left = cells[cells % n == 0].astype(np.int32)
    right = cells[cells % n == n - 1].astype(np.int32)
    rho_el = rho[mesh["cells"]].mean(axis=1)
    E_el = rho_el ** beta
    m.add_side_set(IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, left, np.full(len(left), 3), E_el[left], 0.3,
                   _RULE_QUAD_2x2, MODEL_3D, alpha=NITSCHE_ALPHA, value=(0.0, 0.0, 0.0))
    m.add_side_set(IWG_STRUC_LINEAR_NEUMANN, right, np.full(len(right), 1), E_el[right], 0.3, _RULE_QUAD_2x2,
                   MODEL_3D, value=(TRACTION, 0.0, 0.0))
    if finalize:
        m.finalize()
    return m, mesh, rho


def main():
    """One batched assembly of the XFEM workload (the case profiled in
    profiles/): python -m moris_gb300.workloads --xfem 48 [--warps 4 --split 0]"""
    import argparse
    import json
    import time

    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--xfem", type=int, default=48, help="background cells per edge")
    ap.add_argument("--warps", type=int, default=4)
    ap.add_argument("--split", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args()
    m, x, _ = xfem_spheres(a.xfem, device=True)
    m.set_batched_config(a.warps, a.split)
    dev = torch.device("cuda")
    u = torch.zeros(m.num_adofs, dtype=torch.float64, device=dev)
    vals = torch.zeros(m.nnz, dtype=torch.float64, device=dev)
    rhs = torch.zeros(m.num_adofs, dtype=torch.float64, device=dev)
    times = []
    for _ in range(a.repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.assemble_batched(u, vals, rhs)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    m.check_status()
    print(json.dumps({"n": a.xfem, "adofs": m.num_adofs, "nnz": m.nnz, "seconds": times}))


if __name__ == "__main__":
    main()
