"""Shape sensitivities of the strain energy with respect to B-spline level-set
coefficients (config 4): the workload builder and the adjoint pipeline over
libfem_gpu (fem_gpu_strain_energy, fem_gpu_drdp_adjoint, fem_gen_dqdp).

Pipeline (the reference's sensitivity analysis, with the FD residual
derivative replaced by the exact adjoint kernel):
  p -> phi at the background nodes (cubic B-spline field) -> XFEM
  decomposition -> K u = f -> K^T lambda = dQ/du -> G = d(Q - lambda^T R)/dt
  at the intersection vertices -> dQ/dp = G dt/dp.
"""
import numpy as np

from . import (IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, IWG_STRUC_LINEAR_NEUMANN, NO_JACOBIAN, RULE_QUAD_2x2,
               SHAPE_RECTANGULAR, FemModel, bspline_tmatrix, workloads, xtk)
from .rng import uniform01

LS_ORDER = 3
NOISE = 0.01


def greville(ncoef, order=LS_ORDER):
    """Greville abscissae of a uniform B-spline on [0, 1] with ncoef coefficients
    (HMR numbering: coefficient j spans elements j-order .. j)."""
    h = 1.0 / (ncoef - order)
    return (np.arange(ncoef) - (order - 1) / 2.0) * h


def gaussian(seed, n):
    """Seeded standard normal samples (Box-Muller on the splitmix64 stream)."""
    u = uniform01(seed, 2 * n)
    u1 = np.maximum(u[:n], 1e-300)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u[n:])


def levelset_coefficients(ncoef=32, seed=workloads.BASE_SEED + 4, sphere_seed=workloads.BASE_SEED + 3,
                          noise=NOISE, nspheres=40, rmin=0.03, rmax=0.12):
    """Cubic B-spline level-set coefficients on an ncoef^3 grid: the sphere
    field of config 3 sampled at the Greville points plus seeded Gaussian
    noise smoothed by one 3x3x3 box filter, scaled by `noise`."""
    g = greville(ncoef)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    u = uniform01(sphere_seed, 4 * nspheres)
    cen = u[:3 * nspheres].reshape(nspheres, 3)
    rad = rmin + (rmax - rmin) * u[3 * nspheres:]
    phi = np.full(len(pts), np.inf)
    for k in range(nspheres):
        phi = np.minimum(phi, np.linalg.norm(pts - cen[k], axis=1) - rad[k])
    w = gaussian(seed, ncoef ** 3).reshape(ncoef, ncoef, ncoef)
    gp = np.pad(w, 1, mode="edge")
    acc = np.zeros_like(w)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                acc += gp[dz:dz + ncoef, dy:dy + ncoef, dx:dx + ncoef]
    return phi + noise * (acc / 27.0).ravel()


def node_tmatrix(n, ncoef, order=LS_ORDER):
    """Level-set B-spline basis at the (n+1)^3 background nodes of the unit cube."""
    g = np.arange(n + 1) / n
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    return bspline_tmatrix((ncoef,) * 3, (1.0, 1.0, 1.0), order, pts)


def node_phi(cols, vals, p):
    return (vals * p[cols]).sum(axis=1)


def edge_coordinates(verts, phi_nodes):
    """t of every intersection vertex for nodal level-set values (same topology)."""
    kind, par = verts["kind"], verts["parents"]
    phi_v = np.zeros(len(kind))
    for k, cnt in ((0, 1), (1, 4), (2, 8)):
        sel = kind == k
        phi_v[sel] = phi_nodes[par[sel, :cnt]].mean(axis=1)
    t = verts["value"].copy()
    sel = kind == 3
    f0, f1 = phi_v[par[sel, 0]], phi_v[par[sel, 1]]
    t[sel] = f0 / (f0 - f1)
    return t


def boundary_sets(x, n, E=workloads.XFEM_E, nu=workloads.XFEM_NU, alpha=workloads.NITSCHE_ALPHA,
                  traction=workloads.TRACTION):
    """Clamp (Nitsche) at x = 0 and traction at x = 1 on the faces of uncut
    enriched cells (cut boundary cells carry no boundary condition)."""
    bg, ph = x["cell_background"], x["cell_phase"]
    uncut = np.zeros(len(bg), dtype=bool)
    for p in (0, 1):
        uncut[x["uncut%d" % p]] = True
    i = bg % n
    out = []
    for sel_i, ordinal, iwg, val in ((0, 3, IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, (0.0, 0.0, 0.0)),
                                      (n - 1, 1, IWG_STRUC_LINEAR_NEUMANN, (traction, 0.0, 0.0))):
        cells = np.nonzero(uncut & (i == sel_i))[0].astype(np.int32)
        Ec = np.asarray(E)[ph[cells]]
        out.append(("side", dict(iwg=iwg, ip_cells=cells, ordinals=np.full(len(cells), ordinal), E=Ec, nu=nu,
                                 rule=RULE_QUAD_2x2, alpha=alpha if iwg != IWG_STRUC_LINEAR_NEUMANN else 0.0,
                                 value=val)))
    return out


def build(n=64, ncoef=32, order=2, p=None, finalize=True, stream=None):
    """Config-4 model: n^3 HEX8 unit cube with B-splines of `order` cut by the
    cubic B-spline level set p (ncoef^3).  Returns a dict with the model, the
    decomposition, the set list and the level-set operators."""
    if p is None:
        p = levelset_coefficients(ncoef)
    cols, vals = node_tmatrix(n, ncoef)
    phi = node_phi(cols, vals, p)
    x = xtk.decompose((n, n, n), (1.0, 1.0, 1.0), order, phi)
    sets = workloads.xfem_sets(x)
    # oracle set order: bulk, side, double
    sets = [s for s in sets if s[0] == "bulk"] + boundary_sets(x, n) + [s for s in sets if s[0] == "double"]
    m = FemModel(3, x["mesh"], SHAPE_RECTANGULAR)
    if stream is not None:
        m.set_stream(stream)
    workloads.add_xfem_sets(m, sets)
    v = x["vertices"]
    m.set_ig_vertices(v["kind"], v["parents"], v["coords"], v["value"])
    if finalize:
        m.finalize()
        m.set_level_set_field(cols, vals, len(p))
    return dict(model=m, x=x, sets=sets, p=p, cols=cols, vals=vals, phi=phi, n=n, ncoef=ncoef)


def system(m):
    """CSR graph and operator (device) with b = f (the traction load): R(0) = -f."""
    import torch
    rp = torch.empty(m.num_adofs + 1, dtype=torch.int32, device="cuda")
    ci = torch.empty(m.nnz, dtype=torch.int32, device="cuda")
    m.graph_device(rp, ci)
    vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    r0 = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")
    m.assemble(None, vals, r0)
    return rp, ci, vals, -r0


def _pcg(m, rp, ci, vals, b, x, rel_tol, max_iter):
    from . import FemGpuError
    import time
    t0 = time.perf_counter()
    try:
        r = m.pcg(rp, ci, vals, b, x, rel_tol=rel_tol, max_iter=max_iter)
    except FemGpuError as e:
        if e.status != 10:  # FEM_GPU_NOT_CONVERGED: report instead of raising
            raise
        r = dict(iterations=max_iter, converged=False)
    r["seconds"] = time.perf_counter() - t0
    r["rel_residual"] = true_residual(rp, ci, vals, b, x)
    return r


def true_residual(rp, ci, vals, b, x):
    """||b - A x|| / ||b|| recomputed from the CSR operator"""
    import torch
    A = torch.sparse_csr_tensor(rp.long(), ci.long(), vals, size=(len(b), len(b)))
    rel = float(torch.linalg.norm(b - torch.mv(A, x)) / torch.linalg.norm(b))
    del A
    return rel


def solve_state_adjoint(m, rel_tol=1e-10, max_iter=100000):
    """u (K u = f), lambda (K^T lambda = dQ/du; K is symmetric), Q."""
    import torch
    rp, ci, vals, f = system(m)
    u = torch.zeros_like(f)
    ru = _pcg(m, rp, ci, vals, f, u, rel_tol, max_iter)
    dqdu = torch.empty_like(f)
    q = m.strain_energy(u, dqdu)
    lam = torch.zeros_like(f)
    rl = _pcg(m, rp, ci, vals, dqdu, lam, rel_tol, max_iter)
    return dict(u=u, lam=lam, q=q, dqdu=dqdu, pcg_u=ru, pcg_lambda=rl, csr=(rp, ci, vals, f))


def functional(m, u, lam):
    """F = Q(u) - lambda^T R(u) at fixed u, lambda (device tensors)."""
    import torch
    dqdu = torch.empty_like(u)
    q = m.strain_energy(u, dqdu)
    r = torch.empty_like(u)
    m.assemble(u, None, r, NO_JACOBIAN)
    return q - float(torch.dot(lam, r))


def sensitivities(c, u, lam):
    """G at the intersection vertices and dQ/dp (device tensors)."""
    import torch
    m = c["model"]
    nv = len(c["x"]["vertices"]["kind"])
    G = torch.empty(nv, dtype=torch.float64, device="cuda")
    m.drdp_adjoint(u, lam, G)
    dqdp = torch.empty(len(c["p"]), dtype=torch.float64, device="cuda")
    m.gen_dqdp(G, None, None, len(c["p"]), dqdp)
    return G, dqdp
