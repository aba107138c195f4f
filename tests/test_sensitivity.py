"""Shape sensitivities through the level-set coefficients (config 4 path):
the adjoint dR/dp kernel against central finite differences, the chain to
the B-spline coefficients against central finite differences on 50 random
coefficients, the full dQ/dp with re-solves, and the reference's own
finite-difference sensitivities restated on the oracle."""
import numpy as np
import pytest

import moris_gb300 as mg
from moris_gb300 import sensitivity as S
from moris_gb300.rng import uniform01
from oracle.fd_sensitivity import oracle_model, reference_fd_dfdt

H = 1e-6


def small_case(n=8, ncoef=12, order=2):
    return S.build(n=n, ncoef=ncoef, order=order)


def test_bspline_tmatrix_partition_of_unity():
    cols, vals = S.node_tmatrix(6, 12)
    assert np.allclose(vals.sum(axis=1), 1.0, atol=1e-14)
    assert cols.min() >= 0 and cols.max() < 12 ** 3


def test_edge_coordinates_reproduce_the_decomposition():
    c = S.build(n=8, ncoef=12, finalize=False)
    t = S.edge_coordinates(c["x"]["vertices"], c["phi"])
    k = c["x"]["vertices"]["kind"] == 3
    assert np.max(np.abs(t[k] - c["x"]["vertices"]["value"][k])) < 1e-14


def test_fd_index_finds_every_cluster_of_a_vertex():
    """The FD loop's prebuilt lookups (fd_index) against a scan of every
    integration cell and interface facet: for each IG vertex the background
    cells of the clusters that hold it, and each cell's bounds."""
    from oracle.fd_sensitivity import _cluster_index, fd_index
    c = S.build(n=8, ncoef=12, finalize=False)
    x, sets = c["x"], c["sets"]
    ix = fd_index(sets, x)
    bg = x["cell_background"]
    cut_sets, iface = _cluster_index(sets, x)
    want = {}
    for _, a in cut_sets:
        offs = a["ig_offsets"]
        for e in range(len(offs) - 1):
            for v in np.asarray(a["ig_vertex_ids"])[offs[e]:offs[e + 1]].ravel():
                want.setdefault(int(v), set()).add(int(bg[a["ip_cells"][e]]))
    if iface is not None:
        a = iface[1]
        offs = a["offsets"]
        for e in range(len(offs) - 1):
            for v in np.asarray(a["facet_vertex_ids"])[offs[e]:offs[e + 1]].ravel():
                want.setdefault(int(v), set()).add(int(bg[a["leader"][e]]))
    nv = len(x["vertices"]["kind"])
    for v in range(nv):
        got = set(int(cc) for cc in ix["pair_cells"][ix["vstart"][v]:ix["vstart"][v + 1]])
        assert got == want.get(v, set()), v
    for cell, (lo, hi) in ix["bounds"].items():
        X = x["mesh"]["coords"][x["mesh"]["cells"][np.nonzero(bg == cell)[0][0]]]
        assert np.array_equal(lo, X.min(axis=0)) and np.array_equal(hi, X.max(axis=0))


def oracle_of(c):
    return oracle_model(c["x"], c["sets"])


def random_state(c, seed):
    import torch
    n = c["model"].num_adofs
    u = torch.tensor(uniform01(seed, n) - 0.5, device="cuda") * 1e-2
    lam = torch.tensor(uniform01(seed + 1, n) - 0.5, device="cuda") * 1e-2
    return u, lam


@pytest.mark.gpu
def test_adjoint_kernel_matches_central_fd_in_t():
    """G[v] = d(Q - lambda^T R)/dt_v at fixed u, lambda vs central differences
    of the assembled functional with the geometry update."""
    c = small_case()
    m = c["model"]
    u, lam = random_state(c, 11)
    G, _ = S.sensitivities(c, u, lam)
    G = G.cpu().numpy()
    V = c["x"]["vertices"]
    t0 = V["value"].copy()
    inter = np.nonzero(V["kind"] == 3)[0]
    pick = inter[(uniform01(5, 30) * len(inter)).astype(int)]
    scale = np.max(np.abs(G[inter]))
    for v in pick:
        tp, tm = t0.copy(), t0.copy()
        tp[v] += H
        tm[v] -= H
        m.update_ig_vertices(tp)
        fp = S.functional(m, u, lam)
        m.update_ig_vertices(tm)
        fm = S.functional(m, u, lam)
        fd = (fp - fm) / (2 * H)
        assert abs(fd - G[v]) <= 1e-6 * scale, (v, fd, G[v], scale)
    m.update_ig_vertices(t0)


@pytest.mark.gpu
def test_adjoint_follows_geometry_updates():
    """The vertex table, links and volume items go to the device on the first
    call only, the coordinates after each geometry update: repeated calls
    agree, a moved geometry changes G, and G on the moved geometry equals that
    of a fresh model moved the same way (atomic sums: agreement to 1e-12)."""
    c = small_case()
    m = c["model"]
    u, lam = random_state(c, 12)
    V = c["x"]["vertices"]
    t0 = V["value"].copy()
    inter = V["kind"] == 3
    t1 = t0.copy()
    t1[inter] = 0.9 * t0[inter] + 0.05
    G0 = S.sensitivities(c, u, lam)[0].cpu().numpy()
    G0b = S.sensitivities(c, u, lam)[0].cpu().numpy()
    scale = np.max(np.abs(G0[inter]))
    assert np.max(np.abs(G0b - G0)) <= 1e-12 * scale
    m.update_ig_vertices(t1)
    G1 = S.sensitivities(c, u, lam)[0].cpu().numpy()
    assert np.max(np.abs(G1 - G0)) > 1e-6 * scale
    f = small_case()
    f["model"].update_ig_vertices(t1)
    Gf = S.sensitivities(f, u, lam)[0].cpu().numpy()
    assert np.max(np.abs(G1 - Gf)) <= 1e-12 * scale
    m.update_ig_vertices(t0)
    G2 = S.sensitivities(c, u, lam)[0].cpu().numpy()
    assert np.max(np.abs(G2 - G0)) <= 1e-12 * scale


@pytest.mark.gpu
def test_stored_level_set_field_equals_host_tables():
    """dQ/dp through the field kept on the device equals dQ/dp with the host
    tables passed per call; a call for a field of other sizes is refused."""
    import torch
    c = small_case()
    m = c["model"]
    u, lam = random_state(c, 13)
    G, dq = S.sensitivities(c, u, lam)
    dh = torch.empty_like(dq)
    m.gen_dqdp(G, c["cols"], c["vals"], len(c["p"]), dh)
    scale = float(dq.abs().max())
    assert scale > 0 and float((dq - dh).abs().max()) <= 1e-12 * scale
    m._ls_shape = (c["cols"].shape[0] + 1, c["cols"].shape[1])
    with pytest.raises(mg.FemGpuError):
        m.gen_dqdp(G, None, None, len(c["p"]), dh)


@pytest.mark.gpu
def test_dqdp_chain_matches_central_fd_on_50_coefficients():
    c = small_case()
    m = c["model"]
    u, lam = random_state(c, 21)
    _, dqdp = S.sensitivities(c, u, lam)
    dqdp = dqdp.cpu().numpy()
    p0 = c["p"].copy()
    active = np.nonzero(dqdp != 0.0)[0]
    assert len(active) >= 50
    pick = active[np.unique((uniform01(7, 200) * len(active)).astype(int))[:50]]
    scale = np.max(np.abs(dqdp))
    V = c["x"]["vertices"]
    for j in pick:
        vals = []
        for sgn in (1.0, -1.0):
            p = p0.copy()
            p[j] += sgn * H
            t = S.edge_coordinates(V, S.node_phi(c["cols"], c["vals"], p))
            m.update_ig_vertices(t)
            vals.append(S.functional(m, u, lam))
        fd = (vals[0] - vals[1]) / (2 * H)
        assert abs(fd - dqdp[j]) <= 1e-6 * scale, (j, fd, dqdp[j], scale)
    m.update_ig_vertices(V["value"])


@pytest.mark.gpu
def test_full_dqdp_with_solves_matches_central_fd():
    """dQ/dp with the adjoint solve against central differences of Q(p) with a
    direct solve of K(p) u = f per evaluation."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    import torch
    c = small_case()
    m = c["model"]
    rp, ci = m.graph()

    def solve_q():
        vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
        r0 = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")
        m.assemble(None, vals, r0)
        A = sp.csr_matrix((vals.cpu().numpy(), ci, rp), shape=(m.num_adofs,) * 2)
        u = spla.spsolve(A.tocsc(), -r0.cpu().numpy())
        ud = torch.tensor(u, device="cuda")
        dq = torch.empty_like(ud)
        q = m.strain_energy(ud, dq)
        return q, ud, dq, A

    q0, u, dq, A = solve_q()
    lam = torch.tensor(spla.spsolve(A.T.tocsc(), dq.cpu().numpy()), device="cuda")
    _, dqdp = S.sensitivities(c, u, lam)
    dqdp = dqdp.cpu().numpy()
    active = np.nonzero(dqdp != 0.0)[0]
    pick = active[np.argsort(-np.abs(dqdp[active]))[:8]]
    p0 = c["p"].copy()
    V = c["x"]["vertices"]
    for j in pick:
        qs = []
        for sgn in (1.0, -1.0):
            p = p0.copy()
            p[j] += sgn * H
            m.update_ig_vertices(S.edge_coordinates(V, S.node_phi(c["cols"], c["vals"], p)))
            qs.append(solve_q()[0])
        fd = (qs[0] - qs[1]) / (2 * H)
        # central differences through two direct solves: O(h^2) truncation (1e-4 relative)
        # plus the rounding of Q itself (atomic summation order, the solve), amplified by 1/H
        noise = 1e-11 * abs(q0) / H
        assert abs(fd - dqdp[j]) <= 1e-4 * abs(dqdp[j]) + noise, (j, fd, dqdp[j], noise)
    m.update_ig_vertices(V["value"])


@pytest.mark.gpu
def test_adjoint_matches_reference_fd_geometry_sensitivities():
    """Against the reference's finite-difference dR/dp on the IG vertex
    coordinates (forward, relative step 1e-6), restated on the oracle."""
    c = small_case()
    u, lam = random_state(c, 31)
    G, _ = S.sensitivities(c, u, lam)
    G = G.cpu().numpy()
    orc = oracle_of(c)
    V = c["x"]["vertices"]
    inter = np.nonzero(V["kind"] == 3)[0]
    pick = inter[np.unique((uniform01(9, 24) * len(inter)).astype(int))]
    ref = reference_fd_dfdt(orc, c["sets"], c["x"], u.cpu().numpy(), lam.cpu().numpy(), pick)
    scale = np.max(np.abs(G[inter]))
    assert np.max(np.abs(ref - G[pick])) <= 1e-4 * scale, np.max(np.abs(ref - G[pick])) / scale
