"""Two-phase XFEM path: the decomposition (host), the oracle's interface and
ghost restatement, the MSI graph with double-sided equation objects, and the
cluster kernel (cut clusters, interface, ghost; per set and in the batched
persistent launch) against the oracle."""
import numpy as np
import pytest

import moris_gb300 as mg
from moris_gb300 import workloads, xtk
from oracle import OracleModel

from common import RTOL, csr_row_rel_err, rel_err

N_SMALL = 10


def small_xfem(n=N_SMALL, seed=workloads.BASE_SEED + 3, nspheres=5, rmin=0.15, rmax=0.3, order=1, **set_options):
    phi = workloads.sphere_field(n, seed, nspheres, rmin, rmax)
    x = xtk.decompose((n, n, n), (1.0, 1.0, 1.0), order, phi)
    return x, workloads.xfem_sets(x, **set_options)


# the reference's automatic rules everywhere, and the normal-field ghost with
# SP_Ghost_Displacement in place of the virtual-work ghost
AUTO_NF = dict(tet_rule=mg.RULE_AUTO, tri_rule=mg.RULE_AUTO, hex_rule=mg.RULE_AUTO, ghost_rule=mg.RULE_AUTO,
               ghost_iwg=mg.IWG_GHOST_NORMAL_FIELD)


def oracle_of(x, sets):
    o = OracleModel(3, mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, x["mesh"])
    for kind, a in sets:
        if kind == "bulk":
            o.add_bulk_set(a["ig_cell"], a["rule"], mg.MODEL_3D, a["ip_cells"], a["E"], a["nu"],
                           a.get("ig_offsets"), a.get("ig_coords"), a.get("ig_param"))
    for kind, a in sets:
        if kind == "double":
            o.add_double_side_set(a["iwg"], a["facet_cell"], a["rule"], mg.MODEL_3D, a["leader"], a["follower"],
                                  a["offsets"], a["coords"], a["leader_param"], a["follower_param"], a["EL"], a["EF"],
                                  a["nu"], a["alpha"])
    o.finalize()
    return o


def product_of(x, sets, host_only=False):
    m = mg.FemModel(3, x["mesh"], mg.SHAPE_RECTANGULAR)
    workloads.add_xfem_sets(m, sets)
    m.finalize(host_only=host_only)
    m.kinds = [k for k, _ in sets]
    return m


# ---------------------------------------------------------------------------
# host / oracle (no GPU)

def test_decomposition_partitions_the_cube():
    x, _ = small_xfem()
    s = x["sizes"]
    assert s.num_cut[0] == s.num_cut[1] == s.num_interface > 0
    vol = 0.0
    for p in (0, 1):
        X = x["cut%d" % p]["ig_coords"].reshape(-1, 4, 3)
        a, b, c = X[:, 0] - X[:, 2], X[:, 1] - X[:, 2], X[:, 3] - X[:, 2]
        det = np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0
        assert det.min() > 0.0
        vol += det.sum() + len(x["uncut%d" % p]) / N_SMALL ** 3
    assert abs(vol - 1.0) < 1e-12
    # every cut cell's two phase volumes add up to the cell
    for p in (0, 1):
        off = x["cut%d" % p]["ig_offsets"]
        assert off[0] == 0 and np.all(np.diff(off) > 0)


def test_interface_normals_point_out_of_phase0():
    x, _ = small_xfem()
    it = x["interface"]
    X = it["coords"].reshape(-1, 3, 3)
    n = np.cross(X[:, 0] - X[:, 2], X[:, 1] - X[:, 2])
    c = X.mean(axis=1)
    eps = 1e-3 / N_SMALL
    u = mg.rng.uniform01(workloads.BASE_SEED + 3, 4 * 5)
    cen = u[:15].reshape(5, 3)
    rad = 0.15 + 0.15 * u[15:]
    nn = n / np.linalg.norm(n, axis=1)[:, None]

    def lvl(p):
        return np.min(np.linalg.norm(p[:, None, :] - cen[None], axis=2) - rad[None], axis=1)

    # one step along +n enters phase 1 (phi < 0) for the vast majority of facets
    # (the facet is the linear interpolant, not the sphere itself)
    frac = np.mean(lvl(c + eps * nn) < lvl(c - eps * nn))
    assert frac > 0.99


def test_enrichment_and_graph_match_oracle():
    x, sets = small_xfem()
    prod = product_of(x, sets, host_only=True)
    orc = oracle_of(x, sets)
    assert prod.num_adofs == orc.num_adofs
    rp, ci = prod.graph()
    orp, oci = orc.graph()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    nsets = len(sets)
    for s in range(nsets):
        for e in (0, prod.num_eq(s) // 2, prod.num_eq(s) - 1):
            assert np.array_equal(prod.element_topology(s, e), orc.element_topology(s, e))


def test_oracle_double_sided_jacobian_is_residual_derivative():
    """Restated interface / ghost K against a central difference of the
    restated R (the reference's IWG unit-test check, e.g.
    UT_FEM_IWG_Struc_Linear_Interface.cpp / ..._Virtual_Work_Ghost.cpp)."""
    x, sets = small_xfem()
    orc = oracle_of(x, sets)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(orc.num_adofs) * 1e-2
    nb = sum(1 for k, _ in sets if k == "bulk")
    for s in range(nb, len(sets)):
        ids = orc.element_topology(s, 0)
        K, R = orc.element_matrices(s, 0, u)
        h = 1e-6
        for j in range(0, len(ids), 5):
            up, um = u.copy(), u.copy()
            up[ids[j]] += h
            um[ids[j]] -= h
            _, Rp = orc.element_matrices(s, 0, up)
            _, Rm = orc.element_matrices(s, 0, um)
            fd = (Rp - Rm) / (2 * h)
            # duplicated ids (ghost: shared bases) perturb every copy
            col = K[:, [k for k in range(len(ids)) if ids[k] == ids[j]]].sum(axis=1)
            assert np.max(np.abs(fd - col)) <= 1e-6 * max(1.0, np.max(np.abs(K)))


def test_automatic_rules_match_the_oracle_table():
    """Set::get_auto_integration_order (FEM/INT/src/CORE/cl_FEM_Set.cpp:2983-3185)
    for linear interpolation cells: the library's table against the oracle's"""
    from oracle import OracleLib
    ol = OracleLib()
    cells = (mg.CELL_LINE2, mg.CELL_QUAD4, mg.CELL_HEX8, mg.CELL_TRI3, mg.CELL_TET4)
    for kind in (mg.SET_BULK, mg.SET_SIDESET, mg.SET_DOUBLE_SIDESET):
        for cell in cells:
            want = ol.auto_rule(kind, cell)
            if want < 0:
                with pytest.raises(mg.FemGpuError):
                    mg.auto_integration_rule(kind, cell)
            else:
                assert mg.auto_integration_rule(kind, cell) == want, (kind, cell)
    # the reference's named choices
    assert mg.auto_integration_rule(mg.SET_BULK, mg.CELL_HEX8) == mg.RULE_HEX_2x2x2
    assert mg.auto_integration_rule(mg.SET_BULK, mg.CELL_TET4) == mg.RULE_TET_11
    assert mg.auto_integration_rule(mg.SET_DOUBLE_SIDESET, mg.CELL_TRI3) == mg.RULE_TRI_7
    assert mg.auto_integration_rule(mg.SET_BULK, mg.CELL_HEX8, 2) == mg.RULE_HEX_3x3x3
    with pytest.raises(mg.FemGpuError):  # TET_35 is not one of the library's rules
        mg.auto_integration_rule(mg.SET_BULK, mg.CELL_TET4, 2)


def test_oracle_normal_field_ghost_is_symmetric_and_consistent():
    """IWG_Ghost_Normal_Field restated: K is the derivative of R, symmetric and
    positive semi-definite (it is a penalty on the jump of du/dn)."""
    x, sets = small_xfem(**AUTO_NF)
    orc = oracle_of(x, sets)
    rng = np.random.default_rng(4)
    u = rng.standard_normal(orc.num_adofs) * 1e-2
    ghosts = [s for s, (k, a) in enumerate(sets) if k == "double" and a["iwg"] == mg.IWG_GHOST_NORMAL_FIELD]
    assert ghosts
    for s in ghosts:
        for e in (0, orc.num_eq(s) - 1):
            ids = orc.element_topology(s, e)
            K, R = orc.element_matrices(s, e, u)
            assert np.max(np.abs(K - K.T)) <= 1e-14 * np.max(np.abs(K))
            assert np.min(np.linalg.eigvalsh(0.5 * (K + K.T))) >= -1e-12 * np.max(np.abs(K))
            # R = K u_e (linear in u)
            assert np.max(np.abs(R - K @ u[ids])) <= 1e-12 * np.max(np.abs(R))


# ---------------------------------------------------------------------------
# GPU parity

@pytest.mark.gpu
def test_xfem_automatic_rules_and_normal_field_ghost_match_oracle():
    import torch
    x, sets = small_xfem(**AUTO_NF)
    prod = product_of(x, sets)
    orc = oracle_of(x, sets)
    rng = np.random.default_rng(6)
    u = rng.standard_normal(prod.num_adofs)
    for s in range(len(sets)):
        ne = prod.num_eq(s)
        K, R = prod.element_matrices(s, 0, ne, u)
        for e in range(0, ne, max(1, ne // 40)):
            Ko, Ro = orc.element_matrices(s, e, u)
            idx = compact_index(prod, s, e)
            assert rel_err(K[e][np.ix_(idx, idx)], Ko) <= RTOL, (s, e)
            assert rel_err(R[e][idx], Ro) <= RTOL, (s, e)
    vo, ro = orc.assemble(u)
    rp, _ = prod.graph()
    ud = torch.tensor(u, device="cuda")
    vd = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rd = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble_batched(ud, vd, rd)
    torch.cuda.synchronize()
    assert csr_row_rel_err(rp, vd.cpu().numpy(), vo) <= RTOL
    assert rel_err(rd.cpu().numpy(), ro) <= RTOL
    # AUTO resolves to the reference's named rules: the same system as spelling them out
    explicit = dict(tet_rule=mg.RULE_TET_11, tri_rule=mg.RULE_TRI_7, hex_rule=mg.RULE_HEX_2x2x2,
                    ghost_rule=mg.RULE_QUAD_2x2, ghost_iwg=mg.IWG_GHOST_NORMAL_FIELD)
    prod2 = product_of(x, workloads.xfem_sets(x, **explicit))
    v2, r2 = prod2.assemble_host(u)
    assert csr_row_rel_err(rp, v2, vo) <= RTOL and rel_err(r2, ro) <= RTOL


@pytest.mark.gpu
def test_xfem_element_matrices_match_oracle():
    x, sets = small_xfem()
    prod = product_of(x, sets)
    orc = oracle_of(x, sets)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(prod.num_adofs)
    for s in range(len(sets)):
        ne = prod.num_eq(s)
        K, R = prod.element_matrices(s, 0, ne, u)
        for e in range(0, ne, max(1, ne // 40)):
            ids = prod.element_topology(s, e)
            Ko, Ro = orc.element_matrices(s, e, u)
            n = len(ids)
            # padded product layout: rows side * 3 NB + f NB + i; compact by the topology
            idx = compact_index(prod, s, e)
            assert rel_err(K[e][np.ix_(idx, idx)], Ko) <= RTOL, (s, e)
            assert rel_err(R[e][idx], Ro) <= RTOL, (s, e)
            assert n == len(idx)


def compact_index(prod, s, e):
    nmax = prod.max_element_adofs(s)
    ids = prod.element_topology(s, e)
    sides = 2 if prod.kinds[s] == "double" else 1
    width = nmax // (3 * sides)
    out = []
    pos = 0
    for side in range(sides):
        nb = (len(ids) // sides) // 3
        for f in range(3):
            for i in range(nb):
                out.append(side * 3 * width + f * width + i)
        pos += 3 * nb
    return np.array(out)


@pytest.mark.gpu
def test_xfem_assembly_matches_oracle_per_set_and_batched():
    import torch
    x, sets = small_xfem()
    prod = product_of(x, sets)
    orc = oracle_of(x, sets)
    rng = np.random.default_rng(7)
    u = rng.standard_normal(prod.num_adofs)
    vo, ro = orc.assemble(u)
    rp, _ = prod.graph()
    v, r = prod.assemble_host(u)
    assert csr_row_rel_err(rp, v, vo) <= RTOL
    assert rel_err(r, ro) <= RTOL
    ud = torch.tensor(u, device="cuda")
    vd = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rd = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    for warps, split in ((4, 64), (2, 32), (8, 0)):
        prod.set_batched_config(warps, split)
        for _ in range(2):  # capture, then replay of the graph
            vd.fill_(1.0)
            prod.assemble_batched(ud, vd, rd)
            assert csr_row_rel_err(rp, vd.cpu().numpy(), vo) <= RTOL, (warps, split)
            assert rel_err(rd.cpu().numpy(), ro) <= RTOL


@pytest.mark.gpu
def test_xfem_quadratic_bsplines_match_oracle():
    x, sets = small_xfem(n=6, nspheres=3, rmin=0.25, rmax=0.35, order=2)
    prod = product_of(x, sets)
    orc = oracle_of(x, sets)
    rng = np.random.default_rng(9)
    u = rng.standard_normal(prod.num_adofs)
    vo, ro = orc.assemble(u)
    rp, ci = prod.graph()
    orp, oci = orc.graph()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    v, r = prod.assemble_host(u)
    assert csr_row_rel_err(rp, v, vo) <= RTOL
    assert rel_err(r, ro) <= RTOL


def _assert_same(a, b, path="x"):
    if isinstance(a, dict):
        assert set(a) == set(b), path
        for k in a:
            _assert_same(a[k], b[k], path + "." + str(k))
    elif isinstance(a, np.ndarray):
        assert a.shape == b.shape and a.dtype == b.dtype, path
        assert np.array_equal(a, b), (path, int(np.sum(a != b)))
    elif hasattr(a, "_fields_"):
        for name, _ in a._fields_:
            assert np.array_equal(np.asarray(getattr(a, name)), np.asarray(getattr(b, name))), path + "." + name
    else:
        assert a == b, path


@pytest.mark.gpu
@pytest.mark.parametrize("n,nspheres,rmin,rmax,order", [(10, 5, 0.15, 0.3, 1), (6, 3, 0.25, 0.35, 2),
                                                         (24, 40, 0.03, 0.12, 1)])
def test_device_decomposition_equals_host(n, nspheres, rmin, rmax, order):
    """The GPU decomposition (first-touch numbering by sorts, enrichment and
    unzipping on the device) returns the host decomposition array for array,
    bit for bit."""
    phi = workloads.sphere_field(n, workloads.BASE_SEED + 3, nspheres, rmin, rmax)
    xh = xtk.decompose((n, n, n), (1.0, 1.0, 1.0), order, phi)
    xd = xtk.decompose((n, n, n), (1.0, 1.0, 1.0), order, phi, device=True)
    _assert_same(xh, xd)
