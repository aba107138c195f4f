"""GPU parity: the CUDA element path (through the C ABI) against the oracle.

Bar: element operators, assembled CSR values and residuals agree with the
oracle to a relative error of 1e-12 (tests/common.py RTOL, normwise per
element matrix / per CSR row / per vector); integer data (adof ids, CSR
rowptr/colidx) identical.
"""
import numpy as np
import pytest

import moris_gb300 as mg
from tests.common import RTOL, csr_row_rel_err, problem, rel_err, uniform01

pytestmark = pytest.mark.gpu

CASES = [
    # dim, ne, p, shape, rule, sides
    (2, (6, 5), 1, mg.SHAPE_RECTANGULAR, mg.RULE_QUAD_2x2, True),
    (2, (5, 4), 2, mg.SHAPE_GENERAL, mg.RULE_QUAD_2x2, True),
    (2, (4, 4), 3, mg.SHAPE_RECTANGULAR, mg.RULE_QUAD_2x2, False),
    (3, (3, 3, 2), 1, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_2x2x2, True),
    (3, (3, 2, 3), 2, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_3x3x3, False),
    (3, (3, 3, 3), 2, mg.SHAPE_GENERAL, mg.RULE_HEX_3x3x3, True),
    (3, (2, 3, 2), 2, mg.SHAPE_GENERAL, mg.RULE_HEX_2x2x2, False),
]


def _ids(c):
    return "d%d-p%d-%s-r%d%s" % (c[0], c[2], "rect" if c[3] == 0 else "gen", c[4], "-sides" if c[5] else "")


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_element_operators_match_oracle(torch, case):
    dim, ne, p, shape, rule, sides = case
    prod, orc, _ = problem(dim, ne, p, shape, rule, sides)
    prod.finalize()
    orc.finalize()
    u = uniform01(11, prod.num_adofs) - 0.5
    for s in range(orc.num_sets()):
        n_eq = orc.num_eq(s)
        K, R = prod.element_matrices(s, 0, n_eq, u)
        for eq in range(n_eq):
            ids = orc.element_topology(s, eq)
            assert np.array_equal(prod.element_topology(s, eq), ids)
            Ko, Ro = orc.element_matrices(s, eq, u)
            n = len(ids)
            assert rel_err(K[eq, :n, :n], Ko) <= RTOL, (s, eq)
            assert rel_err(R[eq, :n], Ro) <= RTOL, (s, eq)
            assert np.all(K[eq, n:, :] == 0) and np.all(K[eq, :, n:] == 0)


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_assembly_matches_oracle(torch, case):
    dim, ne, p, shape, rule, sides = case
    prod, orc, _ = problem(dim, ne, p, shape, rule, sides)
    prod.finalize()
    orc.finalize()
    rp, ci = prod.graph()
    rpo, cio = orc.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    u = uniform01(5, prod.num_adofs) - 0.5
    vo, ro = orc.assemble(u, nthreads=4)
    # device buffers through the C ABI
    ut = torch.tensor(u, device="cuda")
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(ut, vals, rhs)
    torch.cuda.synchronize()
    assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL
    # host buffers through the same entry point (the reference-facing call)
    vh, rh = prod.assemble_host(u)
    assert csr_row_rel_err(rp, vh, vo) <= RTOL
    assert rel_err(rh, ro) <= RTOL
    # residual of the linear IWGs is K u - f: check consistency on the device result
    f0 = prod.assemble_host(np.zeros(prod.num_adofs), mg.NO_JACOBIAN)[1]
    import scipy.sparse as sp
    A = sp.csr_matrix((vh, ci, rp), shape=(prod.num_adofs, prod.num_adofs))
    assert rel_err(rh, A @ u + f0) <= 1e-11


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("case", [CASES[1], CASES[4], CASES[5]], ids=_ids)
def test_every_bulk_kernel_variant_matches_oracle(torch, case, variant):
    dim, ne, p, shape, rule, sides = case
    prod, orc, _ = problem(dim, ne, p, shape, rule, sides)
    prod.finalize()
    orc.finalize()
    prod.set_variant(0, variant)
    u = uniform01(17, prod.num_adofs) - 0.5
    n_eq = orc.num_eq(0)
    K, R = prod.element_matrices(0, 0, n_eq, u)
    for eq in range(n_eq):
        Ko, Ro = orc.element_matrices(0, eq, u)
        n = len(Ro)
        assert rel_err(K[eq, :n, :n], Ko) <= RTOL and rel_err(R[eq, :n], Ro) <= RTOL
    rp, _ = prod.graph()
    vo, ro = orc.assemble(u)
    vh, rh = prod.assemble_host(u)
    assert csr_row_rel_err(rp, vh, vo) <= RTOL and rel_err(rh, ro) <= RTOL
    # element sub-ranges go through the same kernel with shifted pointers
    K2, R2 = prod.element_matrices(0, 1, n_eq - 2, u)
    assert np.array_equal(K2, K[1:n_eq - 1]) and np.array_equal(R2, R[1:n_eq - 1])


def test_autotune_keeps_parity(torch):
    prod, orc, _ = problem(3, (4, 4, 3), 2, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_3x3x3, False)
    prod.finalize()
    orc.finalize()
    prod.autotune()
    v, ms, name = prod.variant(0)
    assert 0 <= v < 4 and ms > 0 and name
    u = uniform01(2, prod.num_adofs)
    rp, _ = prod.graph()
    vo, ro = orc.assemble(u)
    vh, rh = prod.assemble_host(u)
    assert csr_row_rel_err(rp, vh, vo) <= RTOL and rel_err(rh, ro) <= RTOL


@pytest.mark.parametrize("case", [(2, (5, 4), 1, mg.SHAPE_RECTANGULAR, mg.RULE_QUAD_2x2),
                                  (3, (3, 3, 2), 1, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_2x2x2),
                                  (3, (3, 2, 3), 1, mg.SHAPE_GENERAL, mg.RULE_HEX_2x2x2),
                                  (3, (2, 3, 2), 2, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_3x3x3)])
@pytest.mark.parametrize("variant", [1, 2, 3])
def test_density_field_material_matches_oracle(torch, case, variant):
    dim, ne, p, shape, rule = case
    prod, orc, _ = problem(dim, ne, p, shape, rule, sides=True, density=True)
    prod.finalize()
    orc.finalize()
    prod.set_variant(0, variant)
    u = uniform01(23, prod.num_adofs) - 0.5
    K, R = prod.element_matrices(0, 0, orc.num_eq(0), u)
    for eq in range(orc.num_eq(0)):
        Ko, Ro = orc.element_matrices(0, eq, u)
        n = len(Ro)
        assert rel_err(K[eq, :n, :n], Ko) <= RTOL and rel_err(R[eq, :n], Ro) <= RTOL, eq
    rp, _ = prod.graph()
    vo, ro = orc.assemble(u)
    vh, rh = prod.assemble_host(u)
    assert csr_row_rel_err(rp, vh, vo) <= RTOL and rel_err(rh, ro) <= RTOL


def test_residual_only_and_jacobian_only_flags(torch):
    prod, orc, _ = problem(2, (4, 4), 2, sides=True)
    prod.finalize()
    orc.finalize()
    u = uniform01(3, prod.num_adofs)
    vo, ro = orc.assemble(u)
    v1, r1 = prod.assemble_host(u, mg.NO_JACOBIAN)
    assert np.all(v1 == 0) and rel_err(r1, ro) <= RTOL
    v2, r2 = prod.assemble_host(u, mg.NO_RESIDUAL)
    assert np.all(r2 == 0)
    rp, _ = prod.graph()
    assert csr_row_rel_err(rp, v2, vo) <= RTOL


@pytest.mark.parametrize("dim,ne,p,shape", [(2, (6, 6), 2, mg.SHAPE_GENERAL), (3, (4, 3, 3), 2, mg.SHAPE_RECTANGULAR),
                                            (3, (3, 3, 3), 1, mg.SHAPE_GENERAL)])
def test_matrix_free_apply_matches_assembled_operator(torch, dim, ne, p, shape):
    prod, orc, _ = problem(dim, ne, p, shape)
    prod.finalize()
    orc.finalize()
    rp, ci = orc.graph()
    vo, _ = orc.assemble(None)
    x = uniform01(9, prod.num_adofs) - 0.5
    import scipy.sparse as sp
    y_ref = sp.csr_matrix((vo, ci, rp), shape=(prod.num_adofs,) * 2) @ x
    xt = torch.tensor(x, device="cuda")
    yt = torch.empty_like(xt)
    prod.apply(xt, yt)
    torch.cuda.synchronize()
    assert rel_err(yt.cpu().numpy(), y_ref) <= RTOL


def test_pcg_solves_plane_strain_cantilever(torch):
    # small version of the 2D elasticity case: clamp x=0 (Nitsche), traction at x=1
    prod, orc, _ = problem(2, (16, 16), 1, sides=True)
    prod.finalize()
    orc.finalize()
    rp, ci = orc.graph()
    vo, ro = orc.assemble(None)
    from oracle.oracle import pcg
    x_ref, it_ref, rr_ref, rc = pcg(rp, ci, vo, -ro, rtol=1e-10)
    assert rc == 0
    rpt = torch.tensor(rp, device="cuda")
    cit = torch.tensor(ci, device="cuda")
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(None, vals, rhs)
    b = -rhs
    x = torch.zeros_like(b)
    rep = prod.pcg(rpt, cit, vals, b, x, rel_tol=1e-10)
    assert rep["converged"] and rep["rel_residual"] <= 1e-10
    assert abs(rep["iterations"] - it_ref) <= max(3, it_ref // 20)
    assert rel_err(x.cpu().numpy(), x_ref) <= 1e-8


def test_pcg_reports_non_convergence(torch):
    prod, _, _ = problem(2, (8, 8), 1, sides=True)
    prod.finalize()
    rp, ci = prod.graph()
    rpt = torch.tensor(rp, device="cuda")
    cit = torch.tensor(ci, device="cuda")
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(None, vals, rhs)
    x = torch.zeros_like(rhs)
    with pytest.raises(mg.FemGpuError) as ei:
        prod.pcg(rpt, cit, vals, -rhs, x, rel_tol=1e-14, max_iter=5)
    assert ei.value.status == 10  # NOT_CONVERGED


def test_nonfinite_input_is_reported(torch):
    prod, _, _ = problem(2, (3, 3), 1)
    prod.finalize()
    u = np.zeros(prod.num_adofs)
    K, R = prod.element_matrices(0, 0, 1, u)
    assert np.isfinite(K).all()
    # a NaN in the solution vector leaves K finite; a NaN modulus does not
    mesh = mg.hmr_uniform_mesh(2, (2, 2), (1.0, 1.0), 1)
    m = mg.FemModel(2, mesh)
    with pytest.raises(mg.FemGpuError) as ei:
        m.add_bulk_set(np.arange(4), [1.0, np.nan, 1.0, 1.0], 0.3, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN)
    assert ei.value.status == 3


@pytest.mark.parametrize("dim", [2, 3])
def test_empty_sets_do_no_work(torch, dim):
    """Sets without equation objects before and after the populated ones: the
    per-set, autotuned, element-level and (3D) batched paths give the oracle's
    system of the populated sets."""
    ne = (5, 4) if dim == 2 else (3, 3, 2)
    rule = mg.RULE_QUAD_2x2 if dim == 2 else mg.RULE_HEX_2x2x2
    prod, orc, _ = problem(dim, ne, 1, mg.SHAPE_RECTANGULAR, rule, True, empty_sets=True)
    prod.finalize()
    orc.finalize()
    bulk = 2 if dim == 2 else 4  # index of the populated bulk set
    assert all(prod.num_eq(k) == 0 for k in range(bulk)) and prod.num_eq(bulk) == orc.num_eq(0)
    u = uniform01(5, prod.num_adofs)
    rp, _ = prod.graph()
    vo, ro = orc.assemble(u)
    vh, rh = prod.assemble_host(u)
    assert csr_row_rel_err(rp, vh, vo) <= RTOL and rel_err(rh, ro) <= RTOL
    prod.autotune()
    vh, rh = prod.assemble_host(u)
    assert csr_row_rel_err(rp, vh, vo) <= RTOL and rel_err(rh, ro) <= RTOL
    K, R = prod.element_matrices(0, 0, 0, u)
    assert K.shape[0] == 0 and R.shape[0] == 0
    if dim == 3:
        ut = torch.tensor(u, dtype=torch.float64, device="cuda")
        vals = torch.zeros(prod.nnz, dtype=torch.float64, device="cuda")
        rhs = torch.zeros(prod.num_adofs, dtype=torch.float64, device="cuda")
        prod.assemble_batched(ut, vals, rhs)
        torch.cuda.synchronize()
        prod.check_status()
        assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL and rel_err(rhs.cpu().numpy(), ro) <= RTOL


def test_host_buffer_assembly_overlaps_the_copy_back(torch):
    """Host-buffer assembly runs the element loop in chunks and copies every
    finished row range while the next chunk computes: with more than one chunk
    (40^3 elements, bulk and side sets) it must equal the device-buffer
    assembly row for row (only the atomic summation order differs)."""
    prod, _, _ = problem(3, (40, 40, 40), 1, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_2x2x2, True)
    prod.finalize()
    u = uniform01(23, prod.num_adofs) - 0.5
    rp, _ = prod.graph()
    vh, rh = prod.assemble_host(u)
    ud = torch.tensor(u, device="cuda")
    vd = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rd = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(ud, vd, rd)
    assert csr_row_rel_err(rp, vh, vd.cpu().numpy()) <= RTOL and rel_err(rh, rd.cpu().numpy()) <= RTOL
    for _ in range(2):  # the cached chunk plan and copy stream are reused
        vh2, rh2 = prod.assemble_host(u)
        assert csr_row_rel_err(rp, vh2, vh) <= RTOL and rel_err(rh2, rh) <= RTOL


SELECT_CASES = [
    # dim, ne, p, shape, rule, iwg
    (2, (5, 4), 2, mg.SHAPE_GENERAL, mg.RULE_QUAD_2x2, mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE),
    (3, (3, 2, 3), 2, mg.SHAPE_GENERAL, mg.RULE_HEX_3x3x3, mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE),
    (3, (3, 3, 2), 1, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_2x2x2, mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE),
]


@pytest.mark.parametrize("case", SELECT_CASES, ids=lambda c: "d%d-p%d-iwg%d" % (c[0], c[2], c[5]))
def test_select_and_thickness_properties_match_oracle(torch, case):
    """Dirichlet sets with a general (non-diagonal) Select matrix and every set
    with a Thickness property (..._Dirichlet.cpp:66-116, ..._Neumann.cpp:66-67,
    ..._Bulk.cpp:84-85): element operators, CSR values and residual."""
    from oracle import OracleModel
    from tests.common import distort
    dim, ne, p, shape, rule, iwg = case
    mesh = mg.hmr_uniform_mesh(dim, ne, [1.0] * dim, p)
    if shape == mg.SHAPE_GENERAL:
        mesh = distort(mesh, dim, ne, 0.2, 8)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 * uniform01(2, nc))
    model = mg.MODEL_3D if dim == 3 else mg.MODEL_PLANE_STRAIN
    ipc = mg.CELL_QUAD4 if dim == 2 else mg.CELL_HEX8
    srule = mg.RULE_BAR_3 if dim == 2 else mg.RULE_QUAD_2x2
    M = np.random.default_rng(4).uniform(-1.0, 1.0, (dim, dim))
    t_bulk, t_dir, t_neu = 0.37, 0.6, 1.7
    cells = np.arange(nc, dtype=np.int32)
    left = cells[cells % ne[0] == 0]
    right = cells[cells % ne[0] == ne[0] - 1]
    prod = mg.FemModel(dim, mesh, shape)
    orc = OracleModel(dim, ipc, shape, mesh)
    prod.add_bulk_set(cells, E, 0.3, rule, model, thickness=t_bulk)
    orc.add_bulk_set(ipc, rule, model, cells, E, 0.3)
    orc.set_bulk_thickness(0, t_bulk)
    g = tuple(0.01 * (k + 1) for k in range(dim))
    prod.add_side_set(iwg, left, np.full(len(left), 3), E[left], 0.3, srule, model, alpha=50.0, value=g,
                      thickness=t_dir, select=M)
    orc.add_side_set(iwg, srule, model, left, np.full(len(left), 3), E[left], 0.3, 50.0, g)
    orc.set_side_options(0, t_dir, M)
    trac = (1e-3,) + (2e-3,) * (dim - 1)
    prod.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, right, np.full(len(right), 1), E[right], 0.3, srule, model,
                      value=trac, thickness=t_neu)
    orc.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, srule, model, right, np.full(len(right), 1), E[right], 0.3, 0.0,
                     trac)
    orc.set_side_options(1, t_neu, None)
    prod.finalize()
    orc.finalize()
    u = uniform01(12, prod.num_adofs) - 0.5
    for s in range(3):
        n_eq = orc.num_eq(s)
        K, R = prod.element_matrices(s, 0, n_eq, u)
        for eq in range(n_eq):
            Ko, Ro = orc.element_matrices(s, eq, u)
            n = len(Ro)
            assert rel_err(K[eq, :n, :n], Ko) <= RTOL, (s, eq)
            assert rel_err(R[eq, :n], Ro) <= RTOL, (s, eq)
    rp, _ = prod.graph()
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(torch.tensor(u, device="cuda"), vals, rhs)
    torch.cuda.synchronize()
    vo, ro = orc.assemble(u)
    assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL


def test_zero_select_adds_nothing(torch):
    """A Dirichlet set whose Select matrix is zero contributes nothing: the
    reference skips the IWG when the projection's norm is below machine
    epsilon (..._Dirichlet.cpp:86, 161).  Its element operators and residuals are
    zero, and the assembled system is the oracle's (brick cells, linear
    B-splines, with a Neumann set beside it)."""
    from oracle import OracleModel
    dim, ne, p = 3, (3, 2, 2), 1
    mesh = mg.hmr_uniform_mesh(dim, ne, [1.0] * dim, p)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 * uniform01(5, nc))
    cells = np.arange(nc, dtype=np.int32)
    left = cells[cells % ne[0] == 0]
    right = cells[cells % ne[0] == ne[0] - 1]
    prod = mg.FemModel(dim, mesh, mg.SHAPE_RECTANGULAR)
    orc = OracleModel(dim, mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, mesh)
    prod.add_bulk_set(cells, E, 0.3, mg.RULE_HEX_2x2x2, mg.MODEL_3D)
    orc.add_bulk_set(mg.CELL_HEX8, mg.RULE_HEX_2x2x2, mg.MODEL_3D, cells, E, 0.3)
    zero = np.zeros((dim, dim))
    iwg = mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE
    prod.add_side_set(iwg, left, np.full(len(left), 3), E[left], 0.3, mg.RULE_QUAD_2x2, mg.MODEL_3D, alpha=50.0,
                      value=(0.01, 0.02, 0.03), select=zero)
    orc.add_side_set(iwg, mg.RULE_QUAD_2x2, mg.MODEL_3D, left, np.full(len(left), 3), E[left], 0.3, 50.0,
                     (0.01, 0.02, 0.03))
    orc.set_side_options(0, 1.0, zero)
    trac = (1e-3, 2e-3, 3e-3)
    prod.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, right, np.full(len(right), 1), E[right], 0.3, mg.RULE_QUAD_2x2,
                      mg.MODEL_3D, value=trac)
    orc.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, mg.RULE_QUAD_2x2, mg.MODEL_3D, right, np.full(len(right), 1),
                     E[right], 0.3, 0.0, trac)
    prod.finalize()
    orc.finalize()
    u = uniform01(13, prod.num_adofs) - 0.5
    K, R = prod.element_matrices(1, 0, orc.num_eq(1), u)
    assert not np.any(K) and not np.any(R)
    rp, _ = prod.graph()
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(torch.tensor(u, device="cuda"), vals, rhs)
    torch.cuda.synchronize()
    vo, ro = orc.assemble(u)
    assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL


def test_tensor_and_general_extraction_paths_match_oracle(torch):
    """Uniform quadratic elements take the bulk kernel's tensor-product path
    (T = P/8, checked per element); an element with a node whose extraction
    weights differ, by 1e-3 or by one unit in the last place, takes the
    column-list path.  Both kinds in one launch: element matrices, CSR values
    and residual against the oracle with the same extraction."""
    from oracle import OracleModel
    dim, ne = 3, (4, 3, 3)
    mesh = mg.hmr_uniform_mesh(dim, ne, [1.0] * dim, 2)
    tw, off = mesh["t_w"].copy(), mesh["t_off"]
    for n in range(0, len(off) - 1, 7):
        tw[off[n]:off[n + 1]] *= 1.0 + 1e-3 * (1 + n % 5)
    tw[off[3]] = np.nextafter(tw[off[3]], 1.0)
    mesh = dict(mesh, t_w=tw)
    nc = len(mesh["cells"])
    touched = {n for n in range(0, len(off) - 1, 7)} | {3}
    tensor_cells = [c for c in range(nc) if not touched & set(mesh["cells"][c].tolist())]
    assert 0 < len(tensor_cells) < nc  # both paths present
    E = 10.0 ** (-3.0 * uniform01(3, nc))
    cells = np.arange(nc, dtype=np.int32)
    prod = mg.FemModel(dim, mesh, mg.SHAPE_RECTANGULAR)
    orc = OracleModel(dim, mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, mesh)
    prod.add_bulk_set(cells, E, 0.3, mg.RULE_HEX_3x3x3, mg.MODEL_3D)
    orc.add_bulk_set(mg.CELL_HEX8, mg.RULE_HEX_3x3x3, mg.MODEL_3D, cells, E, 0.3)
    prod.finalize()
    orc.finalize()
    rp, ci = prod.graph()
    rpo, cio = orc.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    u = uniform01(6, prod.num_adofs) - 0.5
    K, R = prod.element_matrices(0, 0, nc, u)
    for eq in range(nc):
        Ko, Ro = orc.element_matrices(0, eq, u)
        n = len(Ro)
        assert rel_err(K[eq, :n, :n], Ko) <= RTOL, eq
        assert rel_err(R[eq, :n], Ro) <= RTOL, eq
    vo, ro = orc.assemble(u, nthreads=4)
    ut = torch.tensor(u, device="cuda")
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(ut, vals, rhs)
    torch.cuda.synchronize()
    assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL
