"""2D plane-strain cantilever (128 x 128 QUAD4, linear B-splines, Nitsche clamp,
Neumann traction): GPU assembly + Jacobi-PCG to 1e-10 against the oracle's
assembly + CG on the same inputs."""
import numpy as np
import pytest

import moris_gb300 as mg
from moris_gb300 import workloads
from oracle import OracleModel
from oracle.oracle import pcg
from tests.common import csr_row_rel_err, rel_err, RTOL


def oracle_cantilever(n):
    mesh = mg.hmr_uniform_mesh(2, (n, n), (1.0, 1.0), 1)
    nc = len(mesh["cells"])
    E = np.ones(nc)
    o = OracleModel(2, mg.CELL_QUAD4, mg.SHAPE_RECTANGULAR, mesh)
    o.add_bulk_set(mg.CELL_QUAD4, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN, np.arange(nc), E, 0.3)
    left = np.arange(0, nc, n)
    right = np.arange(n - 1, nc, n)
    o.add_side_set(mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, mg.RULE_BAR_3, mg.MODEL_PLANE_STRAIN, left,
                   np.full(len(left), 3), E[left], 0.3, workloads.NITSCHE_ALPHA, (0.0, 0.0))
    o.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, mg.RULE_BAR_3, mg.MODEL_PLANE_STRAIN, right, np.full(len(right), 1),
                   E[right], 0.3, 0.0, (workloads.TRACTION, 0.0))
    o.finalize()
    return o


def test_cantilever_host_setup_matches_oracle():
    m, _, _ = workloads.plane_strain_cantilever(32, finalize=False)
    m.finalize(host_only=True)
    o = oracle_cantilever(32)
    rp, ci = m.graph()
    rpo, cio = o.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)


@pytest.mark.gpu
def test_cantilever_128_solve_matches_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    m, _, _ = workloads.plane_strain_cantilever(128)
    o = oracle_cantilever(128)
    rp, ci = o.graph()
    vo, ro = o.assemble(None, nthreads=8)
    x_ref, it_ref, rr_ref, rc = pcg(rp, ci, vo, -ro, rtol=1e-10)
    assert rc == 0
    rpt = torch.tensor(rp, device="cuda")
    cit = torch.tensor(ci, device="cuda")
    vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")
    m.assemble(None, vals, rhs)
    torch.cuda.synchronize()
    assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL
    x = torch.zeros_like(rhs)
    rep = m.pcg(rpt, cit, vals, -rhs, x, rel_tol=1e-10)
    assert rep["converged"] and rep["rel_residual"] <= 1e-10
    assert abs(rep["iterations"] - it_ref) <= max(5, it_ref // 20)
    xs = x.cpu().numpy()
    import scipy.sparse as sp
    A = sp.csr_matrix((vo, ci, rp), shape=(len(ro),) * 2)
    assert np.linalg.norm(A @ xs + ro) <= 1.0001e-10 * np.linalg.norm(ro)
    assert rel_err(xs, x_ref) <= 1e-6
