"""Geometric multigrid preconditioner (the reference's PCMG path restated for
the GPU): the CPU restatement's own properties (Galerkin operator = coarse
B-spline operator, symmetric positive definite V-cycle, fewer CG iterations
than Jacobi), then the device hierarchy against it level by level (stencils,
smoothing intervals, the V-cycle) and the flexible CG that uses it."""
import numpy as np
import pytest
import scipy.sparse as sp

import moris_gb300 as mg
from oracle import OracleModel
from oracle import mg_oracle as mo

from common import problem


def oracle_csr(orc, n):
    rp, ci = orc.graph()
    vals, rhs = orc.assemble()
    return sp.csr_matrix((vals, ci, rp), shape=(3 * n ** 3,) * 2), rhs


def uniform_operator(ne):
    mesh = mg.hmr_uniform_mesh(3, (ne,) * 3, (1.0,) * 3, 1)
    orc = OracleModel(3, mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, mesh)
    nc = len(mesh["cells"])
    orc.add_bulk_set(mg.CELL_HEX8, mg.RULE_HEX_2x2x2, mg.MODEL_3D, np.arange(nc, dtype=np.int32), np.ones(nc), 0.3)
    orc.finalize()
    return oracle_csr(orc, ne + 1)[0]


def simp_oracle(ne):
    _, orc, _ = problem(3, (ne,) * 3, 1, rule=mg.RULE_HEX_2x2x2, sides=True, density=True)
    orc.finalize()
    return oracle_csr(orc, ne + 1)


# ---------------------------------------------------------------------------
# CPU: the restatement


def test_galerkin_operator_is_the_coarse_bspline_operator():
    """P^T A_h P with the linear B-spline two-scale relation equals the operator
    assembled on the twice coarser mesh (nested spaces, exact 2x2x2 rule)."""
    A8 = uniform_operator(8)
    A4 = uniform_operator(4)
    P = mo.prolongation(9)
    G = (P.T @ A8 @ P).toarray()
    assert np.max(np.abs(G - A4.toarray())) <= 1e-13 * np.max(np.abs(A4.toarray()))


def test_oracle_vcycle_is_symmetric_positive_definite():
    A, _ = simp_oracle(8)
    h = mo.Hierarchy(A, 9, coarse_max=5)
    rng = np.random.default_rng(4)
    r1, r2 = rng.standard_normal(A.shape[0]), rng.standard_normal(A.shape[0])
    v1, v2 = h.vcycle(r1), h.vcycle(r2)
    assert abs(r2 @ v1 - r1 @ v2) <= 1e-12 * abs(r1 @ v1)
    assert r1 @ v1 > 0 and r2 @ v2 > 0


def test_oracle_multigrid_pcg_beats_jacobi_pcg():
    A, b = simp_oracle(16)
    h = mo.Hierarchy(A, 17, coarse_max=5)
    dinv = 1.0 / A.diagonal()
    _, it_j = mo.pcg(A, -b, lambda r: dinv * r)
    x, it_m = mo.pcg(A, -b, h.vcycle)
    assert np.linalg.norm(-b - A @ x) <= 1e-8 * np.linalg.norm(b)
    assert 4 * it_m <= it_j, (it_m, it_j)


# ---------------------------------------------------------------------------
# GPU: the device hierarchy against the restatement


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def device_system(n, beta=3.0):
    from moris_gb300 import learned, workloads
    m, mesh, rho = workloads.simp_3d(n, beta=beta)
    rp, ci, vals, b = learned.assembled_system(m)
    A = sp.csr_matrix((vals.cpu().numpy(), ci.cpu().numpy(), rp.cpu().numpy()), shape=(m.num_adofs,) * 2)
    return m, rp, ci, vals, b, A


@pytest.mark.gpu
@pytest.mark.parametrize("n,coarse_max,beta,tol", [(16, 5, 1.0, 1e-10), (32, 9, 3.0, 1e-7)])
def test_device_hierarchy_matches_oracle(torch, n, coarse_max, beta, tol):
    """Level stencils (1e-12 of the largest coefficient), lambda_max of the
    smoother (1e-10) and one V-cycle.  The V-cycle tolerance is set by the
    dense coarsest inverse: Gauss-Jordan on the device and LAPACK on the host
    agree to about cond(A_L) * 1e-16, 1e-10 at density contrast 1e3 (beta = 1)
    and 1e-7 at the SIMP contrast 1e9 (beta = 3)."""
    from moris_gb300.multigrid import Multigrid
    m, rp, ci, vals, b, A = device_system(n, beta)
    h = Multigrid(m, rp, ci, vals, coarse_max=coarse_max, fp32_levels=0)
    o = mo.Hierarchy(A, n + 1, coarse_max=coarse_max)
    assert h.num_levels == len(o.ns)
    for l, nl in enumerate(o.ns):
        nd, lam = h.level_info(l)
        assert nd == nl
        S = h.stencil(l)
        So = mo.stencil(o.A[l], nl)
        assert np.max(np.abs(S - So)) <= 1e-12 * np.max(np.abs(So)), l
        if l + 1 < len(o.ns):
            assert abs(lam - o.lmax[l]) <= 1e-10 * o.lmax[l], (l, lam, o.lmax[l])
    rng = np.random.default_rng(11)
    r = rng.standard_normal(m.num_adofs)
    z = h.apply(torch.tensor(r, device="cuda"), torch.empty(m.num_adofs, dtype=torch.float64, device="cuda"))
    zo = o.vcycle(r)
    err = float(np.max(np.abs(z.cpu().numpy() - zo)) / np.max(np.abs(zo)))
    assert err <= tol, err
    if beta == 1.0:
        # FP32 smoothing on the two finest levels: the same operator to FP32 rounding
        h32 = Multigrid(m, rp, ci, vals, coarse_max=coarse_max, fp32_levels=2)
        z32 = h32.apply(torch.tensor(r, device="cuda"),
                        torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")).cpu().numpy()
        assert float(np.max(np.abs(z32 - zo)) / np.max(np.abs(zo))) <= 1e-4


@pytest.mark.gpu
def test_multigrid_fcg_beats_jacobi_pcg(torch, record_property):
    """32^3 SIMP (density contrast 1e9): FCG with the V-cycle reaches 1e-8 on
    the true residual in at most a fifth of the Jacobi-PCG iterations, with and
    without the FP32 smoother stencils, and agrees with the Jacobi-PCG solution."""
    from moris_gb300.multigrid import Multigrid, fcg_config, fcg_mg
    m, rp, ci, vals, b, _ = device_system(32)
    xp = torch.zeros_like(b)
    plain = m.pcg(rp, ci, vals, b, xp, rel_tol=1e-8, max_iter=100000)
    fcg_config(1, 200)
    try:
        for fp32 in (0, 2):
            h = Multigrid(m, rp, ci, vals, fp32_levels=fp32)
            x = torch.zeros_like(b)
            rep = fcg_mg(m, rp, ci, vals, b, x, h, rel_tol=1e-8, max_iter=20000)
            assert rep["converged"] and not rep["fallback"], rep
            assert 5 * rep["iterations"] <= plain["iterations"], (rep["iterations"], plain["iterations"])
            assert float(torch.linalg.norm(x - xp) / torch.linalg.norm(xp)) < 1e-5
            record_property("iterations_mg_fp32_%d" % fp32, rep["iterations"])
    finally:
        fcg_config(8, 200)
    record_property("iterations_jacobi", plain["iterations"])


def test_oracle_threaded_pcg_matches_serial():
    """The multithreaded oracle Jacobi-PCG (the CPU baseline of the C5 solve)
    takes the same iterations as the serial one and reaches the same solution."""
    from oracle.oracle import pcg, pcg_mt
    A, b = simp_oracle(8)
    A = A.tocsr()
    x1, it1, r1, rc1 = pcg(A.indptr, A.indices, A.data, -b, rtol=1e-10, max_iter=5000)
    x4, it4, r4, rc4 = pcg_mt(A.indptr, A.indices, A.data, -b, rtol=1e-10, max_iter=5000, nthreads=4)
    assert rc1 == 0 and rc4 == 0 and abs(it1 - it4) <= 1
    assert np.linalg.norm(x4 - x1) <= 1e-8 * np.linalg.norm(x1)


@pytest.mark.gpu
def test_unsymmetric_operator_is_rejected(torch):
    """The hierarchy mirrors half of each Galerkin stencil, so it needs a
    symmetric operator: one perturbed off-diagonal entry is refused."""
    from moris_gb300 import FemGpuError
    from moris_gb300.multigrid import Multigrid
    m, rp, ci, vals, b, A = device_system(8)
    bad = vals.clone()
    row = 5
    cols = ci[int(rp[row]):int(rp[row + 1])].cpu().numpy()
    k = int(rp[row]) + int(np.nonzero(cols != row)[0][0])  # an off-diagonal entry of row 5
    bad[k] *= 1.5
    with pytest.raises(FemGpuError) as e:
        Multigrid(m, rp, ci, bad)
    assert e.value.status == 1
    Multigrid(m, rp, ci, vals).close()  # the symmetric one is accepted
