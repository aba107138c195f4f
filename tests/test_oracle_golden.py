"""Pin the CPU oracle against the reference's own fixtures and checks.

* Lagrange QUAD4/HEX8 values and first derivatives against
  FEM/INT/test/data/lagrange_{quad4,hex8}_*.bin (the reference's
  cl_FEM_Interpolation_Function_Lagrange_{Quad4,Hex8}.cpp, tol 1e-12).
* Gauss rules QUAD_2x2 / HEX_2x2x2 / HEX_3x3x3 against the polynomial
  integrals of integrate_*.bin (cl_FEM_Integrator.cpp, tol 1e-12).
* B-spline extraction: partition of unity of every node's T row (the
  1e-12 checks of HMR/test/ut_HMR_T_Matrix.cpp:100-140) and the basis
  counts n+p per direction (ut_HMR_Lagrange_Mesh.cpp:1048-1049 style).
* Elasticity IWG Jacobians against a 5-point finite difference of the
  residual with relative perturbation 1e-6 and tolerance 1e-6, on the
  deterministic inputs of FEM/INT/test/FEM_Test_Proxy/
  cl_FEM_Inputs_for_Elasticity_UT.cpp (IWG::check_jacobian,
  FEM/INT/src/IWG/cl_FEM_IWG.cpp:2498-2607).
"""
import numpy as np
import pytest

from tests._golden import elasticity_inputs, load_bin
from oracle import OracleLib, OracleModel

QUAD4, HEX8, TRI3, TET4 = 0, 1, 2, 3
BAR_3, QUAD_2x2, HEX_2x2x2, HEX_3x3x3, TRI_7, TET_4, TET_11 = 1, 2, 3, 4, 5, 6, 7
PLANE_STRAIN, PLANE_STRESS, FULL_3D = 0, 1, 2
RECT, GENERAL = 0, 1


@pytest.fixture(scope="module")
def orc():
    return OracleLib()


@pytest.mark.parametrize("cell,name,pts", [(QUAD4, "quad4", "points_2d.bin"), (HEX8, "hex8", "points_3d.bin")])
def test_lagrange_shape_functions_match_reference_fixtures(orc, cell, name, pts):
    xi = load_bin(pts)
    phihat = load_bin("lagrange_%s_phihat.bin" % name)[:, 0]
    phi = load_bin("lagrange_%s_phi.bin" % name)
    dphi = load_bin("lagrange_%s_dphidxi.bin" % name)
    for k in range(xi.shape[1]):
        N, dN = orc.shape(cell, xi[:, k])
        assert abs(N.sum() - 1.0) < 1e-12
        assert abs(N @ phihat - phi.ravel()[k]) < 1e-12
        assert np.linalg.norm(dphi[:, k] - dN @ phihat) < 1e-12


def _poly(path):
    d = load_bin(path)[:, 0]
    ndim, ncoef, integral = int(d[0]), int(d[1]), d[2]
    coef = d[3:3 + ncoef]
    expo = d[3 + ncoef:3 + ncoef + ndim * ncoef].reshape(ncoef, ndim)
    return coef, expo, integral


@pytest.mark.parametrize("rule,path", [(QUAD_2x2, "integrate_quad_2x2.bin"),
                                       (HEX_2x2x2, "integrate_hex_2x2x2.bin"),
                                       (HEX_3x3x3, "integrate_hex_3x3x3.bin")])
def test_gauss_rules_integrate_reference_polynomials(orc, rule, path):
    coef, expo, integral = _poly(path)
    pts, w = orc.rule(rule)
    val = 0.0
    for k in range(len(w)):
        x = pts[:, k]
        val += w[k] * sum(c * np.prod(x ** e) for c, e in zip(coef, expo))
    assert abs(integral - val) < 1e-12


@pytest.mark.parametrize("rule,vol", [(TET_4, 1.0), (TET_11, 1.0), (TRI_7, 1.0), (BAR_3, 2.0)])
def test_simplex_rule_weights(orc, rule, vol):
    _, w = orc.rule(rule)
    assert abs(w.sum() - vol) < 1e-12


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 3)])
def test_bspline_extraction_partition_of_unity(orc, dim, order):
    ne = [3, 4, 2][:dim]
    m = orc.hmr_uniform(dim, ne, [1.0] * dim, order)
    nb = np.prod([n + order for n in ne])
    assert m["num_bases"] == nb
    t_off, t_w = m["t_off"], m["t_w"]
    for n in range(len(t_off) - 1):
        assert abs(t_w[t_off[n]:t_off[n + 1]].sum() - 1.0) < 1e-12
    assert np.all(np.abs(t_w) > 1e-12)
    # linear B-splines interpolate: one basis per node with weight 1
    if order == 1:
        assert np.all(np.diff(t_off) == 1)


def _single_element_model(dim, xhat, rule, model, shape):
    npe = 4 if dim == 2 else 8
    mesh = dict(coords=np.asarray(xhat, dtype=float), cells=np.arange(npe, dtype=np.int32)[None, :],
                num_bases=npe, t_off=np.arange(npe + 1, dtype=np.int64),
                t_bases=np.arange(npe, dtype=np.int32), t_w=np.ones(npe))
    m = OracleModel(dim, QUAD4 if dim == 2 else HEX8, shape, mesh)
    m.add_bulk_set(QUAD4 if dim == 2 else HEX8, rule, model, [0], [1.0], 0.3)
    m.finalize()
    return m


def _fd5_jacobian(m, u):
    n = len(u)
    J = np.zeros((n, n))
    for j in range(n):
        h = 1e-6 * abs(u[j]) if abs(u[j]) > 1e-12 else 1e-6
        rs = []
        for s in (2, 1, -1, -2):
            up = u.copy()
            up[j] += s * h
            rs.append(m.element_pdof_matrices(0, 0, up)[1])
        J[:, j] = (-rs[0] + 8 * rs[1] - 8 * rs[2] + rs[3]) / (12 * h)
    return J


@pytest.mark.parametrize("dim,rule,model,shape", [(2, QUAD_2x2, PLANE_STRESS, GENERAL),
                                                  (2, QUAD_2x2, PLANE_STRAIN, GENERAL),
                                                  (3, HEX_2x2x2, FULL_3D, RECT),
                                                  (3, HEX_3x3x3, FULL_3D, GENERAL)])
def test_bulk_jacobian_matches_fd_on_reference_inputs(dim, rule, model, shape):
    inp = elasticity_inputs()
    npe = 4 if dim == 2 else 8
    xhat = inp["xhat_%dd" % dim]
    uhat = np.asarray(inp["uhat_%dd" % dim])[:npe]      # first time level
    u = uhat.T.ravel().copy()                            # type-major pdof vector
    m = _single_element_model(dim, xhat, rule, model, shape)
    K, R = m.element_pdof_matrices(0, 0, u)
    Kfd = _fd5_jacobian(m, u)
    absd = np.abs(K - Kfd)
    reld = np.abs((Kfd - K) / np.where(Kfd == 0, 1.0, Kfd))
    assert np.all((absd < 1e-6) | (reld < 1e-6))
    # linear elasticity: the residual is exactly K u
    assert np.allclose(R, K @ u, rtol=1e-12, atol=1e-12 * np.abs(K @ u).max())
    assert np.allclose(K, K.T, rtol=0, atol=1e-13 * np.abs(K).max())
