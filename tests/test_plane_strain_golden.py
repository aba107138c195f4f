"""The reference's plane-strain example as a physical golden.

projects/EXA/structure/linear/Plane_Strain (Plane_Strain_Problem.cpp:44-213,
checked by example_test_case.cpp:55-74): the 2 x 2 QUAD4 mesh of
4elements.e on [-1, 1]^2, E = 1, nu = 0.3, plane strain, Thickness 0.1 on
every IWG, rollers by unsymmetric Nitsche (alpha 100) with Select
properties -- u_y = 0 on the bottom edge (SelectY), u_x = 0 on the left edge
(SelectX) -- and the traction (0, -1) on the top edge.  The reference expects
at node (1, 1) U = (0.78, -1.82) and stress (xx, yy, zz) = (0, -1, -0.3)
within 1e-5.  The load is a uniaxial compression whose exact solution is
linear, so a correct plane-strain D matrix, Voigt order and consistent
Nitsche terms reproduce it exactly; a missing Select, a plane-stress D or a
wrong shear term would not.

The reference also adds a Bedding property of 1e-6 (a spring that holds
rigid-body modes) to the bulk IWG; with both roller sets the system is
non-singular without it, and it moves U by about 1e-6, inside the check's
1e-5.  It is left out here, on both sides.

The mesh (node coordinates, connectivity, side sets) is the fixture
tests/golden/plane_strain_4elements.json extracted from 4elements.e by
tests/golden/make_golden.py.  Its elements are rotated by 180 degrees
(local xi runs along -x), so the cells are given as general shapes.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

import moris_gb300 as mg
from oracle import OracleModel

from common import RTOL, csr_row_rel_err, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
MESH = json.load(open(os.path.join(HERE, "golden", "plane_strain_4elements.json")))
U_REF = np.array([0.78, -1.82])
SIGMA_REF = np.array([0.0, -1.0, -0.3])   # xx, yy, zz (transverse)
TOL = 1e-5
THICKNESS = 0.1
SELECT = {"sideset_bottom": [[0.0, 0.0], [0.0, 1.0]], "sideset_left": [[1.0, 0.0], [0.0, 0.0]]}
CORNER = 0  # the mesh node at (1, 1): local node 0 of cell 0


def _mesh():
    X = np.array(MESH["coords"])
    n = len(X)
    return dict(coords=X, cells=np.array(MESH["cells"], dtype=np.int32), num_bases=n,
                t_off=np.arange(n + 1, dtype=np.int64), t_bases=np.arange(n, dtype=np.int32), t_w=np.ones(n))


def _sets(dirichlet_iwg, select=True):
    """(kind, args) of the example: bulk, the two roller sets, the traction"""
    out = [("bulk", dict(cells=np.arange(len(MESH["cells"]), dtype=np.int32)))]
    for name in ("sideset_bottom", "sideset_left"):
        s = MESH["side_sets"][name]
        out.append(("side", dict(iwg=dirichlet_iwg, cells=s["cells"], ordinals=s["ordinals"], alpha=100.0,
                                 value=(0.0, 0.0), select=SELECT[name] if select else None)))
    s = MESH["side_sets"]["sideset_top"]
    out.append(("side", dict(iwg=mg.IWG_STRUC_LINEAR_NEUMANN, cells=s["cells"], ordinals=s["ordinals"], alpha=0.0,
                             value=(0.0, -1.0), select=None)))
    return out


def oracle_model(dirichlet_iwg, select=True):
    o = OracleModel(2, mg.CELL_QUAD4, mg.SHAPE_GENERAL, _mesh())
    k = 0
    for kind, a in _sets(dirichlet_iwg, select):
        if kind == "bulk":
            o.add_bulk_set(mg.CELL_QUAD4, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN, a["cells"], np.ones(len(a["cells"])),
                           0.3)
            o.set_bulk_thickness(0, THICKNESS)
        else:
            o.add_side_set(a["iwg"], mg.RULE_BAR_3, mg.MODEL_PLANE_STRAIN, a["cells"], a["ordinals"], np.ones(2), 0.3,
                           a["alpha"], a["value"])
            o.set_side_options(k, THICKNESS, a["select"])
            k += 1
    o.finalize()
    return o


def product_model(dirichlet_iwg, select=True):
    m = mg.FemModel(2, _mesh(), mg.SHAPE_GENERAL)
    for kind, a in _sets(dirichlet_iwg, select):
        if kind == "bulk":
            m.add_bulk_set(a["cells"], np.ones(len(a["cells"])), 0.3, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN,
                           thickness=THICKNESS)
        else:
            m.add_side_set(a["iwg"], a["cells"], a["ordinals"], np.ones(2), 0.3, mg.RULE_BAR_3, mg.MODEL_PLANE_STRAIN,
                           alpha=a["alpha"], value=a["value"], thickness=THICKNESS, select=a["select"])
    return m


def _solve(rowptr, colidx, vals, rhs):
    """K u = -R(0), dense (18 unknowns; the unsymmetric Nitsche K is not SPD)"""
    n = len(rhs)
    A = sp.csr_matrix((vals, colidx, rowptr), shape=(n, n)).toarray()
    return np.linalg.solve(A, -rhs)


def _corner_u(u, num_used):
    return np.array([u[CORNER], u[num_used + CORNER]])


# ---------------------------------------------------------------------------
# the oracle against the reference's numbers (CPU)

@pytest.mark.parametrize("iwg", [mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE,
                                 mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE])
def test_oracle_reproduces_the_plane_strain_example(iwg):
    o = oracle_model(iwg)
    v, r = o.assemble()
    rp, ci = o.graph()
    u = _solve(rp, ci, v, r)
    nu = o.num_adofs // 2
    assert np.linalg.norm(_corner_u(u, nu) - U_REF) < TOL
    sig = o.element_flux(0, 0, [-1.0, -1.0], u)  # cell 0, local node 0 = (1, 1)
    assert np.max(np.abs(sig[:3] - SIGMA_REF)) < TOL and abs(sig[3]) < TOL


def test_the_select_property_decides_the_example():
    # without SelectX / SelectY the edges are clamped in both directions
    o = oracle_model(mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE, select=False)
    v, r = o.assemble()
    rp, ci = o.graph()
    u = _solve(rp, ci, v, r)
    assert np.linalg.norm(_corner_u(u, o.num_adofs // 2) - U_REF) > 0.05


# ---------------------------------------------------------------------------
# the GPU path on the same problem

@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("iwg", [mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE,
                                 mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE])
def test_gpu_reproduces_the_plane_strain_example(torch, iwg):
    o = oracle_model(iwg)
    m = product_model(iwg)
    m.finalize()
    rp, ci = m.graph()
    rpo, cio = o.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    # element operators of every set at a seeded state
    u0 = np.random.default_rng(3).uniform(-1.0, 1.0, m.num_adofs)
    for s in range(4):
        K, R = m.element_matrices(s, 0, m.num_eq(s), u0)
        for eq in range(m.num_eq(s)):
            Ko, Ro = o.element_matrices(s, eq, u0)
            n = len(Ro)
            assert rel_err(K[eq, :n, :n], Ko) <= RTOL and rel_err(R[eq, :n], Ro) <= RTOL
    vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")
    m.assemble(None, vals, rhs)
    torch.cuda.synchronize()
    vo, ro = o.assemble()
    v, r = vals.cpu().numpy(), rhs.cpu().numpy()
    assert csr_row_rel_err(rp, v, vo) <= RTOL and rel_err(r, ro) <= RTOL
    u = _solve(rp, ci, v, r)
    assert np.linalg.norm(_corner_u(u, m.num_adofs // 2) - U_REF) < TOL
    sig = m.element_flux(0, [0], [[-1.0, -1.0]], torch.tensor(u, device="cuda"))[0]
    assert np.max(np.abs(sig[:3] - SIGMA_REF)) < TOL and abs(sig[3]) < TOL
    if iwg == mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE:
        # symmetric Nitsche: SPD, the library's PCG solves it
        x = torch.zeros_like(rhs)
        rep = m.pcg(torch.tensor(rp, device="cuda"), torch.tensor(ci, device="cuda"), vals, -rhs, x, rel_tol=1e-12)
        assert rep["converged"]
        assert np.linalg.norm(_corner_u(x.cpu().numpy(), m.num_adofs // 2) - U_REF) < TOL
