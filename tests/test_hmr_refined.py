"""Refined (hierarchical) HMR B-spline meshes: the element T matrices and the
node extraction rows of graded meshes (fem_hmr_refined_*), against the
reference's own fixture and the numpy restatement in oracle/hmr_oracle.py.

The fixture is HMR's T-matrix test (projects/HMR/test/ut_HMR_T_Matrix.cpp:
53-196 with data/T-Matrix_test_values.hdf5): one element on [-1, 1]^d with
staircase buffer = refinement buffer = order, its first element refined twice,
the T matrix of the first level-2 element, labels D{2,3}_O{1,2,3}_T{0,1}
(dimension, B-spline order, truncation), compared exactly as the reference
does (CHECK_EQUAL).  The test's Parameters object leaves the polynomial
orders at their default 1, so HMR's padding refinement (ceil(max polynomial /
2)) is 1 there.
"""
import os

import numpy as np
import pytest

import moris_gb300 as mg
from oracle.hmr_oracle import RefinedMesh

from hdf5_min import read_datasets

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = read_datasets(os.path.join(HERE, "golden", "T-Matrix_test_values.hdf5"))
LABELS = [(d, p, t) for d in (2, 3) for p in (1, 2, 3) for t in (0, 1)]


def _label(c):
    return "D%d_O%d_T%d" % c


def test_fixture_is_read():
    assert sorted(FIXTURE) == sorted(_label(c) for c in LABELS)
    assert FIXTURE["D3_O2_T0"].shape == (27, 34)


@pytest.mark.parametrize("case", LABELS, ids=_label)
def test_oracle_reproduces_the_reference_t_matrices(case):
    d, p, t = case
    m = RefinedMesh(d, (1,) * d, (2.0,) * d, p, buffer=p, padding_refinement=1)
    m.refine([(0, (p,) * d)])        # the domain element (mesh indices count the padding)
    m.refine([(1, (2 * p,) * d)])    # its first child
    T, _ = m.element_t_matrix(2, (4 * p,) * d, bool(t))
    assert np.array_equal(T, FIXTURE[_label(case)])


@pytest.mark.parametrize("case", LABELS, ids=_label)
def test_library_reproduces_the_reference_t_matrices(case):
    d, p, t = case
    h = mg.RefinedHmr(d, (1,) * d, (2.0,) * d, p, staircase_buffer=p, padding_refinement=1)
    h.refine([(0, (0,) * d)])
    h.refine([(1, (0,) * d)])
    lv, ijk = h.active_elements()
    assert lv[0] == 2 and not ijk[0].any()   # the first active element, as the reference's get_element( 0 )
    T, dl, di = h.element_t_matrix(2, (0,) * d, bool(t))
    assert np.array_equal(T, FIXTURE[_label(case)])
    o = RefinedMesh(d, (1,) * d, (2.0,) * d, p, buffer=p, padding_refinement=1)
    o.refine([(0, (p,) * d)])
    o.refine([(1, (2 * p,) * d)])
    _, dofs = o.element_t_matrix(2, (4 * p,) * d, bool(t))
    assert [l for l, _ in dofs] == list(dl)
    assert [tuple(np.array(m) - p * 2 ** l) for l, m in dofs] == [tuple(x) for x in di]


# graded meshes: refine a corner region twice and an inner element three times
GRADED = [
    (2, (4, 3), 1), (2, (4, 4), 2), (2, (3, 3), 3), (3, (3, 2, 2), 1), (3, (2, 2, 2), 2),
]


def _graded(cls, d, ne, p, **kw):
    m = cls(d, ne, (1.0,) * d, p, **kw)
    pad = 0 if cls is mg.RefinedHmr else m.pad
    m.refine([(0, tuple(pad + c for c in (0,) * d)), (0, tuple(pad + (1 if k == 0 else 0) for k in range(d)))])
    m.refine([(1, tuple(2 * pad + c for c in (1,) * d))])
    m.refine([(2, tuple(4 * pad + c for c in (2,) * d))])
    return m


@pytest.mark.parametrize("case", GRADED, ids=lambda c: "d%d-p%d-%s" % (c[0], c[2], "x".join(map(str, c[1]))))
@pytest.mark.parametrize("truncate", [True, False], ids=["truncated", "plain"])
def test_refined_mesh_matches_oracle(case, truncate):
    d, ne, p = case
    h = _graded(mg.RefinedHmr, d, ne, p)
    o = _graded(RefinedMesh, d, ne, p)
    lv, ijk = h.active_elements()
    leaves = o.leaves()
    assert [l for l, _ in leaves] == list(lv)
    assert [tuple(np.array(e) - o.pad * 2 ** l) for l, e in leaves] == [tuple(x) for x in ijk]
    assert max(lv) == 3
    a, b = h.mesh(truncate), o.lagrange_mesh(truncate)
    assert a["num_bases"] == b["num_bases"]
    for k in ("cells", "t_off", "t_bases"):
        assert np.array_equal(a[k], b[k]), k
    assert np.max(np.abs(a["coords"] - b["coords"])) <= 1e-15
    assert np.max(np.abs(a["t_w"] - b["t_w"])) <= 1e-14
    if truncate:
        # truncated hierarchical B-splines are a partition of unity
        s = np.add.reduceat(a["t_w"], a["t_off"][:-1])
        assert np.max(np.abs(s - 1.0)) <= 1e-13


def test_refinement_rejects_inactive_elements():
    h = mg.RefinedHmr(2, (2, 2), (1.0, 1.0), 1)
    h.refine([(0, (0, 0))])
    with pytest.raises(mg.FemGpuError):
        h.refine([(0, (0, 0))])   # refined already
    with pytest.raises(mg.FemGpuError):
        h.refine([(0, (5, 0))])   # outside the mesh


# ---------------------------------------------------------------------------
# the element path on refined meshes (GPU)

REFINED_GPU = [(2, (4, 3), 1, True), (2, (4, 3), 1, False), (2, (4, 4), 2, True), (3, (3, 2, 2), 1, True),
               (3, (3, 2, 2), 1, False)]


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("case", REFINED_GPU, ids=lambda c: "d%d-p%d-%s" % (c[0], c[2], "trunc" if c[3] else "plain"))
def test_assembly_on_refined_mesh_matches_oracle(torch, case):
    from oracle import OracleModel
    from common import RTOL, csr_row_rel_err, rel_err
    d, ne, p, truncate = case
    mesh = _graded(mg.RefinedHmr, d, ne, p).mesh(truncate)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 * mg.rng.uniform01(17, nc))
    model = mg.MODEL_3D if d == 3 else mg.MODEL_PLANE_STRAIN
    ipc = mg.CELL_HEX8 if d == 3 else mg.CELL_QUAD4
    cells = np.arange(nc, dtype=np.int32)
    prod = mg.FemModel(d, mesh, mg.SHAPE_RECTANGULAR)
    prod.add_bulk_set(cells, E, 0.3, mg.RULE_AUTO, model)
    prod.finalize()
    orc = OracleModel(d, ipc, mg.SHAPE_RECTANGULAR, mesh)
    orc.add_bulk_set(ipc, mg.RULE_AUTO, model, cells, E, 0.3)
    orc.finalize()
    rp, ci = prod.graph()
    rpo, cio = orc.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    u = np.random.default_rng(5).uniform(-1.0, 1.0, prod.num_adofs)
    K, R = prod.element_matrices(0, 0, nc, u)
    width = prod.max_element_adofs(0) // d  # the padded layout: row f * width + i
    for eq in range(nc):
        ids = orc.element_topology(0, eq)
        assert np.array_equal(prod.element_topology(0, eq), ids)
        Ko, Ro = orc.element_matrices(0, eq, u)
        nb = len(ids) // d
        idx = np.array([f * width + i for f in range(d) for i in range(nb)])
        assert rel_err(K[eq][np.ix_(idx, idx)], Ko) <= RTOL and rel_err(R[eq][idx], Ro) <= RTOL
        pad = np.setdiff1d(np.arange(d * width), idx)
        assert not K[eq][pad].any() and not K[eq][:, pad].any() and not R[eq][pad].any()
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(torch.tensor(u, device="cuda"), vals, rhs)
    torch.cuda.synchronize()
    vo, ro = orc.assemble(u)
    assert csr_row_rel_err(rp, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL


@pytest.mark.gpu
def test_plane_strain_example_on_a_graded_mesh(torch):
    """The reference's plane-strain example (E 1, nu 0.3, rollers by unsymmetric
    Nitsche with Select, traction (0, -1) on top, thickness 0.1; U(1, 1) =
    (0.78, -1.82) and stress (0, -1, -0.3) there) on [-1, 1]^2 with 2 x 2
    coarse elements, the lower-left one refined twice and truncated linear
    hierarchical B-splines: hanging nodes, three levels, and still the exact
    linear solution."""
    import scipy.sparse as sp
    h = mg.RefinedHmr(2, (2, 2), (2.0, 2.0), 1)
    h.refine([(0, (0, 0))])
    h.refine([(1, (0, 0))])
    mesh = h.mesh(True)
    mesh["coords"] = mesh["coords"] - 1.0
    lv, ijk = h.active_elements()
    assert sorted(set(lv)) == [0, 1, 2]
    nc = len(lv)
    m = mg.FemModel(2, mesh, mg.SHAPE_RECTANGULAR)
    m.add_bulk_set(np.arange(nc, dtype=np.int32), np.ones(nc), 0.3, mg.RULE_AUTO, mg.MODEL_PLANE_STRAIN,
                   thickness=0.1)
    n_at = [2 * 2 ** l for l in lv]
    bottom = [i for i in range(nc) if ijk[i, 1] == 0]
    left = [i for i in range(nc) if ijk[i, 0] == 0]
    top = [i for i in range(nc) if ijk[i, 1] == n_at[i] - 1]
    iwg = mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE
    for cells, ordinal, select in ((bottom, 0, [[0, 0], [0, 1]]), (left, 3, [[1, 0], [0, 0]])):
        m.add_side_set(iwg, cells, np.full(len(cells), ordinal), np.ones(len(cells)), 0.3, mg.RULE_AUTO,
                       mg.MODEL_PLANE_STRAIN, alpha=100.0, value=(0.0, 0.0), thickness=0.1, select=select)
    m.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, top, np.full(len(top), 2), np.ones(len(top)), 0.3, mg.RULE_AUTO,
                   mg.MODEL_PLANE_STRAIN, value=(0.0, -1.0), thickness=0.1)
    m.finalize()
    rp, ci = m.graph()
    vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")
    m.assemble(None, vals, rhs)
    torch.cuda.synchronize()
    A = sp.csr_matrix((vals.cpu().numpy(), ci, rp), shape=(m.num_adofs,) * 2).toarray()
    u = np.linalg.solve(A, -rhs.cpu().numpy())
    nu = m.num_adofs // 2
    # displacement at the node (1, 1) through its extraction row
    node = int(np.nonzero(np.all(np.abs(mesh["coords"] - 1.0) < 1e-12, axis=1))[0][0])
    s = slice(mesh["t_off"][node], mesh["t_off"][node + 1])
    ranks = np.searchsorted(np.unique(mesh["t_bases"]), mesh["t_bases"][s])
    U = np.array([np.dot(mesh["t_w"][s], u[f * nu + ranks]) for f in range(2)])
    assert np.linalg.norm(U - np.array([0.78, -1.82])) < 1e-5
    cell = int(np.nonzero(np.any(mesh["cells"] == node, axis=1))[0][0])
    a = int(np.nonzero(mesh["cells"][cell] == node)[0][0])
    xi = [(-1.0, -1.0), (1.0, -1.0), (1.0, 1.0), (-1.0, 1.0)][a]
    sig = m.element_flux(0, [cell], [xi], torch.tensor(u, device="cuda"))[0]
    assert np.max(np.abs(sig[:3] - np.array([0.0, -1.0, -0.3]))) < 1e-5


# ---------------------------------------------------------------------------
# T matrices and node rows evaluated on the GPU


@pytest.mark.gpu
@pytest.mark.parametrize("case", LABELS, ids=_label)
def test_device_t_matrices_reproduce_the_reference(torch, case):
    """The GPU's element T matrix of the fixture element equals the reference's
    values exactly, with the host's columns (levels and ijk)."""
    d, p, t = case
    h = mg.RefinedHmr(d, (1,) * d, (2.0,) * d, p, staircase_buffer=p, padding_refinement=1)
    h.refine([(0, (0,) * d)])
    h.refine([(1, (0,) * d)])
    [(T, dl, di)] = h.element_t_matrices_device([2], [(0,) * d], bool(t))
    assert np.array_equal(T, FIXTURE[_label(case)])
    _, hl, hi = h.element_t_matrix(2, (0,) * d, bool(t))
    assert np.array_equal(dl, hl) and np.array_equal(di, hi)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GRADED, ids=lambda c: "d%d-p%d-%s" % (c[0], c[2], "x".join(map(str, c[1]))))
@pytest.mark.parametrize("truncate", [True, False], ids=["truncated", "plain"])
def test_device_evaluation_equals_host(torch, case, truncate):
    """Graded meshes (levels 0-3, 2-D and 3-D, orders 1-3): the T matrix of
    every active element and the whole node-row mesh computed on the GPU are
    the host's, bit for bit."""
    d, ne, p = case
    h = _graded(mg.RefinedHmr, d, ne, p)
    lv, ijk = h.active_elements()
    dev = h.element_t_matrices_device(lv, ijk, truncate)
    for (l, e), (T, dl, di) in zip(zip(lv, ijk), dev):
        Th, hl, hi = h.element_t_matrix(int(l), e, truncate)
        assert np.array_equal(T, Th) and np.array_equal(dl, hl) and np.array_equal(di, hi), (l, e)
    a, b = h.mesh(truncate, device=True), h.mesh(truncate)
    assert a["num_bases"] == b["num_bases"]
    for k in ("coords", "cells", "t_off", "t_bases", "t_w"):
        assert np.array_equal(a[k], b[k]), k
