"""Host-side parity of the product library against the oracle (no GPU).

The HMR-equivalent mesh generator, the MSI adof numbering / element adof
lists and the CSR sparsity graph of libfem_gpu are compared with the oracle's
independent restatement: integer data must be identical, extraction weights
equal to the last bit or within 1e-15.
"""
import numpy as np
import pytest

import moris_gb300 as mg
from oracle import OracleLib, OracleModel


@pytest.fixture(scope="module")
def orc():
    return OracleLib()


CASES = [(2, (5, 3), 1), (2, (4, 4), 2), (2, (3, 5), 3), (3, (3, 2, 2), 1), (3, (3, 3, 2), 2), (3, (2, 2, 3), 3)]


@pytest.mark.parametrize("dim,ne,p", CASES)
def test_hmr_mesh_matches_oracle(orc, dim, ne, p):
    L = [1.0, 2.0, 0.5][:dim]
    a = mg.hmr_uniform_mesh(dim, ne, L, p)
    b = orc.hmr_uniform(dim, ne, L, p)
    assert a["num_bases"] == b["num_bases"]
    assert np.array_equal(a["cells"], b["cells"])
    assert np.array_equal(a["t_off"], b["t_off"])
    assert np.allclose(a["coords"], b["coords"], rtol=0, atol=1e-15)
    # rows may list bases in a different order: compare as sorted pairs
    for n in range(len(a["t_off"]) - 1):
        s = slice(a["t_off"][n], a["t_off"][n + 1])
        ia, ib = np.argsort(a["t_bases"][s]), np.argsort(b["t_bases"][s])
        assert np.array_equal(a["t_bases"][s][ia], b["t_bases"][s][ib])
        assert np.allclose(a["t_w"][s][ia], b["t_w"][s][ib], rtol=0, atol=1e-15)


def build_pair(dim, ne, p, sides=True, seed=0):
    mesh = mg.hmr_uniform_mesh(dim, ne, [1.0] * dim, p)
    rng = np.random.default_rng(seed)
    nc = len(mesh["cells"])
    E = 10.0 ** rng.uniform(-3, 0, nc)
    model = mg.MODEL_3D if dim == 3 else mg.MODEL_PLANE_STRAIN
    rule = mg.RULE_HEX_3x3x3 if dim == 3 else mg.RULE_QUAD_2x2
    prod = mg.FemModel(dim, mesh)
    orcm = OracleModel(dim, mg.CELL_QUAD4 if dim == 2 else mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, mesh)
    cells = np.arange(nc, dtype=np.int32)
    prod.add_bulk_set(cells, E, 0.3, rule, model)
    orcm.add_bulk_set(mg.CELL_QUAD4 if dim == 2 else mg.CELL_HEX8, rule, model, cells, E, 0.3)
    if sides and dim == 2:
        left = np.arange(0, nc, ne[0], dtype=np.int32)
        right = np.arange(ne[0] - 1, nc, ne[0], dtype=np.int32)
        srule = mg.RULE_BAR_3
        prod.add_side_set(mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, left, np.full(len(left), 3), E[left], 0.3,
                          srule, model, alpha=100.0, value=(0.0, 0.0))
        orcm.add_side_set(mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, srule, model, left,
                          np.full(len(left), 3), E[left], 0.3, 100.0, (0.0, 0.0))
        prod.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, right, np.full(len(right), 1), E[right], 0.3, srule, model,
                          value=(1e-3, 0.0))
        orcm.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, srule, model, right, np.full(len(right), 1), E[right], 0.3,
                          0.0, (1e-3, 0.0))
    return prod, orcm, mesh


@pytest.mark.parametrize("dim,ne,p", CASES)
def test_dof_maps_and_graph_match_oracle(dim, ne, p):
    prod, orcm, _ = build_pair(dim, ne, p)
    prod.finalize(host_only=True)
    orcm.finalize()
    assert prod.num_adofs == orcm.num_adofs
    assert prod.nnz == orcm.nnz
    rp_a, ci_a = prod.graph()
    rp_b, ci_b = orcm.graph()
    assert np.array_equal(rp_a, rp_b)
    assert np.array_equal(ci_a, ci_b)
    for s in range(orcm.num_sets()):
        assert prod.num_eq(s) == orcm.num_eq(s)
        for eq in range(orcm.num_eq(s)):
            assert np.array_equal(prod.element_topology(s, eq), orcm.element_topology(s, eq))


def test_graph_rows_sorted_and_symmetric():
    prod, _, _ = build_pair(3, (3, 3, 3), 2, sides=False)
    prod.finalize(host_only=True)
    rp, ci = prod.graph()
    n = len(rp) - 1
    for r in range(n):
        row = ci[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0)
    # structural symmetry
    pairs = set()
    for r in range(n):
        for c in ci[rp[r]:rp[r + 1]]:
            pairs.add((r, int(c)))
    assert all((c, r) in pairs for (r, c) in pairs)


def test_bad_inputs_are_rejected():
    mesh = mg.hmr_uniform_mesh(2, (2, 2), (1.0, 1.0), 1)
    bad = dict(mesh)
    bad["cells"] = mesh["cells"].copy()
    bad["cells"][0, 0] = 10 ** 6
    with pytest.raises(mg.FemGpuError) as ei:
        mg.FemModel(2, bad)
    assert ei.value.status == 2  # OOB_INDEX
    bad = dict(mesh)
    bad["coords"] = mesh["coords"].copy()
    bad["coords"][1, 0] = np.nan
    with pytest.raises(mg.FemGpuError) as ei:
        mg.FemModel(2, bad)
    assert ei.value.status == 3  # NONFINITE
    m = mg.FemModel(2, mesh)
    with pytest.raises(mg.FemGpuError) as ei:
        m.add_bulk_set([0, 1, 99], [1.0, 1.0, 1.0], 0.3, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN)
    assert ei.value.status == 2
    with pytest.raises(mg.FemGpuError):
        m.add_bulk_set([0], [1.0], 0.6, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN)  # poisson out of range
    with pytest.raises(mg.FemGpuError):
        m.add_bulk_set([0], [1.0], 0.3, mg.RULE_HEX_2x2x2, mg.MODEL_PLANE_STRAIN)  # rule dim mismatch
    with pytest.raises(mg.FemGpuError) as ei:
        m.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, [0], [7], [1.0], 0.3, mg.RULE_BAR_3, mg.MODEL_PLANE_STRAIN)
    assert ei.value.status == 2


def test_empty_sets_keep_indices_and_graph():
    """Sets with no equation objects (a processor without facets on a side set,
    a mesh with no cut cells) are accepted, keep the caller's set indices and
    leave the adof numbering and the graph unchanged."""
    ref, orcm, mesh = build_pair(2, (4, 3), 2)
    ref.finalize(host_only=True)
    orcm.finalize()
    prod = mg.FemModel(2, mesh)
    nc = len(mesh["cells"])
    rng = np.random.default_rng(0)
    E = 10.0 ** rng.uniform(-3, 0, nc)
    empty_i, empty_f = np.zeros(0, np.int32), np.zeros(0)
    assert prod.add_bulk_set(empty_i, empty_f, 0.3, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN) == 0
    assert prod.add_bulk_set(np.arange(nc, dtype=np.int32), E, 0.3, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN) == 1
    assert prod.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, empty_i, empty_i, empty_f, 0.3, mg.RULE_BAR_3,
                             mg.MODEL_PLANE_STRAIN, value=(1.0, 0.0)) == 2
    prod.finalize(host_only=True)
    assert prod.num_eq(0) == 0 and prod.num_eq(2) == 0
    assert prod.num_eq(1) == nc
    rp_a, ci_a = prod.graph()
    # the graph depends only on the cells in use: the full-mesh pair's graph
    rp_b, ci_b = orcm.graph()
    assert np.array_equal(rp_a, rp_b) and np.array_equal(ci_a, ci_b)
    for eq in range(nc):
        assert np.array_equal(prod.element_topology(1, eq), orcm.element_topology(0, eq))
    with pytest.raises(mg.FemGpuError) as ei:
        prod.element_topology(0, 0)
    assert ei.value.status == 2


def test_empty_cut_and_interface_sets_accepted():
    mesh = mg.hmr_uniform_mesh(3, (2, 2, 2), (1.0,) * 3, 1)
    nc = len(mesh["cells"])
    m = mg.FemModel(3, mesh)
    m.add_bulk_set(np.arange(nc, dtype=np.int32), np.ones(nc), 0.3, mg.RULE_HEX_2x2x2, mg.MODEL_3D)
    # a cut set and an interface set of a mesh the geometry does not cut
    m.add_bulk_set(np.zeros(0, np.int32), np.zeros(0), 0.3, mg.RULE_TET_4, mg.MODEL_3D, ig_cell=mg.CELL_TET4,
                   ig_offsets=np.zeros(1, np.int64), ig_coords=np.zeros(0), ig_param=np.zeros(0))
    m.add_double_side_set(mg.IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE, np.zeros(0, np.int32),
                          np.zeros(0, np.int32), np.zeros(1, np.int64), np.zeros(0), np.zeros(0), np.zeros(0),
                          np.zeros(0), np.zeros(0), 0.3, mg.RULE_TRI_3, mg.CELL_TRI3, 10.0)
    m.finalize(host_only=True)
    assert [m.num_eq(s) for s in range(3)] == [nc, 0, 0]


def test_model_without_equation_objects_is_rejected():
    mesh = mg.hmr_uniform_mesh(2, (2, 2), (1.0, 1.0), 1)
    m = mg.FemModel(2, mesh)
    m.add_bulk_set(np.zeros(0, np.int32), np.zeros(0), 0.3, mg.RULE_QUAD_2x2, mg.MODEL_PLANE_STRAIN)
    with pytest.raises(mg.FemGpuError) as ei:
        m.finalize(host_only=True)
    assert ei.value.status == 1


def test_level_set_field_is_validated_on_the_host():
    """fem_gpu_set_level_set_field checks every coefficient id before it
    touches the device, and fem_gen_dqdp refuses a table given by half or a
    stored field of other sizes (the device pointers below are never read)."""
    import ctypes
    mesh = mg.hmr_uniform_mesh(3, (2, 2, 2), [1.0] * 3, 1)
    m = mg.FemModel(3, mesh)
    nodes, width, ncoef = len(mesh["coords"]), 8, 64
    cols = (np.arange(nodes * width, dtype=np.int32) % ncoef).reshape(nodes, width)
    vals = np.full((nodes, width), 0.125)
    for bad in (ncoef, -1):
        c2 = cols.copy()
        c2[5, 3] = bad
        with pytest.raises(mg.FemGpuError) as ei:
            m.set_level_set_field(c2, vals, ncoef)
        assert ei.value.args[0].startswith("fem_gpu status 2 ")  # FEM_GPU_OOB_INDEX
    with pytest.raises(ValueError):
        m.set_level_set_field(cols[:, :4], vals, ncoef)
    with pytest.raises(ValueError):
        m.gen_dqdp(None, None, None, ncoef, None)  # no field stored
    lib = mg.lib()
    dev = ctypes.c_void_p(256)
    tw = vals.ctypes.data_as(ctypes.c_void_p)
    assert lib.fem_gen_dqdp(m.h, dev, nodes, width, None, tw, ncoef, dev) == 1  # FEM_GPU_BAD_ARG
    assert lib.fem_gen_dqdp(m.h, dev, nodes, width, None, None, ncoef, dev) == 1  # no vertex table, no field
