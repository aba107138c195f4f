"""Shared builders for the parity tests: one seeded problem, two models (the
CUDA product through libfem_gpu and the CPU oracle) over identical arrays."""
import numpy as np

import moris_gb300 as mg
from moris_gb300.rng import uniform01 as _uniform01
from oracle import OracleModel

# element operators / residuals: |gpu - oracle| <= RTOL * max|oracle| (per element
# matrix, per assembled CSR row, per vector)
RTOL = 1e-12


def uniform01(seed, n):
    """Seeded inputs shared by the oracle-side and GPU-side models."""
    return _uniform01(seed, n)


def distort(mesh, dim, ne, amount, seed):
    """Move interior nodes by a seeded fraction of the element size."""
    m = dict(mesh)
    x = mesh["coords"].copy()
    h = np.array([1.0 / n for n in ne])
    rng = np.random.default_rng(seed)
    inner = np.all((x > 1e-12) & (x < 1 - 1e-12), axis=1)
    x[inner] += amount * h * rng.uniform(-1, 1, size=(inner.sum(), dim))
    m["coords"] = x
    return m


def _add_empty_sets(prod, dim, rule, model):
    """Sets with no equation objects around the populated ones (product only)."""
    none_i, none_f = np.zeros(0, np.int32), np.zeros(0)
    prod.add_bulk_set(none_i, none_f, 0.3, rule, model)
    prod.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, none_i, none_i, none_f, 0.3,
                      mg.RULE_BAR_3 if dim == 2 else mg.RULE_QUAD_2x2, model, value=(1.0,) + (0.0,) * (dim - 1))
    if dim == 3:
        prod.add_bulk_set(none_i, none_f, 0.3, mg.RULE_TET_4, model, ig_cell=mg.CELL_TET4,
                          ig_offsets=np.zeros(1, np.int64), ig_coords=none_f, ig_param=none_f)
        prod.add_double_side_set(mg.IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE, none_i, none_i,
                                 np.zeros(1, np.int64), none_f, none_f, none_f, none_f, none_f, 0.3, mg.RULE_TRI_3,
                                 mg.CELL_TRI3, 10.0)


def problem(dim, ne, p, shape=mg.SHAPE_RECTANGULAR, rule=None, sides=False, seed=1, distortion=0.2, density=False,
            empty_sets=False):
    """Product and oracle models of one mesh.  empty_sets adds, to the product
    only, sets without equation objects before and after the populated ones."""
    mesh = mg.hmr_uniform_mesh(dim, ne, [1.0] * dim, p)
    if shape == mg.SHAPE_GENERAL:
        mesh = distort(mesh, dim, ne, distortion, seed + 7)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 * uniform01(seed, nc))
    model = mg.MODEL_3D if dim == 3 else mg.MODEL_PLANE_STRAIN
    if rule is None:
        rule = mg.RULE_HEX_3x3x3 if dim == 3 else mg.RULE_QUAD_2x2
    ipc = mg.CELL_QUAD4 if dim == 2 else mg.CELL_HEX8
    prod = mg.FemModel(dim, mesh, shape)
    orc = OracleModel(dim, ipc, shape, mesh)
    cells = np.arange(nc, dtype=np.int32)
    if empty_sets:
        _add_empty_sets(prod, dim, rule, model)
    if density:
        rho = 1e-3 + (1 - 1e-3) * uniform01(seed + 99, len(mesh["coords"]))
        prod.add_bulk_set(cells, E, 0.3, rule, model, node_density=rho, density_exponent=3.0)
        orc.add_bulk_set(ipc, rule, model, cells, E, 0.3)
        orc.set_density(0, rho, 3.0)
    else:
        prod.add_bulk_set(cells, E, 0.3, rule, model)
        orc.add_bulk_set(ipc, rule, model, cells, E, 0.3)
    if sides:
        if dim == 2:
            left = np.arange(0, nc, ne[0], dtype=np.int32)
            right = np.arange(ne[0] - 1, nc, ne[0], dtype=np.int32)
            lo, ro, srule = 3, 1, mg.RULE_BAR_3
        else:
            left = np.array([c for c in range(nc) if c % ne[0] == 0], dtype=np.int32)
            right = np.array([c for c in range(nc) if c % ne[0] == ne[0] - 1], dtype=np.int32)
            lo, ro, srule = 3, 1, mg.RULE_QUAD_2x2
        zero = (0.0,) * dim
        trac = (1e-3,) + (0.0,) * (dim - 1)
        prod.add_side_set(mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, left, np.full(len(left), lo), E[left], 0.3,
                          srule, model, alpha=100.0, value=zero)
        orc.add_side_set(mg.IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE, srule, model, left, np.full(len(left), lo),
                         E[left], 0.3, 100.0, zero)
        prod.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, right, np.full(len(right), ro), E[right], 0.3, srule, model,
                          value=trac)
        orc.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, srule, model, right, np.full(len(right), ro), E[right], 0.3, 0.0,
                         trac)
    if empty_sets:
        _add_empty_sets(prod, dim, rule, model)
    return prod, orc, mesh


def rel_err(a, b):
    scale = np.max(np.abs(b))
    return 0.0 if scale == 0 else float(np.max(np.abs(a - b)) / scale)


def csr_row_rel_err(rowptr, va, vb):
    """max over CSR rows of max|va - vb| / max|vb| in the row (the absolute
    difference for a row whose oracle values are all zero)"""
    rp = np.asarray(rowptr, dtype=np.int64)
    nonempty = rp[1:] > rp[:-1]
    if not np.any(nonempty):
        return 0.0
    starts = rp[:-1][nonempty]
    d = np.maximum.reduceat(np.abs(np.asarray(va) - np.asarray(vb)), starts)
    m = np.maximum.reduceat(np.abs(np.asarray(vb)), starts)
    return float(np.max(np.where(m > 0, d / np.where(m > 0, m, 1.0), d)))
