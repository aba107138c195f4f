"""Parity at the benchmark sizes.

The small parity cases (test_parity_gpu.py, test_xfem.py) cover every kernel
variant on meshes of a few cells.  Some paths only run at size: the in-order
element counter over 262,144 elements, the 16-bit scatter slots with the
basis-union widths of a 64^3 quadratic mesh, the chunked host-buffer pipe on a
2.45 GB CSR, and the cluster kernel's work queue with a million items.  These
tests assemble the exact benchmark workloads on the GPU and compare them with
the oracle's full assembly of the same seeded inputs (the reference's
Solver_Interface::fill_matrix_and_RHS, SOL/DLA/src/cl_DLA_Solver_Interface.cpp:
317-379, restated in oracle/fem_oracle.cpp):

* headline workload: 64^3 hex8, quadratic B-spline extraction, HEX_3x3x3, E
  per element log-uniform in [1e-3, 1] (splitmix64 seed 20261205), nu 0.3;
* XFEM workload: 96^3 hex8 background, linear B-splines, 40 spheres (seed
  20261206), cut TET4 clusters, Nitsche interface, virtual-work ghost.

Bar: identical rowptr / colidx, CSR values per row and the residual within
1e-12 relative, element operators of at least 2,000 equation objects per set
(boundary cells and the largest clusters included) within 1e-12.
"""
import os

import numpy as np
import pytest

import moris_gb300 as mg
from moris_gb300 import workloads
from oracle import OracleModel

from common import RTOL, csr_row_rel_err, rel_err

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def _blocks(n, count, size, seed, must=()):
    """`count` blocks of `size` consecutive equation objects: the first and the
    last block of the set, the rest at seeded positions; plus single objects
    listed in `must`."""
    if n <= count * size:
        return [(0, n)]
    rng = np.random.default_rng(seed)
    starts = {0, n - size}
    while len(starts) < count:
        starts.add(int(rng.integers(0, n - size)))
    out = [(s, size) for s in sorted(starts)]
    out += [(int(i), 1) for i in must]
    return out


def _element_parity(prod, orc, s, u, blocks):
    """worst relative error of the element operators and residuals of set s,
    and the number of equation objects compared"""
    worst, ncmp = 0.0, 0
    for first, count in blocks:
        K, R = prod.element_matrices(s, first, count, u)
        for k in range(count):
            Ko, Ro = orc.element_matrices(s, first + k, u)
            n = len(Ro)
            assert np.array_equal(prod.element_topology(s, first + k), orc.element_topology(s, first + k))
            worst = max(worst, rel_err(K[k, :n, :n], Ko), rel_err(R[k, :n], Ro))
            ncmp += 1
    return worst, ncmp


def test_headline_64cube_assembly_matches_oracle(torch):
    m, mesh, E = workloads.elasticity_3d(64)
    nc = len(mesh["cells"])
    assert nc == 262144 and m.nnz == 306110016
    orc = OracleModel(3, mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, mesh)
    orc.add_bulk_set(mg.CELL_HEX8, mg.RULE_HEX_3x3x3, mg.MODEL_3D, np.arange(nc, dtype=np.int32), E, 0.3)
    orc.finalize()
    rp, ci = m.graph()
    rpo, cio = orc.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    del ci, cio
    u = np.random.default_rng(20261206).uniform(-1.0, 1.0, m.num_adofs)
    vo, ro = orc.assemble(u, nthreads=NTHREADS)

    # device buffers: the benchmark's call
    ut = torch.tensor(u, device="cuda")
    vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")
    m.assemble(ut, vals, rhs)
    torch.cuda.synchronize()
    m.check_status()
    assert csr_row_rel_err(rpo, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL

    # matrix-free operator against the oracle's CSR
    import scipy.sparse as sp
    x = np.random.default_rng(20261207).uniform(-1.0, 1.0, m.num_adofs)
    y = torch.empty_like(ut)
    m.apply(torch.tensor(x, device="cuda"), y)
    A = sp.csr_matrix((vo, orc.graph()[1], rpo), shape=(m.num_adofs,) * 2)
    assert rel_err(y.cpu().numpy(), A @ x) <= RTOL
    del A, vals, rhs, y

    # host buffers: the chunked pipe that copies finished row ranges back
    vh, rh = m.assemble_host(u)
    assert csr_row_rel_err(rpo, vh, vo) <= RTOL
    assert rel_err(rh, ro) <= RTOL
    del vh, vo

    # element operators: first and last 250 cells (boundary rows and faces), six
    # seeded blocks, the eight corner cells
    n = 64
    corners = [i + n * (j + n * k) for i in (0, n - 1) for j in (0, n - 1) for k in (0, n - 1)]
    worst, ncmp = _element_parity(m, orc, 0, u, _blocks(nc, 8, 250, 5, corners))
    assert ncmp >= 2000 and worst <= RTOL


def test_xfem_96cube_assembly_matches_oracle(torch):
    from test_xfem import oracle_of
    m, x, sets = workloads.xfem_spheres(96)
    orc = oracle_of(x, sets)
    rp, ci = m.graph()
    rpo, cio = orc.graph()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    del ci, cio
    u = np.random.default_rng(20261208).uniform(-1.0, 1.0, m.num_adofs)
    vo, ro = orc.assemble(u, nthreads=NTHREADS)
    ut = torch.tensor(u, device="cuda")
    vals = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.num_adofs, dtype=torch.float64, device="cuda")

    # every cluster in the one persistent graph-captured launch (the benchmark's call)
    m.assemble_batched(ut, vals, rhs)
    torch.cuda.synchronize()
    m.check_status()
    assert csr_row_rel_err(rpo, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL

    # one launch per set
    m.assemble(ut, vals, rhs)
    torch.cuda.synchronize()
    assert csr_row_rel_err(rpo, vals.cpu().numpy(), vo) <= RTOL
    assert rel_err(rhs.cpu().numpy(), ro) <= RTOL
    del vals, rhs, vo

    # element operators of every set, the 50 largest cut clusters included
    for s, (kind, a) in enumerate(sets):
        neq = m.num_eq(s)
        must = ()
        if kind == "bulk" and a.get("ig_offsets") is not None:
            sizes = np.diff(a["ig_offsets"])
            must = np.argsort(sizes)[-50:]
        elif kind == "double":
            must = np.argsort(np.diff(a["offsets"]))[-50:]
        worst, ncmp = _element_parity(m, orc, s, u, _blocks(neq, 8, 250, 11 + s, must))
        assert ncmp >= min(2000, neq) and worst <= RTOL, (s, kind, worst)
