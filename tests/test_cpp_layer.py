"""The reference-side integration run end to end: tests/cpp/solver_interface_main
.cpp builds a model through the C++ layer, calls fill_matrix_and_RHS through a
moris::Solver_Interface pointer into MORIS-shaped Dist_Matrix / Dist_Vector
objects (sum_into_values per CSR row, sum_into_global_values), then
get_element_topology and get_equation_object_operator_and_rhs for every
equation object; the results are compared with the oracle.

Model: 2D plane strain on a 5 x 4 mesh with quadratic B-spline extraction,
Young's modulus per element, thickness 0.5, an x-roller on the left edge
(unsymmetric Nitsche with a Select matrix) and a traction on the right edge,
automatic integration rules.
"""
import os
import subprocess

import numpy as np
import pytest

import moris_gb300 as mg
from oracle import OracleLib, OracleModel

from common import RTOL, csr_row_rel_err, rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NE = (5, 4)


def _oracle():
    mesh = OracleLib().hmr_uniform(2, NE, (1.0, 1.0), 2)
    nc = len(mesh["cells"])
    E = 10.0 ** (-2.0 * mg.rng.uniform01(31, nc))
    cells = np.arange(nc, dtype=np.int32)
    left = cells[cells % NE[0] == 0]
    right = cells[cells % NE[0] == NE[0] - 1]
    o = OracleModel(2, mg.CELL_QUAD4, mg.SHAPE_RECTANGULAR, mesh)
    o.add_bulk_set(mg.CELL_QUAD4, mg.RULE_AUTO, mg.MODEL_PLANE_STRAIN, cells, E, 0.3)
    o.set_bulk_thickness(0, 0.5)
    o.add_side_set(mg.IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE, mg.RULE_AUTO, mg.MODEL_PLANE_STRAIN, left,
                   np.full(len(left), 3), E[left], 0.3, 100.0, (0.0, 0.0))
    o.set_side_options(0, 0.5, [[1.0, 0.0], [0.0, 0.0]])
    o.add_side_set(mg.IWG_STRUC_LINEAR_NEUMANN, mg.RULE_AUTO, mg.MODEL_PLANE_STRAIN, right, np.full(len(right), 1),
                   E[right], 0.3, 0.0, (1e-3, -2e-3))
    o.set_side_options(1, 0.5, None)
    o.finalize()
    return o, mesh, E, left, right


@pytest.mark.gpu
def test_integration_program_matches_oracle(tmp_path):
    o, mesh, E, left, right = _oracle()
    u = np.random.default_rng(9).uniform(-1.0, 1.0, o.num_adofs)
    inp, out, exe = tmp_path / "in.bin", tmp_path / "out.bin", tmp_path / "si"
    with open(inp, "wb") as f:
        np.array([2, len(mesh["coords"]), len(mesh["cells"]), mesh["num_bases"], len(mesh["t_bases"]), len(left),
                  len(right)], dtype=np.int32).tofile(f)
        mesh["coords"].astype(np.float64).tofile(f)
        mesh["cells"].astype(np.int32).tofile(f)
        mesh["t_off"].astype(np.int64).tofile(f)
        mesh["t_bases"].astype(np.int32).tofile(f)
        mesh["t_w"].astype(np.float64).tofile(f)
        E.astype(np.float64).tofile(f)
        left.astype(np.int32).tofile(f)
        right.astype(np.int32).tofile(f)
        np.array([o.num_adofs], dtype=np.int64).tofile(f)
        u.tofile(f)
    lib_dir = os.path.join(ROOT, "moris_gb300", "_build")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "tests", "cpp"), os.path.join(ROOT, "tests", "cpp", "solver_interface_main.cpp"),
                        "-L", lib_dir, "-lfem_gpu", "-Wl,-rpath," + lib_dir, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    data = np.fromfile(out, dtype=np.uint8)
    pos = 0

    def take(dtype, n):
        nonlocal pos
        a = data[pos:pos + np.dtype(dtype).itemsize * n].view(dtype)
        pos += np.dtype(dtype).itemsize * n
        return a

    nad, nent = take(np.int64, 2)
    assert nad == o.num_adofs
    rec = np.zeros(nent, dtype=[("r", np.int32), ("c", np.int32), ("v", np.float64)])
    raw = take(np.uint8, nent * 16).reshape(nent, 16)
    rec["r"] = raw[:, 0:4].copy().view(np.int32).ravel()
    rec["c"] = raw[:, 4:8].copy().view(np.int32).ravel()
    rec["v"] = raw[:, 8:16].copy().view(np.float64).ravel()
    rhs = take(np.float64, nad)
    # the matrix written into the distributed object == the oracle's assembly
    rp, ci = o.graph()
    vo, ro = o.assemble(u)
    rows = np.repeat(np.arange(nad), np.diff(rp))
    assert nent == len(ci)
    order = np.lexsort((rec["c"], rec["r"]))
    assert np.array_equal(rec["r"][order], rows) and np.array_equal(rec["c"][order], ci)
    assert csr_row_rel_err(rp, rec["v"][order], vo) <= RTOL
    assert rel_err(rhs, ro) <= RTOL
    # per-object operators in the element topology's order
    for s in range(3):
        neq = take(np.int64, 1)[0]
        assert neq == o.num_eq(s)
        for e in range(neq):
            n = take(np.int32, 1)[0]
            ids = take(np.int32, n)
            K = take(np.float64, n * n).reshape(n, n).T
            R = take(np.float64, n)
            assert np.array_equal(ids, o.element_topology(s, e))
            Ko, Ro = o.element_matrices(s, e, u)
            assert rel_err(K, Ko) <= RTOL and rel_err(R, Ro) <= RTOL
    assert pos == len(data)
