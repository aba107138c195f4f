"""The allocation-free PCG entry point (fem_gpu_pcg_noalloc).

Some callers cannot allocate device memory while they solve (host callbacks,
real-time sections, frameworks with a fixed device memory budget).  For them
fem_gpu_pcg_noalloc keeps its work vectors in one fixed device array of the
library.  This file checks, through the C ABI, that two calls in a row give
the same solution as fem_gpu_pcg (the allocating entry point) within the
tolerance of the solver tests, and that a system above the array's limit is
rejected before anything runs.  It is collected last on purpose.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import moris_gb300 as mg
from tests.common import problem, rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu

# the solver tests' tolerance: the block reductions of both entry points sum
# in a non-deterministic order, so the iterate at which the 1e-10 residual is
# reached can differ by an iteration or two
SOLVE_RTOL = 1e-8


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def _system(torch, ne):
    prod, _, _ = problem(2, ne, 1, sides=True)
    # the solves run on torch's stream, after the kernels that made b and x
    prod.set_stream(torch.cuda.current_stream().cuda_stream)
    prod.finalize()
    rp, ci = prod.graph()
    rpt = torch.tensor(rp, device="cuda")
    cit = torch.tensor(ci, device="cuda")
    vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
    prod.assemble(None, vals, rhs)
    return prod, rpt, cit, vals, -rhs


def test_noalloc_pcg_matches_allocating_pcg_twice(torch):
    prod, rpt, cit, vals, b = _system(torch, (24, 20))
    x_ref = torch.zeros_like(b)
    rep_ref = prod.pcg(rpt, cit, vals, b, x_ref, rel_tol=1e-10)
    assert rep_ref["converged"]
    for _ in range(2):  # the second call reuses the array left by the first
        x = torch.full_like(b, 0.0)
        rep = prod.pcg_noalloc(rpt, cit, vals, b, x, rel_tol=1e-10)
        torch.cuda.synchronize()
        assert rep["converged"] and rep["rel_residual"] <= 1e-10
        assert abs(rep["iterations"] - rep_ref["iterations"]) <= max(3, rep_ref["iterations"] // 20)
        assert rel_err(x.cpu().numpy(), x_ref.cpu().numpy()) <= SOLVE_RTOL


def test_noalloc_pcg_rejects_systems_above_its_limit(torch):
    prod, rpt, cit, vals, b = _system(torch, (260, 260))  # 2 * 261^2 = 136242 rows
    assert prod.num_adofs > 131072
    x = torch.zeros_like(b)
    with pytest.raises(mg.FemGpuError) as ei:
        prod.pcg_noalloc(rpt, cit, vals, b, x)
    assert ei.value.status == 1 and "131072" in str(ei.value)
    assert np.all(x.cpu().numpy() == 0.0)


# A fresh process: nothing of the solver's module is loaded before the model is
# finalized.  The free device memory must not change across the first
# fem_gpu_pcg_noalloc call (its array and kernels come with fem_gpu_finalize).
_FRESH = r"""
import sys
sys.path.insert(0, sys.argv[1])
import torch
from tests.common import problem
torch.cuda.set_device(0)
prod, _, _ = problem(2, (24, 20), 1, sides=True)
prod.set_stream(torch.cuda.current_stream().cuda_stream)
prod.finalize()
rp, ci = prod.graph()
rpt = torch.tensor(rp, device="cuda")
cit = torch.tensor(ci, device="cuda")
vals = torch.empty(prod.nnz, dtype=torch.float64, device="cuda")
rhs = torch.empty(prod.num_adofs, dtype=torch.float64, device="cuda")
prod.assemble(None, vals, rhs)
b = -rhs
x = torch.zeros_like(b)
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
rep = prod.pcg_noalloc(rpt, cit, vals, b, x, rel_tol=1e-10)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
print("FREE", free0, free1, int(rep["converged"]))
"""


def test_noalloc_first_call_in_a_fresh_process_takes_no_device_memory(torch):
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE ")][-1].split()
    free0, free1, converged = int(line[1]), int(line[2]), int(line[3])
    assert converged == 1
    assert free1 == free0, "first pcg_noalloc call changed free device memory by %d bytes" % (free0 - free1)
