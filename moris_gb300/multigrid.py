"""Geometric multigrid preconditioner (fem_mg_*) and the flexible CG that uses
it (fem_gpu_fcg_mg) for 3D linear-B-spline models on a cubic node grid.

The hierarchy is the reference's PCMG preconditioner (Preconditioner_PETSc::
build_multigrid_preconditioner, SOL/DLA/src/cl_DLA_Preconditioner_PETSc.cpp:
77-345) built on the device: Galerkin coarse operators through the linear
B-spline two-scale relation, Chebyshev-Jacobi smoothing, dense coarsest solve.
"""
import ctypes as C

import numpy as np

from . import FemGpuError, PcgOpts, PcgReport, _dev_ptr, lib
from ._lib import MgOpts


def _check(st, what):
    if st:
        raise FemGpuError(st, what)


def fcg_config(depth=8, window=200):
    """truncation depth of FCG(m) and the stagnation window before the fallback"""
    _check(lib().fem_gpu_fcg_config(depth, window), "fcg_config")


class Multigrid:
    def __init__(self, model, rp, ci, vals, coarse_max=5, degree=2, lo_frac=0.1, hi_frac=1.1, power_iters=12,
                 fp32_levels=8):
        self.L = lib()
        o = MgOpts(coarse_max, degree, lo_frac, hi_frac, power_iters, fp32_levels)
        h = C.c_void_p()
        model._check(self.L.fem_mg_create(model.h, _dev_ptr(rp), _dev_ptr(ci), _dev_ptr(vals), C.byref(o),
                                          C.byref(h)), "fem_mg_create")
        self.h = h
        self.num_adofs = model.num_adofs

    def close(self):
        if getattr(self, "h", None):
            self.L.fem_mg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def num_levels(self):
        return self.L.fem_mg_num_levels(self.h)

    @property
    def setup_seconds(self):
        return self.L.fem_mg_setup_seconds(self.h)

    def level_info(self, level):
        n = C.c_int32()
        lam = C.c_double()
        _check(self.L.fem_mg_level_info(self.h, level, C.byref(n), C.byref(lam)), "mg_level_info")
        return n.value, lam.value

    def stencil(self, level):
        n, _ = self.level_info(level)
        out = np.zeros((27, 3, 3, n ** 3))
        _check(self.L.fem_mg_get_stencil(self.h, level, out.ctypes.data_as(C.c_void_p)), "mg_get_stencil")
        return out

    def apply(self, r, z):
        _check(self.L.fem_mg_apply(self.h, _dev_ptr(r), _dev_ptr(z)), "mg_apply")
        return z


def fcg_mg(model, rp, ci, vals, b, x, mg, cnn=None, factor=4, rho_dev=None, rel_tol=1e-8, max_iter=200000):
    o = PcgOpts(rel_tol, max_iter, 1)
    r = PcgReport()
    fb = C.c_int32()
    st = lib().fem_gpu_fcg_mg(model.h, _dev_ptr(rp), _dev_ptr(ci), _dev_ptr(vals), _dev_ptr(b), _dev_ptr(x), mg.h,
                              cnn.h if cnn is not None else None, factor, _dev_ptr(rho_dev), C.byref(o),
                              C.byref(r), C.byref(fb))
    model._check(st, "fcg_mg")
    return dict(iterations=r.iterations, converged=bool(r.converged), rel_residual=r.rel_residual, seconds=r.seconds,
                fallback=fb.value == 1, net_switched_off=fb.value == 2)


def main():
    """python -m moris_gb300.multigrid [--n 128] [--repeat 1]: the SIMP density
    problem (n^3 hex8, linear B-splines, E = rho^3 with rho in [1e-3, 1]) solved
    to 1e-8 with FCG and the V-cycle; prints one JSON line per repeat."""
    import argparse
    import json
    import time

    import torch

    from . import learned, workloads
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--fp32-levels", type=int, default=8)
    a = ap.parse_args()
    m, mesh, rho = workloads.simp_3d(a.n)
    rp, ci, vals, b = learned.assembled_system(m)
    fcg_config(1, 200)
    for _ in range(a.repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = Multigrid(m, rp, ci, vals, fp32_levels=a.fp32_levels)
        torch.cuda.synchronize()
        ts = time.perf_counter() - t0
        x = torch.zeros_like(b)
        r = fcg_mg(m, rp, ci, vals, b, x, h, rel_tol=1e-8, max_iter=20000)
        r.update(n=a.n, setup_seconds=ts, levels=[h.level_info(lv)[0] for lv in range(h.num_levels)])
        print(json.dumps(r), flush=True)
        h.close()


if __name__ == "__main__":
    main()
