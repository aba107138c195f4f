#!/usr/bin/env python
"""Benchmark of the GB300 element hot path: elements/s of full Jacobian +
residual assembly into CSR (fill_matrix_and_RHS) on the 3D linear-elasticity
workload: 64^3 hex8 cells on the unit cube, quadratic B-spline extraction
(27 bases / 81 adofs per element, dense 8x27 extraction per element),
HEX_3x3x3 Gauss points, FP64, Young's modulus per element drawn log-uniform
in [1e-3, 1] from a seeded generator, nu = 0.3.  Also times the matrix-free
Jacobian-vector product of the same operator.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica of the
workload (the element path has no cross-GPU exchange on one node: replicas
only); value = elements of all ranks / max time over ranks.

``--impl reference`` times the reference's algorithm on the host cores: the
C++ restatement in oracle/ (the reference itself needs Trilinos/PETSc/MPI
and does not build here), all host threads, a bounded sample of the same
elements per step.
"""
import argparse
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20261203 + 2  # base seed + config index of the 3D quadratic workload
NE = 64
NU_P = 0.3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ne", type=int, default=NE, help="elements per direction (64 = the benchmark workload)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--c5-cpu-iterations", type=int, default=60,
                    help="Jacobi-PCG iterations of the C5 CPU baseline sample")
    ap.add_argument("--c4-max-iter", type=int, default=6000,
                    help="Jacobi-PCG iteration cap of the config-4 state and adjoint solves")
    ap.add_argument("--no-c3", action="store_true", help="skip the XFEM (config 3) record")
    ap.add_argument("--no-c4", action="store_true", help="skip the adjoint-sensitivity (config 4) record")
    ap.add_argument("--no-c5", action="store_true", help="skip the learned-preconditioner (config 5) record")
    return ap.parse_args()


def workload(ne):
    import moris_gb300 as mg
    from moris_gb300.rng import uniform01
    mesh = mg.hmr_uniform_mesh(3, (ne, ne, ne), (1.0, 1.0, 1.0), 2)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 + 3.0 * uniform01(SEED, nc))
    return mesh, E


def workload_host(ne):
    """The same mesh and moduli built by the oracle's own generator, so that the
    host-core reference loads no product code."""
    from oracle import OracleLib
    from oracle.rng import uniform01
    mesh = OracleLib().hmr_uniform(3, (ne, ne, ne), (1.0, 1.0, 1.0), 2)
    nc = len(mesh["cells"])
    E = 10.0 ** (-3.0 + 3.0 * uniform01(SEED, nc))
    return mesh, E


def c2_config(ne, adofs, nnz):
    """The config object of the headline workload (identical in both arms)."""
    return {"workload": "3D elasticity %d^3 hex8, quadratic B-spline extraction (27 bases, 8x27 T per element), "
                        "HEX_3x3x3, E log-uniform [1e-3,1], nu 0.3" % ne,
            "elements": ne ** 3, "adofs": int(adofs), "csr_nnz": int(nnz),
            "l2": "inputs exceed L2 (CSR values %.2f GB, element data > 1 GB)" % (8 * nnz / 1e9)}


def flops_per_element(order=2, ngp=27, rect=True, density=False):
    """FP64 flop count (FMA = 2, other ops 1) of the bulk kernel's formulation
    for one interior hex8 element with B-spline extraction of `order` and
    `ngp` Gauss points.

    Column counts of the extraction T (8 nodes x (order+1)^3 bases): per
    direction the two end nodes of a quadratic element see bases 0, 1, 2 with
    (1, 2, 1) nonzeros, so column j has tc_j = product over directions (sum 64
    = 8 nonzeros per node row); linear extraction at level 0 is the identity
    (one nonzero per column and per node row).
    rect=True is the constant-Jacobian (brick) path: the Gram matrix is a
    scaled per-rule table; rect=False the per-Gauss-point path.  density=True
    is the SIMP path: E(x_q) = E0 rho(x_q)^beta per Gauss point, so the Gram
    matrix is summed per element over the points with those weights.
    Quadratic extraction is the tensor product of (1/2, 1/2, 0) / (0, 1/2, 1/2):
    K is formed as K/64, K T / 8 as (K/64) P summed axis by axis (19 additions
    per row of K and column field, 8 node values -> 27 bases), and each entry
    of T^T K T = P^T (K/64) P as a plain sum over the sparser column's nodes
    (count - 1 additions)."""
    tc1, nzrow = {1: ([1, 1], 1), 2: ([1, 2, 1], 8)}[order]
    tc = [a * b * c for c in tc1 for b in tc1 for a in tc1]
    NGP, NPD, NB, D = ngp, 24, len(tc), 3
    nsym = NPD * (NPD + 1) // 2
    if rect:
        geo = D * 8 * 2 + 2 + D + 4                           # diagonal J, detJ, 3 divisions, products
        gram = nsym * NGP * 2 + NGP * (8 * 2 + 3) if density else 0  # rho(x_q)^3, sum_q w_q E_q dN dN^T
        kiso = nsym * 4 + 3 * 36 * 8                          # c_fg (lam G0 + mu G0') (+ trace on diagonal blocks)
    else:
        geo = NGP * (D * D * 8 * 2 + 40 + D * D * 8 * 2 + 1 + NPD)  # J, inverse, g = J^-1 dN, w*, w*g
        gram = nsym * NGP * 2 + (NGP * (8 * 2 + 3) if density else 0)  # upper triangle of A
        kiso = nsym * 3 + 3 * 36 * 4
    upd = NPD * nzrow * 2                                     # u_pdof = T u_adof
    resid = NPD * NPD * 2 + D * sum(tc) * 2                   # R_p = K u, R_a = T^T R_p
    if order == 2:
        kt = NPD * D * 19                                     # K T summed axis by axis (y, x, z stages)
    else:
        kt = (D * (D + 1) // 2) * 8 * sum(tc) * 2             # K T over the T column nonzeros
    ka = 0                                                    # upper triangle of T^T (K T)
    nad = D * NB
    if order == 2:
        # count-ordered adofs: the row holds the sparser column, count - 1 additions
        srt = sorted(tc)
        for x in range(nad):
            ka += (srt[x // D] - 1) * (nad - x)
    else:
        for r in range(nad):
            ka += tc[r % NB] * (nad - r) * 2
    return geo + gram + kiso + upd + resid + kt + ka


def flops_per_element_c2(rect=True):
    """the headline workload: quadratic B-splines, HEX_3x3x3"""
    return flops_per_element(2, 27, rect)


def dense_gp_flops(ngp, npd=24, nv=6):
    """the per-Gauss-point dense count of the reference's IWG (D B then B^T (D B)
    per point), the algorithmic figure the Gram formulation replaces"""
    return ngp * (nv * nv * npd * 2 + npd * nv * npd * 2)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None
        # the raw samples (the JSON line carries their summary); BENCH_CLOCKS_DIR keeps them
        self.path = os.path.join(os.environ.get("BENCH_CLOCKS_DIR", tempfile.gettempdir()),
                                 "clocks_bench_%d.csv" % gpu_index)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return ""


def oracle_c2(mesh, E):
    """The oracle model of the headline workload and its input vector (the same
    seeded u as the GPU leg)."""
    from oracle import OracleModel
    nc = len(mesh["cells"])
    orc = OracleModel(3, 1, 0, mesh)
    orc.add_bulk_set(1, 4, 2, np.arange(nc, dtype=np.int32), E, NU_P)
    orc.finalize()
    u = np.random.default_rng(SEED + 1).uniform(-1.0, 1.0, orc.num_adofs)
    return orc, u


def cpu_reference(orc, u, nc, seconds, steps=1, warmup=0, nthreads=None):
    """Time the oracle's restated reference assembly (fill_matrix_and_RHS: every
    element's T^T K T and T^T R scattered into CSR) on host threads.  A step is
    the full assembly when it fits in `seconds`, else every k-th element with
    the smallest such k (a bounded sample of the same workload).  For a full
    assembly the last step's CSR values and residual are returned."""
    nthreads = nthreads or os.cpu_count() or 1
    out = (np.zeros(orc.nnz), np.zeros(orc.num_adofs))
    # calibrate on a sample of about 1/32 of the elements (at least 2 s of work)
    stride = 32
    while True:
        t0 = time.perf_counter()
        orc.assemble(u, nthreads=nthreads, eq_stride=stride, out=out)
        dt = time.perf_counter() - t0
        if dt > 2.0 or stride == 1:
            break
        stride = max(1, stride // 4)
    rate = ((nc + stride - 1) // stride) / dt
    stride = max(1, int(np.ceil(nc / max(1.0, rate * seconds))))
    n_el = (nc + stride - 1) // stride
    for _ in range(warmup):
        orc.assemble(u, nthreads=nthreads, eq_stride=stride, out=out)
    times = []
    for _ in range(steps):
        out[0][:] = 0.0
        out[1][:] = 0.0
        t0 = time.perf_counter()
        orc.assemble(u, nthreads=nthreads, eq_stride=stride, out=out)
        times.append(time.perf_counter() - t0)
    return dict(value=n_el / float(np.median(times)), cores=nthreads, n_el=n_el, stride=stride,
                step_seconds=float(np.median(times)), cpu=cpu_model(), adofs=orc.num_adofs, nnz=orc.nnz,
                output=out if stride == 1 else None)


def row_rel_err(rowptr, a, b):
    """max over CSR rows of max|a - b| / max|b| in the row"""
    rp = np.asarray(rowptr, dtype=np.int64)
    starts = rp[:-1][rp[1:] > rp[:-1]]
    d = np.maximum.reduceat(np.abs(a - b), starts)
    m = np.maximum.reduceat(np.abs(b), starts)
    ok = m > 0
    return float(np.max(d[ok] / m[ok])) if np.any(ok) else float(np.max(d))


def cpu_sample_text(r, nc):
    what = "all %d elements" % nc if r["stride"] == 1 else "every %d-th of the %d elements (%d)" % (
        r["stride"], nc, r["n_el"])
    return "%s per step, oracle restatement of the reference assembly, %d host threads (%s)" % (
        what, r["cores"], r["cpu"] or "cpu model unknown")


NE_C3 = 96


def c3_stats(x):
    """Work counts of the XFEM workload: integration points of uncut cells,
    cut clusters, interface facets and ghost faces."""
    s = x["sizes"]
    uncut = int(s.num_uncut[0] + s.num_uncut[1])
    cut_gp = int(4 * (s.num_ig_cells[0] + s.num_ig_cells[1]))
    return dict(uncut_cells=uncut, cut_clusters=int(s.num_cut[0] + s.num_cut[1]), cut_points=cut_gp,
                tets=int(s.num_ig_cells[0] + s.num_ig_cells[1]), interface_clusters=int(s.num_interface),
                interface_facets=int(s.num_interface_facets), ghost_faces=int(s.num_ghost[0] + s.num_ghost[1]))


def c3_flops(st):
    """FP64 operations of the cluster kernel's formulation per step (counted
    from the kernel code, FMA = 2):
      uncut cell      5,050 (Gram from the rule table, isotropic K, R = K u, K T, T^T K T)
      cut point         120 (IG->IP map, detJ, w*, monomials, 28 moment FMAs)
      cut cluster    16,750 (Gram from the moments: 300 entries x 20 FMAs; epilogue
                             as for an uncut cell)
      interface facet 22,100 (7 points x 460 geometry, facet moments P and Q,
                              normal-weighted cluster moments A1)
      interface clus. 47,000 (K from A1 and Q, R = K u, K T, T^T K T on 48 x 48)
      ghost cluster   86,000 (4 points geometry, n.D.B operators, 4 x 3 rank-1
                              updates of the 48 x 48 block, epilogue)"""
    return (5050 * st["uncut_cells"] + 120 * st["cut_points"] + 16750 * st["cut_clusters"] +
            22100 * st["interface_facets"] + 47000 * st["interface_clusters"] + 86000 * st["ghost_faces"])


def cpu_reference_c3(x, sets, seconds):
    """Oracle assembly of the XFEM workload on all host threads over a bounded
    sample (every k-th equation object of every set)."""
    from oracle import OracleModel
    import moris_gb300 as mg
    nthreads = os.cpu_count() or 1
    orc = OracleModel(3, mg.CELL_HEX8, mg.SHAPE_RECTANGULAR, x["mesh"])
    for kind, a in sets:
        if kind == "bulk":
            orc.add_bulk_set(a["ig_cell"], a["rule"], mg.MODEL_3D, a["ip_cells"], a["E"], a["nu"],
                             a.get("ig_offsets"), a.get("ig_coords"), a.get("ig_param"))
    for kind, a in sets:
        if kind == "double":
            orc.add_double_side_set(a["iwg"], a["facet_cell"], a["rule"], mg.MODEL_3D, a["leader"], a["follower"],
                                    a["offsets"], a["coords"], a["leader_param"], a["follower_param"], a["EL"],
                                    a["EF"], a["nu"], a["alpha"])
    orc.finalize()
    u = np.random.default_rng(SEED + 11).uniform(-1.0, 1.0, orc.num_adofs)
    out = (np.zeros(orc.nnz), np.zeros(orc.num_adofs))
    stride = 4096
    for _ in range(2):  # calibrate the stride to about `seconds` of work
        t0 = time.perf_counter()
        orc.assemble(u, nthreads=nthreads, eq_stride=stride, out=out)
        dt = time.perf_counter() - t0
        stride = max(1, int(stride * dt / seconds))
    t0 = time.perf_counter()
    orc.assemble(u, nthreads=nthreads, eq_stride=stride, out=out)
    dt = time.perf_counter() - t0
    # every set sampled with the same stride: the full assembly takes ~stride x dt
    return dict(value=NE_C3 ** 3 / (stride * dt), cores=nthreads, stride=stride, seconds=dt)


def run_c3(timed, stream, world, args):
    """Config 3: two-phase XFEM, 96^3 background cut by 40 spheres; every
    cluster in one persistent graph-captured launch (fem_gpu_assemble_batched)."""
    import torch
    import moris_gb300 as mg
    from moris_gb300 import workloads
    from moris_gb300 import xtk
    # the decomposition itself, host and device (identical arrays)
    phi = workloads.sphere_field(NE_C3, workloads.BASE_SEED + 3, 40, 0.03, 0.12)
    t0 = time.perf_counter()
    xh = xtk.decompose((NE_C3,) * 3, (1.0,) * 3, 1, phi)
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    xd = xtk.decompose((NE_C3,) * 3, (1.0,) * 3, 1, phi, device=True)
    t_dev = time.perf_counter() - t0
    same = all(np.array_equal(xh[k][j], xd[k][j]) for k in ("mesh", "interface", "vertices", "cut0", "cut1")
               for j in xh[k] if isinstance(xh[k][j], np.ndarray))
    del xh, xd
    t0 = time.perf_counter()
    m, x, sets = workloads.xfem_spheres(NE_C3, finalize=False, device=True)
    m.set_stream(stream.cuda_stream)
    m.finalize()
    warps, split, tuned_ms = m.autotune_batched()
    setup = time.perf_counter() - t0
    st = c3_stats(x)
    nad, nnz = m.num_adofs, m.nnz
    u = torch.tensor(np.random.default_rng(SEED + 11).uniform(-1.0, 1.0, nad), device="cuda")
    vals = torch.empty(nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(nad, dtype=torch.float64, device="cuda")
    fn = lambda: m.assemble_batched(u, vals, rhs, mg.ASYNC)
    for _ in range(3):
        fn()
    m.check_status()
    l0 = m.launch_count()
    steps = max(5, args.steps // 3)
    ms = timed(fn, steps, 0)
    launches = (m.launch_count() - l0) / steps
    m.check_status()
    n_el = NE_C3 ** 3
    fl = c3_flops(st)
    peak = fp64_peak()
    rec = {"workload": "XFEM two-phase %d^3 hex8 unit cube, linear B-splines, 40 spheres r in [0.03,0.12] "
                       "(seed %d), E 1 / 0.1, nu 0.3, uncut HEX_2x2x2, cut TET4 cells TET_4, Nitsche interface "
                       "TRI_7 alpha 100, virtual-work ghost QUAD_2x2 alpha 0.01" % (NE_C3, workloads.BASE_SEED + 3),
           "elements": n_el, "elements_per_s": n_el / (ms * 1e-3), "ms_per_step": ms, "steps": steps,
           "adofs": nad, "csr_nnz": nnz, "counts": st, "gpu_launches_per_step": launches,
           "batched_config": {"warps": warps, "split_points": split, "tuned_ms": tuned_ms},
           "roofline": {"bound": "fp64", "achieved": fl / (ms * 1e-3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                        "frac": fl / (ms * 1e-3) / 1e12 / peak, "flops_per_step": fl,
                        "peak_source": "measured in-run (FP64 FMA-chain probe)"},
           "setup_seconds": setup,
           "decomposition": {"host_seconds": t_host, "device_seconds": t_dev, "identical_arrays": bool(same)}}
    if world == 1 and not args.no_cpu:
        r = cpu_reference_c3(x, sets, min(args.cpu_seconds, 10.0))
        rec["cpu_baseline"] = {"value": r["value"], "unit": "elements/s", "cores": r["cores"], "kind": "port",
                               "sample": "every %d-th equation object of every set, oracle restatement, %d threads"
                                         % (r["stride"], r["cores"])}
        rec["speedup_vs_cpu"] = rec["elements_per_s"] / r["value"]
    del m
    torch.cuda.empty_cache()
    return rec


# analysis B-splines of the sensitivity workload: quadratic, the config-2 mesh.
# Jacobi-PCG does not reach 1e-10 on this XFEM system (first-order ghost
# penalty), so the state and adjoint solves stop at --c4-max-iter and report the
# residual they reached; the adjoint kernel and its FD check are evaluated at
# those fixed (u, lambda), which they do not depend on being converged.
C4_ORDER = 2


def secondary_record(fn):
    """One of the extra records (C3, C4, C5): a failure is reported in its place
    (type and message, with the traceback on stderr) so that the headline line
    is still printed."""
    try:
        return fn()
    except Exception as exc:
        import traceback
        traceback.print_exc(file=sys.stderr)
        return {"error": "%s: %s" % (type(exc).__name__, exc)}


def run_c4(stream, args):
    """Config 4: adjoint shape sensitivities of the strain energy with respect
    to a 32^3 cubic B-spline level set on the 64^3 quadratic-B-spline mesh."""
    import torch
    from moris_gb300 import sensitivity as S
    from moris_gb300.rng import uniform01
    t0 = time.perf_counter()
    c = S.build(n=64, ncoef=32, order=C4_ORDER, stream=stream.cuda_stream)
    m = c["model"]
    setup = time.perf_counter() - t0
    sol = S.solve_state_adjoint(m, rel_tol=1e-10, max_iter=args.c4_max_iter)
    u, lam = sol["u"], sol["lam"]
    nv = len(c["x"]["vertices"]["kind"])
    G = torch.empty(nv, dtype=torch.float64, device="cuda")
    dqdp = torch.empty(len(c["p"]), dtype=torch.float64, device="cuda")
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    m.drdp_adjoint(u, lam, G)  # warm-up
    torch.cuda.synchronize()
    e0.record(stream)
    reps = 3
    for _ in range(reps):
        m.drdp_adjoint(u, lam, G)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_adj = e0.elapsed_time(e1) / reps
    t1 = time.perf_counter()
    m.gen_dqdp(G, None, None, len(c["p"]), dqdp)  # the field stored at build
    ms_chain = (time.perf_counter() - t1) * 1e3
    dq = dqdp.cpu().numpy()
    # central FD (h = 1e-6) of Q - lambda^T R at fixed u, lambda on 50 random active coefficients
    active = np.nonzero(dq != 0.0)[0]
    pick = active[np.unique((uniform01(SEED + 40, 400) * len(active)).astype(int))[:50]]
    V = c["x"]["vertices"]
    worst = 0.0
    h = 1e-6
    for j in pick:
        f = []
        for sgn in (1.0, -1.0):
            p = c["p"].copy()
            p[j] += sgn * h
            m.update_ig_vertices(S.edge_coordinates(V, S.node_phi(c["cols"], c["vals"], p)))
            f.append(S.functional(m, u, lam))
        worst = max(worst, abs((f[0] - f[1]) / (2 * h) - dq[j]) / np.max(np.abs(dq)))
    m.update_ig_vertices(V["value"])
    n_inter = int(np.sum(V["kind"] == 3))
    rec = {"workload": "64^3 hex8 unit cube, %s B-splines, XFEM two-phase cut by a 32^3 cubic B-spline "
                       "level set (sphere field of config 3 + 0.01 x smoothed Gaussian noise, seed %d), strain energy"
                       % ({1: "linear", 2: "quadratic"}[C4_ORDER], SEED + 2),
           "adofs": m.num_adofs, "level_set_coefficients": len(c["p"]), "intersection_vertices": n_inter,
           "Q": sol["q"], "pcg_iterations": {"state": sol["pcg_u"]["iterations"],
                                             "adjoint": sol["pcg_lambda"]["iterations"]},
           "pcg_seconds": {"state": sol["pcg_u"]["seconds"], "adjoint": sol["pcg_lambda"]["seconds"]},
           "pcg_converged": {"state": sol["pcg_u"]["converged"], "adjoint": sol["pcg_lambda"]["converged"]},
           "pcg_rel_residual_reached": {"state": sol["pcg_u"]["rel_residual"],
                                        "adjoint": sol["pcg_lambda"]["rel_residual"]},
           "adjoint_kernel_ms": ms_adj, "vertices_per_s": n_inter / (ms_adj * 1e-3), "chain_ms": ms_chain,
           "fd_check": {"coefficients": int(len(pick)), "h": h, "max_abs_err_over_max_dqdp": worst},
           "setup_seconds": setup}
    if not args.no_cpu:
        # the reference's finite-difference dR/dp (forward FD of IG vertex coordinates),
        # restated on the oracle, timed on a sample of intersection vertices
        from oracle.fd_sensitivity import fd_index, oracle_model, reference_fd_dfdt
        t2 = time.perf_counter()
        orc = oracle_model(c["x"], c["sets"])
        fdix = fd_index(c["sets"], c["x"])  # cluster lookups, built once like the model
        build_s = time.perf_counter() - t2
        inter = np.nonzero(V["kind"] == 3)[0]
        sample = inter[np.unique((uniform01(SEED + 41, 40) * len(inter)).astype(int))]
        Gh = G.cpu().numpy()
        t2 = time.perf_counter()
        ref = reference_fd_dfdt(orc, c["sets"], c["x"], u.cpu().numpy(), lam.cpu().numpy(), sample, index=fdix)
        dt = time.perf_counter() - t2
        rec["cpu_baseline"] = {"value": len(sample) / dt, "unit": "vertices/s", "cores": 1, "kind": "port",
                               "sample": "%d intersection vertices, the reference's forward-FD geometric dR/dp "
                                         "restated on the oracle (model and cluster lookups built once, %.1f s, not timed)"
                                         % (len(sample), build_s),
                               "note": "a Python-driven loop of oracle residual evaluations on one core: the ratio "
                                       "compares the reference's finite-difference method with the adjoint kernel, "
                                       "not two implementations of one kernel"}
        rec["reference_fd_agreement"] = float(np.max(np.abs(ref - Gh[sample])) / np.max(np.abs(Gh[inter])))
        rec["speedup_vs_cpu"] = rec["vertices_per_s"] / rec["cpu_baseline"]["value"]
    return rec, c


LPC_WEIGHTS = os.path.join(ROOT, "moris_gb300", "data", "lpc_simp128.bin")


def run_c5(timed, stream, args):
    """Config 5: SIMP 128^3 (density contrast 1e9), wall time to 1e-8 relative
    residual (true residual, recomputed at the end) of
      - Jacobi-PCG, the plain method (fem_gpu_pcg);
      - flexible CG with one multigrid V-cycle per iteration (fem_mg_create +
        fem_gpu_fcg_mg; the hierarchy setup is inside the wall time);
      - the same with the learned correction added (weights trained on the GPU by
        moris_gb300/train_lpc.py on other density seeds), when a weight file exists.
    Each solve starts from x = 0 on device-resident CSR and right-hand side."""
    import torch
    from moris_gb300 import ACCUMULATE, learned, workloads
    from moris_gb300.multigrid import Multigrid, fcg_config, fcg_mg
    m, mesh, rho = workloads.simp_3d(128, finalize=False)
    m.set_stream(stream.cuda_stream)
    m.finalize()
    rho_d = torch.tensor(rho, device="cuda")
    t0 = time.perf_counter()
    rp, ci, vals, b = learned.assembled_system(m)
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t0
    # the per-Gauss-point assembly path (SIMP modulus at every point), CUDA events
    # on the launching stream; the CSR values (4.1 GB) exceed L2 between steps
    rhs_t = torch.empty_like(b)
    nel = len(mesh["cells"])
    ms_asm = timed(lambda: m.assemble(None, vals, rhs_t), 10, 3)
    ms_asm_kernel = timed(lambda: m.assemble(None, vals, rhs_t, ACCUMULATE), 10, 2)
    fpe = flops_per_element(1, 8, rect=True, density=True)
    peak = fp64_peak()
    asm = {"path": "per-Gauss-point E0 rho(x_q)^3 on HEX_2x2x2 (density-weighted Gram matrix per element), "
                   "linear B-splines", "elements": nel, "ms_per_assembly": ms_asm,
           "elements_per_s": nel / (ms_asm * 1e-3), "kernel_ms": ms_asm_kernel,
           "roofline": {"bound": "fp64", "achieved": fpe * nel / (ms_asm_kernel * 1e-3) / 1e12, "peak": peak,
                        "unit": "TFLOP/s", "frac": fpe * nel / (ms_asm_kernel * 1e-3) / 1e12 / peak,
                        "flops_per_element": fpe, "dense_gp_flops_per_element": dense_gp_flops(8),
                        "csr_bytes_per_assembly": 8 * m.nnz,
                        "csr_write_gbs": 8 * m.nnz / (ms_asm_kernel * 1e-3) / 1e9}}
    rhs_t = None
    m.assemble(None, vals, b)
    b.neg_()
    x_plain = torch.zeros_like(b)
    plain = m.pcg(rp, ci, vals, b, x_plain, rel_tol=1e-8, max_iter=100000)
    nx = float(torch.linalg.norm(x_plain))

    def mg_solve(cnn=None, factor=2, depth=1):
        fcg_config(depth, 200)
        try:
            torch.cuda.synchronize()
            t = time.perf_counter()
            h = Multigrid(m, rp, ci, vals)
            torch.cuda.synchronize()
            ts = time.perf_counter() - t
            x = torch.zeros_like(b)
            r = fcg_mg(m, rp, ci, vals, b, x, h, cnn=cnn, factor=factor, rho_dev=rho_d, rel_tol=1e-8, max_iter=20000)
        finally:
            fcg_config(8, 200)
        r.update(setup_seconds=ts, wall_seconds=ts + r["seconds"], fcg_depth=depth,
                 levels=[h.level_info(lv)[0] for lv in range(h.num_levels)],
                 solution_rel_diff_vs_jacobi=float(torch.linalg.norm(x - x_plain)) / nx)
        h.close()
        return r

    mgr = mg_solve()
    out = {"workload": "SIMP 128^3 hex8, linear B-splines, rho smoothed noise in [1e-3,1] (seed %d), E = rho^3, "
                       "Nitsche clamp x=0, traction x=1" % (workloads.BASE_SEED + 5),
           "adofs": m.num_adofs, "nnz": m.nnz, "assembly_seconds_with_setup": t_asm, "assembly": asm,
           "jacobi_pcg": plain,
           "fcg_multigrid": mgr, "wall_time_ratio_jacobi_over_multigrid": plain["seconds"] / mgr["wall_seconds"]}
    if not args.no_cpu:
        # CPU Jacobi-PCG on the same CSR (the oracle, all host threads), a bounded
        # sample of iterations projected to the iteration count of the full solve
        from oracle.oracle import pcg_mt
        host = [t.cpu().numpy() for t in (rp, ci, vals, b)]
        nthreads = os.cpu_count() or 1
        t = time.perf_counter()
        _, it, _, _ = pcg_mt(*host, rtol=1e-8, max_iter=args.c5_cpu_iterations, nthreads=nthreads)
        dt = time.perf_counter() - t
        per_it = dt / max(it, 1)
        projected = per_it * plain["iterations"]
        out["cpu_baseline"] = {"value": projected, "unit": "s to 1e-8 (projected)", "cores": nthreads, "kind": "port",
                               "sample": "%d Jacobi-PCG iterations of the oracle on the same CSR, %d threads, "
                                         "%.1f ms each, times the %d iterations of the full solve"
                                         % (it, nthreads, per_it * 1e3, plain["iterations"])}
        out["speedup_multigrid_vs_cpu_jacobi_pcg"] = projected / mgr["wall_seconds"]
        out["speedup_jacobi_pcg_vs_cpu_jacobi_pcg"] = projected / plain["seconds"]
    out["learned_conv"] = conv_record()
    if os.path.exists(LPC_WEIGHTS):
        cnn, factor, meta = learned.load_cnn(LPC_WEIGHTS)
        meta = json.loads(meta) if meta else {}
        if meta.get("base") == "multigrid":
            lrn = mg_solve(cnn, factor, depth=8)
        else:
            x = torch.zeros_like(b)
            lrn = learned.fcg(m, rp, ci, vals, b, x, cnn, factor, rho_d, rel_tol=1e-8, max_iter=100000)
            lrn["wall_seconds"] = lrn["seconds"]
            lrn["solution_rel_diff_vs_jacobi"] = float(torch.linalg.norm(x - x_plain)) / nx
        out.update(fcg_learned=lrn, training=meta,
                   wall_time_ratio_jacobi_over_learned=plain["seconds"] / lrn["wall_seconds"],
                   learned_gain_over_method_without_it=mgr["wall_seconds"] / lrn["wall_seconds"]
                   if meta.get("base") == "multigrid" else None)
    else:
        out["fcg_learned"] = {"unavailable": "no trained weights (python -m moris_gb300.train_lpc)"}
    return out


def bf16_peak():
    """the measured dense bf16 burst peak of this GPU type (TFLOP/s) and its source"""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "of measured (cuBLAS bf16 burst)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "of fallback (1.9 PFLOP/s bf16 burst)"


def conv_record(n=65, batches=(1, 8), reps=20):
    """Tensor-core roofline of the learned correction's convolutions on the
    n^3 coarse grid of the SIMP solve (65^3 for 128^3 elements): device time
    per call (CUDA events on the net's stream) of each 3x3x3 layer, forward
    and data gradient, and TFLOP/s of the algorithmic work 2*27*cin*cout per
    voxel (real channels, real voxels) against the measured dense bf16 peak
    (burst: each call is timed alone)."""
    from moris_gb300 import learned
    layers = [(4, 32), (32, 32), (32, 32), (32, 3)]
    names = ["fwd%d %d->%d" % (l, a, b) for l, (a, b) in enumerate(layers)] + \
            ["dgrad%d %d->%d" % (l, b, a) for l, (a, b) in enumerate(layers) if l > 0]
    work = [layers[l] for l in range(4)] + [layers[l] for l in range(1, 4)]
    peak, note = bf16_peak()
    rec = {"kernel": "conv_umma_pipe_kernel (tcgen05.mma kind::f16 M=128 N=3*cout (x taps folded into N), bf16 "
                     "operands, f32 TMEM accumulators, TMA halo blocks 16x10x3 voxels x 8 channels)", "grid": "%d^3" % n, "peak_bf16_tflops": peak,
           "peak_note": note, "batches": {}}
    cnn = learned.Cnn(n, batch_max=max(batches), seed=3)
    for nb in batches:
        ms = cnn.profile(nb, reps)
        rows = []
        for name, (a, b), t in zip(names, work, ms):
            fl = 2.0 * 27 * a * b * n ** 3 * nb
            rows.append({"layer": name, "ms": float(t), "tflops": fl / (t * 1e-3) / 1e12,
                         "frac": fl / (t * 1e-3) / 1e12 / peak})
        tot_fl = sum(2.0 * 27 * a * b * n ** 3 * nb for a, b in work)
        rec["batches"][str(nb)] = {"layers": rows, "total_ms": float(ms.sum()),
                                   "total_tflops": tot_fl / (ms.sum() * 1e-3) / 1e12}
    del cnn
    return rec


_FP64_PEAK = []


def fp64_peak():
    """the FP64 FMA-chain probe of this GPU (TFLOP/s), measured once per run"""
    if not _FP64_PEAK:
        import moris_gb300 as mg
        _FP64_PEAK.append(mg.probe_fp64_tflops())
    return _FP64_PEAK[0]


def max_over_ranks(v, world, device="cuda"):
    """The largest value over the ranks (the job's time is its slowest rank's);
    device is where the collective's tensor lives (cuda for NCCL, cpu for gloo)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, seconds):
    """Weak scaling: every rank processes the same units; the job's throughput is
    all of them over the slowest rank's time."""
    return units_per_rank * world / seconds


def c2_parity(model, orc, u, vals, rhs, oracle_out):
    """GPU assembly of the benchmark workload against the oracle's full
    assembly of the same inputs: identical rowptr / colidx, CSR values per row
    and the residual within 1e-12 relative."""
    import torch
    model.assemble(u, vals, rhs)
    torch.cuda.synchronize()
    rp_g, ci_g = model.graph()
    rp_o, ci_o = orc.graph()
    same_graph = bool(np.array_equal(rp_g, rp_o) and np.array_equal(ci_g, ci_o))
    del ci_g, ci_o
    v = vals.cpu().numpy()
    csr = row_rel_err(rp_o, v, oracle_out[0])
    del v
    rg = rhs.cpu().numpy()
    res = float(np.max(np.abs(rg - oracle_out[1])) / np.max(np.abs(oracle_out[1])))
    return {"against": "oracle full assembly, same seeded inputs", "rowptr_colidx_identical": same_graph,
            "csr_max_row_rel_err": csr, "residual_rel_err": res, "tolerance": 1e-12,
            "pass": bool(same_graph and csr <= 1e-12 and res <= 1e-12)}


def run_reference(args):
    """The reference's CPU assembly of the headline workload on the host cores:
    the oracle restatement (the reference itself needs Trilinos/PETSc/MPI and
    does not build here), inputs from the oracle's own generator, all host
    threads.  Rank 0 alone runs it."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, E = workload_host(args.ne)
    nc = len(mesh["cells"])
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    # bounded: the whole --steps/--warmup run stays within about four minutes
    per_step = max(0.5, 240.0 / (steps + warm))
    orc, u = oracle_c2(mesh, E)
    r = cpu_reference(orc, u, nc, per_step, steps=steps, warmup=warm)
    line = {
        "metric": "elements/s assembled (FP64 full Jacobian + residual into CSR)",
        "value": r["value"], "unit": "elements/s", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": r["step_seconds"] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded splitmix64, seed %d)" % SEED,
        "impl": "reference", "config": c2_config(args.ne, r["adofs"], r["nnz"]), "parallelism": "host threads",
        "cpu_baseline": {"value": r["value"], "unit": "elements/s", "cores": r["cores"], "kind": "port",
                         "sample": cpu_sample_text(r, nc), "cpu": r["cpu"]},
        "e2e": {"value": r["value"], "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist
    import moris_gb300 as mg
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    mesh, E = workload(args.ne)
    nc = len(mesh["cells"])
    model = mg.FemModel(3, mesh, mg.SHAPE_RECTANGULAR)
    model.add_bulk_set(np.arange(nc, dtype=np.int32), E, NU_P, mg.RULE_HEX_3x3x3, mg.MODEL_3D)
    stream = torch.cuda.current_stream()
    model.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    model.finalize()
    model.autotune()
    variant = model.variant(0)
    setup_s = time.perf_counter() - t0
    nad, nnz = model.num_adofs, model.nnz
    rng = np.random.default_rng(SEED + 1)
    u_host = rng.uniform(-1.0, 1.0, nad)
    u = torch.tensor(u_host, device="cuda")
    vals = torch.empty(nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(nad, dtype=torch.float64, device="cuda")

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps  # ms

    # --- headline: fill_matrix_and_RHS on device-resident inputs -------------------
    sampler = ClockSampler(local)
    for _ in range(args.warmup):
        model.assemble(u, vals, rhs)
    torch.cuda.synchronize()
    barrier()
    l0 = model.launch_count()
    sampler.start()
    ms = timed(lambda: model.assemble(u, vals, rhs), args.steps, 0)
    clocks = sampler.stop()
    launches = model.launch_count() - l0
    # kernel alone (accumulate: no zero fill) for the roofline
    ms_kernel = timed(lambda: model.assemble(u, vals, rhs, mg.ACCUMULATE), max(5, args.steps // 4), 2)
    # matrix-free Jv
    x = torch.tensor(rng.uniform(-1.0, 1.0, nad), device="cuda")
    y = torch.empty_like(x)
    ms_jv = timed(lambda: model.apply(x, y), max(5, args.steps // 2), 2)
    # check Jv against the assembled CSR operator (same seeded input)
    rowptr = torch.empty(nad + 1, dtype=torch.int32, device="cuda")
    colidx = torch.empty(nnz, dtype=torch.int32, device="cuda")
    model.graph_device(rowptr, colidx)
    model.assemble(u, vals, rhs)
    model.apply(x, y)
    Acsr = torch.sparse_csr_tensor(rowptr.long(), colidx.long(), vals, size=(nad, nad))
    y_ref = torch.mv(Acsr, x)
    jv_err = float((y - y_ref).abs().max() / y_ref.abs().max())
    del Acsr, rowptr, colidx
    # --- e2e: the same call with host buffers (pinned), copies inside the timed region -------
    e2e = None
    if not args.no_e2e:
        u_p = torch.tensor(u_host).pin_memory()
        vals_p = torch.empty(nnz, dtype=torch.float64).pin_memory()
        rhs_p = torch.empty(nad, dtype=torch.float64).pin_memory()
        fn = lambda: model.assemble_raw(u_p.data_ptr(), vals_p.data_ptr(), rhs_p.data_ptr(), mg.HOST_BUFFERS)
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        barrier()
        n_e2e = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            fn()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / n_e2e
        barrier()
        e2e = {"seconds_per_step": dt, "h2d_bytes_per_step": 8 * nad, "d2h_bytes_per_step": 8 * (nnz + nad)}

    # max over ranks
    ms = max_over_ranks(ms, world)
    ms_kernel = max_over_ranks(ms_kernel, world)
    ms_jv = max_over_ranks(ms_jv, world)
    if e2e:
        e2e["seconds_per_step"] = max_over_ranks(e2e["seconds_per_step"], world)
    value = job_throughput(nc, world, ms * 1e-3)
    if rank != 0:
        barrier()
        if world > 1:
            dist.destroy_process_group()
        return
    # roofline of the dominant kernel against the FP64 pipe, on the formulation's
    # flop count (the tensor-product path leaves so few FP64 operations that the
    # kernel is bound by shared-memory latency instead, as the limiter says)
    peak = fp64_peak()
    dmma_alone = mg.probe_dmma_tflops()
    dmma_mixed = mg.probe_dmma_tflops(mixed=True)
    fpe = flops_per_element_c2()
    achieved = fpe * nc / (ms_kernel * 1e-3) / 1e12
    traffic = None
    prof = os.path.join(ROOT, "profiles", "bulk_kernel_hex8_q2_traffic.json")
    if os.path.exists(prof) and args.ne == NE:
        try:
            traffic = json.load(open(prof)).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    line = {
        "metric": "elements/s assembled (FP64 full Jacobian + residual into CSR)",
        "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded splitmix64, seed %d)" % SEED,
        "config": c2_config(args.ne, nad, nnz), "parallelism": "replicas" if world > 1 else "1 GPU",
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "measured in-run (FP64 FMA-chain probe, fem_gpu_probe_fp64_tflops)",
                     "limiter": "latency of the shared-memory load chains of T^T K T; ncu at 32^3: FP64 pipe 52 %, "
                                "L1 72 %, L2 68 %, issue 36 %",
                     "flops_per_element": fpe, "kernel_ms": ms_kernel,
                     "fp64_tensor_probe_tflops": {"dmma": dmma_alone, "dmma_plus_dfma": dmma_mixed}},
        "kernel_variant": {"index": variant[0], "name": variant[2], "tuned_ms": variant[1]},
        "jv": {"ms_per_apply": ms_jv, "elements_per_s": nc / (ms_jv * 1e-3), "rel_err_vs_csr": jv_err},
        "setup_seconds": setup_s,
    }
    if e2e:
        line["e2e"] = {"value": job_throughput(nc, world, e2e["seconds_per_step"]), "unit": "elements/s",
                       "h2d_bytes_per_step": e2e["h2d_bytes_per_step"], "d2h_bytes_per_step": e2e["d2h_bytes_per_step"]}
    if clocks:
        line["clocks"] = clocks
    # config 1: 2D plane-strain cantilever, assembly + Jacobi-PCG to 1e-10
    if world == 1:
        from moris_gb300 import workloads
        m1, _, _ = workloads.plane_strain_cantilever(128)
        m1.set_stream(stream.cuda_stream)
        rp1 = torch.empty(m1.num_adofs + 1, dtype=torch.int32, device="cuda")
        ci1 = torch.empty(m1.nnz, dtype=torch.int32, device="cuda")
        m1.graph_device(rp1, ci1)
        v1 = torch.empty(m1.nnz, dtype=torch.float64, device="cuda")
        r1 = torch.empty(m1.num_adofs, dtype=torch.float64, device="cuda")
        ms_a1 = timed(lambda: m1.assemble(None, v1, r1), 10, 3)
        x1 = torch.zeros_like(r1)
        t0 = time.perf_counter()
        rep1 = m1.pcg(rp1, ci1, v1, -r1, x1, rel_tol=1e-10)
        line["c1_solve"] = {"workload": "2D plane strain 128^2 quad4, linear B-splines, Nitsche clamp, traction 1e-3",
                            "adofs": m1.num_adofs, "assembly_ms": ms_a1, "pcg_ms": (time.perf_counter() - t0) * 1e3,
                            "pcg_iterations": rep1["iterations"], "rel_residual": rep1["rel_residual"]}
    if world == 1 and not args.no_cpu:
        # the reference's CPU assembly on the host cores (all threads, and one core),
        # and the full oracle assembly as a parity check of the GPU's CSR at this size
        orc, u_o = oracle_c2(mesh, E)
        assert np.array_equal(u_o, u_host)
        r = cpu_reference(orc, u_o, nc, args.cpu_seconds)
        r1 = cpu_reference(orc, u_o, nc, min(args.cpu_seconds, 10.0), nthreads=1)
        line["cpu_baseline"] = {"value": r["value"], "unit": "elements/s", "cores": r["cores"], "kind": "port",
                                "sample": cpu_sample_text(r, nc), "cpu": r["cpu"],
                                "one_core": {"value": r1["value"], "cores": 1, "sample": cpu_sample_text(r1, nc)}}
        if r["output"] is not None:
            line["parity"] = c2_parity(model, orc, u, vals, rhs, r["output"])
        del orc, r, r1
    if world == 1 and not args.no_c4:
        line["c4_adjoint"] = secondary_record(lambda: run_c4(stream, args)[0])
        torch.cuda.empty_cache()
    if world == 1 and not args.no_c5:
        line["c5_simp_solve"] = secondary_record(lambda: run_c5(timed, stream, args))
        torch.cuda.empty_cache()
    # the XFEM record goes last: the end of the line is what a truncated log keeps
    if world == 1 and not args.no_c3:
        line["c3_xfem"] = secondary_record(lambda: run_c3(timed, stream, world, args))
    print(json.dumps(line), flush=True)
    barrier()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
