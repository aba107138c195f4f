"""Learned coarse-grid correction for PCG on uniform linear-B-spline hex
meshes (config 5): data generation from the solver's own iterates, GPU
training, weight files, and the flexible CG that uses the net.

Everything here drives libfem_gpu entry points (fem_cnn_*, fem_lpc_*,
fem_gpu_pcg_snapshots, fem_gpu_fcg); tensors are torch CUDA tensors used as
device buffers.
"""
import ctypes as C
import os
import struct
import time

import numpy as np

from . import FemGpuError, PcgOpts, PcgReport, _dev_ptr, lib

WEIGHT_MAGIC = b"MGBLPC01"
DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def _check(st, what):
    if st:
        raise FemGpuError(st, what)


class Cnn:
    """fem_cnn: 4-layer 3D conv net on an n^3 coarse grid."""

    def __init__(self, n, batch_max=1, seed=1):
        self.L = lib()
        self.n = n
        self.V = n ** 3
        h = C.c_void_p()
        _check(self.L.fem_cnn_create(n, batch_max, seed, C.byref(h)), "fem_cnn_create")
        self.h = h
        self.num_weights = self.L.fem_cnn_num_weights()

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fem_cnn_destroy(self.h)
            self.h = None

    def weights(self):
        w = np.zeros(self.num_weights, dtype=np.float32)
        _check(self.L.fem_cnn_get_weights(self.h, w.ctypes.data_as(C.c_void_p)), "get_weights")
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.num_weights
        _check(self.L.fem_cnn_set_weights(self.h, w.ctypes.data_as(C.c_void_p)), "set_weights")

    def forward(self, x4, nb):
        import torch
        y = torch.empty(nb * self.V * 3, dtype=torch.float32, device="cuda")
        _check(self.L.fem_cnn_forward(self.h, _dev_ptr(x4), nb, _dev_ptr(y)), "cnn_forward")
        return y

    @property
    def output_scale(self):
        return self.L.fem_cnn_get_output_scale(self.h)

    @output_scale.setter
    def output_scale(self, v):
        _check(self.L.fem_cnn_set_output_scale(self.h, float(v)), "set_output_scale")

    def profile(self, nb, reps=20):
        """Device time (ms per call) of each convolution on nb samples: the
        forward of layers 0..3, then the data gradients of layers 1..3."""
        ms = np.zeros(7, dtype=np.float64)
        _check(self.L.fem_cnn_profile(self.h, nb, reps, ms.ctypes.data_as(C.c_void_p)), "cnn_profile")
        return ms

    def loss_grad(self, x4, t3, nb):
        loss = C.c_double()
        g = np.zeros(self.num_weights, dtype=np.float32)
        _check(self.L.fem_cnn_loss_grad(self.h, _dev_ptr(x4), _dev_ptr(t3), nb, C.byref(loss),
                                        g.ctypes.data_as(C.c_void_p)), "cnn_loss_grad")
        return loss.value, g

    def train_step(self, x4, t3, nb, lr):
        loss = C.c_double()
        _check(self.L.fem_cnn_train_step(self.h, _dev_ptr(x4), _dev_ptr(t3), nb, C.c_float(lr), C.byref(loss)),
               "cnn_train_step")
        return loss.value


def save_weights(path, w, n, factor, scale, meta=""):
    """flat weight file: magic, n, factor, count, output scale, metadata, FP32 weights"""
    w = np.ascontiguousarray(w, dtype=np.float32)
    m = meta.encode()
    with open(path, "wb") as f:
        f.write(WEIGHT_MAGIC)
        f.write(struct.pack("<iiqdi", n, factor, w.size, float(scale), len(m)))
        f.write(m)
        f.write(w.tobytes())


def load_weights(path):
    with open(path, "rb") as f:
        if f.read(8) != WEIGHT_MAGIC:
            raise ValueError("not a learned-preconditioner weight file: %s" % path)
        n, factor, size, scale, lm = struct.unpack("<iiqdi", f.read(28))
        meta = f.read(lm).decode()
        w = np.frombuffer(f.read(4 * size), dtype=np.float32).copy()
    return w, n, factor, scale, meta


def load_cnn(path):
    w, n, factor, scale, meta = load_weights(path)
    cnn = Cnn(n)
    cnn.set_weights(w)
    cnn.output_scale = scale
    return cnn, factor, meta


def grid_sizes(model):
    """edge length of the cubic node grid of a 3D linear-B-spline model"""
    nu = model.num_adofs // 3
    nf = int(round(nu ** (1.0 / 3.0)))
    assert nf ** 3 == nu, "needs a cubic node grid"
    return nf


def restrict(nf, factor, r, rho):
    """coarse input [Vc][4] (FP32 device) and the scale ||R r||"""
    import torch
    nc = (nf - 1) // factor + 1
    out = torch.zeros(nc ** 3 * 4, dtype=torch.float32, device="cuda")
    s = C.c_double()
    _check(lib().fem_lpc_restrict(nf, factor, _dev_ptr(r), _dev_ptr(rho), _dev_ptr(out), C.byref(s)), "lpc_restrict")
    return out, s.value


def inject(nf, factor, e, scale):
    import torch
    nc = (nf - 1) // factor + 1
    out = torch.zeros(nc ** 3 * 3, dtype=torch.float32, device="cuda")
    _check(lib().fem_lpc_inject(nf, factor, _dev_ptr(e), scale, _dev_ptr(out)), "lpc_inject")
    return out


def assembled_system(model):
    """CSR (device) of a finalized model and b = -R(0)."""
    import torch
    rp = torch.empty(model.num_adofs + 1, dtype=torch.int32, device="cuda")
    ci = torch.empty(model.nnz, dtype=torch.int32, device="cuda")
    model.graph_device(rp, ci)
    vals = torch.empty(model.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(model.num_adofs, dtype=torch.float64, device="cuda")
    model.assemble(None, vals, rhs)
    return rp, ci, vals, -rhs


def pcg_snapshots(model, rp, ci, vals, b, every, max_snaps, rel_tol=1e-8, max_iter=200000):
    import torch
    x = torch.zeros_like(b)
    snaps = torch.empty(max_snaps * model.num_adofs, dtype=torch.float64, device="cuda")
    o = PcgOpts(rel_tol, max_iter, 1)
    r = PcgReport()
    ns = C.c_int32()
    st = lib().fem_gpu_pcg_snapshots(model.h, _dev_ptr(rp), _dev_ptr(ci), _dev_ptr(vals), _dev_ptr(b), _dev_ptr(x),
                                     C.byref(o), C.byref(r), every, _dev_ptr(snaps), max_snaps, C.byref(ns))
    model._check(st, "pcg_snapshots")
    return x, snaps.view(max_snaps, model.num_adofs)[:ns.value], r.iterations


def training_pairs(model, rho_dev, factor, every, max_snaps):
    """(coarse input, coarse target) pairs of one density field: residuals
    r_k = b - A x_k and errors e_k = x* - x_k of the plain-PCG iterates x_k."""
    import torch
    rp, ci, vals, b = assembled_system(model)
    x_star, snaps, iters = pcg_snapshots(model, rp, ci, vals, b, every, max_snaps)
    nf = grid_sizes(model)
    A = torch.sparse_csr_tensor(rp.long(), ci.long(), vals, size=(model.num_adofs,) * 2)
    ins, tgts = [], []
    for k in range(snaps.shape[0]):
        xk = snaps[k].contiguous()
        rk = (b - torch.mv(A, xk)).contiguous()
        ek = (x_star - xk).contiguous()
        cin, s = restrict(nf, factor, rk, rho_dev)
        if not s > 0:
            continue
        ins.append(cin)
        tgts.append(inject(nf, factor, ek, s))
    return ins, tgts, iters


def train(cnn, inputs, targets, epochs, batch, lr, seed=0, log=None):
    """Adam on shuffled mini-batches; returns the per-epoch mean losses."""
    import torch
    n = len(inputs)
    X = torch.stack(inputs)
    Y = torch.stack(targets)
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        perm = rng.permutation(n)
        tot, cnt = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            idx = torch.as_tensor(perm[i:i + batch], device="cuda")
            xb = X[idx].reshape(-1).contiguous()
            yb = Y[idx].reshape(-1).contiguous()
            tot += cnn.train_step(xb, yb, batch, lr)
            cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log("epoch %d loss %.4e" % (ep, hist[-1]))
    return hist


def fcg(model, rp, ci, vals, b, x, cnn=None, factor=4, rho_dev=None, rel_tol=1e-8, max_iter=200000):
    o = PcgOpts(rel_tol, max_iter, 1)
    r = PcgReport()
    fb = C.c_int32()
    st = lib().fem_gpu_fcg(model.h, _dev_ptr(rp), _dev_ptr(ci), _dev_ptr(vals), _dev_ptr(b), _dev_ptr(x),
                           cnn.h if cnn is not None else None, factor, _dev_ptr(rho_dev), C.byref(o), C.byref(r),
                           C.byref(fb))
    model._check(st, "fcg")
    return dict(iterations=r.iterations, converged=bool(r.converged), rel_residual=r.rel_residual, seconds=r.seconds,
                fallback=bool(fb.value))


def train_simp(n=128, factor=4, fields=10, per_field=200, every=None, epochs=30, batch=16, lr=2e-3, seed=1,
               log=print):
    """Train the correction on plain-PCG iterates of `fields` seeded density
    fields (seeds other than the benchmark's) of the n^3 SIMP problem."""
    import torch
    from . import workloads
    nc = n // factor + 1
    cnn = Cnn(nc, batch_max=batch, seed=seed)
    ins, tgts = [], []
    t0 = time.time()
    for f in range(fields):
        m, mesh, rho = workloads.simp_3d(n, seed=workloads.BASE_SEED + 1000 + f)
        rho_dev = torch.tensor(rho, device="cuda")
        ev = every or max(1, 2000 // per_field)
        a, b_, iters = training_pairs(m, rho_dev, factor, ev, per_field)
        ins += a
        tgts += b_
        log("field %d: %d pcg iterations, %d pairs (%.1f s)" % (f, iters, len(a), time.time() - t0))
        del m
        torch.cuda.empty_cache()
    # output scale: RMS size of the targets, so that the net learns O(1) values
    sq = sum(float((t.double() ** 2).mean()) for t in tgts) / max(1, len(tgts))
    sigma = float(np.sqrt(sq)) if sq > 0 else 1.0
    tgts = [(t / sigma).contiguous() for t in tgts]
    cnn.output_scale = sigma
    hist = train(cnn, ins, tgts, epochs, batch, lr, seed=seed, log=log)
    return cnn, hist, len(ins)


# ---------------------------------------------------------------------------
# correction on top of the multigrid V-cycle, trained on the energy functional


def spmv(rp, ci, vals, x, y):
    _check(lib().fem_gpu_spmv(x.numel(), _dev_ptr(rp), _dev_ptr(ci), _dev_ptr(vals), _dev_ptr(x), _dev_ptr(y)),
           "gpu_spmv")
    return y


def prolong_add(nf, factor, c3, scale, z):
    _check(lib().fem_lpc_prolong_add(nf, factor, _dev_ptr(c3), float(scale), _dev_ptr(z)), "lpc_prolong_add")
    return z


def prolong_transpose(nf, factor, fine, scale, out3):
    _check(lib().fem_lpc_prolong_transpose(nf, factor, _dev_ptr(fine), float(scale), _dev_ptr(out3)),
           "lpc_prolong_transpose")
    return out3


def plain_pcg_residuals(model, rp, ci, vals, b, every, max_snaps):
    """unit-norm residuals r_k = b - A x_k (FP32, device) of the plain-PCG
    iterates x_k taken every `every` iterations"""
    import torch
    _, snaps, iters = pcg_snapshots(model, rp, ci, vals, b, every, max_snaps)
    out = []
    q = torch.empty_like(b)
    for k in range(snaps.shape[0]):
        spmv(rp, ci, vals, snaps[k].contiguous(), q)
        r = b - q
        nr = float(torch.linalg.norm(r))
        if nr > 0:
            out.append((r / nr).float())
    del snaps
    return out, iters


class EnergyStep:
    """One field's system (CSR, V-cycle, density) and the energy functional of
    y = V r + P sigma s f(R r / s): E(y) = 1/2 y.A y - y.r, whose minimum over y
    is at the error e = A^-1 r (E(y) = 1/2 |e - y|_A^2 - 1/2 |e|_A^2).  CG picks
    the step length itself, so training minimises the energy after the optimal
    scaling, E_opt(y) = min_a E(a y): only the direction of y counts."""

    def __init__(self, rp, ci, vals, mg, rho, nf, factor, cnn):
        import torch
        self.rp, self.ci, self.vals, self.mg, self.rho = rp, ci, vals, mg, rho
        self.nf, self.factor, self.cnn = nf, factor, cnn
        self.nadof = 3 * nf ** 3
        self.Vc = cnn.V
        self.q = torch.empty(self.nadof, dtype=torch.float64, device="cuda")

    def energy(self, y, r):
        """(E(y), E_opt(y), dE_opt/dy) with E_opt(y) = min_a E(a y) =
        -1/2 (y.r)^2 / y.A y, the energy after the step-length choice of CG
        (scale-free in y), and dE_opt/dy = a (a A y - r), a = y.r / y.A y"""
        spmv(self.rp, self.ci, self.vals, y, self.q)
        yAy, yr = float(y @ self.q), float(y @ r)
        if not yAy > 0:
            return 0.5 * yAy - yr, 0.0, -r
        a = yr / yAy
        return 0.5 * yAy - yr, -0.5 * yr * a, a * (a * self.q - r)

    def inputs(self, rs):
        """coarse inputs and scales of a list of fine residuals"""
        import torch
        cin = torch.zeros(len(rs), self.Vc * 4, dtype=torch.float32, device="cuda")
        sc = []
        for j, r in enumerate(rs):
            c, s = restrict(self.nf, self.factor, r, self.rho)
            cin[j] = c
            sc.append(s)
        return cin, sc

    def corrected(self, z0, f, s):
        y = z0.clone()
        if s > 0:
            prolong_add(self.nf, self.factor, f, self.cnn.output_scale * s, y)
        return y


def mg_pcg_residuals(rp, ci, vals, b, mg, rel_tol=1e-8, max_iter=200, cnn=None, factor=2, rho=None):
    """unit-norm residuals (FP32, device) of the iterates of flexible CG (one
    previous direction) with M(r) = V r, or V r + P sigma s f(R r / s) when a
    net is given -- the residuals the correction meets inside that solver"""
    import torch
    nf = int(round((b.numel() // 3) ** (1.0 / 3.0)))
    x = torch.zeros_like(b)
    r = b.clone()
    z = torch.empty_like(b)
    q = torch.empty_like(b)
    bn = float(torch.linalg.norm(b))
    out = []
    p_prev = q_prev = None
    pq_prev = 1.0
    for _ in range(max_iter):
        nr = float(torch.linalg.norm(r))
        if nr <= rel_tol * bn:
            break
        out.append((r / nr).float())
        mg.apply(r, z)
        if cnn is not None:
            cin, s = restrict(nf, factor, r, rho)
            if s > 0:
                prolong_add(nf, factor, cnn.forward(cin, 1), cnn.output_scale * s, z)
        p = z.clone()
        if p_prev is not None:
            p.add_(p_prev, alpha=-float(z @ q_prev) / pq_prev)
        spmv(rp, ci, vals, p, q)
        pq = float(p @ q)
        a = float(p @ r) / pq
        x.add_(p, alpha=a)
        r.add_(q, alpha=-a)
        p_prev, q_prev, pq_prev = p, q.clone(), pq
    return out


def mg_field(n, seed, factor, cnn=None, closed_loop_iters=20):
    """one SIMP density field: (model, CSR, V-cycle, density, training
    residuals).  The residuals are those of V-cycle-preconditioned CG and, when
    a net is given, also those of the first closed_loop_iters iterations of
    the solver with the net's correction in the loop (its own feedback)."""
    import torch
    from . import workloads
    from .multigrid import Multigrid
    m, mesh, rho = workloads.simp_3d(n, seed=seed)
    rho_d = torch.tensor(rho, device="cuda")
    rp, ci, vals, b = assembled_system(m)
    mg = Multigrid(m, rp, ci, vals)
    res = mg_pcg_residuals(rp, ci, vals, b, mg)
    if cnn is not None:
        res += mg_pcg_residuals(rp, ci, vals, b, mg, max_iter=closed_loop_iters, cnn=cnn, factor=factor, rho=rho_d)
    return m, rp, ci, vals, mg, rho_d, res


def train_energy_mg(cnn, n, factor, seeds, epochs=2, batch=4, lr=3e-4, seed=1, log=None):
    """Adam on E_opt, streaming the density fields: every epoch builds each
    field's system and V-cycle, takes the residuals of its V-cycle-preconditioned
    CG iterates (from the second epoch on also those of the solver with the
    current net in the loop) and makes one shuffled pass over them.  Returns per-epoch means
    of E_opt(V r + c) / E_opt(V r) (both negative: above 1 means the correction
    lowers the energy, i.e. helps)."""
    import torch
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        ratios = []
        for fs in seeds:
            # from the second epoch on, the data include the net's own closed loop
            model, rp, ci, vals, mg, rho, res = mg_field(n, fs, factor, cnn if ep > 0 else None)
            nf = grid_sizes(model)
            st = EnergyStep(rp, ci, vals, mg, rho, nf, factor, cnn)
            z = torch.empty(st.nadof, dtype=torch.float64, device="cuda")
            perm = rng.permutation(len(res))
            for i in range(0, len(res) - batch + 1, batch):
                idx = perm[i:i + batch]
                rs = [res[j].double() for j in idx]
                cin, sc = st.inputs(rs)
                f = cnn.forward(cin.reshape(-1), batch).view(batch, -1)
                tgt = torch.empty_like(f)
                for k in range(batch):
                    z0 = mg.apply(rs[k], z).clone()
                    e0 = st.energy(z0, rs[k])[1]
                    y = st.corrected(z0, f[k].contiguous(), sc[k])
                    _, eopt, g = st.energy(y, rs[k])
                    if e0 < 0:
                        ratios.append(eopt / e0)
                    gc = torch.zeros(st.Vc * 3, dtype=torch.float32, device="cuda")
                    prolong_transpose(nf, factor, g.contiguous(), cnn.output_scale * sc[k], gc)
                    tgt[k] = gc
                # MSE target whose gradient is the energy gradient (Adam is scale-free)
                kappa = 1.0 / max(float(tgt.abs().mean()), 1e-30)
                cnn.train_step(cin.reshape(-1).contiguous(), (f - kappa * tgt).reshape(-1).contiguous(), batch, lr)
            del st, res, mg, model, rp, ci, vals
            torch.cuda.empty_cache()
        hist.append(float(np.mean(ratios)))
        count = len(ratios)
        if log:
            log("epoch %d: E_opt(V r + c) / E_opt(V r) = %.4f over %d residuals" % (ep, hist[-1], count))
    return hist, count


def calibrate_output_scale(cnn, n, factor, seed, samples=8):
    """sigma = median over residuals of the optimal step |alpha*| of the
    initial net's correction c = P s f: alpha* = -c.(A V r - r) / c.A c"""
    import torch
    model, rp, ci, vals, mg, rho, res = mg_field(n, seed, factor)
    nf = grid_sizes(model)
    st = EnergyStep(rp, ci, vals, mg, rho, nf, factor, cnn)
    cnn.output_scale = 1.0
    al = []
    for r in res[:: max(1, len(res) // samples)]:
        r = r.double()
        z0 = mg.apply(r, torch.empty(st.nadof, dtype=torch.float64, device="cuda"))
        cin, sc = st.inputs([r])
        f = cnn.forward(cin.reshape(-1), 1)
        c = torch.zeros_like(z0)
        prolong_add(nf, factor, f, sc[0], c)
        spmv(rp, ci, vals, z0, st.q)
        g0 = st.q - r
        spmv(rp, ci, vals, c, st.q)
        cAc = float(c @ st.q)
        if cAc > 0:
            al.append(abs(float(c @ g0)) / cAc)
    sigma = float(np.median(al)) if al else 1.0
    cnn.output_scale = sigma
    return sigma


def train_simp_mg(n=128, factor=2, fields=167, epochs=2, batch=4, lr=3e-4, seed=1, log=print):
    """Correction on top of the V-cycle, trained on the residuals of
    V-cycle-preconditioned CG on `fields` seeded density fields other than the
    benchmark's (about 12 residuals per field at 128^3).  Returns the net, the
    per-epoch energy ratios and the number of residuals per epoch."""
    from . import workloads
    nc = (n // factor) + 1
    cnn = Cnn(nc, batch_max=batch, seed=seed)
    seeds = [workloads.BASE_SEED + 1000 + f for f in range(fields)]
    sigma = calibrate_output_scale(cnn, n, factor, seeds[0])
    if log:
        log("output scale sigma = %.4e" % sigma)
    hist, count = train_energy_mg(cnn, n, factor, seeds, epochs=epochs, batch=batch, lr=lr, seed=seed, log=log)
    return cnn, hist, count
