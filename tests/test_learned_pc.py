"""Learned coarse-grid correction (config 5): the GPU network against the CPU
oracle (forward, loss, weight gradients), the oracle against finite
differences, training, and what the trained correction gains inside flexible
CG over the same solver without it."""
import numpy as np
import pytest

from oracle import cnn_oracle as co


def _inputs(nb, n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(nb, n, n, n, 4)).astype(np.float32)
    t = rng.normal(size=(nb, n, n, n, 3)).astype(np.float32)
    return x, t


def _weights(seed):
    rng = np.random.default_rng(seed)
    ws = []
    for cin, cout in co.LAYERS:
        ws.append(rng.normal(scale=np.sqrt(2.0 / (27 * cin)), size=27 * cin * cout))
    return np.concatenate(ws).astype(np.float32)


def test_oracle_gradient_matches_finite_differences():
    x, t = _inputs(1, 4, 1)
    w = _weights(2).astype(np.float64)
    loss, g, _ = co.loss_grad(w, x, t, quantized=False)
    rng = np.random.default_rng(3)
    for i in rng.choice(len(w), 12, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (co.loss_grad(wp, x, t, quantized=False)[0] - co.loss_grad(wm, x, t, quantized=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
def test_gpu_network_matches_oracle(torch):
    from moris_gb300.learned import Cnn
    nb, n = 2, 6
    x, t = _inputs(nb, n, 5)
    w = _weights(6)
    cnn = Cnn(n, batch_max=nb)
    cnn.set_weights(w)
    xd = torch.tensor(x.ravel(), device="cuda")
    td = torch.tensor(t.ravel(), device="cuda")
    y = cnn.forward(xd, nb).cpu().numpy().reshape(nb, n, n, n, 3)
    loss, g = cnn.loss_grad(xd, td, nb)
    loss_o, g_o, y_o = co.loss_grad(w, x, t, quantized=True)
    # forward: bf16 operands and activations, fp32 accumulation in another
    # order; a hidden activation can round to the neighbouring bf16 value
    # (relative 2^-8), so the bound is a bf16 ulp on the largest output and
    # almost every entry agrees far more closely
    err = np.abs(y - y_o)
    assert err.max() <= 2e-2 * np.abs(y_o).max()
    assert np.linalg.norm(y - y_o) <= 5e-3 * np.linalg.norm(y_o)
    assert abs(loss - loss_o) <= 5e-3 * loss_o
    off = 0
    for cin, cout in co.LAYERS:
        m = 27 * cin * cout
        ga, gb = g[off:off + m], g_o[off:off + m]
        assert np.linalg.norm(ga - gb) <= 2e-2 * np.linalg.norm(gb), (cin, cout)
        off += m


@pytest.mark.gpu
def test_gpu_forward_is_exact_on_exactly_representable_data(torch):
    """Weights in {-1, 0, 1}/8 and inputs in (1/16) Z keep every product and
    partial sum exact in fp32, so the tensor-core forward must equal the
    oracle; this pins the fragment layouts and the tap / channel order."""
    from moris_gb300.learned import Cnn
    nb, n = 2, 5
    rng = np.random.default_rng(11)
    x = (rng.integers(-8, 9, size=(nb, n, n, n, 4)) / 16.0).astype(np.float32)
    w = (rng.integers(-1, 2, size=_weights(0).size) / 8.0).astype(np.float32)
    cnn = Cnn(n, batch_max=nb)
    cnn.set_weights(w)
    y = cnn.forward(torch.tensor(x.ravel(), device="cuda"), nb).cpu().numpy().reshape(nb, n, n, n, 3)
    y_o, _, _ = co.forward(w, x, quantized=True)
    assert np.array_equal(y, y_o.astype(np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [17, 33, 65])
def test_tensor_core_convolution_matches_warp_mma(torch, monkeypatch, n):
    """The tcgen05 convolution (TMA halo blocks, TMEM accumulators) against
    the warp-level mma.sync kernel on grids of several 8 x 16 tiles with
    partial edge tiles and two samples: forward output and weight gradient
    (both read BF16 operands and accumulate in FP32, in different orders)."""
    from moris_gb300.learned import Cnn
    nb = 2
    x, t = _inputs(nb, n, 21)
    w = _weights(22)
    xd = torch.tensor(x.ravel(), device="cuda")
    td = torch.tensor(t.ravel(), device="cuda")
    monkeypatch.delenv("FEM_CNN_CONV_KERNEL", raising=False)
    a = Cnn(n, batch_max=nb)
    monkeypatch.setenv("FEM_CNN_CONV_KERNEL", "mma")
    b = Cnn(n, batch_max=nb)
    monkeypatch.delenv("FEM_CNN_CONV_KERNEL")
    outs = []
    for cnn in (a, b):
        cnn.set_weights(w)
        y = cnn.forward(xd, nb).cpu().numpy()
        loss, g = cnn.loss_grad(xd, td, nb)
        outs.append((y, loss, g))
    (ya, la, ga), (yb, lb, gb) = outs
    assert np.linalg.norm(ya - yb) <= 5e-3 * np.linalg.norm(yb)
    assert abs(la - lb) <= 5e-3 * lb
    assert np.linalg.norm(ga - gb) <= 2e-2 * np.linalg.norm(gb)


@pytest.mark.gpu
def test_convolution_profile_times_every_layer(torch):
    """fem_cnn_profile: a positive device time for each of the four forward
    convolutions and the three data gradients."""
    from moris_gb300.learned import Cnn
    ms = Cnn(17, batch_max=2, seed=4).profile(2, reps=2)
    assert ms.shape == (7,) and np.all(np.isfinite(ms)) and np.all(ms > 0)


@pytest.mark.gpu
def test_training_reduces_loss(torch):
    from moris_gb300.learned import Cnn, train
    n = 6
    rng = np.random.default_rng(9)
    ins, tgts = [], []
    for _ in range(16):
        x = rng.normal(size=(n, n, n, 4)).astype(np.float32)
        # a learnable target: a smoothed copy of the first three channels
        tt = 0.5 * x[..., :3] + 0.25 * np.roll(x[..., :3], 1, axis=0)
        ins.append(torch.tensor(x.ravel(), device="cuda"))
        tgts.append(torch.tensor(tt.ravel().astype(np.float32), device="cuda"))
    cnn = Cnn(n, batch_max=4, seed=3)
    hist = train(cnn, ins, tgts, epochs=40, batch=4, lr=3e-3)
    assert hist[-1] < 0.3 * hist[0]


@pytest.mark.gpu
def test_prolongation_transpose_is_the_adjoint(torch):
    """<P c, v> = <c, P^T v> for the net's grid transfer (factors 2 and 4)."""
    from moris_gb300 import learned
    nf = 17
    rng = np.random.default_rng(21)
    for factor in (2, 4):
        nc = (nf - 1) // factor + 1
        c = torch.tensor(rng.standard_normal(nc ** 3 * 3).astype(np.float32), device="cuda")
        v = torch.tensor(rng.standard_normal(3 * nf ** 3), device="cuda")
        pc = learned.prolong_add(nf, factor, c, 1.0, torch.zeros(3 * nf ** 3, dtype=torch.float64, device="cuda"))
        ptv = learned.prolong_transpose(nf, factor, v, 1.0, torch.zeros(nc ** 3 * 3, dtype=torch.float32,
                                                                          device="cuda"))
        lhs, rhs = float(pc @ v), float(c.double() @ ptv.double())
        assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + 1.0), (factor, lhs, rhs)


@pytest.mark.gpu
def test_energy_training_gradient_matches_finite_differences(torch):
    """The training signal of the correction on top of the V-cycle: dE_opt/df =
    sigma s P^T (a (a A y - r)), y = V r + P sigma s f, against central
    differences of E_opt in single entries of the net's output f."""
    from moris_gb300 import learned
    from moris_gb300.learned import Cnn, EnergyStep
    n, factor = 16, 2
    model, rp, ci, vals, mg, rho, res = learned.mg_field(n, 7, factor)
    nf = learned.grid_sizes(model)
    cnn = Cnn((nf - 1) // factor + 1)
    cnn.output_scale = 0.05
    st = EnergyStep(rp, ci, vals, mg, rho, nf, factor, cnn)
    r = res[1].double()
    z0 = mg.apply(r, torch.empty_like(r)).clone()
    cin, sc = st.inputs([r])
    rng = np.random.default_rng(3)
    f = torch.tensor(rng.standard_normal(cnn.V * 3).astype(np.float32) * 0.1, device="cuda")
    _, e0, g = st.energy(st.corrected(z0, f, sc[0]), r)
    gc = learned.prolong_transpose(nf, factor, g.contiguous(), cnn.output_scale * sc[0],
                                   torch.zeros(cnn.V * 3, dtype=torch.float32, device="cuda")).double()
    h = 1e-2
    for j in rng.choice(cnn.V * 3, 6, replace=False):
        fp, fm = f.clone(), f.clone()
        fp[j] += h
        fm[j] -= h
        ep = st.energy(st.corrected(z0, fp, sc[0]), r)[1]
        em = st.energy(st.corrected(z0, fm, sc[0]), r)[1]
        fd = (ep - em) / (2 * h)
        assert abs(fd - float(gc[j])) <= 1e-3 * float(gc.abs().max()) + 1e-6 * abs(e0), (j, fd, float(gc[j]))


@pytest.mark.gpu
def test_learned_correction_gain_is_measured(torch, record_property):
    """Trains the correction on top of the V-cycle (energy after the optimal step,
    residuals of V-cycle-preconditioned CG on other density seeds, 32^3 SIMP),
    then solves the benchmark-seed field with FCG and the V-cycle, with and
    without the net.  Both must reach 1e-8 on the true residual and agree with
    Jacobi-PCG; the iteration and time ratios are what the trained network
    gains over the method without it (recorded, not asserted: measured at
    32^3-128^3 the net does not pay off on top of the V-cycle)."""
    from moris_gb300 import learned, workloads
    from moris_gb300.multigrid import Multigrid, fcg_config, fcg_mg
    cnn, hist, _ = learned.train_simp_mg(n=32, factor=2, fields=12, epochs=2, batch=4, lr=3e-4, log=lambda s: None)
    assert all(np.isfinite(hist))
    m, mesh, rho = workloads.simp_3d(32)
    rho_d = torch.tensor(rho, device="cuda")
    rp, ci, vals, b = learned.assembled_system(m)
    xp = torch.zeros_like(b)
    plain = m.pcg(rp, ci, vals, b, xp, rel_tol=1e-8, max_iter=100000)
    h = Multigrid(m, rp, ci, vals)
    reps = {}
    fcg_config(8, 200)
    for name, net in (("multigrid", None), ("learned", cnn)):
        x = torch.zeros_like(b)
        rep = fcg_mg(m, rp, ci, vals, b, x, h, cnn=net, factor=2, rho_dev=rho_d, rel_tol=1e-8, max_iter=20000)
        assert rep["converged"] and rep["rel_residual"] <= 1e-8 * 1.0001
        assert float(torch.linalg.norm(x - xp) / torch.linalg.norm(xp)) < 1e-5
        reps[name] = rep
    record_property("energy_ratio_per_epoch", hist)
    record_property("iterations_jacobi", plain["iterations"])
    record_property("iterations_multigrid", reps["multigrid"]["iterations"])
    record_property("iterations_learned", reps["learned"]["iterations"])
    record_property("fallback", reps["learned"]["fallback"])
    record_property("time_ratio_multigrid_over_learned", reps["multigrid"]["seconds"] / reps["learned"]["seconds"])
