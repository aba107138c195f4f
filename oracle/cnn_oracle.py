"""CPU oracle of the learned-correction network (test infrastructure only).

Restates the net computed by libfem_gpu's fem_cnn_* on numpy arrays:
channels-last grids [samples, n, n, n, c], 3x3x3 taps k = dx+1 + 3(dy+1) +
9(dz+1), zero padding, weights [27][cout][cin], ReLU between layers, no
biases, mean-squared loss over 3 output channels.  `quantized=True` rounds
inputs, weights, hidden activations and back-propagated gradients to bfloat16
(round to nearest even) where the GPU stores them in bfloat16; arithmetic is
float64.
"""
import numpy as np

LAYERS = [(4, 32), (32, 32), (32, 32), (32, 3)]


def bf16(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def split_weights(w):
    out, o = [], 0
    for cin, cout in LAYERS:
        n = 27 * cin * cout
        out.append(np.asarray(w[o:o + n], dtype=np.float64).reshape(27, cout, cin))
        o += n
    return out


def shift(x, off):
    """y[v] = x[v + off] with zero padding; x [nb, n, n, n, c], off (dx, dy, dz)"""
    dx, dy, dz = off
    y = np.zeros_like(x)
    n = x.shape[1]

    def sl(d):
        return (slice(max(0, -d), n - max(0, d)), slice(max(0, d), n - max(0, -d)))

    (zo, zi), (yo, yi), (xo, xi) = sl(dz), sl(dy), sl(dx)
    y[:, zo, yo, xo, :] = x[:, zi, yi, xi, :]
    return y


def taps():
    return [(k % 3 - 1, (k // 3) % 3 - 1, k // 9 - 1) for k in range(27)]


def conv(x, W, sign=1):
    out = np.zeros(x.shape[:4] + (W.shape[1],))
    for k, (dx, dy, dz) in enumerate(taps()):
        out += shift(x, (sign * dx, sign * dy, sign * dz)) @ W[k].T
    return out


def forward(w, x4, quantized=True):
    q = bf16 if quantized else (lambda a: np.asarray(a, dtype=np.float64))
    Ws = [q(W) for W in split_weights(w)]
    acts = [q(x4)]
    for l, W in enumerate(Ws):
        z = conv(acts[-1], W)
        if l < len(Ws) - 1:
            acts.append(q(np.maximum(z, 0.0)))
        else:
            y = z
    return y, acts, Ws


def loss_grad(w, x4, t3, quantized=True):
    q = bf16 if quantized else (lambda a: np.asarray(a, dtype=np.float64))
    y, acts, Ws = forward(w, x4, quantized)
    count = y.size
    d = y - t3
    loss = float((d * d).sum() / count)
    g = q(2.0 * d / count)
    grads = [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        a = acts[l]
        dW = np.zeros_like(Ws[l])
        for k, off in enumerate(taps()):
            s = shift(a, off)
            dW[k] = np.einsum("bzyxo,bzyxi->oi", g, s)
        grads[l] = dW
        if l > 0:
            da = np.zeros_like(a)
            for k, (dx, dy, dz) in enumerate(taps()):
                da += shift(g, (-dx, -dy, -dz)) @ Ws[l][k]
            g = q(da * (a > 0))
    return loss, np.concatenate([gr.ravel() for gr in grads]), y
