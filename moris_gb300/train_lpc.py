"""Train the learned correction for the SIMP density problem on the GPU (the
project's own convolution forward / backward kernels and Adam) and write the
weight file that bench.py and the tests load.

    python -m moris_gb300.train_lpc [--n 128] [--base multigrid] [--factor 2]
                                    [--fields 8] [--pairs 2000] [--out moris_gb300/data/lpc_simp128.bin]

Training data: residuals (and, for --base jacobi, errors) of plain Jacobi-PCG
iterates on seeded density fields (seeds BASE_SEED + 1000 + f, never the
benchmark's field).
  --base multigrid  the correction is added to one multigrid V-cycle and trained
                    on the energy functional 1/2 y.A y - y.r of y = V r + c(r)
                    (default);
  --base jacobi     the correction is added to D^-1 r and trained on the
                    mean-squared error against the injected coarse error.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--base", choices=("multigrid", "jacobi"), default="multigrid")
    ap.add_argument("--factor", type=int, default=None, help="coarsening of the net's grid (2 multigrid, 4 jacobi)")
    ap.add_argument("--fields", type=int, default=8)
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--every", type=int, default=8, help="PCG iterations between residual snapshots")
    ap.add_argument("--epochs", type=int, default=20, help="jacobi base: epochs")
    ap.add_argument("--passes", type=int, default=2, help="multigrid base: passes per field and round")
    ap.add_argument("--rounds", type=int, default=2, help="multigrid base: rounds over the fields")
    ap.add_argument("--batch", type=int, default=None)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=os.path.join(HERE, "data", "lpc_simp%d.bin" % 128))
    a = ap.parse_args()
    from moris_gb300 import learned
    t0 = time.time()
    log = lambda s: print(s, flush=True)  # noqa: E731
    per_field = max(1, a.pairs // a.fields)
    if a.base == "multigrid":
        factor = a.factor or 2
        batch = a.batch or 4
        cnn, hist, npairs = learned.train_simp_mg(n=a.n, factor=factor, fields=a.fields, per_field=per_field,
                                                  every=a.every, passes=a.passes, rounds=a.rounds, batch=batch,
                                                  lr=a.lr, log=log)
        summary = {"objective": "energy", "energy_opt_first": hist[0], "energy_opt_last": hist[-1],
                   "passes": a.passes, "rounds": a.rounds}
    else:
        factor = a.factor or 4
        batch = a.batch or 16
        cnn, hist, npairs = learned.train_simp(n=a.n, factor=factor, fields=a.fields, per_field=per_field,
                                               epochs=a.epochs, batch=batch, lr=a.lr, log=log)
        summary = {"objective": "mse", "loss_first": hist[0], "loss_last": hist[-1], "epochs": a.epochs}
    meta = dict(n=a.n, base=a.base, factor=factor, fields=a.fields, pairs=npairs, batch=batch, lr=a.lr,
                train_seconds=time.time() - t0, **summary)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    learned.save_weights(a.out, cnn.weights(), cnn.n, factor, cnn.output_scale, json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
