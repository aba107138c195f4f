"""Train the learned correction for the SIMP density problem on the GPU (the
project's own convolution forward / backward kernels and Adam) and write the
weight file that bench.py and the tests load.

    python -m moris_gb300.train_lpc [--n 128] [--base multigrid] [--factor 2]
                                    [--fields 84] [--epochs 3] [--out moris_gb300/data/lpc_simp128.bin]

Training data come from the solver's own iterates on seeded density fields
(seeds BASE_SEED + 1000 + f, never the benchmark's field):
  --base multigrid  the correction is added to one multigrid V-cycle and trained
                    on the energy functional 1/2 y.A y - y.r of y = V r + c(r)
                    over the residuals of V-cycle-preconditioned CG (about 12
                    per field at 128^3) and, from the second epoch on, those of
                    the solver with the net in the loop (about 20 more per
                    field): 84 fields give about 2,300 per epoch (default);
  --base jacobi     the correction is added to D^-1 r and trained on the
                    mean-squared error against the injected coarse error of
                    2,000 residual / error pairs of Jacobi-PCG iterates.
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
    ap.add_argument("--fields", type=int, default=None, help="density fields (84 multigrid, 10 jacobi)")
    ap.add_argument("--pairs", type=int, default=2000, help="jacobi base: residual / error pairs")
    ap.add_argument("--epochs", type=int, default=None, help="passes over the data (3 multigrid, 20 jacobi)")
    ap.add_argument("--batch", type=int, default=None)
    ap.add_argument("--lr", type=float, default=None)
    ap.add_argument("--out", default=os.path.join(HERE, "data", "lpc_simp%d.bin" % 128))
    a = ap.parse_args()
    from moris_gb300 import learned
    t0 = time.time()
    log = lambda s: print(s, flush=True)  # noqa: E731
    if a.base == "multigrid":
        factor, fields, epochs = a.factor or 2, a.fields or 84, a.epochs or 3
        batch, lr = a.batch or 4, a.lr or 3e-4
        cnn, hist, npairs = learned.train_simp_mg(n=a.n, factor=factor, fields=fields, epochs=epochs, batch=batch,
                                                  lr=lr, log=log)
        summary = {"objective": "energy", "data": "residuals of V-cycle-preconditioned CG iterates; from epoch 1 "
                                                  "also those of the solver with the net in the loop",
                   "energy_ratio_per_epoch": hist, "epochs": epochs}
    else:
        factor, fields, epochs = a.factor or 4, a.fields or 10, a.epochs or 20
        batch, lr = a.batch or 16, a.lr or 1e-3
        cnn, hist, npairs = learned.train_simp(n=a.n, factor=factor, fields=fields,
                                               per_field=max(1, a.pairs // fields), epochs=epochs, batch=batch,
                                               lr=lr, log=log)
        summary = {"objective": "mse", "data": "residual / error pairs of Jacobi-PCG iterates",
                   "loss_first": hist[0], "loss_last": hist[-1], "epochs": epochs}
    meta = dict(n=a.n, base=a.base, factor=factor, fields=fields, pairs=npairs, batch=batch, lr=lr,
                train_seconds=time.time() - t0, **summary)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    learned.save_weights(a.out, cnn.weights(), cnn.n, factor, cnn.output_scale, json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
