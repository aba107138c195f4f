"""Train the learned coarse-grid correction for the SIMP density problem on the
GPU (the project's own convolution forward / backward kernels and Adam) and
write the weight file that bench.py and the tests load.

    python -m moris_gb300.train_lpc [--n 128] [--fields 10] [--pairs 2000]
                                    [--epochs 20] [--out moris_gb300/data/lpc_simp128.bin]

Training pairs: residual / error pairs of plain Jacobi-PCG iterates on seeded
density fields (seeds BASE_SEED + 1000 + f, never the benchmark's field).
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
    ap.add_argument("--factor", type=int, default=4)
    ap.add_argument("--fields", type=int, default=10)
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=os.path.join(HERE, "data", "lpc_simp%d.bin" % 128))
    a = ap.parse_args()
    from moris_gb300 import learned
    t0 = time.time()
    cnn, hist, npairs = learned.train_simp(n=a.n, factor=a.factor, fields=a.fields,
                                           per_field=max(1, a.pairs // a.fields), epochs=a.epochs, batch=a.batch,
                                           lr=a.lr, log=lambda s: print(s, flush=True))
    meta = json.dumps({"n": a.n, "factor": a.factor, "fields": a.fields, "pairs": npairs, "epochs": a.epochs,
                       "batch": a.batch, "lr": a.lr, "loss_first": hist[0], "loss_last": hist[-1],
                       "train_seconds": time.time() - t0})
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    learned.save_weights(a.out, cnn.weights(), cnn.n, a.factor, cnn.output_scale, meta)
    print(meta)


if __name__ == "__main__":
    main()
