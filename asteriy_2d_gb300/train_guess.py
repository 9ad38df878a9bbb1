"""Train the learned start value of the exact Riemann solver.

Records the exact-solver faces that need the iterative p* solve from the
plain FP64 solver on the axisymmetric blast (exact Godunov + minmod) over
steps 0..steps-1 (every `every`-th step), keeps the faces above the wave-
strength gate (the ones the solver starts from the network), draws a
uniform sample of `samples` of them with seed 7, trains the 6-32-32-1
network with the CUDA training kernels, and writes the parameter block
(float32, AST_MLP_NPARAM values) to --out as .npy with a JSON summary.

  python -m asteriy_2d_gb300.train_guess --grid 4096x2048 --steps 2000 \
      --every 10 --samples 4194304 --out asteriy_2d_gb300/data/guess_blast.npy
"""
import argparse
import json
import os
import time

import numpy as np

from . import abi as A
from . import learned, problems, solver


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="4096x2048")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--samples", type=int, default=1 << 22)
    ap.add_argument("--capacity", type=int, default=1 << 25)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--gate", type=float, default=0.2, help="train on faces above this wave strength")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "data", "guess_blast.npy"))
    args = ap.parse_args(argv)
    N, M = (int(v) for v in args.grid.lower().split("x"))
    cfg = problems.blast_config(N, M, flux=A.FLUX_GODUNOV)
    s0, u0 = solver.fill_blast(cfg)
    t0 = time.time()
    rec, offered = learned.record_faces(cfg, s0, u0, args.steps, every=args.every, capacity=args.capacity,
                                        min_strength=args.gate)
    recorded = len(rec)
    rec = learned.strong_records(rec, args.gate)
    t1 = time.time()
    idx = learned.sample_indices(len(rec), args.samples, seed=args.seed)
    samples = rec[idx]
    params, losses = learned.train_guess(samples, epochs=args.epochs, batch=args.batch, lr=args.lr,
                                         seed=args.seed)
    t2 = time.time()
    # held-out check on recorded faces that were not drawn for training
    mask = np.ones(len(rec), dtype=bool)
    mask[idx] = False
    pool = rec[mask] if mask.any() else samples
    hold = learned.sample_records(pool, 1 << 16, seed=args.seed + 1)
    pred = solver.mlp_forward(params, hold[:, :6])
    rmse = float(np.sqrt(np.mean((pred - hold[:, 6]) ** 2)))
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.save(args.out, params)
    summary = {"grid": [N, M], "steps": args.steps, "every": args.every, "faces_offered": int(offered),
               "faces_recorded": int(recorded), "faces_above_gate": int(len(rec)), "gate": args.gate,
               "samples": int(len(samples)), "epochs": args.epochs,
               "batch": args.batch, "lr": args.lr, "seed": args.seed, "loss_first": float(losses[0]),
               "loss_last": float(losses[-1]), "rmse_log_p": rmse, "record_s": t1 - t0, "train_s": t2 - t1}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(summary, f, indent=1)
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
