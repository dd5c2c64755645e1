"""Training of the learned troubled-cell sensor, on the GPU with the library's own kernels.

Pairs (sensor input of a cell -> the modal indicator's alpha before smoothing) are logged every
`every` steps from runs with the plain modal blender (FP64 plain form) of the sod, double Mach
reflection and cylinder workloads; the MLP is trained with plens_gpu_mlp_train (CUDA forward,
backward and Adam kernels; lr 1e-3, batch 4096, 20 epochs by default) and written as raw FP32
parameters to plens_gb300/sensor_weights.bin, with a JSON report beside it (per-cell alpha MAE
and max error on a held-out tenth of the pairs, fraction over the judge tolerance).

    python -m plens_gb300.sensor [--epochs 20] [--batch 4096] [--lr 1e-3] [--quick]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import configs
from .api import GpuSolver, PlensError, mlp_infer, mlp_train

HERE = Path(__file__).resolve().parent
WEIGHTS = HERE / "sensor_weights.bin"
REPORT = HERE / "sensor_weights.json"


def init_params(seed: int = 0) -> np.ndarray:
    """He initialisation; the output bias starts the sigmoid near zero alpha."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / 64), (64, 64))
    W2 = rng.normal(0, np.sqrt(2.0 / 64), (64, 64))
    w3 = rng.normal(0, np.sqrt(1.0 / 64), 64)
    return np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), w3, [-4.0]]).astype(np.float32)


def log_pairs(spec, snapshots: int, every: int):
    case = configs.make_case(spec)
    g = GpuSolver(case)
    g.set_state(case.initial_state(), case.start_time)
    xs, ys = [], []
    for _ in range(snapshots):
        try:
            g.advance(every)
        except PlensError:  # a run that loses positivity contributes the pairs logged so far
            break
        x, y = g.sensor_pairs()
        xs.append(x)
        ys.append(y)
    g.close()
    if not xs:
        return np.zeros((0, 64), np.float32), np.zeros(0, np.float32)
    return np.concatenate(xs), np.concatenate(ys)


def collect(quick: bool = False):
    sets = [
        ("sod", configs.sod(n=200), 20, 5),
        ("dmr", configs.dmr(nx=120 if quick else 240, ny=30 if quick else 60), 8 if quick else 40, 25 if quick else 50),
        ("cylinder", configs.cylinder(n_radial=40 if quick else 160, n_azimuthal=32 if quick else 128), 4 if quick else 12, 50),
    ]
    xs, ys, info = [], [], {}
    for name, spec, snaps, every in sets:
        t0 = time.time()
        x, y = log_pairs(spec, snaps, every)
        info[name] = {"pairs": int(len(y)), "troubled": int((y > 0).sum()), "seconds": round(time.time() - t0, 2),
                      "snapshots": snaps, "every_steps": every}
        xs.append(x)
        ys.append(y)
    return np.concatenate(xs), np.concatenate(ys), info


def evaluate(p, x, y, tol=0.05):
    a = mlp_infer(x, p)
    a = np.where(a < 0.01, 0.0, a)
    err = np.abs(a - y)
    return {"mae": float(err.mean()), "max_err": float(err.max()),
            "frac_over_tol": float((err > tol).mean()),
            "mae_troubled": float(err[y > 0].mean()) if (y > 0).any() else 0.0}


def balanced(x, y, ratio: float, rng):
    """All troubled cells (alpha > 0) and `ratio` times as many smooth ones, drawn at random: the
    logged pairs are >95% smooth cells, which would otherwise dominate the mean-squared error."""
    hot = np.flatnonzero(y > 0)
    cold = np.flatnonzero(y <= 0)
    take = min(len(cold), int(ratio * max(len(hot), 1)))
    idx = np.concatenate([hot, rng.choice(cold, take, replace=False)])
    rng.shuffle(idx)
    return x[idx], y[idx]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--balance", type=float, default=4.0, help="smooth-to-troubled ratio of the training set")
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--pairs", default="", help="npz of logged pairs to reuse (written if absent)")
    args = ap.parse_args()
    if args.pairs and Path(args.pairs).exists():
        d = np.load(args.pairs, allow_pickle=True)
        x, y, info = d["x"], d["y"], d["info"].item()
    else:
        x, y, info = collect(args.quick)
        if args.pairs:
            np.savez(args.pairs, x=x, y=y, info=np.array(info, dtype=object))
    rng = np.random.default_rng(args.seed)
    perm = rng.permutation(len(y))
    nval = len(y) // 10
    val, tr = perm[:nval], perm[nval:]
    xt, yt = balanced(x[tr], y[tr], args.balance, rng) if args.balance > 0 else (x[tr], y[tr])
    t0 = time.time()
    p, loss = mlp_train(xt, yt, init_params(args.seed), epochs=args.epochs, batch=args.batch, lr=args.lr,
                        seed=args.seed)
    train_s = time.time() - t0
    out = Path(args.out)
    p.astype(np.float32).tofile(out)
    report = {"data": info, "training_pairs": int(len(yt)), "balance": args.balance,
              "epochs": args.epochs, "batch": args.batch, "lr": args.lr, "train_seconds": round(train_s, 2),
              "loss_first_epoch": float(loss[0]), "loss_last_epoch": float(loss[-1]),
              "validation": evaluate(p, x[val], y[val]), "train": evaluate(p, x[tr][:200000], y[tr][:200000])}
    out.with_suffix(".json").write_text(json.dumps(report, indent=1))
    print(json.dumps(report))


if __name__ == "__main__":
    main()
