"""Offline training of the learned leaf priority (the MLP behind mdas_learned_*).

For each training scene (seeds 1-32 by default) the plain sampler renders the
workload; at every pass a random subset of the leaves gives one batch of
training rows: the leaves' features (mdas_leaf_features) and their true
reconstruction error (mdas_leaf_true_errors: the leaf's mean sample value
against the integrand's mean over the leaf's box from 64 points).  The MLP is
trained on log2(true error / plain error) / 32 (the correction the learned
priority applies to the plain error) with the library's own tensor-core
gradient kernel and Adam kernel, and the weights are written as raw float32
(MDAS_MLP_PARAMS values) beside a JSON record of how they were made.

    python -m pmdas_gb300.train_priority --workload mbdof1080 \\
        --out pmdas_gb300/weights/priority_mbdof1080.f32

Needs a GPU (the sampler and the kernels are the library's).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import _native as N
from .kdgrid import KDGrid, Scene, mlp_adam, mlp_forward, mlp_gradients
from .workloads import WORKLOADS

SCALE = 32.0  # priorities, network outputs and targets are log2 quantities / 32


def collect(wl, seed: int, rows_per_pass: int, samples: int, rng):
    """Features and targets of random leaves at every pass of one plain render."""
    import torch
    g = KDGrid(wl.dim, wl.maxSamples, wl.candidatesNum, wl.bitsPerDim, wl.extraImgBits, wl.alpha, wl.scaleX,
               wl.scaleY)
    sc = Scene(wl.scene_kind, seed, wl.scene_count, wl.scaleX, wl.scaleY, wl.width, wl.height)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    xs, ys = [], []
    while True:
        n, _, l, _ = g._counts()
        if n >= wl.budget or n + l > wl.maxSamples:
            break
        g.ComputeErrors()
        feats = g.LeafFeatures()
        k = min(rows_per_pass, l)
        idx = torch.from_numpy(rng.choice(l, size=k, replace=False).astype(np.int32)).cuda()
        true = g.LeafTrueErrors(sc, samples=samples, seed=int(rng.integers(1 << 62)), leaves=idx)
        x = feats[idx.long()].clone()
        # target: log2(true error / plain error) / 32, within [-8, 8] bits (feature 10 = log2(plain error) / 32)
        y = (torch.log2(true + 1e-12) / SCALE - x[:, 10]).clamp(-8.0 / SCALE, 8.0 / SCALE)
        xs.append(x)
        ys.append(y)
        g.AdaptiveSampling()
        n2, nn, _, _ = g._counts()
        sc.evaluate(g, n2 - nn, nn)
    g.close()
    sc.close()
    return torch.cat(xs), torch.cat(ys)


def init_params(seed: int) -> np.ndarray:
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for the weights and biases of each layer."""
    rng = np.random.default_rng(seed)
    H, IN = 64, 16
    p = np.zeros(N.MLP_PARAMS, np.float32)
    off = 0
    for n, fan in ((H * IN, IN), (H, IN), (H * H, H), (H, H), (H, H), (1, H)):
        p[off:off + n] = rng.uniform(-1, 1, n) / math.sqrt(fan)
        off += n
    return p


def train(x, y, steps: int, batch: int, lr: float, seed: int, log_every: int = 200):
    import torch
    gen = torch.Generator(device="cuda").manual_seed(seed)
    p = torch.from_numpy(init_params(seed)).cuda()
    m1 = torch.zeros_like(p)
    m2 = torch.zeros_like(p)
    losses = []
    for step in range(1, steps + 1):
        idx = torch.randint(0, x.shape[0], (batch,), device="cuda", generator=gen)
        g, loss = mlp_gradients(p, x[idx].contiguous(), y[idx].contiguous())
        mlp_adam(p, m1, m2, g, step, lr * 0.5 * (1 + math.cos(math.pi * step / steps)))  # cosine schedule
        if step % log_every == 0 or step == steps:
            losses.append((step, loss))
    return p, losses


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="mbdof1080")
    ap.add_argument("--seeds", default="1-32")
    ap.add_argument("--eval-seed", type=int, default=100)
    ap.add_argument("--rows-per-pass", type=int, default=16384)
    ap.add_argument("--samples", type=int, default=64)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    import torch
    a, b = (int(v) for v in args.seeds.split("-"))
    wl = WORKLOADS[args.workload]
    rng = np.random.default_rng(12345)
    t0 = time.time()
    xs, ys = [], []
    for s in range(a, b + 1):
        x, y = collect(wl, s, args.rows_per_pass, args.samples, rng)
        xs.append(x)
        ys.append(y)
    x, y = torch.cat(xs), torch.cat(ys)
    ex, ey = collect(wl, args.eval_seed, args.rows_per_pass, args.samples, rng)
    t1 = time.time()
    p, losses = train(x, y, args.steps, args.batch, args.lr, seed=1)
    t2 = time.time()
    with torch.no_grad():
        eval_mse = float(((mlp_forward(p, ex) - ey) ** 2).mean())
        base_mse = float((ey ** 2).mean())  # no correction: the plain error as the predictor
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    p.cpu().numpy().astype("<f4").tofile(args.out)
    rec = {"workload": args.workload, "train_seeds": args.seeds, "eval_seed": args.eval_seed,
           "rows": int(x.shape[0]), "rows_per_pass": args.rows_per_pass, "samples_per_leaf": args.samples,
           "steps": args.steps, "batch": args.batch, "lr": args.lr, "schedule": "cosine",
           "target": "log2(true error / plain error) / 32, clamped to 8 bits", "train_loss": losses[-1][1],
           "eval_mse": eval_mse, "eval_mse_plain_error_as_predictor": base_mse,
           "collect_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1)}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec))


if __name__ == "__main__":
    main()
