"""Train the plan selector on the GPU and save its weights.

  python mixed-mlx_gb300/train_selector.py --train 4096 --test 1024 \
      --out mixed-mlx_gb300/selector_weights.npz

Training data: SPD matrices of three spectrum families (log-uniform,
clustered, power law), n log-uniform in [--n-lo, --n-hi] (default [32, 512]),
condition log-uniform in [1e1, 1e8]; every plan is run on every matrix by msq_solve_batched and
scored by its own float-float residual at the tolerance.  The network is
trained by the library's CUDA kernels (msq_mlp_backward / msq_mlp_step).
Prints accept rate, fallback rate and solves/s on held-out seeds for the
selector and for the FP32 path alone.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--test", type=int, default=1024)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--threshold", type=float, default=0.9)
    ap.add_argument("--n-lo", type=int, default=32)
    ap.add_argument("--n-hi", type=int, default=512)
    ap.add_argument("--out", default=os.path.join(HERE, "selector_weights.npz"))
    args = ap.parse_args()
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    sel = importlib.import_module("mixed-mlx_gb300.selector")
    ctx = msq.Context(0)

    chunks_f, chunks_y, secs = [], [], np.zeros(len(sel.PLANS))
    for c, start in enumerate(range(0, args.train, 1024)):
        count = min(1024, args.train - start)
        orders, mats = sel.generate(torch, count, seed=1000 + c, n_lo=args.n_lo, n_hi=args.n_hi)
        batch, flat = sel.pack(msq, torch, orders, mats)
        chunks_f.append(sel.features(ctx, torch, batch, flat, args.tol))
        out = sel.score_plans(ctx, msq, torch, batch, flat, args.tol)
        chunks_y.append(torch.from_numpy(out.accepted).cuda())
        secs += out.seconds
        del mats, flat
    feats = torch.cat(chunks_f)
    targets = torch.cat(chunks_y)
    selector = sel.Selector(msq, torch, ctx, seed=0)
    selector.cost_order = [int(k) for k in np.argsort(secs)]
    losses = selector.fit(feats, targets, epochs=args.epochs)

    orders, mats = sel.generate(torch, args.test, seed=999_999, n_lo=args.n_lo, n_hi=args.n_hi)
    batch, flat = sel.pack(msq, torch, orders, mats)
    feats_t = sel.features(ctx, torch, batch, flat, args.tol)
    choice = selector.choose(feats_t, args.threshold)
    plans = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15) if k < 0 else sel.plan_structs(msq, [int(k)])[0]
             for k in choice]
    fp32 = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15)] * batch.count
    report = {}
    for name, p in (("selector", plans), ("fp32_path", fp32)):
        outb = torch.empty_like(flat)
        ctx.solve_batched(flat, batch, p, args.tol, out=outb)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        _, res = ctx.solve_batched(flat, batch, p, args.tol, out=outb)
        e.record()
        torch.cuda.synchronize()
        ms = s.elapsed_time(e)
        report[name] = {"ms": ms, "solves_per_s": batch.count / (ms / 1e3),
                        "accept_rate": float(np.mean([r.accepted for r in res])),
                        "fallback_rate": float(np.mean([r.fallback for r in res])),
                        "met_tolerance": float(np.mean([r.final_residual <= args.tol for r in res]))}
    report["plan_histogram"] = {str(k): int(np.sum(choice == k)) for k in range(-1, len(sel.PLANS))}
    report["train_loss_first_last"] = [losses[0], losses[-1]]
    report["plan_seconds_on_training_set"] = secs.tolist()
    np.savez(args.out, params=selector.params.cpu().numpy(), mean=selector.mean.cpu().numpy(),
             std=selector.std.cpu().numpy(), cost_order=np.array(selector.cost_order),
             tol=np.array([args.tol]), threshold=np.array([args.threshold]))
    print(json.dumps(report))


if __name__ == "__main__":
    main()
