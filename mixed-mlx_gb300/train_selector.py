"""Train the plan selector on the GPU and save its weights.

  python mixed-mlx_gb300/train_selector.py --out mixed-mlx_gb300/selector_weights.npz

Training data: SPD matrices of three spectrum families (log-uniform,
clustered, power law i^-2), n log-uniform in [--n-lo, --n-hi] (default
[64, 2048]), condition log-uniform in [1e1, 1e8], plus --wishart Wishart
covariances (n log-uniform in [16, 512], the batched workload's family);
every plan is run by msq_solve_batched and scored by its own float-float
residual at the tolerance.  Every plan runs on the first --probe matrices
(the Wishart set first); a plan that met the tolerance on none of them is
not run on the rest and scores 0 there (at 1e-5 the plans without a
correction, and FP8 / MXFP4 with one, never do: the quantization error of
X0 is above the tolerance), and the plan costs come from the probe, where
every plan ran on the same matrices.  Orders up to 1024 are solved in
batches of 1024; each order above 1024 takes the whole GPU (grid
eigensolver), so of those only the first --max-large drawn are run (the
count is recorded).  The network is trained by
the library's CUDA kernels (msq_mlp_backward / msq_mlp_step).  Then held-out
seeds (--test, drawn the same way) are solved with the selected plans and
with the FP32 path alone; accept rate, fallback rate, met-tolerance rate and
solves/s are printed as JSON and stored with the weights.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

BATCHED_MAX = 1024  # orders the batched eigensolver takes


def draw_orders(count: int, seed: int, n_lo: int, n_hi: int, max_large: int):
    """Orders log-uniform on [n_lo, n_hi]; the ones above BATCHED_MAX beyond
    the first max_large are dropped.  Returns (small, large, drawn_large)."""
    rng = np.random.default_rng(seed)
    n = np.floor(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi + 1), count))).astype(np.int32)
    n = np.clip(n, n_lo, n_hi)
    small, large = n[n <= BATCHED_MAX], n[n > BATCHED_MAX]
    return small, large[:max_large], int(large.size)


def chunks(orders, size: int):
    for s in range(0, len(orders), size):
        yield s, orders[s:s + size]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=200_000)
    ap.add_argument("--probe", type=int, default=8192,
                    help="matrices on which every plan runs (plans that never meet the "
                         "tolerance there are not run on the rest)")
    ap.add_argument("--test", type=int, default=20480)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--threshold", type=float, default=0.9)
    ap.add_argument("--n-lo", type=int, default=64)
    ap.add_argument("--n-hi", type=int, default=2048)
    ap.add_argument("--max-large", type=int, default=512,
                    help="orders above 1024 run per set (each takes the whole GPU)")
    ap.add_argument("--wishart", type=int, default=4096,
                    help="Wishart covariances (n in [16, 512]) added to the training set")
    ap.add_argument("--out", default=os.path.join(HERE, "selector_weights.npz"))
    args = ap.parse_args()
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    sel = importlib.import_module("mixed-mlx_gb300.selector")
    ctx = msq.Context(0)
    t_start = time.time()

    small, large, drawn_large = draw_orders(args.train, 1000, args.n_lo, args.n_hi, args.max_large)
    chunks_f, chunks_y = [], []
    secs = np.zeros(len(sel.PLANS))        # every plan, probe matrices only
    secs_all = np.zeros(len(sel.PLANS))    # whatever ran
    probe_acc = np.zeros(len(sel.PLANS))
    state = {"scored": 0, "run": list(range(len(sel.PLANS)))}

    def score(orders, mats):
        batch, flat = sel.pack(msq, torch, orders, mats)
        chunks_f.append(sel.features(ctx, torch, batch, flat, args.tol))
        probing = state["scored"] < args.probe
        out = sel.score_plans(ctx, msq, torch, batch, flat, args.tol,
                              None if probing else state["run"])
        chunks_y.append(torch.from_numpy(out.accepted).cuda())
        secs_all[:] += out.seconds
        if probing:
            secs[:] += out.seconds
            probe_acc[:] += out.accepted.sum(0)
        state["scored"] += batch.count
        if probing and state["scored"] >= args.probe:
            state["run"] = [k for k in range(len(sel.PLANS)) if probe_acc[k] > 0]
        del flat

    for c, start in enumerate(range(0, args.wishart, 1024)):
        orders, mats = sel.generate_wishart(torch, min(1024, args.wishart - start), seed=30_000 + c)
        score(orders, mats)
        del mats
    for part, size in ((small, 1024), (large, 16)):
        for c, (start, orders) in enumerate(chunks(part, size)):
            if len(orders) == 0:
                continue
            seed = 10_000 * (1 + (part is large)) + c
            _, mats = sel.generate(torch, len(orders), seed=seed, orders=orders)
            score(orders, mats)
            del mats
    feats = torch.cat(chunks_f)
    targets = torch.cat(chunks_y)
    selector = sel.Selector(msq, torch, ctx, seed=0)
    selector.cost_order = sel.cost_order(secs)
    losses = selector.fit(feats, targets, epochs=args.epochs)
    t_train = time.time() - t_start
    save(args, selector, {"train": {"matrices": int(small.size + large.size), "drawn": args.train,
                                    "seconds": t_train, "plan_seconds_probe": secs.tolist()}})

    # held-out seeds: selected plans against the FP32 path alone
    small_t, large_t, drawn_large_t = draw_orders(args.test, 999_999, args.n_lo, args.n_hi,
                                                  args.max_large // 2)
    totals = {name: {"ms": 0.0, "met": 0, "accepted": 0, "fallback": 0, "count": 0}
              for name in ("selector", "fp32_path")}
    hist = np.zeros(len(sel.PLANS) + 1, dtype=np.int64)
    for part, size in ((small_t, 1024), (large_t, 16)):
        for c, (start, orders) in enumerate(chunks(part, size)):
            if len(orders) == 0:
                continue
            seed = 500_000 + 1000 * (part is large_t) + c
            _, mats = sel.generate(torch, len(orders), seed=seed, orders=orders)
            batch, flat = sel.pack(msq, torch, orders, mats)
            del mats
            choice = selector.choose(sel.features(ctx, torch, batch, flat, args.tol),
                                     args.threshold)
            hist += np.bincount(choice + 1, minlength=len(sel.PLANS) + 1)
            plans = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15) if k < 0 else
                     sel.plan_structs(msq, [int(k)])[0] for k in choice]
            fp32 = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15)] * batch.count
            for name, p in (("selector", plans), ("fp32_path", fp32)):
                outb = torch.empty_like(flat)
                for _ in range(2):  # plan caches, then the solve's graph capture
                    ctx.solve_batched(flat, batch, p, args.tol, out=outb)
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record()
                _, res = ctx.solve_batched(flat, batch, p, args.tol, out=outb)
                e.record()
                torch.cuda.synchronize()
                t = totals[name]
                t["ms"] += s.elapsed_time(e)
                t["met"] += sum(r.final_residual <= args.tol for r in res)
                t["accepted"] += sum(r.accepted for r in res)
                t["fallback"] += sum(r.fallback for r in res)
                t["count"] += batch.count
            del flat
    report = {"train": {"matrices": int(small.size + large.size), "drawn": args.train,
                        "wishart": args.wishart, "wishart_n": [16, 512],
                        "above_1024_drawn": drawn_large, "above_1024_run": int(large.size),
                        "n": [args.n_lo, args.n_hi], "cond": [1e1, 1e8],
                        "families": ["log-uniform", "clustered", "power law i^-2"],
                        "loss_first_last": [losses[0], losses[-1]], "epochs": args.epochs,
                        "probe": int(min(state["scored"], max(args.probe, 1))),
                        "probe_accept_rate": (probe_acc / max(1, min(state["scored"], args.probe))).tolist(),
                        "plans_run_after_probe": state["run"],
                        "plan_seconds_probe": secs.tolist(),
                        "plan_seconds_all": secs_all.tolist(), "seconds": t_train},
              "held_out": {"matrices": int(small_t.size + large_t.size), "drawn": args.test,
                           "above_1024_drawn": drawn_large_t, "above_1024_run": int(large_t.size),
                           "tolerance": args.tol, "threshold": args.threshold,
                           "plan_histogram": {("fp32+1" if k < 0 else
                                               "%s+%d" % (("bf16", "fp8", "mxfp4")[sel.PLANS[k][0] - 1],
                                                          sel.PLANS[k][1])): int(hist[k + 1])
                                              for k in range(-1, len(sel.PLANS))}}}
    for name, t in totals.items():
        report["held_out"][name] = {
            "solves_per_s": t["met"] / (t["ms"] / 1e3), "ms": t["ms"],
            "accept_rate": t["accepted"] / t["count"], "fallback_rate": t["fallback"] / t["count"],
            "met_tolerance": t["met"] / t["count"]}
    report["held_out"]["speedup_vs_fp32_path"] = (report["held_out"]["selector"]["solves_per_s"] /
                                                  report["held_out"]["fp32_path"]["solves_per_s"])
    save(args, selector, report)
    print(json.dumps(report))


def save(args, selector, report):
    """Weights, normalisation, plan order and the report (written once after
    training and again with the held-out results)."""
    np.savez(args.out, params=selector.params.cpu().numpy(), mean=selector.mean.cpu().numpy(),
             std=selector.std.cpu().numpy(), cost_order=np.array(selector.cost_order),
             tol=np.array([args.tol]), threshold=np.array([args.threshold]),
             metadata=np.array(json.dumps(report)))


if __name__ == "__main__":
    main()
