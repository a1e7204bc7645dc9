"""Learned plan selector: data generation, GPU training and plan choice.

The network (msq_mlp.cu) maps 16 per-matrix features to 8 logits, one per
plan, each the probability that the plan meets the requested tolerance.
Training data come from the method itself: every plan is run on every
training matrix through msq_solve_batched and scored by its own float-float
residual.  At inference the cheapest plan whose predicted probability clears
`threshold` is chosen (plans are ordered by measured cost); the solver's
residual check still re-solves any miss with the FP32 fallback.

The reference chooses plans by fixed rules (runAdaptiveMetalCase always FP32,
src/metal_solver.cpp:976-1001; low-bit products only below condition 1000,
3_spectral/spectral.cpp:837-838); this replaces those rules.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# The 8 plans: {BF16, FP8-rowscale, MXFP4} x {0, 1, 2} sweeps minus MXFP4
# with 0 sweeps (4-bit storage cannot meet a tight tolerance uncorrected).
# The Jacobi tolerance loosens as more Sylvester sweeps follow it: one
# correction of a BF16 root lands near 7e-6 whatever the basis (off-norm
# 1e-3 is as good as 1e-4 there, one sweep fewer), two reach 1e-7 from a
# basis with off-norm 1e-2 (two Jacobi sweeps fewer than 1e-4).
JACOBI_TOL = {0: 1e-7, 1: 1e-3, 2: 1e-2}
PLANS = [(1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2), (3, 1), (3, 2)]


def cost_order(seconds, tie: float = 0.02) -> list:
    """Plans from cheapest to dearest by measured GPU time; plans within
    `tie` (relative) of each other count as equally cheap and are ordered by
    basis precision (BF16, then FP8, then MXFP4), so a near-tie never trades
    accuracy for noise."""
    seconds = np.asarray(seconds, dtype=np.float64)
    base = seconds.min()
    buckets = np.floor(np.log(seconds / base) / np.log1p(tie)).astype(np.int64)
    return sorted(range(len(PLANS)), key=lambda k: (buckets[k], PLANS[k][0], seconds[k]))


def load(msq, torch, ctx, path):
    """A Selector with the weights, normalisation and plan costs saved by
    train_selector.py; returns (selector, threshold, metadata)."""
    import json
    w = np.load(path)
    selector = Selector(msq, torch, ctx)
    selector.params = torch.from_numpy(w["params"]).cuda()
    selector.mean = torch.from_numpy(w["mean"]).cuda()
    selector.std = torch.from_numpy(w["std"]).cuda()
    meta = json.loads(str(w["metadata"])) if "metadata" in w.files else {}
    train = meta.get("train", {})
    secs = train.get("plan_seconds_probe", train.get("plan_seconds"))
    selector.cost_order = cost_order(secs) if secs else [int(k) for k in w["cost_order"]]
    return selector, float(w["threshold"][0]), meta


def plan_structs(msq, index_list):
    return [msq.plan(PLANS[k][0], PLANS[k][1], JACOBI_TOL[PLANS[k][1]], 15) for k in index_list]


def generate(torch, count: int, seed: int, n_lo: int = 32, n_hi: int = 512,
             cond_lo: float = 1e1, cond_hi: float = 1e8, device="cuda", orders=None):
    """SPD matrices of three spectrum families (log-uniform, clustered, power
    law i^-2) with n log-uniform in [n_lo, n_hi] (or the given orders) and
    condition log-uniform in [cond_lo, cond_hi]; Q from QR of a seeded
    Gaussian.  Returns (orders, list of FP64 tensors)."""
    rng = np.random.default_rng(seed)
    drawn = np.floor(np.exp(rng.uniform(math.log(n_lo), math.log(n_hi + 1), count))).astype(np.int32)
    orders = np.clip(drawn, n_lo, n_hi) if orders is None else np.asarray(orders, np.int32)
    conds = np.exp(rng.uniform(math.log(cond_lo), math.log(cond_hi), count))
    fams = rng.integers(0, 3, count)
    g = torch.Generator(device=device).manual_seed(seed)
    mats = []
    for n, cond, fam in zip(orders, conds, fams):
        n = int(n)
        if fam == 0:
            lam = np.exp(rng.uniform(-math.log(cond), 0.0, n))
            lam[0], lam[-1] = 1.0 / cond, 1.0
        elif fam == 1:
            k = max(1, n // 10)
            lam = np.concatenate([rng.uniform(0.9, 1.1, n - k),
                                  np.exp(rng.uniform(-math.log(cond), math.log(0.9), k))])
            lam[-1] = 1.0 / cond
        else:
            lam = 1.0 / np.arange(1, n + 1, dtype=np.float64) ** 2
            lam = np.maximum(lam, 1.0 / cond)
        q, r = torch.linalg.qr(torch.randn(n, n, generator=g, device=device, dtype=torch.float64))
        q = q * torch.sign(torch.diagonal(r))
        lt = torch.as_tensor(lam, device=device, dtype=torch.float64)
        a = (q * lt) @ q.T
        mats.append(0.5 * (a + a.T))
    return orders, mats


def generate_wishart(torch, count: int, seed: int, n_lo: int = 16, n_hi: int = 512,
                     device="cuda"):
    """Wishart covariances A = X^T X / m + 1e-6 I, X ~ N(0,1) of shape m x n,
    m = 2n, n log-uniform in [n_lo, n_hi] (the batched workload's family).
    Returns (orders, list of FP64 tensors)."""
    rng = np.random.default_rng(seed)
    orders = np.floor(np.exp(rng.uniform(math.log(n_lo), math.log(n_hi + 1), count))).astype(np.int32)
    orders = np.clip(orders, n_lo, n_hi)
    g = torch.Generator(device=device).manual_seed(seed)
    mats = []
    for n in orders:
        n = int(n)
        x = torch.randn(2 * n, n, generator=g, device=device, dtype=torch.float64)
        a = x.T @ x / (2 * n) + 1e-6 * torch.eye(n, device=device, dtype=torch.float64)
        mats.append(0.5 * (a + a.T))
    return orders, mats


def pack(msq, torch, orders, mats):
    batch = msq.Batch.from_orders(orders)
    flat = torch.zeros(batch.total, dtype=torch.float32, device=mats[0].device)
    for i, a in enumerate(mats):
        n = int(orders[i])
        o = int(batch.offset[i])
        flat[o:o + n * n] = a.T.reshape(-1).to(torch.float32)
    return batch, flat


def features(ctx, torch, batch, flat, tolerance: float):
    f = ctx.features(flat, batch).clone()
    f[:, 14] = math.log10(tolerance)
    return f


@dataclass
class Outcomes:
    accepted: np.ndarray  # [count, 8] 1 if plan k met the tolerance itself
    seconds: np.ndarray   # [8] GPU seconds per plan for the whole set


def score_plans(ctx, msq, torch, batch, flat, tolerance: float, plans_run=None) -> Outcomes:
    """Runs every plan (or those in `plans_run`; the others score 0 and 0 s)
    on every matrix; records which plans met the tolerance on their own (the
    plan's final float-float residual) and the GPU time each plan took.  The
    solve runs with a tolerance every plan meets (1e30), so no fallback
    spends time on the misses; the plan's own residual is compared with
    `tolerance` here."""
    acc = np.zeros((batch.count, len(PLANS)), dtype=np.float32)
    secs = np.zeros(len(PLANS))
    out = torch.empty_like(flat)
    for k in (range(len(PLANS)) if plans_run is None else plans_run):
        plans = plan_structs(msq, [k] * batch.count)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        _, res = ctx.solve_batched(flat, batch, plans, 1e30, out=out)
        end.record()
        torch.cuda.synchronize()
        secs[k] = start.elapsed_time(end) / 1e3
        acc[:, k] = [r.plan_residual <= tolerance for r in res]
    return Outcomes(acc, secs)


class Selector:
    """MLP parameters (FP32 masters on the GPU) plus the plan cost order."""

    def __init__(self, msq, torch, ctx, seed: int = 0):
        self.msq, self.torch, self.ctx = msq, torch, ctx
        rng = np.random.default_rng(seed)
        p = np.zeros(msq.MLP_PARAMS, dtype=np.float32)
        i, h, o = msq.MLP_IN, msq.MLP_HIDDEN, msq.MLP_OUT
        off = 0
        for rows, cols in ((h, i), (h, h), (o, h)):
            w = rng.standard_normal((rows, cols)) * math.sqrt(2.0 / cols)
            p[off:off + rows * cols] = w.reshape(-1)
            off += rows * cols + rows  # weights then bias (bias stays 0)
        self.params = torch.from_numpy(p).cuda()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.cost_order = list(range(len(PLANS)))
        self.mean = None
        self.std = None

    def normalise(self, f):
        return (f - self.mean) / self.std

    def fit(self, feats, targets, epochs: int = 200, batch_rows: int = 256, lr: float = 3e-3,
            seed: int = 0):
        torch = self.torch
        self.mean = feats.mean(0, keepdim=True)
        self.std = feats.std(0, keepdim=True).clamp_min(1e-3)
        self.mean[:, 15] = 0.0
        self.std[:, 15] = 1.0
        x = self.normalise(feats).contiguous()
        y = targets.contiguous()
        grad = torch.zeros_like(self.params)
        g = torch.Generator(device="cpu").manual_seed(seed)
        losses = []
        for _ in range(epochs):
            perm = torch.randperm(x.shape[0], generator=g).to(x.device)
            total = 0.0
            for s in range(0, x.shape[0], batch_rows):
                idx = perm[s:s + batch_rows]
                xb, yb = x[idx].contiguous(), y[idx].contiguous()
                grad.zero_()
                loss = self.ctx.mlp_backward(self.params, xb, yb, grad)
                self.step += 1
                self.ctx.mlp_step(self.params, grad, self.m, self.v, self.step, lr)
                total += float(loss.item()) * xb.shape[0]
            losses.append(total / x.shape[0])
        return losses

    def probabilities(self, feats):
        z = self.ctx.mlp_forward(self.params, self.normalise(feats).contiguous())
        return self.torch.sigmoid(z)

    def choose(self, feats, threshold: float = 0.9):
        """Cheapest plan per row whose probability clears the threshold;
        -1 (the FP32 fallback plan) when none does."""
        p = self.probabilities(feats).cpu().numpy()
        choice = np.full(p.shape[0], -1, dtype=np.int64)
        for k in reversed(self.cost_order):
            choice = np.where(p[:, k] >= threshold, k, choice)
        return choice
