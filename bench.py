"""Benchmark: batched SPD square roots on one GB300 (or N replicas).

Workload (the batched configuration the throughput target is stated on):
4096 Wishart covariances A = X^T X / m + 1e-6 I, X ~ N(0,1) of shape m x n,
m = 2n, n log-uniform integer in [16, 512], FP32 input, seeded.  One step =
one msq_solve_batched call over the whole batch with the low-bit plan (BF16
factor on tcgen05 + Sylvester sweeps, FP32 fallback for any matrix whose
float-float residual misses 1e-5).  value = matrices meeting
||A - X^2||_F/||A||_F <= 1e-5 per second.  The plain FP32 path (Jacobi to
1e-7, FP32 reconstruction) is timed beside it as the denominator of the
low-bit speed-up.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank solves its own batch (weak scaling, no collective
on the data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("SPD sqrt solves/s at rel. residual ≤1e-5: low-bit+Sylvester vs plain FP32, "
          "1×GB300")
TOL = 1e-5
COUNT = 4096
N_LO, N_HI = 16, 512


PROFILE_STEPS = 1  # serialized step whose per-kernel times give the roofline

# Size classes of the Jacobi sweep launches (the library's launch names).
SWEEP_CLASS_NAMES = ["jacobi sweep n<=16", "jacobi sweep n<=32", "jacobi sweep n<=64",
                     "jacobi sweep n<=128", "jacobi sweep n<=256", "jacobi sweep n<=320",
                     "jacobi sweep n<=512 (global)", "jacobi sweep n<=1024 (global)",
                     "jacobi sweep n<=2048 (global)"]
# DRAM bytes (read + write) per matrix-sweep of the global-tile sweep kernel,
# 320 < n <= 512: ncu dram__bytes_read.sum + dram__bytes_write.sum of one
# 67-matrix launch of `bench.py --count 512` (the roofline's `traffic`)
GLOBAL_SWEEP_DRAM_PER_MATRIX_SWEEP = 80.5e6 / 67


def _tiles_fit_shared(n: int) -> bool:
    """The sweep keeps the packed tiles in shared memory when they fit 227 KB."""
    m = (n + 7) // 8 * 8
    nb, p = m // 4, m // 8
    # reduction scratch, tile table, counters, done flags, three 16-bit round
    # tables; two rotation buffers (68-float stride); the packed tiles
    head = (32 * 8 + (nb + 1 + 2 + p) * 4 + 3 * (3 * p + 2 * nb) * 2 + 15) // 16 * 16
    return head + 2 * p * 68 * 4 + nb * (nb + 1) // 2 * 16 * 4 <= 227 * 1024 - 256


def sweep_class(n: int) -> int:
    for c, hi in enumerate((16, 32, 64, 128, 256)):
        if n <= hi:
            return c
    if _tiles_fit_shared(n):
        return 5
    return 6 if n <= 512 else (7 if n <= 1024 else 8)


def workload_orders(count: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n = np.floor(np.exp(rng.uniform(np.log(N_LO), np.log(N_HI + 1), count))).astype(np.int32)
    return np.clip(n, N_LO, N_HI)


def rank_shard(count: int, rank: int):
    """Weak scaling: rank r solves its own seeded batch of `count` matrices
    (orders seed 1234 + r, matrix seed 99 + r); no data crosses ranks."""
    return workload_orders(count, 1234 + rank), 99 + rank


def whole_job(accepted: float, ms: float, world: int, device) -> tuple:
    """Sum of accepted solves over the ranks and the slowest rank's time."""
    if world == 1:
        return float(accepted), float(ms)
    import torch
    import torch.distributed as dist
    acc = torch.tensor([float(accepted)], dtype=torch.float64, device=device)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(acc, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(acc.item()), float(t.item())


def wishart_matrix(n: int, seed: int) -> np.ndarray:
    """Matrix `seed` of the workload: A = X^T X / m + 1e-6 I, X ~ N(0,1) of
    shape m x n (m = 2n) from numpy's default_rng(seed), FP64, symmetrised.
    Both arms of the benchmark solve these same matrices."""
    x = np.random.default_rng(seed).standard_normal((2 * n, n))
    a = x.T @ x / (2 * n) + 1e-6 * np.eye(n)
    return 0.5 * (a + a.T)


def matrix_seed(base: int, i: int) -> int:
    return base * 1_000_003 + i


def make_batch(msq, torch, orders, seed, device):
    """The workload's Wishart matrices (wishart_matrix, generated on the
    host), stored FP32, packed column-major, copied to the device."""
    batch = msq.Batch.from_orders(orders)
    flat = np.zeros(batch.total, dtype=np.float32)
    for i, n in enumerate(orders):
        n = int(n)
        o = int(batch.offset[i])
        flat[o:o + n * n] = wishart_matrix(n, matrix_seed(seed, i)).reshape(-1, order="F")
    return batch, torch.from_numpy(flat).to(device)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def stratified(orders, k: int = 64) -> np.ndarray:
    """k matrices of the batch spread evenly over the sorted orders."""
    order = np.argsort(orders, kind="stable")
    return order[:: max(1, len(order) // k)][:k]


def time_plain(oracle, mats: dict, sample, budget_s: float):
    """Times the reference's CPU plain method (runAccelerateCase restated in
    the oracle) on `sample`, stopping once budget_s is used.  Returns
    (seconds per solve, fraction meeting the tolerance, solves timed)."""
    done, ok, t_used = 0, 0, 0.0
    for idx in sample:
        t0 = time.perf_counter()
        root, hist = oracle.plain_method(mats[int(idx)], 12, TOL)
        t_used += time.perf_counter() - t0
        done += 1
        ok += hist[-1] <= TOL
        if t_used > budget_s:
            break
    return t_used / done, ok / done, done


def cpu_baseline(oracle, mats, budget_s: float) -> dict:
    """The reference's CPU plain method on a stratified sample of the batch
    (every order range in proportion), bounded to ~budget_s."""
    sample = stratified([m.shape[0] for m in mats])
    per_solve, ok, done = time_plain(oracle, dict(enumerate(mats)), sample, budget_s)
    cores = os.cpu_count() or 1
    return {"value": ok / per_solve, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"{done} of {len(mats)} matrices (stratified by n), "
                      f"{per_solve * done:.1f}s, OpenBLAS threads={os.environ.get('OPENBLAS_NUM_THREADS', cores)}"}


def run_reference(args):
    """--impl reference: the reference's CPU plain method (runAccelerateCase,
    src/accelerate_backend.cpp:803-1091, as the oracle's numpy/LAPACK port:
    the reference's own C++ is compiled only where its sources are, and the
    GPU host has none) on the host cores.  Same matrices as the GPU arm
    (wishart_matrix with the same seeds), same tolerance.  A step is one
    pass over a stratified sample of 64 of the 4096 matrices; ms_per_step is
    that pass's measured time and value its accepted solves per second."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    orders, base = rank_shard(COUNT, 0)
    sample = stratified(orders)
    # the FP32 rounding the GPU arm's input has, back in FP64
    mats = {int(i): wishart_matrix(int(orders[i]), matrix_seed(base, int(i)))
            .astype(np.float32).astype(np.float64) for i in sample}
    for _ in range(args.warmup):
        O.plain_method(mats[int(sample[0])], 12, TOL)
    ms_steps, oks = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ok = 0
        for idx in sample:
            _, hist = O.plain_method(mats[int(idx)], 12, TOL)
            ok += hist[-1] <= TOL
        ms_steps.append((time.perf_counter() - t0) * 1e3)
        oks.append(ok)
    ms = statistics.mean(ms_steps)
    value = statistics.mean(oks) / (ms / 1e3)
    cores = os.cpu_count() or 1
    sample_text = (f"{len(sample)} of the {COUNT} matrices per step (stratified by n, the GPU "
                   f"arm's matrices and seeds), OpenBLAS threads="
                   f"{os.environ.get('OPENBLAS_NUM_THREADS', cores)}")
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded Wishart, same matrices as the GPU arm)", "impl": "reference",
            "config": {"workload": f"{COUNT} Wishart SPD A=X^T X/m+1e-6 I (m=2n), n log-uniform "
                                   f"[{N_LO},{N_HI}], FP32 input, tol 1e-5",
                       "sample_per_step": len(sample)},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": sample_text},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_codec(args):
    """Secondary line: MXFP4 (E2M1 + E8M0 per 32) encode + decode of 2^26
    N(0,1) FP32 values, inputs resident in HBM (256 MB > L2).  Algorithmic
    bytes per element: encode 4 + 0.5 + 1/32, decode 0.5 + 1/32 + 4."""
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    ctx = msq.Context(0)
    stream = torch.cuda.current_stream()
    n = 1 << 26
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn(n, device="cuda", generator=g)
    vals = torch.empty(msq.storage_bytes(msq.MXFP4_E2M1, n), dtype=torch.uint8, device="cuda")
    scales = torch.empty(msq.scale_bytes(msq.MXFP4_E2M1, n), dtype=torch.uint8, device="cuda")
    out = torch.empty_like(x)
    lib = msq.lib()

    def encode():
        ctx.check(lib.msq_encode(ctx.handle, msq.MXFP4_E2M1, x.data_ptr(), n, 0, vals.data_ptr(),
                                 scales.data_ptr()), "encode")

    def decode():
        ctx.check(lib.msq_decode(ctx.handle, msq.MXFP4_E2M1, vals.data_ptr(), scales.data_ptr(),
                                 n, 0, out.data_ptr()), "decode")

    def step():
        encode()
        decode()

    def kernel_ms(fn, reps):
        # back-to-back launches of one kernel between two events on the
        # launching stream: its average duration
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    lib.msq_timing_begin(ctx.handle)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        s.record(stream)
        for _ in range(args.steps):
            step()
        e.record(stream)
        torch.cuda.synchronize()
    rows = timing_report(msq, ctx)
    ms = s.elapsed_time(e) / args.steps
    enc_bytes = n * (4 + 0.5 + 1 / 32)
    dec_bytes = n * (0.5 + 1 / 32 + 4)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    enc_ms = kernel_ms(encode, 4 * args.steps)
    dec_ms = kernel_ms(decode, 4 * args.steps)
    # bit-exact spot check against the oracle on sampled blocks (untimed)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    blocks = np.random.default_rng(0).integers(0, n // 32, 256)
    sel = torch.from_numpy((blocks[:, None] * 32 + np.arange(32)).reshape(-1)).cuda()
    ov, os_ = O.encode(msq.MXFP4_E2M1, x[sel].cpu().numpy())
    exact = bool(np.array_equal(out[sel].cpu().numpy().view(np.uint32),
                                O.decode(msq.MXFP4_E2M1, ov, os_, sel.numel()).view(np.uint32)))
    line = {"metric": "MXFP4 codec round trip (encode+decode) throughput", "value": n / (ms / 1e3),
            "unit": "elements/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8", "data": "synthetic N(0,1), seeded",
            "config": {"workload": "MXFP4 E2M1 + E8M0/32 round trip, 2^26 FP32 elements",
                       "l2": "inputs larger than L2 (268 MB)"},
            "roofline": {"bound": "hbm", "achieved": enc_bytes / (enc_ms / 1e3) / 1e9, "peak": hbm,
                         "unit": "GB/s", "frac": enc_bytes / (enc_ms / 1e3) / 1e9 / hbm,
                         "traffic": None, "kernel": "msq_encode (encodeMxfp4Kernel)",
                         "decode_achieved": dec_bytes / (dec_ms / 1e3) / 1e9,
                         "decode_frac": dec_bytes / (dec_ms / 1e3) / 1e9 / hbm},
            "bit_exact_sampled_blocks": exact, "clocks": clocks.summary(),
            "gpu_launches": sum(v[0] for v in rows.values())}
    print(json.dumps(line), flush=True)


def selector_eval(msq, torch, ctx, count: int, steps: int = 1, warmup: int = 2):
    """Learned plan selection on held-out seeds: SPD matrices of the three
    spectrum families, n log-uniform in [64, 1024], condition log-uniform in
    [1e1, 1e8]; each matrix gets the cheapest plan the MLP predicts to meet
    1e-5 (FP32 fallback on a miss); compared with every matrix on the plain
    FP32 path (device time of one call after the warm-ups that build the
    plan caches and the solve graph)."""
    sel = importlib.import_module("mixed-mlx_gb300.selector")
    weights = os.path.join(ROOT, "mixed-mlx_gb300", "selector_weights.npz")
    if not os.path.exists(weights):
        return None
    selector, threshold, meta = sel.load(msq, torch, ctx, weights)
    orders, mats = sel.generate(torch, count, seed=777_777, n_lo=64, n_hi=1024)
    batch, flat = sel.pack(msq, torch, orders, mats)
    del mats
    choice = selector.choose(sel.features(ctx, torch, batch, flat, TOL), threshold)
    plans = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15) if k < 0 else sel.plan_structs(msq, [int(k)])[0]
             for k in choice]
    fp32 = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15)] * batch.count
    out = torch.empty_like(flat)

    def timed(p):
        for _ in range(max(2, warmup)):  # caches, then the solve's graph capture
            ctx.solve_batched(flat, batch, p, TOL, out=out)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(steps):
            _, res = ctx.solve_batched(flat, batch, p, TOL, out=out)
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / steps, res

    ms_sel, res_sel = timed(plans)
    ms_fp32, res_fp32 = timed(fp32)
    met = lambda res: sum(r.final_residual <= TOL for r in res)
    hist = {("fp32+1" if k < 0 else "%s+%d" % (("bf16", "fp8", "mxfp4")[sel.PLANS[k][0] - 1], sel.PLANS[k][1])):
            int(np.sum(choice == k)) for k in sorted(set(choice.tolist()))}
    return {"matrices": batch.count, "ms": ms_sel,
            "solves_s": met(res_sel) / (ms_sel / 1e3),
            "fp32_path": {"solves_s": met(res_fp32) / (ms_fp32 / 1e3), "ms": ms_fp32},
            "speedup_vs_fp32_path": (met(res_sel) / ms_sel) / max(met(res_fp32) / ms_fp32, 1e-30),
            "accept_rate": float(np.mean([r.accepted for r in res_sel])),
            "fallback_rate": float(np.mean([r.fallback for r in res_sel])),
            "met_tolerance": float(met(res_sel)) / batch.count,
            "plan_histogram": hist,
            "training": meta.get("train"), "held_out_at_training": meta.get("held_out")}


def run_selector(args):
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    ctx = msq.Context(0)
    count = args.count if args.count != COUNT else 2048
    r = selector_eval(msq, torch, ctx, count, max(1, args.steps // 2), args.warmup)
    if r is None:
        print(json.dumps({"metric": "selector", "unavailable": "no trained selector weights"}))
        return
    print(json.dumps({
        "metric": "SPD sqrt solves/s at rel. residual <=1e-5 with learned plan selection (held-out seeds)",
        "value": r["solves_s"], "unit": "solves/s", "n_gpus": 1,
        "steps": max(1, args.steps // 2), "warmup": max(2, args.warmup), "ms_per_step": r["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded Gaussian-QR spectra: log-uniform, clustered, power law)",
        "config": {"workload": f"{count} held-out SPD, n log-uniform [64,1024], cond [1e1,1e8], tol 1e-5",
                   "selector": "MLP 16-64-64-8, trained by the library's CUDA kernels"},
        **{k: v for k, v in r.items() if k not in ("ms", "solves_s")}}), flush=True)


def _spd_gpu(torch, lam, seed, device):
    """A = Q diag(lam) Q^T in FP64 on the GPU, Q from QR of a seeded N(0,1)
    matrix with the signs of R's diagonal fixed; returned rounded to FP32
    (what the solver sees) and as the FP64 image of that rounding."""
    n = lam.numel()
    g = torch.Generator(device=device).manual_seed(seed)
    q, r = torch.linalg.qr(torch.randn(n, n, generator=g, device=device, dtype=torch.float64))
    q = q * torch.sign(torch.diagonal(r))
    a = (q * lam) @ q.T
    a32 = (0.5 * (a + a.T)).to(torch.float32)
    return a32, a32.to(torch.float64)


def _fp64_errors(torch, a64, x32, root):
    """||A - X^2||_F / ||A||_F and ||X - X_fp64||_F / ||X_fp64||_F in FP64."""
    x = x32.to(torch.float64)
    resid = float(torch.linalg.norm(a64 - x @ x) / torch.linalg.norm(a64))
    err = None if root is None else float(torch.linalg.norm(x - root) / torch.linalg.norm(root))
    return resid, err


def _plan_flops(n: int, jacobi_sweeps: int, corrections: int) -> float:
    """Algorithmic flops of one solve: Jacobi 6 n^3 per sweep (A and V
    updates), reconstruction 2 n^3, per correction 8 n^3 (four GEMMs) + 2 n^3
    (residual), and the residual of X0 2 n^3."""
    n3 = float(n) ** 3
    return 6 * n3 * jacobi_sweeps + 2 * n3 + 10 * n3 * corrections + 2 * n3


def _time_solve(torch, ctx, a, batch, plan, out, reps: int = 1, warm: bool = True):
    if warm:
        ctx.solve_batched(a, batch, [plan], TOL, out=out)  # layouts, graphs, tuner
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        _, res = ctx.solve_batched(a, batch, [plan], TOL, out=out)
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps, res[0]


C2_ALL = [(n, c, p) for n in (1024, 2048, 4096) for c in (1e2, 1e4, 1e6)
          for p in ("fp32", "bf16+0", "bf16+1", "bf16+2", "fp8row+0", "fp8row+1", "fp8row+2")]
# the default line's share of the grid (about half a minute of GPU time):
# every plan at n = 1024 and 2048, the two-sweep plans and FP32 at n = 4096
C2_DEFAULT = [(n, c, p) for (n, c, p) in C2_ALL
              if n < 4096 or (c == 1e2 and p in ("fp32", "bf16+2", "fp8row+2"))]


def c2_table(msq, torch, ctx, cases=C2_ALL) -> list:
    """The single-matrix low-bit grid: per (n, condition) one seeded
    Gaussian-QR matrix with log-uniform spectrum, its FP64 root (dsyevd of the
    FP32-rounded matrix, cuSOLVER, untimed), then each plan of `cases` among
    {FP32 plain, BF16, FP8 per-row} x {0, 1, 2} corrections: device time of
    one solve (after a warm-up below n = 2048, where first-call set-up is not
    negligible), solves/s, algorithmic TFLOP/s, FP64 residual and forward
    error, and whether the plan met 1e-5 itself or fell back to FP32."""
    jt = {0: 1e-4, 1: 1e-4, 2: 1e-3}
    fmt_id = {"fp32": msq.PLAN_FP32, "bf16": msq.PLAN_BF16, "fp8row": msq.PLAN_FP8}
    rows = []
    for n, cond in sorted({(n, c) for n, c, _ in cases}):
        seed = n + int(np.log10(cond))
        g = torch.Generator(device="cuda").manual_seed(seed + 1)
        lam = torch.exp(torch.empty(n, dtype=torch.float64, device="cuda").uniform_(
            float(np.log(1.0 / cond)), 0.0, generator=g))
        lam[0], lam[-1] = 1.0, 1.0 / cond
        a32, a64 = _spd_gpu(torch, lam, seed, "cuda")
        w, v = torch.linalg.eigh(a64)
        root = (v * torch.sqrt(w)) @ v.T
        root = 0.5 * (root + root.T)
        del w, v
        batch = msq.Batch.from_orders([n])
        a = a32.T.contiguous().reshape(-1)  # column-major (symmetric anyway)
        out = torch.empty_like(a)
        for nn, cc, p in cases:
            if (nn, cc) != (n, cond):
                continue
            name, k = (p.split("+") + ["1"])[:2]
            k = int(k)
            plan = msq.plan(fmt_id[name], k, 1e-7 if name == "fp32" else jt[k], 20)
            ms, r = _time_solve(torch, ctx, a, batch, plan, out, warm=n < 2048)
            resid, err = _fp64_errors(torch, a64, out.view(n, n).T, root)
            flops = _plan_flops(n, r.jacobi_sweeps, r.corrections)
            rows.append({"n": n, "cond": cond, "format": name, "sweeps": k,
                         "ms": round(ms, 3), "solves_s": round(1e3 / ms, 2),
                         "tflops": round(flops / (ms / 1e3) / 1e12, 2),
                         "residual_fp64": resid, "error_fp64": err,
                         "plan_residual": r.plan_residual, "accepted": bool(r.accepted),
                         "fallback": bool(r.fallback), "jacobi_sweeps": r.jacobi_sweeps,
                         "corrections": r.corrections})
        del a32, a64, root, a, out
        torch.cuda.empty_cache()
    return rows


def c1_entry(msq, torch, ctx) -> dict:
    """The plain method on one matrix: n = 256, A = Q diag(lambda) Q^T with Q
    from QR of a seeded N(0,1) matrix and lambda log-uniform on [1e-3, 1]
    (condition 1e3), FP32 input; Jacobi to off-norm 1e-7 ||A||_F, FP32
    reconstruction, no correction (plan FP32 + 0).  Device time of one solve
    after warm-ups (latency) and of 1024 such matrices (different seeds) in
    one call (throughput); FP64 residual and forward error of the single
    solve against dsyevd of the FP32-rounded matrix."""
    n, cond = 256, 1e3

    def matrix(seed):
        g = torch.Generator(device="cuda").manual_seed(seed)
        lam = torch.exp(torch.empty(n, dtype=torch.float64, device="cuda").uniform_(
            float(np.log(1.0 / cond)), 0.0, generator=g))
        lam[0], lam[-1] = 1.0, 1.0 / cond
        return _spd_gpu(torch, lam, seed, "cuda")

    a32, a64 = matrix(257)
    w, v = torch.linalg.eigh(a64)
    root = (v * torch.sqrt(w)) @ v.T
    batch = msq.Batch.from_orders([n])
    a = a32.T.contiguous().reshape(-1)
    out = torch.empty_like(a)
    plan = msq.plan(msq.PLAN_FP32, 0, 1e-7, 20)
    for _ in range(2):
        ctx.solve_batched(a, batch, [plan], 1.0, out=out)
    ms, r = _time_solve(torch, ctx, a, batch, plan, out, reps=5)
    resid, err = _fp64_errors(torch, a64, out.view(n, n).T, root)
    count = 1024
    flat = torch.cat([matrix(10_000 + i)[0].T.contiguous().reshape(-1) for i in range(count)])
    big = msq.Batch.from_orders([n] * count)
    outb = torch.empty_like(flat)
    plans = [plan] * count
    for _ in range(3):
        ctx.solve_batched(flat, big, plans, TOL, out=outb)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    _, res = ctx.solve_batched(flat, big, plans, TOL, out=outb)
    e.record()
    torch.cuda.synchronize()
    ms_b = s.elapsed_time(e)
    met = sum(x.final_residual <= TOL for x in res)
    sweeps = float(np.mean([x.jacobi_sweeps for x in res]))
    return {"n": n, "cond": cond, "plan": "FP32: Jacobi to 1e-7, FP32 reconstruction",
            "latency_ms": round(ms, 3), "jacobi_sweeps": r.jacobi_sweeps,
            "residual_fp64": resid, "error_fp64": err,
            "batch": {"matrices": count, "ms": round(ms_b, 2), "solves_s": met / (ms_b / 1e3),
                      "met_tolerance": int(met),
                      "tflops": count * (6.0 * n ** 3 * sweeps + 4.0 * n ** 3) / (ms_b / 1e3) / 1e12}}


def c3_entry(msq, torch, ctx, warm: bool = False) -> dict:
    """n = 8192, condition 1e4, clustered spectrum (90% of the eigenvalues in
    [0.9, 1.1], 10% log-uniform down to 1e-4), MXFP4 basis + 2 corrections:
    device time of one solve, whether the plan met 1e-5 or fell back, the
    FP64 residual of the returned root, and the block-scaled reconstruction
    stage (kind::mxf4) timed alone over five launches on an order-8192 FP32
    factor (the launch timer), as TFLOP/s of its 2 n^3 flops."""
    n, cond = 8192, 1e4
    g = torch.Generator(device="cuda").manual_seed(8193)
    k = n // 10
    lam = torch.empty(n, dtype=torch.float64, device="cuda")
    lam[: n - k].uniform_(0.9, 1.1, generator=g)
    lam[n - k:] = torch.exp(torch.empty(k, dtype=torch.float64, device="cuda").uniform_(
        float(np.log(1.0 / cond)), float(np.log(0.9)), generator=g))
    lam[-1] = 1.0 / cond
    a32, a64 = _spd_gpu(torch, lam, 8192, "cuda")
    batch = msq.Batch.from_orders([n])
    a = a32.T.contiguous().reshape(-1)
    del a32
    out = torch.empty_like(a)
    plan = msq.plan(msq.PLAN_MXFP4, 2, 1e-3, 20)
    ms, r = _time_solve(torch, ctx, a, batch, plan, out, warm=warm)
    resid, _ = _fp64_errors(torch, a64, out.view(n, n).T, None)
    del a64
    ctx.reconstruct_factor(msq.PLAN_MXFP4, a, batch, out=out)  # the stage, warm
    torch.cuda.synchronize()
    msq.lib().msq_timing_begin(ctx.handle)
    for _ in range(5):
        ctx.reconstruct_factor(msq.PLAN_MXFP4, a, batch, out=out)
    torch.cuda.synchronize()
    rows = timing_report(msq, ctx)
    rec = rows.get("tcgen05 reconstruction", (0, 0.0))
    rec_ms = rec[1] / max(rec[0], 1)
    pack = rows.get("pack block-scaled operand", (0, 0.0))
    return {"n": n, "cond": cond, "plan": "MXFP4 + 2 corrections", "ms": round(ms, 2),
            "solves_s": 1e3 / ms,
            "tflops": _plan_flops(n, r.jacobi_sweeps, r.corrections) / (ms / 1e3) / 1e12,
            "residual_fp64": resid, "plan_residual": r.plan_residual,
            "initial_residual": r.initial_residual,
            "accepted": bool(r.accepted), "fallback": bool(r.fallback),
            "jacobi_sweeps": r.jacobi_sweeps, "corrections": r.corrections,
            "reconstruction": {"kernel": "tcGemmKernel kind::mxf4 block_scale", "ms": rec_ms,
                               "tflops": 2.0 * n ** 3 / (rec_ms / 1e3) / 1e12 if rec_ms > 0 else None,
                               "pack_ms": pack[1] / max(pack[0], 1)}}


def run_mxf4(args):
    """Secondary line: the block-scaled reconstruction stage X = Q(W) Q(W)^T of
    one order-8192 FP32 factor (256 MB, larger than L2) with W quantized to
    MXFP4 per row block of 32 (kind::mxf4) and, for comparison, to BF16
    (kind::f16).  2 n^3 flops per launch; device time of each stage's GEMM
    kernel from the launch timer (CUDA events on the launching stream)."""
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    ctx = msq.Context(0)
    n = 8192
    g = torch.Generator(device="cuda").manual_seed(11)
    f = torch.randn(n * n, generator=g, device="cuda") / float(np.sqrt(n))
    batch = msq.Batch.from_orders([n])
    out = torch.empty_like(f)
    res = {}
    for name, plan in (("mxfp4", msq.PLAN_MXFP4), ("bf16", msq.PLAN_BF16)):
        for _ in range(max(1, args.warmup)):
            ctx.reconstruct_factor(plan, f, batch, out=out)
        torch.cuda.synchronize()
        msq.lib().msq_timing_begin(ctx.handle)
        for _ in range(args.steps):
            ctx.reconstruct_factor(plan, f, batch, out=out)
        torch.cuda.synchronize()
        rows = timing_report(msq, ctx)
        cnt, tot = rows.get("tcgen05 reconstruction", (0, 0.0))
        res[name] = {"gemm_ms": tot / max(cnt, 1), "launches": cnt,
                     "tflops": 2.0 * n ** 3 / (tot / max(cnt, 1) / 1e3) / 1e12,
                     "pack_ms": sum(v[1] for k, v in rows.items() if k.startswith("pack")) / max(cnt, 1)}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    fp4_nominal = 13500.0
    m = res["mxfp4"]
    print(json.dumps({
        "metric": "block-scaled MXFP4 reconstruction X = Q(W) Q(W)^T, n = 8192", "value": m["tflops"],
        "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": max(1, args.warmup),
        "ms_per_step": m["gemm_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "e2m1 (ue8m0 / 32)", "data": "synthetic N(0,1)/sqrt(n), seeded",
        "config": {"workload": "order-8192 FP32 factor quantized per row block of 32, tcgen05 kind::mxf4",
                   "l2": "factor 256 MB > L2"},
        "roofline": {"bound": "tensor", "achieved": m["tflops"], "peak": fp4_nominal,
                     "unit": "TFLOP/s", "frac": m["tflops"] / fp4_nominal, "traffic": None,
                     "kernel": "tcGemmKernel<kOpMxf4> (kind::mxf4 block_scale)",
                     "peak_source": "nominal dense FP4 (no FP4 figure among the measured peaks); "
                                    "of measured BF16 %.0f TFLOP/s: %.2f" % (
                                        peaks.get("bf16_tflops", 1900.0),
                                        m["tflops"] / peaks.get("bf16_tflops", 1900.0))},
        "stages": res}), flush=True)


def run_c2(args):
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    ctx = msq.Context(0)
    t0 = time.perf_counter()
    rows = c2_table(msq, torch, ctx)
    t1 = time.perf_counter()
    c3 = c3_entry(msq, torch, ctx)
    print(json.dumps({"metric": "single-matrix low-bit grid (C2) and n=8192 MXFP4 (C3)",
                      "c2": rows, "c3": c3, "wall_s": {"c2": t1 - t0, "c3": time.perf_counter() - t1}}),
          flush=True)


def timing_report(msq, ctx) -> dict:
    import ctypes
    buf = ctypes.create_string_buffer(1 << 16)
    msq.lib().msq_timing_end(ctx.handle, buf, len(buf))
    rows = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split("\t")
        rows[name] = (int(cnt), float(ms))
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=COUNT)
    ap.add_argument("--sweeps", type=int, default=1)
    ap.add_argument("--jacobi-tol", type=float, default=1e-3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c2", action="store_true",
                    help="skip the single-matrix grid and the n=8192 MXFP4 legs of the line")
    ap.add_argument("--selector", type=int, default=1,
                    help="batched workload: plans from the trained selector (default); 0: the "
                         "fixed BF16 plan with --sweeps corrections and --jacobi-tol")
    ap.add_argument("--workload", default="batched", choices=["batched", "codec", "selector", "c2", "mxf4"],
                    help="codec: MXFP4 round trip of 2^26 N(0,1) values; selector: learned plan "
                         "selection on held-out matrices (secondary lines)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "codec":
        return run_codec(args)
    if args.workload == "selector":
        return run_selector(args)
    if args.workload == "c2":
        return run_c2(args)
    if args.workload == "mxf4":
        return run_mxf4(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    msq = importlib.import_module("mixed-mlx_gb300")
    ctx = msq.Context(local)
    stream = torch.cuda.current_stream(device)

    orders, matrix_seed = rank_shard(args.count, rank)
    batch, a = make_batch(msq, torch, orders, matrix_seed, device)
    torch.cuda.synchronize()
    low_plan = [msq.plan(msq.PLAN_BF16, args.sweeps, args.jacobi_tol, 15)] * batch.count
    plan_source = f"fixed BF16 + {args.sweeps} sweep(s)"
    weights = os.path.join(ROOT, "mixed-mlx_gb300", "selector_weights.npz")
    if args.selector and os.path.exists(weights):
        # learned plan selection: features + MLP forward on the GPU (outside
        # the timed region, like the plan choice of a serving loop)
        sel = importlib.import_module("mixed-mlx_gb300.selector")
        selector, threshold, _ = sel.load(msq, torch, ctx, weights)
        choice = selector.choose(sel.features(ctx, torch, batch, a, TOL), threshold)
        low_plan = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15) if k < 0 else
                    sel.plan_structs(msq, [int(k)])[0] for k in choice]
        plan_source = "learned selector (" + ", ".join(
            f"{('fp32+1' if k < 0 else '%s+%d' % (('bf16', 'fp8', 'mxfp4')[sel.PLANS[k][0] - 1], sel.PLANS[k][1]))}:{int(np.sum(choice == k))}"
            for k in sorted(set(choice.tolist()))) + ")"
    # the plain FP32 path: Jacobi to 1e-7, FP32 reconstruction and one FP32
    # Sylvester correction (the reference's plain method corrects until the
    # tolerance is met, src/accelerate_backend.cpp:803-1091; FP32 Jacobi +
    # reconstruction alone misses 1e-5 on a quarter of this batch)
    fp32_plan = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15)] * batch.count
    root = torch.empty_like(a)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(plans, steps, warmup, collect_timing=False):
        for _ in range(warmup):
            ctx.solve_batched(a, batch, plans, TOL, out=root)
        barrier()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = ctx.launches
        if collect_timing:
            msq.lib().msq_timing_begin(ctx.handle)
        accepted = []
        start.record(stream)
        for _ in range(steps):
            _, res = ctx.solve_batched(a, batch, plans, TOL, out=root)
            accepted.append(sum(r.final_residual <= TOL for r in res))
        end.record(stream)
        barrier()
        rows = timing_report(msq, ctx) if collect_timing else {}
        ms = start.elapsed_time(end) / steps
        return ms, statistics.mean(accepted), ctx.launches - l0, res, rows

    # plain FP32 path (denominator)
    ms_plain, acc_plain, _, res_plain, _ = timed(fp32_plan, max(1, args.steps // 2), 2)
    plain_all, ms_plain_max = whole_job(acc_plain, ms_plain, world, device)
    plain_value = plain_all / (ms_plain_max / 1e3)
    # low-bit + Sylvester path (headline), clocks sampled while it runs
    with ClockSampler(local) as clocks:
        ms, acc, launches, res, _ = timed(low_plan, args.steps, args.warmup, False)
    # per-kernel times from one more step with every launch on one stream
    # (outside the timed region: concurrent launches would share the GPU)
    ctx.set_concurrency(False)
    _, _, _, _, rows = timed(low_plan, PROFILE_STEPS, 0, True)
    ctx.set_concurrency(True)
    # whole job: solves of all ranks over the slowest rank's time
    acc_all, ms_max = whole_job(acc, ms, world, device)
    value = acc_all / (ms_max / 1e3)

    # end to end: every step copies its inputs host -> device from pinned
    # memory and its roots device -> host, double-buffered on a copy stream
    # so the copies of neighbouring steps overlap the solve (all inside the
    # timed region)
    host_in = torch.empty(batch.total, dtype=torch.float32, pin_memory=True)
    host_in.copy_(a.cpu())
    host_out = [torch.empty(batch.total, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    dev_in = [torch.empty_like(a), torch.empty_like(a)]
    dev_out = [torch.empty_like(a), torch.empty_like(a)]
    copy = torch.cuda.Stream(device)
    # the solves on a stream of their own: on the legacy default stream each
    # solve would also wait for the copy stream's device -> host copy of the
    # previous step (implicit synchronisation), serialising what overlaps
    default_stream = stream
    stream = torch.cuda.Stream(device)
    stream.wait_stream(default_stream)
    ctx.set_stream(stream)
    ev_in = [torch.cuda.Event(), torch.cuda.Event()]
    ev_solved = [torch.cuda.Event(), torch.cuda.Event()]
    ev_out = [None, None]  # D2H of the buffer's previous step done
    # untimed warm-up: two solves per buffer pair (launch graphs are captured
    # per set of buffers on the second call, so both pairs' graphs exist
    # before the clock starts)
    for k in range(2):
        dev_in[k].copy_(host_in, non_blocking=True)  # on the default stream
        stream.wait_stream(default_stream)
        for _ in range(2):
            ctx.solve_batched(dev_in[k], batch, low_plan, TOL, out=dev_out[k])
    torch.cuda.synchronize(device)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_steps = args.steps
    e2e_acc = []
    e0.record(stream)
    copy.wait_stream(stream)
    with torch.cuda.stream(copy):
        dev_in[0].copy_(host_in, non_blocking=True)
        ev_in[0].record(copy)
    for k in range(e2e_steps):
        cur, nxt = k % 2, (k + 1) % 2
        if k + 1 < e2e_steps:
            with torch.cuda.stream(copy):
                dev_in[nxt].copy_(host_in, non_blocking=True)
                ev_in[nxt].record(copy)
        stream.wait_event(ev_in[cur])
        if ev_out[cur] is not None:
            stream.wait_event(ev_out[cur])
        _, r_e = ctx.solve_batched(dev_in[cur], batch, low_plan, TOL, out=dev_out[cur])
        ev_solved[cur].record(stream)
        with torch.cuda.stream(copy):
            copy.wait_event(ev_solved[cur])
            host_out[cur].copy_(dev_out[cur], non_blocking=True)
            ev_out[cur] = torch.cuda.Event()
            ev_out[cur].record(copy)
        e2e_acc.append(sum(r.final_residual <= TOL for r in r_e))
    stream.wait_stream(copy)
    e1.record(stream)
    default_stream.wait_stream(stream)
    ctx.set_stream(default_stream)
    stream = default_stream
    barrier()
    e2e_acc_all, e2e_ms = whole_job(statistics.mean(e2e_acc), e0.elapsed_time(e1) / e2e_steps,
                                    world, device)
    e2e_value = e2e_acc_all / (e2e_ms / 1e3)

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    # accuracy (outside timing): every root's FP64 residual on the host,
    # ||A - X^2||_F / ||A||_F, and the forward error against the FP64
    # eigendecomposition root (dsyevd) on a stratified sample of 512
    roots = root.cpu().numpy()
    a_host = a.cpu().numpy()
    mats = batch.unpack(a_host)
    xs = batch.unpack(roots)
    resid_all = np.array([np.linalg.norm(m - x @ x) / np.linalg.norm(m) for m, x in zip(mats, xs)])
    idx = np.argsort(orders)[:: max(1, batch.count // 512)]

    def fp64_root(m):
        w, v = np.linalg.eigh(m)
        return (v * np.sqrt(w)) @ v.T

    errs = [float(np.linalg.norm(xs[i] - fp64_root(mats[i])) / np.linalg.norm(fp64_root(mats[i])))
            for i in idx]
    fallback = sum(r.fallback for r in res)
    reported = np.array([r.final_residual for r in res])
    # matrices the solver counted as meeting 1e-5 whose FP64 residual of the
    # returned (FP32-rounded) root is above it
    miscounted = int(np.sum((reported <= TOL) & (resid_all > TOL * (1 + 1e-2) + 1e-7)))
    # the single-matrix grid and the order-8192 MXFP4 case (untimed legs)
    c1 = c2 = c3 = None
    selector_key = selector_eval(msq, torch, ctx, 1024) if not args.no_c2 else None
    if not args.no_c2:
        c1 = c1_entry(msq, torch, ctx)
        c2 = c2_table(msq, torch, ctx, C2_DEFAULT)
        c3 = c3_entry(msq, torch, ctx)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # the CPU baseline leg only

    # roofline of the dominant kernel (largest share of the timed region)
    top = max(rows.items(), key=lambda kv: kv[1][1]) if rows else ("", (0, 0.0))
    total_ms = sum(v[1] for v in rows.values()) or 1.0
    sweeps = np.array([r.jacobi_sweeps for r in res], dtype=np.float64)
    n64 = orders.astype(np.float64)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops", 1900.0)
    name, (cnt, tot) = top
    avg_ms = tot / max(cnt, 1)
    # Jacobi kernels are FP32 CUDA-core work (the eigensolver stays FP32):
    # their roofline is the FP32 FMA rate, which the measured-peaks file does
    # not hold, so it is measured here (and the nominal rate at the sampled
    # SM clock reported beside it).  Per
    # sweep of an order-n matrix (m = n padded to 8, nb = m/4 blocks, P = m/8
    # pivots): super-tile updates 2 * 512 FMA for each of P(P-1)/2 tiles in
    # each of nb-1 rounds; the V replay 64 FMA per row and pivot per round.
    m64 = np.ceil(n64 / 8.0) * 8.0
    nb64, p64 = m64 / 4.0, m64 / 8.0
    sm_mhz = clocks.summary().get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    fp32_nominal = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s
    # measured FP32 FMA rate of this GPU (independent FMA chains on every SM,
    # best of three launches), the denominator of the FP32 rooflines
    fp32_peak = ctx.fma_rate()
    if name.startswith("jacobi sweep") or name.startswith("jacobi replay"):
        if name.startswith("jacobi sweep"):
            # the sweep launches are named by size class: count only that class
            in_class = np.array([SWEEP_CLASS_NAMES[sweep_class(int(n))] == name for n in orders])
            fma = (nb64 - 1) * p64 * (p64 - 1) / 2.0 * 1024.0 * in_class
            hbm_bytes = 4.0 * 2.0 * m64 * m64 / 2.0 * in_class  # packed tiles read + written
        else:
            fma = (nb64 - 1) * n64 * p64 * 64.0
            hbm_bytes = 8.0 * n64 * n64  # V read + written once per sweep
        per_launch = float(np.sum(2.0 * fma * sweeps)) * PROFILE_STEPS / max(cnt, 1)
        achieved = per_launch / (avg_ms / 1e3) / 1e12
        hbm_launch = float(np.sum(hbm_bytes * sweeps)) * PROFILE_STEPS / max(cnt, 1)
        traffic = None
        if name == SWEEP_CLASS_NAMES[6]:
            # DRAM read + write per matrix-sweep of the global-tile class from
            # one ncu capture (80.5 MB over a 67-matrix launch of the
            # 512-matrix workload), times this launch's matrix-sweeps
            msweeps = float(np.sum(sweeps * in_class)) * PROFILE_STEPS / max(cnt, 1)
            traffic = GLOBAL_SWEEP_DRAM_PER_MATRIX_SWEEP * msweeps
        roof = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": traffic, "kernel": name,
                "peak_source": "measured FP32 FMA rate (msq_fma_rate, in this run); nominal "
                               "152 SMs x 128 lanes x 2 flop x %.0f MHz = %.1f" % (sm_mhz, fp32_nominal),
                "frac_of_nominal": achieved / fp32_nominal,
                "hbm_view": {"achieved": hbm_launch / (avg_ms / 1e3) / 1e9, "peak": hbm,
                             "unit": "GB/s", "frac": hbm_launch / (avg_ms / 1e3) / 1e9 / hbm}}
    else:
        flops = float(np.sum(2.0 * n64 ** 3)) * PROFILE_STEPS / max(cnt, 1)
        achieved = flops / (avg_ms / 1e3) / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                "frac": achieved / bf16, "traffic": None, "kernel": name,
                "peak_source": "measured (MEASURED_PEAKS.json)" if peaks else "fallback"}
    roof["share"] = tot / total_ms

    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(O, mats, 15.0)

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded Wishart, generated on the host, the reference arm's matrices)",
        "config": {"workload": f"{batch.count} Wishart SPD A=X^T X/m+1e-6 I (m=2n), n log-uniform "
                               f"[{N_LO},{N_HI}], FP32 input, low-bit plan + Sylvester sweeps, "
                               f"FP32 fallback, tol 1e-5",
                   "plans": plan_source,
                   "matrices": batch.count, "sum_n3": float(np.sum(n64 ** 3)),
                   "l2": "inputs larger than L2 (%.0f MB)" % (batch.total * 4 / 1e6),
                   "jacobi_tolerance": ("per plan: 1e-7 / 1e-3 / 1e-2 for 0 / 1 / 2 corrections"
                                        if plan_source.startswith("learned") else args.jacobi_tol)},
        "e2e": {"value": e2e_value, "unit": "solves/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": batch.total * 4, "d2h_bytes_per_step": batch.total * 4},
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "gpu_launches": launches,
        "plain_fp32": {"value": plain_value, "ms_per_step": ms_plain_max,
                       "accepted": acc_plain, "fallback": int(sum(r.fallback for r in res_plain)),
                       "plan": "FP32: Jacobi to 1e-7, FP32 reconstruction, one FP32 Sylvester sweep"},
        "speedup_vs_plain_fp32": (value / plain_value) if plain_value > 0 else None,
        "accepted": acc, "fallback": int(fallback),
        "error_vs_fp64": {"p50": float(np.percentile(errs, 50)), "p99": float(np.percentile(errs, 99)),
                          "forward_error_sample": len(idx),
                          "residual_p50": float(np.percentile(resid_all, 50)),
                          "residual_p99": float(np.percentile(resid_all, 99)),
                          "residual_max": float(resid_all.max()),
                          "residual_checked": int(resid_all.size),
                          "met_tolerance_fp64": int(np.sum(resid_all <= TOL * (1 + 1e-2) + 1e-7)),
                          "counted_but_missed": miscounted},
        "c1": c1, "c2": c2, "c3": c3, "selector": selector_key,
        "kernels": {k: {"launches": v[0], "ms": v[1], "share": v[1] / total_ms} for k, v in rows.items()},
        "kernels_source": "launch timer over one extra step with concurrency off (serial)",
        "autotune": [l for l in ctx.autotune_report().splitlines() if l],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()


if __name__ == "__main__":
    main()
