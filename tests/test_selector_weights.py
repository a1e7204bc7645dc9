"""The committed selector weights: shapes the MLP kernels expect, and the
training record the weights carry (the learned-selector specification:
200k method-generated matrices, n in [64, 2048], condition in [1e1, 1e8],
three spectrum families; 20k held-out seeds at tolerance 1e-5)."""
import importlib
import json
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WEIGHTS = os.path.join(ROOT, "mixed-mlx_gb300", "selector_weights.npz")


def _load():
    w = np.load(WEIGHTS)
    return w, json.loads(str(w["metadata"]))


def test_weights_have_the_network_shape():
    w, _ = _load()
    # 16 -> 64 -> 64 -> 8: weights and biases of three layers
    params = 16 * 64 + 64 + 64 * 64 + 64 + 64 * 8 + 8
    assert w["params"].shape == (params,)
    assert w["mean"].shape == (1, 16) and w["std"].shape == (1, 16)
    assert np.all(np.isfinite(w["params"])) and np.all(w["std"] > 0)
    assert float(w["tol"][0]) == 1e-5 and 0.5 <= float(w["threshold"][0]) < 1.0


def test_training_record_matches_the_specification():
    _, meta = _load()
    train, held = meta["train"], meta["held_out"]
    assert train["drawn"] >= 200_000
    assert train["n"] == [64, 2048] and train["cond"] == [10.0, 1e8]
    assert sorted(train["families"]) == ["clustered", "log-uniform", "power law i^-2"]
    # every plan ran on the probe; the ones never accepted there were not run on the rest
    probe = np.asarray(train["probe_accept_rate"])
    assert sorted(train["plans_run_after_probe"]) == sorted(np.flatnonzero(probe > 0).tolist())
    assert held["drawn"] >= 20_000 and held["tolerance"] == 1e-5
    sel, fp32 = held["selector"], held["fp32_path"]
    assert abs(sel["accept_rate"] + sel["fallback_rate"] - 1.0) < 1e-9
    # no matrix the FP32 path solves is lost by the selector (fallback)
    assert sel["met_tolerance"] >= fp32["met_tolerance"] - 1e-9
    assert held["speedup_vs_fp32_path"] > 1.0


def test_cost_order_comes_from_the_probe():
    sel = importlib.import_module("mixed-mlx_gb300.selector")
    w, meta = _load()
    order = sel.cost_order(meta["train"]["plan_seconds_probe"])
    assert sorted(order) == list(range(8))
    secs = np.asarray(meta["train"]["plan_seconds_probe"])
    # plans more than 2% apart keep their measured order
    for a, b in zip(order, order[1:]):
        assert secs[a] <= secs[b] * 1.02 or sel.PLANS[a][0] < sel.PLANS[b][0]


def test_cost_order_ties_prefer_the_more_precise_basis():
    """Plans within 2% of each other count as equally cheap and are ordered
    by basis precision (BF16, then FP8, then MXFP4); otherwise by time."""
    sel = importlib.import_module("mixed-mlx_gb300.selector")
    # PLANS: 0 bf16+0, 1 bf16+1, 2 bf16+2, 3 fp8+0, 4 fp8+1, 5 fp8+2, 6 mxfp4+1, 7 mxfp4+2
    secs = [4.0, 2.6, 2.10, 4.0, 2.5, 2.09, 2.5, 2.08]
    order = sel.cost_order(secs)
    # 2.08 / 2.09 / 2.10 tie: bf16+2 first, then fp8+2, then mxfp4+2
    assert order[:3] == [2, 5, 7]
    # fp8+1 and mxfp4+1 tie at 2.5 (FP8 first); bf16+1 at 2.6 is 4% dearer
    assert order[3:6] == [4, 6, 1]
    # the two 4.0 plans tie: BF16 before FP8
    assert order[6:] == [0, 3]
    # far apart: plain time order
    assert sel.cost_order([1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0]) == list(range(8))
