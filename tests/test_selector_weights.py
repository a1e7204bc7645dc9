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
