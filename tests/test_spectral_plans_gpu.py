"""The reference's stage-3 precision plans (precision_plans / run_spectral,
3_spectral/spectral.cpp:769-1385) through the C++ mirror runCudaSpectral,
against the oracle's restatement of run_spectral (oracle.spectral_plan) on
the same matrix: the reference's controlled family at order 128 and the
conditions its driver runs (3_spectral/main.cpp: 4, 100, 1e4).  Both sides
start from the same FP32 eigenbasis (the blocked Jacobi, bit-exact between
GPU and oracle) and quantize with the same codecs, so the quantization
errors and the basis condition agree to rounding; the corrections run FP32
products on the GPU and FP64 products in the oracle, so the residual
histories agree to a small factor and the iteration counts to a couple of
corrections (exactly where neither side is near the tolerance)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "tests", "cpp", "cuda_backend_check")
TOL = 1e-12
ORDER = 128


@pytest.fixture(scope="module", autouse=True)
def exe():
    if not os.path.exists(EXE):
        pytest.skip("cuda_backend_check was not built")


def _run(tmp_path, a, plan, cond, tol=TOL, max_corrections=30):
    n = a.shape[0]
    path = tmp_path / f"s{n}_{plan}.bin"
    with open(path, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.asfortranarray(a, np.float64).tobytes(order="F"))
        f.write(np.asfortranarray(O.reference_root(a), np.float64).tobytes(order="F"))
    out = subprocess.run([EXE, str(path), "spectral", plan, str(tol), str(max_corrections),
                          str(cond)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return dict(kv.split("=", 1) for kv in out.stdout.split())


@pytest.mark.parametrize("cond", [4.0, 100.0, 1e4])
@pytest.mark.parametrize("plan,basis,spectrum", O.SPECTRAL_PLANS)
def test_stage3_plan_against_the_oracle(tmp_path, plan, basis, spectrum, cond):
    a = O.controlled(ORDER, cond)
    r = _run(tmp_path, a, plan, cond)
    o = O.spectral_plan(a, basis, spectrum, cond, 30, TOL)
    assert r["plan"] == plan
    assert (r["accepted"] == "1") == o["accepted"], (r, o["reason"])
    if not o["accepted"]:
        assert r["reason"] == o["reason"]
        return
    # same operands: quantization errors and basis condition agree
    assert float(r["basis_error"]) == pytest.approx(o["basis_error"], rel=1e-6, abs=1e-12)
    assert float(r["spectrum_error"]) == pytest.approx(o["spectrum_error"], rel=1e-6, abs=1e-12)
    assert float(r["basis_condition"]) == pytest.approx(o["basis_condition"], rel=1e-4)
    # the initial root's residual (FP32 vs FP64 product of the same operands)
    res = [float(x) for x in r["residuals"].split(",")]
    assert res[0] == pytest.approx(o["residuals"][0], rel=1e-2)
    # outcome: identical unless the oracle's final residual is within a
    # factor 4 of the tolerance (then FP32 products may land either side)
    marginal = o["final_residual"] > TOL / 4 and o["reason"] in ("converged", "correction_limit")
    if not marginal:
        assert r["reason"] == o["reason"], (r["reason"], o["reason"], res, o["residuals"])
    if r["reason"] == "converged":
        assert float(r["final_residual"]) <= TOL
        assert float(r["final_error"]) < 1e-8
        if not marginal:
            assert abs(int(r["iterations"]) - o["iterations"]) <= max(2, o["iterations"] // 5)
    # low-bit products only for a low-bit basis below condition 1000
    lowbit = basis in ("fp8_e4m3", "fp8_e5m2", "mxfp8_e4m3", "mxfp4_e2m1") and cond < 1000
    assert (int(r["low_product_corrections"]) > 0) == (lowbit and o["low_product_corrections"] > 0)


def test_stage3_storage_bits_follow_the_formats(tmp_path):
    a = O.controlled(64, 100.0)
    bits = {"fp32": 32.0, "fp16": 16.0, "bf16": 16.0, "fp8_e4m3": 8.0, "fp8_e5m2": 8.0,
            "mxfp8_e4m3": 8.25, "mxfp4_e2m1": 4.25}
    for plan, basis, spectrum in O.SPECTRAL_PLANS[:8]:
        r = _run(tmp_path, a, plan, 100.0, max_corrections=1)
        assert float(r["basis_bits"]) == pytest.approx(bits[basis])
        assert float(r["spectrum_bits"]) == pytest.approx(bits[spectrum])


def test_stage3_stall_fallback_leaves_low_products(tmp_path):
    """basis_mxfp4 at condition 100: the 4-bit products stop contracting; after
    two corrections without halving the residual the plan continues on FP32
    products (the reference's stall fallback), as the oracle does."""
    a = O.controlled(ORDER, 100.0)
    r = _run(tmp_path, a, "basis_mxfp4", 100.0)
    o = O.spectral_plan(a, "mxfp4_e2m1", "fp32", 100.0, 30, TOL)
    low = int(r["low_product_corrections"])
    assert 0 < low < int(r["iterations"])
    assert abs(low - o["low_product_corrections"]) <= 1
