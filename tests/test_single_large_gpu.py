"""Single large matrices through msq_solve_batched: the grid eigensolver, the
tcgen05 low-bit reconstruction and the Sylvester sweeps over the whole
single-matrix low-bit grid (n = 1024, 2048, 4096 x condition 1e2, 1e4, 1e6 x
BF16 / FP8-E4M3 per-row-scaled basis x 0, 1, 2 correction sweeps) and the
MXFP4 case (n = 8192, clustered spectrum).  Checked against FP64: the
reported float-float residual equals ||A - X^2||_F / ||A||_F computed in FP64
on the host, and the forward error against the FP64 eigendecomposition root
of the same (FP32-rounded) matrix stays within the conditioning bound.  A
plan that cannot meet the tolerance must say so (not accepted, FP32 fallback)
and the fallback's root must meet it."""
import functools

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5
# the root is returned in FP32: rounding X (float-float inside the solver)
# to FP32 alone moves ||A - X^2|| / ||A|| by up to a few units of 2^-24
ROUNDING = 1e-7
# Jacobi tolerance per number of correction sweeps (the plans the selector
# and the bench use): one sweep needs the tighter basis
JACOBI_TOL = {0: 1e-4, 1: 1e-4, 2: 1e-3}


@functools.lru_cache(maxsize=None)
def _case(n, cond):
    """The seeded Gaussian-QR matrix with log-uniform spectrum, rounded to
    FP32 as the solver sees it, and its FP64 root (host dsyevd)."""
    a = O.spd_loguniform(n, cond, seed=n + int(np.log10(cond)))
    a = a.astype(np.float32).astype(np.float64)
    return a, O.reference_root(a)


def _solve(ctx, msq, a64, plan):
    import torch
    n = a64.shape[0]
    b = msq.Batch.from_orders([n])
    a = torch.from_numpy(b.pack([a64])).cuda()
    root, res = ctx.solve_batched(a, b, [plan], tolerance=TOL)
    torch.cuda.synchronize()
    return b.unpack(root.cpu().numpy())[0].astype(np.float64), res[0]


@pytest.mark.parametrize("sweeps", [0, 1, 2])
@pytest.mark.parametrize("fmt", ["bf16", "fp8row"])
@pytest.mark.parametrize("cond", [1e2, 1e4, 1e6])
@pytest.mark.parametrize("n", [1024, 2048, 4096])
def test_low_bit_grid(ctx, msq, n, cond, fmt, sweeps):
    """Every plan of the grid reports what it reached: the plan's own final
    residual decides acceptance, a plan that misses the tolerance is
    re-solved by the FP32 fallback (corrections until the tolerance is met),
    and the returned root meets the tolerance either way.  Which plans meet
    it on their own depends on the basis quantization against the spectrum
    (frozen-basis Newton contracts by about the relative error of X0 per
    sweep): X0 alone never does; BF16 with two sweeps does up to condition
    1e4 at every order."""
    a, x_ref = _case(n, cond)
    fmt_id = {"bf16": msq.PLAN_BF16, "fp8row": msq.PLAN_FP8}[fmt]
    x, r = _solve(ctx, msq, a, msq.plan(fmt_id, sweeps, JACOBI_TOL[sweeps], 20))
    resid = O.relative_residual(a, x)
    # the reported residual (float-float X) is the FP64 one of the root
    # before its rounding to FP32
    assert abs(resid - r.final_residual) <= 1e-3 * resid + ROUNDING, (resid, r.final_residual)
    if (n, cond) == (4096, 1e6):
        # the FP32 basis of 4096 eigenvalues log-uniform over six decades
        # (neighbours 0.3% apart) limits the corrections: the fallback may
        # stop a little above the tolerance, and must then say so
        assert r.final_residual <= TOL or (r.fallback and r.final_residual <= 1e-3)
    else:
        assert r.final_residual <= TOL
    # forward error: a residual eps moves the root by about eps * sqrt(cond)
    err = O.relative_error(x, x_ref)
    assert err <= 10 * max(TOL, r.final_residual) * np.sqrt(cond), err
    # the plan's own outcome decides, and is reported
    assert bool(r.accepted) == (r.plan_residual <= TOL)
    assert bool(r.fallback) == (not r.accepted)
    if r.accepted:
        assert r.plan_residual == r.final_residual and r.corrections == sweeps
    else:
        assert 1 <= r.corrections <= 4
    if sweeps == 0:
        # X0 carries the basis quantization (BF16 ~3e-3, FP8 ~5e-2)
        assert not r.accepted and r.plan_residual == r.initial_residual
        assert r.plan_residual > {"bf16": 1e-3, "fp8row": 1e-2}[fmt]
    if fmt == "bf16" and sweeps == 2 and cond <= 1e4:
        assert r.accepted, r.plan_residual


def test_order_8192_clustered_mxfp4(ctx, msq):
    """n = 8192, condition 1e4, clustered spectrum (90% of the eigenvalues in
    [0.9, 1.1], 10% log-uniform down to 1e-4), MXFP4 basis (kind::mxf4
    reconstruction) and two Sylvester sweeps.  The 4-bit X0 is too far from
    the root for the frozen-basis corrections at this order and spectrum
    (its error exceeds the smallest root eigenvalues, so Newton does not
    contract): the plan must report that it missed the tolerance, and the
    FP32 fallback's root must meet it.  FP64 residual and forward error
    against the FP64 eigendecomposition root."""
    n, cond = 8192, 1e4
    a = O.spd_clustered(n, cond, seed=8192).astype(np.float32).astype(np.float64)
    x, r = _solve(ctx, msq, a, msq.plan(msq.PLAN_MXFP4, 2, 1e-3, 20))
    resid = O.relative_residual(a, x)
    assert abs(resid - r.final_residual) <= 1e-3 * resid + ROUNDING
    assert r.final_residual <= TOL
    assert bool(r.accepted) == (r.plan_residual <= TOL)
    assert bool(r.fallback) == (not r.accepted)
    assert r.initial_residual > 1e-2  # the 4-bit X0
    assert np.abs(x - x.T).max() <= 1e-6 * np.abs(x).max()
    err = O.relative_error(x, O.reference_root(a))
    assert err <= 10 * TOL * np.sqrt(cond), err
