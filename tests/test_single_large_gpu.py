"""Single large matrices through msq_solve_batched: the grid eigensolver, the
tcgen05 low-bit reconstruction and the Sylvester sweeps at the orders of the
single-matrix low-bit sweep (n = 1024 ... 4096, condition 1e2 ... 1e6) and of
the MXFP4 case (n = 8192, clustered spectrum).  Checked against FP64: the
reported float-float residual equals ||A - X^2||_F / ||A||_F computed in FP64
on the host, and the forward error against the FP64 eigendecomposition root
stays within the conditioning bound."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5
# the root is returned in FP32: rounding X (float-float inside the solver)
# to FP32 alone moves ||A - X^2|| / ||A|| by up to a few units of 2^-24
ROUNDING = 1e-7


def _solve(ctx, msq, a64, plan):
    import torch
    n = a64.shape[0]
    b = msq.Batch.from_orders([n])
    a = torch.from_numpy(b.pack([a64])).cuda()
    root, res = ctx.solve_batched(a, b, [plan], tolerance=TOL)
    torch.cuda.synchronize()
    return b.unpack(root.cpu().numpy())[0].astype(np.float64), res[0]


@pytest.mark.parametrize("n,cond", [(1024, 1e2), (1024, 1e6), (2048, 1e4)])
@pytest.mark.parametrize("fmt,sweeps", [("bf16", 1), ("fp8row", 2)])
def test_low_bit_plans_at_large_order(ctx, msq, n, cond, fmt, sweeps):
    a = O.spd_loguniform(n, cond, seed=n + int(np.log10(cond)))
    fmt_id = {"bf16": msq.PLAN_BF16, "fp8row": msq.PLAN_FP8}[fmt]
    jac_tol = {1: 1e-4, 2: 1e-3}[sweeps]
    x, r = _solve(ctx, msq, a, msq.plan(fmt_id, sweeps, jac_tol, 20))
    resid = O.relative_residual(a, x)
    # the reported residual (float-float X) is the FP64 one of the root
    # before its rounding to FP32
    assert abs(resid - r.final_residual) <= 1e-3 * resid + ROUNDING, (resid, r.final_residual)
    assert r.final_residual <= TOL
    # forward error: a residual eps moves the root by about eps * sqrt(cond)
    err = O.relative_error(x, O.reference_root(a))
    assert err <= 10 * TOL * np.sqrt(cond), err


def test_order_4096_bf16_two_sweeps(ctx, msq):
    n = 4096
    a = O.spd_loguniform(n, 1e2, seed=7)
    x, r = _solve(ctx, msq, a, msq.plan(msq.PLAN_BF16, 2, 1e-3, 20))
    resid = O.relative_residual(a, x)
    assert abs(resid - r.final_residual) <= 1e-3 * resid + ROUNDING
    assert r.final_residual <= TOL and not r.fallback


def test_order_8192_clustered_mxfp4(ctx, msq):
    """n = 8192, condition 1e4, clustered spectrum (90% of the eigenvalues in
    [0.9, 1.1]), MXFP4 basis and two Sylvester sweeps.  The FP64 check is the
    residual of the returned root on the host (no FP64 eigendecomposition
    at this order in a test)."""
    n = 8192
    a = O.spd_clustered(n, 1e4, seed=8192)
    x, r = _solve(ctx, msq, a, msq.plan(msq.PLAN_MXFP4, 2, 1e-3, 20))
    resid = O.relative_residual(a, x)
    assert abs(resid - r.final_residual) <= 1e-3 * resid + ROUNDING
    assert r.final_residual <= TOL
    assert np.abs(x - x.T).max() <= 1e-6 * np.abs(x).max()
