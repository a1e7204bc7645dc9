"""Batched Jacobi for 256 < n <= 512 in the two-level pairing.

VECTORS_BLOCKED (FP32 replay) must agree bit for bit with the oracle's
blocked Jacobi in the same order.  VECTORS_TENSOR keeps those rotations of A
(bit-exact) and accumulates V with split-BF16 tcgen05 GEMMs.
VECTORS_TENSOR_A rotates only the 64x64 diagonal blocks on the CUDA cores
and brings the rest of A up to date once per stage on the tensor cores too.
The tensor-core results are checked within the split-BF16 error (about
2^-16 relative per product): against FP64 (orthonormal V, A V = V diag(w),
eigenvalues) and against the oracle."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

# nine orders above 256 keep the batch on the one-CTA-per-matrix kernels;
# block counts 66, 76, 84, 84, 100, 112, 118, 128, 66: ragged and empty
# super-blocks, shared- and global-tile sweep classes
ORDERS = [257, 300, 330, 336, 400, 448, 470, 512, 264]


def _mats():
    return [O.wishart(n, seed=1000 + n) for n in ORDERS]


def _run(ctx, msq, mats, mode, tol, max_sweeps):
    import torch
    b = msq.Batch.from_orders([m.shape[0] for m in mats])
    a = torch.from_numpy(b.pack(mats)).cuda()
    ctx.set_jacobi_vectors(mode)
    try:
        v, w, sweeps, off = ctx.jacobi(a, b, tol, max_sweeps)
        torch.cuda.synchronize()
        ctx.synchronize()
    finally:
        ctx.set_jacobi_vectors(msq.VECTORS_AUTO)
    vs = b.unpack(v.cpu().numpy())
    eo = b.eig_offset
    ws = [w.cpu().numpy()[eo[i]:eo[i] + b.n[i]] for i in range(b.count)]
    return vs, ws, sweeps.cpu().numpy(), off.cpu().numpy(), b.unpack(a.cpu().numpy())


def test_blocked_mode_bit_exact(ctx, msq):
    mats = _mats()
    vs, ws, sweeps, _, af = _run(ctx, msq, mats, msq.VECTORS_BLOCKED, 0.0, 3)
    for i, a in enumerate(mats):
        w_o, v_o, sw_o, _, a_o = O.jacobi_blocked(a, 0.0, 3, with_matrix=True, two_level=True)
        assert int(sweeps[i]) == sw_o == 3
        assert np.array_equal(ws[i], w_o), ORDERS[i]
        assert np.array_equal(vs[i], v_o), ORDERS[i]
        assert np.array_equal(af[i], a_o), ORDERS[i]


def test_tensor_vectors_against_oracle(ctx, msq):
    """VECTORS_TENSOR: the rotations of A are the FP32 two-level ones
    (eigenvalues and rotated matrix bit-exact with the oracle); V is
    accumulated with split-BF16 tcgen05 GEMMs, within the split's error of
    the oracle's FP32 V (about 2^-16 relative per stage product; the entries
    of V are O(n^-1/2))."""
    mats = _mats()
    vs, ws, sweeps, _, af = _run(ctx, msq, mats, msq.VECTORS_TENSOR, 0.0, 3)
    for i, a in enumerate(mats):
        n = ORDERS[i]
        w_o, v_o, _, _, a_o = O.jacobi_blocked(a, 0.0, 3, with_matrix=True, two_level=True)
        assert int(sweeps[i]) == 3
        assert np.array_equal(ws[i], w_o), n
        assert np.array_equal(af[i], a_o), n
        err = np.abs(vs[i].astype(np.float64) - v_o).max()
        assert err <= 2e-3 / np.sqrt(n), (n, err)
        v = vs[i].astype(np.float64)
        assert np.abs(v.T @ v - np.eye(n)).max() <= 1e-4, n


def test_tensor_blocks_fixed_sweeps(ctx, msq):
    """VECTORS_TENSOR_A, three sweeps: the diagonal blocks rotate on the CUDA
    cores, the rest of A and V on the tensor cores.  The returned matrix is
    V^T A V (to the split-BF16 accuracy), V is orthonormal, and the off-norm
    falls like the oracle's two-level FP32 sweeps."""
    mats = _mats()
    vs, ws, sweeps, off, af = _run(ctx, msq, mats, msq.VECTORS_TENSOR_A, 0.0, 3)
    for i, a in enumerate(mats):
        n = ORDERS[i]
        _, _, _, off_o, _ = O.jacobi_blocked(a, 0.0, 3, with_matrix=True, two_level=True)
        assert int(sweeps[i]) == 3
        v = vs[i].astype(np.float64)
        assert np.abs(v.T @ v - np.eye(n)).max() <= 1e-4, (n, np.abs(v.T @ v - np.eye(n)).max())
        dev = np.linalg.norm(af[i] - v.T @ a @ v) / np.linalg.norm(a)
        assert dev <= 1e-4, (n, dev)
        assert off[i] <= 2 * off_o + 1e-4, (n, off[i], off_o)


@pytest.mark.parametrize("mode", ["VECTORS_TENSOR", "VECTORS_TENSOR_A"])
def test_tensor_modes_converged_eigenpairs(ctx, msq, mode):
    mats = _mats()
    vs, ws, sweeps, off, _ = _run(ctx, msq, mats, getattr(msq, mode), 1e-4, 15)
    for i, a in enumerate(mats):
        n = ORDERS[i]
        assert off[i] <= 1e-4 and sweeps[i] < 15
        v, w = vs[i].astype(np.float64), ws[i].astype(np.float64)
        lam = np.linalg.eigvalsh(a)
        assert np.abs(np.sort(w) - lam).max() <= 3 * n * 2.0 ** -24 * lam.max() + 2e-4 * lam.max()
        assert np.abs(v.T @ v - np.eye(n)).max() <= 2e-4, n
        assert np.linalg.norm(a @ v - v * w) / np.linalg.norm(a) <= 3e-4, n


def test_bf16_plan_solves_with_tensor_vectors(ctx, msq):
    """msq_solve_batched picks the tensor-core eigenvectors for low-bit plans
    (automatic mode); every matrix still meets 1e-5 after one Sylvester
    sweep, checked in FP64 on the host."""
    import torch
    mats = _mats() + [O.wishart(n, seed=7 + n) for n in (290, 380, 500)]
    b = msq.Batch.from_orders([m.shape[0] for m in mats])
    a = torch.from_numpy(b.pack(mats)).cuda()
    plans = [msq.plan(msq.PLAN_BF16, 1, 1e-4, 20)] * len(mats)
    root, res = ctx.solve_batched(a, b, plans, tolerance=1e-5)
    torch.cuda.synchronize()
    xs = b.unpack(root.cpu().numpy())
    for i, m in enumerate(mats):
        r = O.relative_residual(m, xs[i].astype(np.float64))
        assert r <= 1e-5 + 1e-7, (m.shape[0], r, res[i].fallback)
