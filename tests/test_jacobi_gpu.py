"""GPU Jacobi parity: eigenpairs against the FP64 oracle and the CPU
restatement of the reference's parallel-order Jacobi."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
U32 = 2.0 ** -24  # FP32 unit roundoff


def _run(ctx, msq, mats, tol=1e-7, max_sweeps=15):
    import torch
    b = msq.Batch.from_orders([m.shape[0] for m in mats])
    a = torch.from_numpy(b.pack(mats)).cuda()
    v, w, sweeps, off = ctx.jacobi(a, b, tol, max_sweeps)
    torch.cuda.synchronize()
    ctx.synchronize()
    vs = b.unpack(v.cpu().numpy())
    eo = b.eig_offset
    ws = [w.cpu().numpy()[eo[i]:eo[i] + b.n[i]].astype(np.float64) for i in range(b.count)]
    return vs, ws, sweeps.cpu().numpy(), off.cpu().numpy(), b.unpack(a.cpu().numpy())


@pytest.mark.parametrize("n", [1, 2, 3, 16, 17, 31, 32, 33, 96, 128, 255, 256, 336])
def test_single_matrix_eigenpairs(ctx, msq, n):
    a = O.spd_loguniform(n, 1e3, seed=100 + n)
    vs, ws, sweeps, off, af = _run(ctx, msq, [a])
    v, w = vs[0], ws[0]
    ref = np.linalg.eigvalsh(a)
    scale = np.abs(ref).max()
    # FP32 Jacobi: eigenvalue error grows like n * u * ||A||_2
    np.testing.assert_allclose(np.sort(w), ref, rtol=0, atol=max(5e-6, 3 * n * U32) * scale)
    np.testing.assert_allclose(v.T @ v, np.eye(n), atol=5e-6 * max(1, np.sqrt(n) / 4))
    # A V = V diag(w)
    resid = np.linalg.norm(a @ v - v * w) / np.linalg.norm(a)
    assert resid < max(1e-5, n * U32)
    assert off[0] <= 1e-7 or n == 1
    # the converged matrix is written back, nearly diagonal
    assert np.linalg.norm(af[0] - np.diag(np.diag(af[0]))) <= 1e-6 * np.linalg.norm(a)


@pytest.mark.parametrize("n", [329, 400, 512, 1000])
def test_global_path_orders(ctx, msq, n):
    a = O.wishart(n, seed=n)
    vs, ws, sweeps, off, _ = _run(ctx, msq, [a])
    ref = np.linalg.eigvalsh(a)
    # FP32 Jacobi: eigenvalue error of order n * u * ||A|| (the CPU
    # restatement of the same rotations measures 1.3-1.5 n u on Wishart input)
    np.testing.assert_allclose(np.sort(ws[0]), ref, rtol=0, atol=3 * n * U32 * np.abs(ref).max())
    assert np.linalg.norm(a @ vs[0] - vs[0] * ws[0]) / np.linalg.norm(a) < n * U32


@pytest.mark.parametrize("n", [8, 24, 65, 130, 400])
def test_bit_exact_against_cpu_restatement(ctx, msq, n):
    """Same blocked round-robin order, same rotations, same FP32 roundings:
    after the same number of sweeps (tolerance 0, fixed budget) the GPU and
    the CPU restatement return identical eigenvalues, eigenvectors and
    rotated matrix, bit for bit (n = 400 runs the global-memory tile path)."""
    a = O.spd_loguniform(n, 1e2, seed=n) if n < 400 else O.wishart(n, seed=n)
    sweeps_fixed = 3
    w_o, v_o, sw_o, _, a_o = O.jacobi_blocked(a, 0.0, sweeps_fixed, with_matrix=True)
    vs, ws, sweeps, off, af = _run(ctx, msq, [a], tol=0.0, max_sweeps=sweeps_fixed)
    assert sw_o == sweeps_fixed and int(sweeps[0]) == sweeps_fixed
    assert np.array_equal(ws[0].astype(np.float32), w_o)
    assert np.array_equal(vs[0], v_o)
    assert np.array_equal(af[0], a_o)


def test_converged_sweeps_match_cpu_restatement(ctx, msq):
    """With a tolerance, both stop after the same number of sweeps (the FP64
    off-norms differ only in summation order) and agree on the spectrum."""
    for n in (8, 24, 65, 130):
        a = O.spd_loguniform(n, 1e2, seed=n)
        w_o, v_o, sw_o, off_o = O.jacobi_blocked(a, 1e-7, 15)
        vs, ws, sweeps, off, _ = _run(ctx, msq, [a])
        assert sw_o < 15 and abs(int(sweeps[0]) - sw_o) <= 1
        if int(sweeps[0]) == sw_o:
            assert np.array_equal(ws[0].astype(np.float32), w_o)
        np.testing.assert_allclose(np.sort(ws[0]), np.sort(w_o), rtol=0,
                                   atol=3 * n * U32 * np.abs(w_o).max())


def test_uneven_batch(ctx, msq):
    orders = O.wishart_orders(64, 16, 512, seed=4)
    mats = [O.wishart(int(n), seed=i) for i, n in enumerate(orders)]
    vs, ws, sweeps, off, _ = _run(ctx, msq, mats)
    for a, v, w in zip(mats, vs, ws):
        ref = np.linalg.eigvalsh(a)
        np.testing.assert_allclose(np.sort(w), ref, rtol=0,
                                   atol=max(1e-5, 3 * len(w) * U32) * np.abs(ref).max())
    assert np.all(off <= 1e-7)


def test_sweep_budget_and_tolerance(ctx, msq):
    a = O.spd_loguniform(64, 1e4, seed=1)
    _, _, sweeps, off, _ = _run(ctx, msq, [a], tol=1e-7, max_sweeps=2)
    assert sweeps[0] == 2 and off[0] > 1e-7
    _, _, sweeps, off, _ = _run(ctx, msq, [a], tol=1e-2, max_sweeps=15)
    assert off[0] <= 1e-2 and sweeps[0] < 8


# ---- grid kernels (every SM on one matrix) --------------------------------

@pytest.mark.parametrize("n", [300, 400, 1040])
def test_grid_path_bit_exact_against_cpu_restatement(ctx, msq, n):
    """A lone matrix above 256 (or any above 1024) is solved by the grid
    kernels: same rotations, same roundings as the CPU restatement."""
    a = O.wishart(n, seed=n)
    sweeps_fixed = 2 if n < 1000 else 1
    w_o, v_o, sw_o, _, a_o = O.jacobi_blocked(a, 0.0, sweeps_fixed, with_matrix=True)
    vs, ws, sweeps, off, af = _run(ctx, msq, [a], tol=0.0, max_sweeps=sweeps_fixed)
    assert int(sweeps[0]) == sweeps_fixed
    assert np.array_equal(ws[0].astype(np.float32), w_o)
    assert np.array_equal(vs[0], v_o)
    assert np.array_equal(af[0], a_o)


def test_grid_path_equals_batched_path(ctx, msq):
    """Nine matrices above 256 go to the batched kernels, one alone to the
    grid kernels: identical bits for the same matrix."""
    mats = [O.spd_loguniform(300, 1e3, seed=s) for s in range(9)]
    vs_b, ws_b, sw_b, _, af_b = _run(ctx, msq, mats, tol=0.0, max_sweeps=3)
    vs_g, ws_g, sw_g, _, af_g = _run(ctx, msq, mats[:1], tol=0.0, max_sweeps=3)
    assert np.array_equal(ws_b[0], ws_g[0])
    assert np.array_equal(vs_b[0], vs_g[0])
    assert np.array_equal(af_b[0], af_g[0])


@pytest.mark.parametrize("n", [2048, 4096])
def test_grid_path_large_orders(ctx, msq, n):
    a = O.spd_loguniform(n, 1e4, seed=n)
    vs, ws, sweeps, off, _ = _run(ctx, msq, [a], tol=1e-7, max_sweeps=20)
    ref = np.linalg.eigvalsh(a)
    assert off[0] <= 1e-7 and int(sweeps[0]) < 20
    np.testing.assert_allclose(np.sort(ws[0]), ref, rtol=0, atol=3 * n * U32 * np.abs(ref).max())
    v = vs[0].astype(np.float64)
    assert np.linalg.norm(a @ v - v * ws[0]) / np.linalg.norm(a) < n * U32
    assert np.abs(v.T @ v - np.eye(n)).max() < 1e-4


def test_batched_global_tiles_bit_exact(ctx, msq):
    """Nine matrices of order 400 stay on the batched kernels (tiles in the
    global workspace): bit-identical to the CPU restatement."""
    mats = [O.wishart(400, seed=s) for s in range(9)]
    w_o, v_o, _, _, a_o = O.jacobi_blocked(mats[0], 0.0, 2, with_matrix=True)
    vs, ws, sweeps, off, af = _run(ctx, msq, mats, tol=0.0, max_sweeps=2)
    assert np.array_equal(ws[0].astype(np.float32), w_o)
    assert np.array_equal(vs[0], v_o)
    assert np.array_equal(af[0], a_o)
