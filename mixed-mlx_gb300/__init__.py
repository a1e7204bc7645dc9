"""Python host side of the GB300 SPD square-root pipeline.

A thin ctypes layer over the C ABI declared in include/msq_cuda.h
(libmsq_cuda.so, built in-tree by build.py).  PyTorch supplies device memory
and streams only; every computation runs in this library's CUDA kernels.
There is no CPU fallback: if the shared library is missing, or no GPU is
present, the calls raise.

The names mirror the reference's operator/codec API:
  * copy_to_storage / storage_values  -> copyToStorage / storageValueAt
    (src/storage_codecs.hpp:20-24)
  * Context.solve_batched             -> solveGpuResidentSpd over a batch
    (src/metal_solver.cpp:92-336)
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmsq_cuda.so")

# Storage formats; ids 0..7 equal the reference's HostStorageCodec.
FP32, BF16, FP8_E4M3FN, FP8_E5M2, MXFP8_E4M3FN, MXFP8_E5M2, FP4_E2M1, MXFP4_E2M1, \
    FP8_E4M3FN_ROWSCALE = range(9)
FORMAT_NAMES = {
    FP32: "fp32", BF16: "bf16", FP8_E4M3FN: "fp8_e4m3fn", FP8_E5M2: "fp8_e5m2",
    MXFP8_E4M3FN: "mxfp8_e4m3fn", MXFP8_E5M2: "mxfp8_e5m2", FP4_E2M1: "fp4_e2m1",
    MXFP4_E2M1: "mxfp4_e2m1", FP8_E4M3FN_ROWSCALE: "fp8_e4m3fn_rowscale",
}
# Rounding modes of msq_spectrum_encode (the reference's --rounding).
ROUND_NEAREST = 0
ROUND_STOCHASTIC = 1

# Plans (msq_plan_format)
PLAN_FP32, PLAN_BF16, PLAN_FP8, PLAN_MXFP4 = range(4)
# msq_set_jacobi_vectors modes
VECTORS_AUTO, VECTORS_REPLAY, VECTORS_BLOCKED, VECTORS_TENSOR, VECTORS_TENSOR_A = -1, 0, 1, 2, 3

MLP_IN, MLP_HIDDEN, MLP_OUT = 16, 64, 8
MLP_PARAMS = (MLP_IN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN +
              MLP_HIDDEN + MLP_HIDDEN * MLP_OUT + MLP_OUT)


class MsqError(RuntimeError):
    pass


class Plan(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int32), ("sweeps", ctypes.c_int32),
                ("jacobi_tolerance", ctypes.c_double),
                ("jacobi_max_sweeps", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class SolveResult(ctypes.Structure):
    _fields_ = [("final_residual", ctypes.c_double),
                ("initial_residual", ctypes.c_double),
                ("jacobi_sweeps", ctypes.c_int32), ("corrections", ctypes.c_int32),
                ("accepted", ctypes.c_int32), ("fallback", ctypes.c_int32),
                ("plan_residual", ctypes.c_double)]


_LIB = None

_P = ctypes.c_void_p
_SIGS = {
    "msq_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    "msq_destroy": (None, [_P]),
    "msq_last_error": (ctypes.c_char_p, [_P]),
    "msq_set_stream": (ctypes.c_int, [_P, _P]),
    "msq_synchronize": (ctypes.c_int, [_P]),
    "msq_debug_expire_waits": (ctypes.c_int, [ctypes.c_int]),
    "msq_launch_count": (ctypes.c_uint64, [_P]),
    "msq_graph_launch_count": (ctypes.c_uint64, [_P]),
    "msq_fma_rate": (ctypes.c_int, [_P, _P]),
    "msq_storage_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_size_t]),
    "msq_scale_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]),
    "msq_encode": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_size_t, _P, _P]),
    "msq_decode": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, ctypes.c_size_t, ctypes.c_size_t, _P]),
    "msq_encode_stochastic": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_size_t,
                                             ctypes.c_uint32, ctypes.c_uint32, _P, _P]),
    "msq_spectrum_metadata_bytes": (ctypes.c_size_t, [ctypes.c_size_t]),
    "msq_spectrum_encode": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_int,
                                           ctypes.c_uint32, ctypes.c_uint32, _P, _P]),
    "msq_spectrum_decode": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, ctypes.c_size_t, _P]),
    "msq_native_sylvester_sweep": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P,
                                                  ctypes.c_int, _P, _P, _P, _P, _P]),
    "msq_jacobi_batched": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int, _P, _P]),
    "msq_jacobi_noalloc": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_int, _P, _P, _P]),
    "msq_set_concurrency": (ctypes.c_int, [_P, ctypes.c_int]),
    "msq_set_graphs": (ctypes.c_int, [_P, ctypes.c_int]),
    "msq_set_jacobi_vectors": (ctypes.c_int, [_P, ctypes.c_int]),
    "msq_jacobi_schedule": (ctypes.c_int, [ctypes.c_int, _P, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_int)]),
    "msq_jacobi_route": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P]),
    "msq_autotune_report": (ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]),
    "msq_autotune_reset": (ctypes.c_int, [ctypes.c_int]),
    "msq_timing_begin": (ctypes.c_int, [_P]),
    "msq_timing_end": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "msq_make_factor": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int, _P]),
    "msq_reconstruct": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, _P, ctypes.c_int, _P]),
    "msq_reconstruct_factor": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_int, _P]),
    "msq_residual": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, ctypes.c_int, _P, _P]),
    "msq_sylvester_sweep": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, _P, _P,
                                           ctypes.c_int, _P, _P, _P]),
    "msq_solve_batched": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, _P,
                                         ctypes.c_double, _P, _P]),
    "msq_features": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, _P]),
    "msq_mlp_forward": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P]),
    "msq_mlp_backward": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, _P, _P]),
    "msq_mlp_step": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_float]),
}


def lib() -> ctypes.CDLL:
    """Load libmsq_cuda.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise MsqError(f"{LIB_PATH} is missing: run mixed-mlx_gb300/build.py "
                           "(there is no CPU fallback)")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(handle, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


def storage_bytes(fmt: int, elements: int) -> int:
    return int(lib().msq_storage_bytes(fmt, elements))


def scale_bytes(fmt: int, elements: int, row_length: int = 0) -> int:
    return int(lib().msq_scale_bytes(fmt, elements, row_length))


def _ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


@dataclass
class Batch:
    """Packed batch of square matrices (column-major, back to back)."""
    n: np.ndarray        # int32 [count]
    offset: np.ndarray   # int64 [count] element offsets
    total: int

    @property
    def count(self) -> int:
        return int(self.n.shape[0])

    @property
    def eig_offset(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum(self.n[:-1].astype(np.int64))]).astype(np.int64)

    @staticmethod
    def from_orders(orders: Sequence[int], align: int = 4) -> "Batch":
        n = np.asarray(orders, dtype=np.int32)
        sizes = n.astype(np.int64) ** 2
        padded = (sizes + align - 1) // align * align  # 16-byte aligned starts
        offset = np.concatenate([[0], np.cumsum(padded[:-1])]).astype(np.int64)
        return Batch(n, offset, int(padded.sum()))

    def pack(self, mats: Sequence[np.ndarray]) -> np.ndarray:
        flat = np.zeros(self.total, dtype=np.float32)
        for i, m in enumerate(mats):
            k = int(self.n[i])
            flat[self.offset[i]:self.offset[i] + k * k] = np.asarray(m, np.float32).reshape(-1, order="F")
        return flat

    def unpack(self, flat: np.ndarray, dtype=np.float64) -> list[np.ndarray]:
        out = []
        for i in range(self.count):
            k = int(self.n[i])
            out.append(np.asarray(flat[self.offset[i]:self.offset[i] + k * k], dtype).reshape(k, k, order="F"))
        return out


def jacobi_schedule(blocks: int) -> np.ndarray:
    """The library's two-level pair table for `blocks` 4-index blocks
    (host-side, no GPU): (rounds, blocks/2, 2) int32 pairs (I, J), with
    J = -1 - J for an identity pair."""
    rounds = ctypes.c_int()
    status = lib().msq_jacobi_schedule(blocks, None, 0, ctypes.byref(rounds))
    if status != 0:
        raise MsqError(f"msq_jacobi_schedule({blocks}): status {status}")
    out = np.zeros(rounds.value * blocks, dtype=np.int32)
    status = lib().msq_jacobi_schedule(blocks, out.ctypes.data, out.size, ctypes.byref(rounds))
    if status != 0:
        raise MsqError(f"msq_jacobi_schedule({blocks}): status {status}")
    return out.reshape(rounds.value, blocks // 2, 2)


def jacobi_route(orders, mode: int = 0) -> np.ndarray:
    """Which eigensolver path each matrix of a batch takes (host-side, no
    GPU): 1 = the grid kernels with every SM, 0 = the batched kernels one CTA
    each, under eigenvector mode `mode` (VECTORS_REPLAY .. VECTORS_TENSOR_A)."""
    n = np.ascontiguousarray(orders, dtype=np.int32)
    out = np.zeros(n.size, dtype=np.int32)
    status = lib().msq_jacobi_route(n.ctypes.data, n.size, mode, out.ctypes.data)
    if status != 0:
        raise MsqError(f"msq_jacobi_route: status {status}")
    return out


class Context:
    """Owns one msq_ctx bound to a CUDA device and torch's current stream."""

    def __init__(self, device: int = 0):
        import torch
        if not torch.cuda.is_available():
            raise MsqError("CUDA device required: this library has no CPU path")
        self.torch = torch
        self.device = device
        torch.cuda.set_device(device)
        handle = _P()
        status = lib().msq_create(ctypes.byref(handle), device)
        if status != 0:
            raise MsqError(f"msq_create failed with status {status}")
        self.handle = handle
        self.set_stream(torch.cuda.current_stream(device))

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().msq_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status: int, what: str) -> None:
        if status != 0:
            msg = lib().msq_last_error(self.handle)
            raise MsqError(f"{what}: status {status}: {msg.decode() if msg else ''}")

    def set_stream(self, stream) -> None:
        self.stream = stream
        self.check(lib().msq_set_stream(self.handle, ctypes.c_void_p(stream.cuda_stream)),
                   "msq_set_stream")

    def set_concurrency(self, enable: bool) -> None:
        self.check(lib().msq_set_concurrency(self.handle, int(bool(enable))), "msq_set_concurrency")

    def set_graphs(self, enable: bool) -> None:
        self.check(lib().msq_set_graphs(self.handle, int(bool(enable))), "msq_set_graphs")

    def set_jacobi_vectors(self, mode: int) -> None:
        """Eigenvector mode of the batched Jacobi for 256 < n <= 512:
        VECTORS_AUTO, VECTORS_REPLAY, VECTORS_BLOCKED, VECTORS_TENSOR or
        VECTORS_TENSOR_A."""
        self.check(lib().msq_set_jacobi_vectors(self.handle, int(mode)), "msq_set_jacobi_vectors")

    def synchronize(self) -> None:
        self.check(lib().msq_synchronize(self.handle), "msq_synchronize")

    @property
    def launches(self) -> int:
        return int(lib().msq_launch_count(self.handle))

    @property
    def graph_launches(self) -> int:
        return int(lib().msq_graph_launch_count(self.handle))

    def fma_rate(self) -> float:
        """Measured FP32 FMA throughput of the device, TFLOP/s."""
        out = ctypes.c_double()
        self.check(lib().msq_fma_rate(self.handle, ctypes.byref(out)), "msq_fma_rate")
        return out.value

    def autotune_report(self) -> str:
        """The launch-shape autotuner's decisions for this context's device."""
        buf = ctypes.create_string_buffer(4096)
        self.check(lib().msq_autotune_report(self.device, buf, len(buf)), "msq_autotune_report")
        return buf.value.decode()

    # ---- codecs -------------------------------------------------------
    def copy_to_storage(self, fmt: int, source, row_length: int = 0):
        """copyToStorage: returns (values uint8, scales uint8 or None)."""
        torch = self.torch
        n = source.numel()
        values = torch.empty(max(storage_bytes(fmt, n), 1), dtype=torch.uint8, device=source.device)
        sb = scale_bytes(fmt, n, row_length)
        scales = torch.empty(sb, dtype=torch.uint8, device=source.device) if sb else None
        self.check(lib().msq_encode(self.handle, fmt, _ptr(source), n, row_length,
                                    _ptr(values), _ptr(scales)), "msq_encode")
        return values, scales

    def storage_values(self, fmt: int, values, scales, elements: int, row_length: int = 0):
        """storageValueAt for every index: FP32 tensor of `elements`."""
        out = self.torch.empty(elements, dtype=self.torch.float32, device=values.device)
        self.check(lib().msq_decode(self.handle, fmt, _ptr(values), _ptr(scales), elements,
                                    row_length, _ptr(out)), "msq_decode")
        return out

    def copy_to_storage_stochastic(self, fmt: int, source, seed: int, stream: int,
                                   row_length: int = 0):
        """The device quantizers' stochastic rounding (--rounding stochastic):
        returns (values uint8, scales uint8 or None) as copy_to_storage."""
        torch = self.torch
        n = source.numel()
        values = torch.empty(max(storage_bytes(fmt, n), 1), dtype=torch.uint8, device=source.device)
        sb = scale_bytes(fmt, n, row_length)
        scales = torch.empty(sb, dtype=torch.uint8, device=source.device) if sb else None
        self.check(lib().msq_encode_stochastic(self.handle, fmt, _ptr(source), n, row_length,
                                               seed & 0xffffffff, stream & 0xffffffff,
                                               _ptr(values), _ptr(scales)),
                   "msq_encode_stochastic")
        return values, scales

    def copy_spectrum_to_storage(self, fmt: int, spectrum, rounding: int = ROUND_NEAREST,
                                 seed: int = 0, stream: int = 0):
        """Log-spectrum storage (copySpectrumToStorage, device form) of finite
        positive root eigenvalues: returns (codes uint8, metadata float32 of
        (min, span) per block of 8)."""
        torch = self.torch
        n = spectrum.numel()
        values = torch.empty(max(storage_bytes(fmt, n), 1), dtype=torch.uint8, device=spectrum.device)
        meta = torch.empty(max(lib().msq_spectrum_metadata_bytes(n) // 4, 2), dtype=torch.float32,
                           device=spectrum.device)
        self.check(lib().msq_spectrum_encode(self.handle, fmt, _ptr(spectrum), n, rounding,
                                             seed & 0xffffffff, stream & 0xffffffff,
                                             _ptr(values), _ptr(meta)), "msq_spectrum_encode")
        return values, meta

    def spectrum_values(self, fmt: int, values, meta, elements: int):
        """spectrumValueAt for every index (device form): FP32 tensor."""
        out = self.torch.empty(elements, dtype=self.torch.float32, device=values.device)
        self.check(lib().msq_spectrum_decode(self.handle, fmt, _ptr(values), _ptr(meta), elements,
                                             _ptr(out)), "msq_spectrum_decode")
        return out

    # ---- pipeline stages -----------------------------------------------
    def jacobi(self, a_flat, batch: Batch, tolerance: float = 1e-7, max_sweeps: int = 15):
        torch = self.torch
        v = torch.empty_like(a_flat)
        w = torch.empty(int(batch.n.sum()), dtype=torch.float32, device=a_flat.device)
        sweeps = torch.empty(batch.count, dtype=torch.int32, device=a_flat.device)
        off = torch.empty(batch.count, dtype=torch.float32, device=a_flat.device)
        self.check(lib().msq_jacobi_batched(
            self.handle, _ptr(a_flat), _ptr(v), _ptr(w),
            batch.n.ctypes.data, batch.offset.ctypes.data, batch.count,
            tolerance, max_sweeps, _ptr(sweeps), _ptr(off)), "msq_jacobi_batched")
        return v, w, sweeps, off

    def make_factor(self, v, w, batch: Batch):
        f = self.torch.empty_like(v)
        self.check(lib().msq_make_factor(self.handle, _ptr(v), _ptr(w), batch.n.ctypes.data,
                                         batch.offset.ctypes.data, batch.count, _ptr(f)),
                   "msq_make_factor")
        return f

    def reconstruct(self, fmt: int, values, scales, batch: Batch, out=None):
        if out is None:
            out = self.torch.empty(batch.total, dtype=self.torch.float32, device=values.device)
        self.check(lib().msq_reconstruct(self.handle, fmt, _ptr(values), _ptr(scales),
                                         batch.n.ctypes.data, batch.offset.ctypes.data,
                                         batch.count, _ptr(out)), "msq_reconstruct")
        return out

    def reconstruct_factor(self, plan_format: int, factor_t, batch: Batch, out=None):
        """X0 from the FP32 factor quantized to a plan format (the solver's stage)."""
        if out is None:
            out = self.torch.empty(batch.total, dtype=self.torch.float32, device=factor_t.device)
        self.check(lib().msq_reconstruct_factor(self.handle, plan_format, _ptr(factor_t),
                                                batch.n.ctypes.data, batch.offset.ctypes.data,
                                                batch.count, _ptr(out)), "msq_reconstruct_factor")
        return out

    def residual(self, a, x_hi, x_lo, batch: Batch, want_r: bool = True, a_lo=None):
        """R = (a + a_lo) - (x_hi + x_lo)^2 in float-float; returns (R, norms)
        with norms[2i] = ||R_i||^2, norms[2i+1] = ||A_i||^2 (FP64)."""
        torch = self.torch
        r = torch.empty_like(a) if want_r else None
        norms = torch.empty(2 * batch.count, dtype=torch.float64, device=a.device)
        self.check(lib().msq_residual(self.handle, _ptr(a), _ptr(a_lo), _ptr(x_hi), _ptr(x_lo),
                                      batch.n.ctypes.data, batch.offset.ctypes.data,
                                      batch.count, _ptr(r), _ptr(norms)), "msq_residual")
        return r, norms

    def native_sylvester_sweep(self, fmt: int, v, vt, s, r, batch: Batch, x_hi, x_lo):
        """One native-quantized correction (every operand and intermediate
        in `fmt`); v / vt: decoded stored V and V^T, s: decoded root
        eigenvalues (sum of n floats); updates x_hi / x_lo."""
        torch = self.torch
        workspace = torch.empty(3 * batch.total, dtype=torch.float32, device=v.device)
        self.check(lib().msq_native_sylvester_sweep(
            self.handle, fmt, _ptr(v), _ptr(vt), _ptr(s), _ptr(r), batch.n.ctypes.data,
            batch.offset.ctypes.data, batch.count, _ptr(x_hi), _ptr(x_lo), _ptr(workspace),
            None, None), "msq_native_sylvester_sweep")

    def sylvester_sweep(self, gemm_fmt: int, v, w, r, batch: Batch, x_hi, x_lo, workspace=None):
        if workspace is None:
            workspace = self.torch.empty(2 * batch.total, dtype=self.torch.float32, device=v.device)
        self.check(lib().msq_sylvester_sweep(self.handle, gemm_fmt, _ptr(v), _ptr(w), _ptr(r),
                                             batch.n.ctypes.data, batch.offset.ctypes.data,
                                             batch.count, _ptr(x_hi), _ptr(x_lo),
                                             _ptr(workspace)), "msq_sylvester_sweep")

    def solve_batched(self, a_flat, batch: Batch, plans=None, tolerance: float = 1e-5,
                      out=None, results: bool = True):
        torch = self.torch
        if out is None:
            out = torch.empty_like(a_flat)
        plan_arr = None
        if plans is not None:
            plan_arr = (Plan * batch.count)()
            for i, p in enumerate(plans):
                plan_arr[i] = p
        res_arr = (SolveResult * batch.count)() if results else None
        self.check(lib().msq_solve_batched(
            self.handle, _ptr(a_flat), batch.n.ctypes.data, batch.offset.ctypes.data,
            batch.count, ctypes.cast(plan_arr, _P) if plan_arr is not None else None,
            tolerance, _ptr(out), ctypes.cast(res_arr, _P) if res_arr is not None else None),
            "msq_solve_batched")
        return out, res_arr

    # ---- learned plan selector --------------------------------------------
    def features(self, a_flat, batch: Batch):
        f = self.torch.empty(batch.count * MLP_IN, dtype=self.torch.float32, device=a_flat.device)
        self.check(lib().msq_features(self.handle, _ptr(a_flat), batch.n.ctypes.data,
                                      batch.offset.ctypes.data, batch.count, _ptr(f)),
                   "msq_features")
        return f.view(batch.count, MLP_IN)

    def mlp_forward(self, params, features):
        rows = features.shape[0]
        out = self.torch.empty(rows, MLP_OUT, dtype=self.torch.float32, device=features.device)
        self.check(lib().msq_mlp_forward(self.handle, _ptr(params), _ptr(features), rows,
                                         _ptr(out)), "msq_mlp_forward")
        return out

    def mlp_backward(self, params, features, targets, grad):
        loss = self.torch.zeros(1, dtype=self.torch.float32, device=features.device)
        self.check(lib().msq_mlp_backward(self.handle, _ptr(params), _ptr(features),
                                          _ptr(targets), features.shape[0], _ptr(grad),
                                          _ptr(loss)), "msq_mlp_backward")
        return loss

    def mlp_step(self, params, grad, m, v, step: int, lr: float):
        self.check(lib().msq_mlp_step(self.handle, _ptr(params), _ptr(grad), _ptr(m), _ptr(v),
                                      step, lr), "msq_mlp_step")


def plan(fmt: int, sweeps: int, jacobi_tolerance: float = 1e-7,
         jacobi_max_sweeps: int = 15) -> Plan:
    return Plan(fmt, sweeps, jacobi_tolerance, jacobi_max_sweeps, 0)
