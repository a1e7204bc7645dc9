// Learned plan selector: per-matrix features and a 16 -> 64 -> 64 -> 8 MLP
// with hand-written forward, backward and Adam kernels.
//
// The reference picks precision plans by fixed rules: runAdaptiveMetalCase
// always takes FP32 ("latency_first", src/metal_solver.cpp:976-1001), stage 3
// allows low-bit products only below condition 1000
// (3_spectral/spectral.cpp:837-838), and a low-precision factor that fails
// its gate escalates to FP32 (src/metal_solver.cpp:225-235).  This network
// replaces the rules: output k is the logit of "plan k meets the requested
// tolerance" for the matrix described by the features, trained with a
// sigmoid cross-entropy on outcomes the solver itself produced; the caller
// picks the cheapest plan whose probability clears a threshold and the
// float-float residual check still falls back to FP32 on a miss.
//
// Parameters: one FP32 master array (W1[64][16], b1[64], W2[64][64], b2[64],
// W3[8][64], b3[8]); forward and backward read BF16-rounded weights (the
// codec's RNE, src/storage_codecs.cpp:16-28) and accumulate in FP32.
#include "msq_codec_device.cuh"
#include "msq_internal.cuh"

namespace msq {
namespace {

constexpr int kIn = MSQ_MLP_IN, kHid = MSQ_MLP_HIDDEN, kOut = MSQ_MLP_OUT;
constexpr int kW1 = 0, kB1 = kW1 + kHid * kIn, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid,
              kW3 = kB2 + kHid, kB3 = kW3 + kOut * kHid, kParams = kB3 + kOut;
static_assert(kParams == MSQ_MLP_PARAMS, "parameter layout");

__device__ __forceinline__ float bf16Round(float x) { return decodeBf16(encodeBf16(x)); }

// Features of one matrix (one CTA), all from O(n^2) passes:
//  0 log2 n            1 log10 trace/n        2 log10 ||A||_F / n
//  3 log10 min diag    4 log10 max diag       5 log10(max/min diag)
//  6 Gershgorin lower / (trace/n) (clamped)   7 log10 Gershgorin upper/(trace/n)
//  8 off-diagonal Frobenius mass / ||A||_F    9 max row off-diag sum / min diag
// 10 mean |a_ij| off-diagonal / mean diag     11 log10 (||A||_F^2 / trace^2 * n)
// 12 std diag / mean diag                     13 fraction of rows diagonally dominant
// 14 log10 tolerance (filled by the caller; 0 here)   15 bias term 1
__global__ void featuresKernel(const float *__restrict__ a, const int32_t *__restrict__ nn,
                               const int64_t *__restrict__ off, float *__restrict__ out) {
  const int mi = blockIdx.x;
  const int n = nn[mi];
  const float *A = a + off[mi];
  __shared__ double red[8][32];
  double tr = 0, fro = 0, offm = 0, offabs = 0, dmin = 1e300, dmax = -1e300, d2 = 0;
  double glo = 1e300, ghi = -1e300, rowmax = 0, dom = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = A[i + static_cast<int64_t>(i) * n];
    double rs = 0, ro2 = 0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const double v = A[j + static_cast<int64_t>(i) * n];  // row i = column i (symmetric)
      rs += fabs(v);
      ro2 += v * v;
    }
    tr += d;
    d2 += d * d;
    fro += d * d + ro2;
    offm += ro2;
    offabs += rs;
    dmin = fmin(dmin, d);
    dmax = fmax(dmax, d);
    glo = fmin(glo, d - rs);
    ghi = fmax(ghi, d + rs);
    rowmax = fmax(rowmax, rs);
    dom += d > rs ? 1.0 : 0.0;
  }
  double vals[8] = {tr, fro, offm, offabs, d2, dom, 0, 0};
  double mins[2] = {dmin, glo}, maxs[3] = {dmax, ghi, rowmax};
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32, warps = blockDim.x / 32;
  for (int k = 0; k < 6; ++k) {
    double v = vals[k];
    for (int s = 16; s; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (lane == 0) red[k][warp] = v;
  }
  for (int k = 0; k < 2; ++k) {
    double v = mins[k];
    for (int s = 16; s; s >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, s));
    mins[k] = v;
  }
  for (int k = 0; k < 3; ++k) {
    double v = maxs[k];
    for (int s = 16; s; s >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, s));
    maxs[k] = v;
  }
  __shared__ double rmin[2][32], rmax[3][32];
  if (lane == 0) {
    rmin[0][warp] = mins[0]; rmin[1][warp] = mins[1];
    rmax[0][warp] = maxs[0]; rmax[1][warp] = maxs[1]; rmax[2][warp] = maxs[2];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) {
      double s = 0;
      for (int w = 0; w < warps; ++w) s += red[k][w];
      vals[k] = s;
    }
    double mn0 = 1e300, mn1 = 1e300, mx0 = -1e300, mx1 = -1e300, mx2 = 0;
    for (int w = 0; w < warps; ++w) {
      mn0 = fmin(mn0, rmin[0][w]); mn1 = fmin(mn1, rmin[1][w]);
      mx0 = fmax(mx0, rmax[0][w]); mx1 = fmax(mx1, rmax[1][w]); mx2 = fmax(mx2, rmax[2][w]);
    }
    const double trace = vals[0], fnorm = sqrt(vals[1]), mean_d = trace / n;
    const double tiny = 1e-30;
    float *f = out + static_cast<int64_t>(mi) * kIn;
    f[0] = static_cast<float>(log2(static_cast<double>(n)));
    f[1] = static_cast<float>(log10(fmax(mean_d, tiny)));
    f[2] = static_cast<float>(log10(fmax(fnorm / n, tiny)));
    f[3] = static_cast<float>(log10(fmax(mn0, tiny)));
    f[4] = static_cast<float>(log10(fmax(mx0, tiny)));
    f[5] = static_cast<float>(log10(fmax(mx0, tiny) / fmax(mn0, tiny)));
    f[6] = static_cast<float>(fmax(-10.0, fmin(1.0, mn1 / fmax(mean_d, tiny))));
    f[7] = static_cast<float>(log10(fmax(mx1, tiny) / fmax(mean_d, tiny)));
    f[8] = static_cast<float>(sqrt(vals[2]) / fmax(fnorm, tiny));
    f[9] = static_cast<float>(fmin(100.0, mx2 / fmax(mn0, tiny)));
    f[10] = static_cast<float>(n > 1 ? (vals[3] / (static_cast<double>(n) * (n - 1))) / fmax(mean_d, tiny) : 0.0);
    f[11] = static_cast<float>(log10(fmax(vals[1] * n / fmax(trace * trace, tiny), tiny)));
    f[12] = static_cast<float>(sqrt(fmax(vals[4] / n - mean_d * mean_d, 0.0)) / fmax(mean_d, tiny));
    f[13] = static_cast<float>(vals[5] / n);
    f[14] = 0.0f;
    f[15] = 1.0f;
  }
}

// Forward for rows of features: thread block of 64 threads, 8 rows per block
// iteration; h1 and h2 staged in shared memory.  Logits are FP32.
template <bool kKeep>
__device__ void mlpForwardRow(const float *__restrict__ p, const float *__restrict__ x,
                              float *h1, float *h2, float *z) {
  const int t = threadIdx.x;  // hidden unit
  float s = bf16Round(p[kB1 + t]);
  for (int i = 0; i < kIn; ++i) s = fmaf(bf16Round(p[kW1 + t * kIn + i]), x[i], s);
  h1[t] = fmaxf(s, 0.0f);
  __syncthreads();
  s = bf16Round(p[kB2 + t]);
  for (int i = 0; i < kHid; ++i) s = fmaf(bf16Round(p[kW2 + t * kHid + i]), h1[i], s);
  h2[t] = fmaxf(s, 0.0f);
  __syncthreads();
  if (t < kOut) {
    s = bf16Round(p[kB3 + t]);
    for (int i = 0; i < kHid; ++i) s = fmaf(bf16Round(p[kW3 + t * kHid + i]), h2[i], s);
    z[t] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(64) mlpForwardKernel(const float *__restrict__ p,
                                                       const float *__restrict__ x, int rows,
                                                       float *__restrict__ logits) {
  __shared__ float xs[kIn], h1[kHid], h2[kHid], z[kOut];
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    if (threadIdx.x < kIn) xs[threadIdx.x] = x[static_cast<int64_t>(r) * kIn + threadIdx.x];
    __syncthreads();
    mlpForwardRow<false>(p, xs, h1, h2, z);
    if (threadIdx.x < kOut) logits[static_cast<int64_t>(r) * kOut + threadIdx.x] = z[threadIdx.x];
    __syncthreads();
  }
}

// Backward of L = mean over rows and outputs of softplus(z) - y z (sigmoid
// cross-entropy), accumulating dL/dparams (w.r.t. the FP32 masters, through
// the BF16 rounding as a straight-through identity) with block-local
// partial sums flushed by atomics.  loss gets the mean loss.
__global__ void __launch_bounds__(64) mlpBackwardKernel(const float *__restrict__ p,
                                                        const float *__restrict__ x,
                                                        const float *__restrict__ y, int rows,
                                                        float *__restrict__ grad,
                                                        float *__restrict__ loss) {
  __shared__ float xs[kIn], h1[kHid], h2[kHid], z[kOut], dz[kOut], dh2[kHid], dh1[kHid];
  const int t = threadIdx.x;
  // per-thread accumulators for the rows this block handles
  float gW1[kIn], gB1 = 0.0f, gW2[kHid], gB2 = 0.0f, gW3[kHid], gB3 = 0.0f;
  for (int i = 0; i < kIn; ++i) gW1[i] = 0.0f;
  for (int i = 0; i < kHid; ++i) { gW2[i] = 0.0f; gW3[i] = 0.0f; }
  float lsum = 0.0f;
  const float inv = 1.0f / (static_cast<float>(rows) * kOut);
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    if (t < kIn) xs[t] = x[static_cast<int64_t>(r) * kIn + t];
    __syncthreads();
    mlpForwardRow<true>(p, xs, h1, h2, z);
    if (t < kOut) {
      const float zz = z[t], yy = y[static_cast<int64_t>(r) * kOut + t];
      const float sig = 1.0f / (1.0f + expf(-zz));
      dz[t] = (sig - yy) * inv;
      lsum += (fmaxf(zz, 0.0f) + log1pf(expf(-fabsf(zz))) - yy * zz) * inv;
    }
    __syncthreads();
    // layer 3: thread t < 8 owns output t
    if (t < kOut) {
      for (int i = 0; i < kHid; ++i) gW3[i] += dz[t] * h2[i];
      gB3 += dz[t];
    }
    // dh2
    {
      float s = 0.0f;
      for (int o = 0; o < kOut; ++o) s = fmaf(bf16Round(p[kW3 + o * kHid + t]), dz[o], s);
      dh2[t] = h2[t] > 0.0f ? s : 0.0f;
    }
    __syncthreads();
    for (int i = 0; i < kHid; ++i) gW2[i] += dh2[t] * h1[i];
    gB2 += dh2[t];
    {
      float s = 0.0f;
      for (int o = 0; o < kHid; ++o) s = fmaf(bf16Round(p[kW2 + o * kHid + t]), dh2[o], s);
      dh1[t] = h1[t] > 0.0f ? s : 0.0f;
    }
    __syncthreads();
    for (int i = 0; i < kIn; ++i) gW1[i] += dh1[t] * xs[i];
    gB1 += dh1[t];
    __syncthreads();
  }
  for (int i = 0; i < kIn; ++i) atomicAdd(&grad[kW1 + t * kIn + i], gW1[i]);
  atomicAdd(&grad[kB1 + t], gB1);
  for (int i = 0; i < kHid; ++i) atomicAdd(&grad[kW2 + t * kHid + i], gW2[i]);
  atomicAdd(&grad[kB2 + t], gB2);
  if (t < kOut) {
    for (int i = 0; i < kHid; ++i) atomicAdd(&grad[kW3 + t * kHid + i], gW3[i]);
    atomicAdd(&grad[kB3 + t], gB3);
    atomicAdd(loss, lsum);
  }
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on the FP32 masters.
__global__ void adamKernel(float *__restrict__ p, const float *__restrict__ g,
                           float *__restrict__ m, float *__restrict__ v, int step, float lr) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, static_cast<float>(step));
  const float c2 = 1.0f - powf(b2, static_cast<float>(step));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
    m[i] = b1 * m[i] + (1.0f - b1) * g[i];
    v[i] = b2 * v[i] + (1.0f - b2) * g[i] * g[i];
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + 1e-8f);
  }
}

}  // namespace
}  // namespace msq

using namespace msq;

extern "C" int msq_features(msq_ctx *ctx, const float *a, const int32_t *n, const int64_t *offset,
                            int count, float *features) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!a || !features) return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_features: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  featuresKernel<<<count, 128, 0, ctx->stream>>>(a, b->n, b->offset, features);
  return launched(ctx, "mlp features");
}

extern "C" int msq_mlp_forward(msq_ctx *ctx, const float *params, const float *features, int rows,
                               float *logits) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!params || !features || !logits || rows < 0)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_mlp_forward: bad argument");
  if (rows == 0) return MSQ_OK;
  mlpForwardKernel<<<std::min(rows, kSmCount * 16), 64, 0, ctx->stream>>>(params, features, rows,
                                                                          logits);
  return launched(ctx, "mlp forward");
}

extern "C" int msq_mlp_backward(msq_ctx *ctx, const float *params, const float *features,
                                const float *targets, int rows, float *grad_params, float *loss) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!params || !features || !targets || !grad_params || !loss || rows <= 0)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_mlp_backward: bad argument");
  mlpBackwardKernel<<<std::min(rows, kSmCount * 4), 64, 0, ctx->stream>>>(
      params, features, targets, rows, grad_params, loss);
  return launched(ctx, "mlp backward");
}

extern "C" int msq_mlp_step(msq_ctx *ctx, float *params, const float *grad_params, float *adam_m,
                            float *adam_v, int step, float learning_rate) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!params || !grad_params || !adam_m || !adam_v || step < 1)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_mlp_step: bad argument");
  adamKernel<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(params, grad_params, adam_m, adam_v,
                                                             step, learning_rate);
  return launched(ctx, "mlp adam");
}
