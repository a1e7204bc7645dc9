// Dense batched kernels of the square-root pipeline that run on the CUDA
// cores: the FP32 "TN" GEMM of the plain FP32 path, the float-float residual
// R = A - X*X, the eigen-factor W^T = (V diag(lambda^(1/4)))^T, transposes
// and the symmetric float-float update X <- X + (E + E^T)/2.
//
// Every GEMM of the pipeline is written as C_ij = sum_k A[k + i*lda] *
// B[k + j*ldb] ("TN": both operands column-major with K contiguous), which
// the symmetry of A, X, R, C lets us use everywhere:
//   X   = F^T F            (F = W^T, reconstruction; metal_mixed_sqrt.metal
//                           :162-206 scale_columns + matmul_tiled_f32)
//   G   = R^T V = R V      (R symmetric)
//   C   = (V^T G) o H      (matmul_tiled_scaled_f32, :208-255)
//   Z^T = C^T V^T = C V^T  (C symmetric)
//   E   = Z V^T
// Work is a flat list of (matrix, tile row, tile column) items so one launch
// covers an uneven batch.
#include "msq_dense.cuh"
#include "msq_internal.cuh"
#include "msq_f32x2.cuh"

#include <algorithm>
#include <vector>

namespace msq {
namespace {

constexpr int kTile = 64;    // output tile
constexpr int kBK = 16;      // K step
constexpr int kThreads = 256;  // 16 x 16 threads, 4 x 4 outputs each

__device__ __forceinline__ float rootOf(float lambda) {
  return sqrtf(fmaxf(lambda, 0.0f));
}

// C tile (64 x 64) of C = A^T B (both K-contiguous), FP32 FMA, with an
// epilogue.  Shared-memory tiles are stored [k][m] so the 4x4 register
// micro-tile reads broadcast-free rows.
template <int kEpilogue>
__global__ void __launch_bounds__(kThreads)
gemmTNKernel(GemmArgs args) {
  __shared__ __align__(16) float As[2][kBK][kTile + 4];
  __shared__ __align__(16) float Bs[2][kBK][kTile + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  for (int item = blockIdx.x; item < args.items; item += gridDim.x) {
    const int4 w = args.work[item];  // matrix, tile_i, tile_j, unused
    const int mi = w.x;
    const int n = args.n[mi];
    const int i0 = w.y * kTile, j0 = w.z * kTile;
    const float *A = args.a + args.a_offset[mi];
    const float *B = args.b + args.b_offset[mi];
    float acc[4][4] = {};
    // loader mapping: each thread loads 4 (k, row) elements per operand
    // Operand layouts: K-major (element (i, k) at k + i*n) loads with k
    // fastest; M-major (at i + k*n) with i fastest; both coalesced.
    auto load = [&](int buf, int k0) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int idx = threadIdx.x + e * kThreads;  // 0..1023
        {
          const int kk = args.a_mmajor ? idx / kTile : idx % kBK;
          const int r = args.a_mmajor ? idx % kTile : idx / kBK;
          const int k = k0 + kk, gi = i0 + r;
          const int64_t at = args.a_mmajor ? gi + static_cast<int64_t>(k) * n
                                           : k + static_cast<int64_t>(gi) * n;
          As[buf][kk][r] = (k < n && gi < n) ? A[at] : 0.0f;
        }
        {
          const int kk = args.b_nmajor ? idx / kTile : idx % kBK;
          const int r = args.b_nmajor ? idx % kTile : idx / kBK;
          const int k = k0 + kk, gj = j0 + r;
          const int64_t at = args.b_nmajor ? gj + static_cast<int64_t>(k) * n
                                           : k + static_cast<int64_t>(gj) * n;
          Bs[buf][kk][r] = (k < n && gj < n) ? B[at] : 0.0f;
        }
      }
    };
    const int ksteps = (n + kBK - 1) / kBK;
    load(0, 0);
    __syncthreads();
    for (int ks = 0; ks < ksteps; ++ks) {
      const int buf = ks & 1;
      if (ks + 1 < ksteps) load(buf ^ 1, (ks + 1) * kBK);
#pragma unroll
      for (int kk = 0; kk < kBK; ++kk) {
        const float4 a4 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
        const float4 b4 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
        const float av[4] = {a4.x, a4.y, a4.z, a4.w};
        const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
      }
      __syncthreads();
    }
    float *C = args.c + args.c_offset[mi];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = j0 + tx * 4 + c;
      if (j >= n) continue;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty * 4 + r;
        if (i >= n) continue;
        float v = acc[r][c];
        if (kEpilogue == kEpilogueInverseH) {
          const float *lam = args.eigenvalues + args.eig_offset[mi];
          // an FP32 eigenvalue <= 0 (below FP32 resolution of a nearly
          // singular input) has root 0; the pair of two such gets no correction
          const float d = rootOf(lam[i]) + rootOf(lam[j]);
          v = d > 0.0f ? v / d : 0.0f;
        }
        C[i + static_cast<int64_t>(j) * n] = v;
      }
    }
  }
}

// Float-float residual R = A - X X (X = hi + lo), the reference's
// working_residual (metal_mixed_sqrt.metal:1927-1942) as a tiled product:
// each product is split exactly with an FMA, sums are two-sums, and the
// low-order terms accumulate in a separate FP32 compensation (Ogita-Rump-
// Oishi Dot2).  Per-matrix ||R||_F^2 and ||A||_F^2 reduce into FP64.
// X is symmetric, so X X is too: only tiles on or above the diagonal are
// computed, and an off-diagonal tile also writes R_ji = A_ji - (X X)_ij
// (the same products in the same order as a direct (j, i) tile).
// kGeneral: X need not be symmetric (the stage-3 plans with an explicit
// basis inverse): the left operand is read as rows of X, every tile is
// computed and nothing is mirrored.
template <bool kGeneral>
__global__ void __launch_bounds__(kThreads)
residualFFKernel(ResidualArgs args) {
  __shared__ __align__(16) float Hs[kBK][kTile + 4];
  __shared__ __align__(16) float Ls[kBK][kTile + 4];
  __shared__ __align__(16) float Hb[kBK][kTile + 4];
  __shared__ __align__(16) float Lb[kBK][kTile + 4];
  __shared__ double red[2][kThreads / 32];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  for (int item = blockIdx.x; item < args.items; item += gridDim.x) {
    const int4 w = args.work[item];
    const int mi = w.x;
    const int n = args.n[mi];
    const int i0 = w.y * kTile, j0 = w.z * kTile;
    const int64_t off = args.offset[mi];
    const float *Xh = args.x_hi + off;
    const float *Xl = args.x_lo ? args.x_lo + off : nullptr;
    // accumulators in pairs of adjacent columns: s (leading part) and comp
    // (low-order terms), two outputs per packed FP32 instruction
    f32x2 s2[4][2], comp2[4][2];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 2; ++q) s2[r][q] = comp2[r][q] = f2zero();
    for (int k0 = 0; k0 < n; k0 += kBK) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int idx = threadIdx.x + e * kThreads;
        const int kk = idx % kBK, r = idx / kBK;
        const int k = k0 + kk, gi = i0 + r, gj = j0 + r;
        // (X X)_ij = sum_k X_ki X_kj (X symmetric): column-contiguous loads;
        // general X: X_ik from row i
        const bool vi = k < n && gi < n, vj = k < n && gj < n;
        const int64_t ai = kGeneral ? gi + static_cast<int64_t>(k) * n
                                    : k + static_cast<int64_t>(gi) * n;
        Hs[kk][r] = vi ? Xh[ai] : 0.0f;
        Ls[kk][r] = vi && Xl ? Xl[ai] : 0.0f;
        Hb[kk][r] = vj ? Xh[k + static_cast<int64_t>(gj) * n] : 0.0f;
        Lb[kk][r] = vj && Xl ? Xl[k + static_cast<int64_t>(gj) * n] : 0.0f;
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < kBK; ++kk) {
        const float4 ah4 = *reinterpret_cast<const float4 *>(&Hs[kk][ty * 4]);
        const float4 al4 = *reinterpret_cast<const float4 *>(&Ls[kk][ty * 4]);
        const ulonglong2 bh2 = *reinterpret_cast<const ulonglong2 *>(&Hb[kk][tx * 4]);
        const ulonglong2 bl2 = *reinterpret_cast<const ulonglong2 *>(&Lb[kk][tx * 4]);
        const float ah[4] = {ah4.x, ah4.y, ah4.z, ah4.w}, al[4] = {al4.x, al4.y, al4.z, al4.w};
        const f32x2 bh[2] = {bh2.x, bh2.y}, bl[2] = {bl2.x, bl2.y};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const f32x2 a2 = f2make(ah[r], ah[r]), na2 = f2make(-ah[r], -ah[r]);
          const f32x2 l2 = f2make(al[r], al[r]);
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            // p = a b (carried negated: m = -p, exact), its error e = a b - p,
            // the two-sum t + se = s + p, and the low-order terms into comp
            const f32x2 m = f2mul(na2, bh[q]);
            const f32x2 pe = f2fma(a2, bh[q], m);
            const f32x2 t = f2sub(s2[r][q], m);
            const f32x2 z = f2sub(t, s2[r][q]);
            const f32x2 se = f2sub(f2sub(s2[r][q], f2sub(t, z)), f2add(m, z));
            s2[r][q] = t;
            // low-order terms: the cross products hi*lo' and lo*hi' fused into
            // comp (comp is ~2^-24 of s, so its roundings stay ~2^-48 of s)
            f32x2 c = f2fma(a2, bl[q], comp2[r][q]);
            c = f2fma(l2, bh[q], c);
            comp2[r][q] = f2add(c, f2add(se, pe));
          }
        }
      }
      __syncthreads();
    }
    float s[4][4], comp[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        f2split(s2[r][q], s[r][2 * q], s[r][2 * q + 1]);
        f2split(comp2[r][q], comp[r][2 * q], comp[r][2 * q + 1]);
      }
    const float *A = args.a + off;
    const float *AL = args.a_lo ? args.a_lo + off : nullptr;
    float *R = args.r ? args.r + off : nullptr;
    const bool mirror = !kGeneral && w.z > w.y;
    double rn = 0.0, an = 0.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = j0 + tx * 4 + c;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty * 4 + r;
        if (i >= n || j >= n) continue;
        const int64_t idx = i + static_cast<int64_t>(j) * n;
        const float a = A[idx];
        const float a_lo = AL ? AL[idx] : 0.0f;  // A = a + a_lo (float-float input)
        // (a + a_lo) - (s + comp) with a two-sum so the FP32 output rounds once
        const float hi = -s[r][c], lo = a_lo - comp[r][c];
        const float t = a + hi;
        const float z = t - a;
        const float e = (a - (t - z)) + (hi - z) + lo;
        const double rv = static_cast<double>(t) + static_cast<double>(e);
        if (R) R[idx] = t + e;
        rn += rv * rv;
        const double av = static_cast<double>(a) + a_lo;
        an += av * av;
        if (mirror) {
          const int64_t idt = j + static_cast<int64_t>(i) * n;
          const float a2 = A[idt];
          const float lo2 = (AL ? AL[idt] : 0.0f) - comp[r][c];
          const float t2 = a2 + hi;
          const float z2 = t2 - a2;
          const float e2 = (a2 - (t2 - z2)) + (hi - z2) + lo2;
          const double rv2 = static_cast<double>(t2) + static_cast<double>(e2);
          if (R) R[idt] = t2 + e2;
          rn += rv2 * rv2;
          const double av2 = static_cast<double>(a2) + (AL ? AL[idt] : 0.0f);
          an += av2 * av2;
        }
      }
    }
#pragma unroll
    for (int sft = 16; sft > 0; sft >>= 1) {
      rn += __shfl_xor_sync(0xffffffffu, rn, sft);
      an += __shfl_xor_sync(0xffffffffu, an, sft);
    }
    if (threadIdx.x % 32 == 0) {
      red[0][threadIdx.x / 32] = rn;
      red[1][threadIdx.x / 32] = an;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a0 = 0.0, a1 = 0.0;
      for (int q = 0; q < kThreads / 32; ++q) {
        a0 += red[0][q];
        a1 += red[1][q];
      }
      atomicAdd(&args.norms[2 * mi], a0);
      atomicAdd(&args.norms[2 * mi + 1], a1);
    }
    __syncthreads();
  }
}

// F^T (K-major factor): F[k + i*n] = V[i + k*n] * lambda_k^(1/4), so that
// X = F^T F = V diag(sqrt(lambda)) V^T (scale_columns_f32,
// metal_mixed_sqrt.metal:21-38, split symmetrically over both factors).
__global__ void makeFactorKernel(const float *__restrict__ v, const float *__restrict__ lam,
                                 const int32_t *__restrict__ nn, const int64_t *__restrict__ off,
                                 const int64_t *__restrict__ eoff, float *__restrict__ f,
                                 const int4 *__restrict__ work, int items) {
  __shared__ float tile[32][33];
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
  const int mi = work[item].x;
  const int n = nn[mi];
  const int i0 = work[item].y * 32, k0 = work[item].z * 32;
  __syncthreads();
  const float *V = v + off[mi];
  float *F = f + off[mi];
  const float *L = lam + eoff[mi];
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int k = k0 + r, i = i0 + threadIdx.x;
    tile[r][threadIdx.x] = (k < n && i < n) ? V[i + static_cast<int64_t>(k) * n] * sqrtf(rootOf(L[k])) : 0.0f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = i0 + r, k = k0 + threadIdx.x;
    if (i < n && k < n) F[k + static_cast<int64_t>(i) * n] = tile[threadIdx.x][r];
  }
  }
}

__global__ void transposeKernel(const float *__restrict__ src, const int32_t *__restrict__ nn,
                                const int64_t *__restrict__ off, float *__restrict__ dst,
                                const int4 *__restrict__ work, int items) {
  __shared__ float tile[32][33];
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
  const int mi = work[item].x;
  const int n = nn[mi];
  const int i0 = work[item].y * 32, j0 = work[item].z * 32;
  __syncthreads();
  const float *S = src + off[mi];
  float *D = dst + off[mi];
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int j = j0 + r, i = i0 + threadIdx.x;
    tile[r][threadIdx.x] = (i < n && j < n) ? S[i + static_cast<int64_t>(j) * n] : 0.0f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = i0 + r, j = j0 + threadIdx.x;
    if (i < n && j < n) D[j + static_cast<int64_t>(i) * n] = tile[threadIdx.x][r];
  }
  }
}

// X <- X + (E + E^T)/2 in float-float (working_add_symmetric_correction,
// metal_mixed_sqrt.metal:1955-1970).
__global__ void symmetricAddKernel(float *__restrict__ x_hi, float *__restrict__ x_lo,
                                   const float *__restrict__ e, const int32_t *__restrict__ nn,
                                   const int64_t *__restrict__ off, const int4 *__restrict__ work,
                                   int items) {
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
  const int mi = work[item].x;
  const int n = nn[mi];
  const int i = work[item].y * 32 + threadIdx.x;
  for (int jj = threadIdx.y; jj < 32; jj += blockDim.y) {
  const int j = work[item].z * 32 + jj;
  if (i >= n || j >= n) continue;
  const int64_t o = off[mi];
  const int64_t idx = o + i + static_cast<int64_t>(j) * n;
  const float corr = 0.5f * (e[idx] + e[o + j + static_cast<int64_t>(i) * n]);
  const float h = x_hi[idx], l = x_lo[idx];
  const float s = h + corr;
  const float vr = s - h;
  const float err = (h - (s - vr)) + (corr - vr) + l;
  const float hi = s + err;
  x_hi[idx] = hi;
  x_lo[idx] = err - (hi - s);
  }
  }
}

// X <- X + E in float-float (the reference's working_add,
// metal_mixed_sqrt.metal:1955-1970): two-sum of the high word and E, the
// error and the low word renormalised into (hi, lo).
__global__ void workingAddKernel(float *__restrict__ x_hi, float *__restrict__ x_lo,
                                 const float *__restrict__ e, const int32_t *__restrict__ nn,
                                 const int64_t *__restrict__ off, const int4 *__restrict__ work,
                                 int items) {
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int mi = work[item].x;
    const int n = nn[mi];
    const int i = work[item].y * 32 + threadIdx.x;
    for (int jj = threadIdx.y; jj < 32; jj += blockDim.y) {
      const int j = work[item].z * 32 + jj;
      if (i >= n || j >= n) continue;
      const int64_t idx = off[mi] + i + static_cast<int64_t>(j) * n;
      const float corr = e[idx];
      const float h = x_hi[idx], l = x_lo[idx];
      const float s = h + corr;
      const float vr = s - h;
      const float err = (h - (s - vr)) + (corr - vr) + l;
      const float hi = s + err;
      x_hi[idx] = hi;
      x_lo[idx] = err - (hi - s);
    }
  }
}

}  // namespace

int gemmWork(msq_ctx *ctx, const DeviceBatch *b, int tile, const int4 **work, int *items) {
  // One list per (layout, tile size); cached on the batch.  A negative tile
  // size asks for the upper triangle of tiles only (tj >= ti).
  auto &cache = const_cast<DeviceBatch *>(b)->work_cache;
  for (auto &e : cache) {
    if (e.tile == tile) {
      *work = e.work;
      *items = e.items;
      return MSQ_OK;
    }
  }
  std::vector<int4> list;
  // largest matrices first: their long K loops start early
  std::vector<int> ids(b->count);
  for (int i = 0; i < b->count; ++i) ids[i] = i;
  std::stable_sort(ids.begin(), ids.end(),
                   [&](int x, int y) { return b->host_n[x] > b->host_n[y]; });
  const bool upper = tile < 0;
  const int size = upper ? -tile : tile;
  for (int mi : ids) {
    const int t = (b->host_n[mi] + size - 1) / size;
    for (int ti = 0; ti < t; ++ti)
      for (int tj = upper ? ti : 0; tj < t; ++tj) list.push_back(make_int4(mi, ti, tj, 0));
  }
  int4 *dev = nullptr;
  MSQ_TRY(cudaCheck(ctx, cudaMalloc(&dev, list.size() * sizeof(int4)), "work list alloc"));
  MSQ_TRY(cudaCheck(ctx, cudaMemcpy(dev, list.data(), list.size() * sizeof(int4),
                                    cudaMemcpyHostToDevice), "work list upload"));
  cache.push_back({tile, dev, static_cast<int>(list.size())});
  *work = dev;
  *items = static_cast<int>(list.size());
  return MSQ_OK;
}

int gemmTN(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *bm, float *c,
           int epilogue, const float *eigenvalues, bool a_mmajor, bool b_nmajor) {
  GemmArgs args{};
  args.a_mmajor = a_mmajor;
  args.b_nmajor = b_nmajor;
  MSQ_TRY(gemmWork(ctx, b, kTile, &args.work, &args.items));
  args.a = a;
  args.b = bm;
  args.c = c;
  args.a_offset = b->offset;
  args.b_offset = b->offset;
  args.c_offset = b->offset;
  args.n = b->n;
  args.eigenvalues = eigenvalues;
  args.eig_offset = b->eig_offset;
  const unsigned grid = std::min<unsigned>(args.items, kSmCount * 8);
  if (epilogue == kEpilogueInverseH) {
    gemmTNKernel<kEpilogueInverseH><<<grid, kThreads, 0, ctx->stream>>>(args);
  } else {
    gemmTNKernel<kEpilogueStore><<<grid, kThreads, 0, ctx->stream>>>(args);
  }
  return launched(ctx, "gemm TN fp32");
}

int residualFF(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *x_hi,
               const float *x_lo, float *r, double *norms, const float *a_lo) {
  ResidualArgs args{};
  MSQ_TRY(gemmWork(ctx, b, -kTile, &args.work, &args.items));  // upper tiles
  args.a = a;
  args.a_lo = a_lo;
  args.x_hi = x_hi;
  args.x_lo = x_lo;
  args.r = r;
  args.norms = norms;
  args.offset = b->offset;
  args.n = b->n;
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(norms, 0, 2 * b->count * sizeof(double), ctx->stream),
                    "norm reset"));
  const unsigned grid = std::min<unsigned>(args.items, kSmCount * 8);
  residualFFKernel<false><<<grid, kThreads, 0, ctx->stream>>>(args);
  return launched(ctx, "residual float-float");
}

int makeFactor(msq_ctx *ctx, const DeviceBatch *b, const float *v, const float *lam, float *f) {
  const int4 *work;
  int items;
  MSQ_TRY(gemmWork(ctx, b, 32, &work, &items));
  makeFactorKernel<<<std::min(items, kSmCount * 16), dim3(32, 8), 0, ctx->stream>>>(
      v, lam, b->n, b->offset, b->eig_offset, f, work, items);
  return launched(ctx, "make factor");
}

int transpose(msq_ctx *ctx, const DeviceBatch *b, const float *src, float *dst) {
  const int4 *work;
  int items;
  MSQ_TRY(gemmWork(ctx, b, 32, &work, &items));
  transposeKernel<<<std::min(items, kSmCount * 16), dim3(32, 8), 0, ctx->stream>>>(
      src, b->n, b->offset, dst, work, items);
  return launched(ctx, "transpose");
}

// C = A B for one n x n column-major matrix, each element the FMA chain
// sum = fma(A[r, k], B[k, c], sum) over k = 0..n-1 in order, as the
// reference's matmul kernels accumulate (metal_mixed_sqrt.metal:39-56,
// matmul_tiled_*: decoded operands, FP32).  16 x 16 outputs per CTA, K
// staged through shared memory 16 at a time (the chain order is kept).
namespace {
constexpr int kMmTile = 16;

__global__ void __launch_bounds__(kMmTile * kMmTile)
matmulFmaKernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ c,
                int n) {
  __shared__ float as[kMmTile][kMmTile + 1];
  __shared__ float bs[kMmTile][kMmTile + 1];
  const int tr = threadIdx.x, tc = threadIdx.y;  // row fastest: coalesced column reads
  const int row = blockIdx.x * kMmTile + tr, col = blockIdx.y * kMmTile + tc;
  float sum = 0.0f;
  for (int k0 = 0; k0 < n; k0 += kMmTile) {
    // A[row, k0 + tc] and B[k0 + tr, col]
    as[tr][tc] = row < n && k0 + tc < n ? a[row + static_cast<int64_t>(k0 + tc) * n] : 0.0f;
    bs[tr][tc] = k0 + tr < n && col < n ? b[(k0 + tr) + static_cast<int64_t>(col) * n] : 0.0f;
    __syncthreads();
    const int kend = min(kMmTile, n - k0);
    for (int k = 0; k < kend; ++k) sum = fmaf(as[tr][k], bs[k][tc], sum);
    __syncthreads();
  }
  if (row < n && col < n) c[row + static_cast<int64_t>(col) * n] = sum;
}

// The same product for every matrix of a batch: one CTA per 16 x 16 output
// tile of a (matrix, tile_i, tile_j) work list, the same FMA chains.
__global__ void __launch_bounds__(kMmTile * kMmTile)
matmulFmaBatchKernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ c,
                     const int64_t *__restrict__ offset, const int32_t *__restrict__ n,
                     const int4 *__restrict__ work, int items) {
  __shared__ float as[kMmTile][kMmTile + 1];
  __shared__ float bs[kMmTile][kMmTile + 1];
  const int tr = threadIdx.x, tc = threadIdx.y;
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int4 w = work[item];
    const int nn = n[w.x];
    const int64_t o = offset[w.x];
    const int row = w.y * kMmTile + tr, col = w.z * kMmTile + tc;
    float sum = 0.0f;
    for (int k0 = 0; k0 < nn; k0 += kMmTile) {
      as[tr][tc] = row < nn && k0 + tc < nn ? a[o + row + static_cast<int64_t>(k0 + tc) * nn] : 0.0f;
      bs[tr][tc] = k0 + tr < nn && col < nn ? b[o + (k0 + tr) + static_cast<int64_t>(col) * nn] : 0.0f;
      __syncthreads();
      const int kend = min(kMmTile, nn - k0);
      for (int k = 0; k < kend; ++k) sum = fmaf(as[tr][k], bs[k][tc], sum);
      __syncthreads();
    }
    if (row < nn && col < nn) c[o + row + static_cast<int64_t>(col) * nn] = sum;
  }
}

// C_ij = W_ij / (s_i + s_j) (diagonal_sylvester_*, metal_mixed_sqrt.metal:58-74).
__global__ void diagonalSylvesterKernel(const float *__restrict__ w, const float *__restrict__ s,
                                        float *__restrict__ c, int n) {
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
       idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int i = static_cast<int>(idx % n), j = static_cast<int>(idx / n);
    c[idx] = __fdiv_rn(w[idx], s[i] + s[j]);
  }
}
// The same for every matrix of a batch (grid.y = matrix); s of matrix i at
// eig_offset[i].
__global__ void diagonalSylvesterBatchKernel(const float *__restrict__ w, const float *__restrict__ s,
                                             float *__restrict__ c, const int64_t *__restrict__ offset,
                                             const int64_t *__restrict__ eig_offset,
                                             const int32_t *__restrict__ n, int count) {
  for (int mi = blockIdx.y; mi < count; mi += gridDim.y) {
    const int nn = n[mi];
    const int64_t total = static_cast<int64_t>(nn) * nn, o = offset[mi];
    const float *sm = s + eig_offset[mi];
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
      const int i = static_cast<int>(idx % nn), j = static_cast<int>(idx / nn);
      c[o + idx] = __fdiv_rn(w[o + idx], sm[i] + sm[j]);
    }
  }
}
}  // namespace

int matmulFmaBatch(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *bm, float *c) {
  const int4 *work = nullptr;
  int items = 0;
  MSQ_TRY(gemmWork(ctx, b, kMmTile, &work, &items));
  matmulFmaBatchKernel<<<std::min(items, kSmCount * 16), dim3(kMmTile, kMmTile), 0, ctx->stream>>>(
      a, bm, c, b->offset, b->n, work, items);
  return launched(ctx, "native matmul");
}

int diagonalSylvesterBatch(msq_ctx *ctx, const DeviceBatch *b, const float *w, const float *s,
                           float *c) {
  const int64_t nn = static_cast<int64_t>(b->max_n) * b->max_n;
  const dim3 grid(static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((nn + 255) / 256, 64))),
                  static_cast<unsigned>(std::min(b->count, 65535)));
  diagonalSylvesterBatchKernel<<<grid, 256, 0, ctx->stream>>>(w, s, c, b->offset, b->eig_offset,
                                                              b->n, b->count);
  return launched(ctx, "native diagonal sylvester");
}

int matmulFma(msq_ctx *ctx, const float *a, const float *b, float *c, int n) {
  const dim3 grid((n + kMmTile - 1) / kMmTile, (n + kMmTile - 1) / kMmTile);
  matmulFmaKernel<<<grid, dim3(kMmTile, kMmTile), 0, ctx->stream>>>(a, b, c, n);
  return launched(ctx, "native matmul");
}

int diagonalSylvester(msq_ctx *ctx, const float *w, const float *s, float *c, int n) {
  const int64_t total = static_cast<int64_t>(n) * n;
  const int grid = static_cast<int>(std::min<int64_t>((total + 255) / 256, kSmCount * 8));
  diagonalSylvesterKernel<<<grid, 256, 0, ctx->stream>>>(w, s, c, n);
  return launched(ctx, "native diagonal sylvester");
}

int residualFFGeneral(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *x_hi,
                      const float *x_lo, float *r, double *norms, const float *a_lo) {
  ResidualArgs args{};
  MSQ_TRY(gemmWork(ctx, b, kTile, &args.work, &args.items));  // every tile
  args.a = a;
  args.a_lo = a_lo;
  args.x_hi = x_hi;
  args.x_lo = x_lo;
  args.r = r;
  args.norms = norms;
  args.offset = b->offset;
  args.n = b->n;
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(norms, 0, 2 * b->count * sizeof(double), ctx->stream),
                    "norm reset"));
  const unsigned grid = std::min<unsigned>(args.items, kSmCount * 8);
  residualFFKernel<true><<<grid, kThreads, 0, ctx->stream>>>(args);
  return launched(ctx, "residual float-float (general X)");
}

int workingAdd(msq_ctx *ctx, const DeviceBatch *b, float *x_hi, float *x_lo, const float *e) {
  const int4 *work;
  int items;
  MSQ_TRY(gemmWork(ctx, b, 32, &work, &items));
  workingAddKernel<<<std::min(items, kSmCount * 16), dim3(32, 8), 0, ctx->stream>>>(
      x_hi, x_lo, e, b->n, b->offset, work, items);
  return launched(ctx, "working add");
}

int symmetricAdd(msq_ctx *ctx, const DeviceBatch *b, float *x_hi, float *x_lo, const float *e) {
  const int4 *work;
  int items;
  MSQ_TRY(gemmWork(ctx, b, 32, &work, &items));
  symmetricAddKernel<<<std::min(items, kSmCount * 16), dim3(32, 8), 0, ctx->stream>>>(
      x_hi, x_lo, e, b->n, b->offset, work, items);
  return launched(ctx, "symmetric add");
}

}  // namespace msq
