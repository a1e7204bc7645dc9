// Grid-parallel Jacobi for one large matrix.
//
// The batched eigensolver gives each matrix one CTA, which leaves a single
// large matrix (or a handful) on a few SMs.  Here every SM works on the same
// matrix, with the same blocked rotations and the same bits:
//  * A is kept as the same packed, row-swizzled 4x4 tiles of the upper
//    triangle, in global memory (L2-resident up to n ~ 4096);
//  * a round is two launches: gridPivotKernel sweeps the P pivots (a quad of
//    lanes each, writing the round's rotations), gridUpdateKernel applies
//    every super-tile update T' = Q_k^T T Q_l (two lanes each) and the V
//    update V <- V Q on row-major V (lanes = rows, so Q_k is a broadcast);
//  * the rounds of one sweep are captured once into a CUDA graph and the
//    graph is launched once per sweep;
//  * after each sweep the FP64 off-norm is reduced on the device and read by
//    the host, which decides whether another sweep is needed (the reference
//    runs a fixed 8 sweeps, MetalRuntime::symmetricJacobi,
//    src/metal_runtime.cpp:584-646).
// Every element update is the same ordered FP32 chain as in the batched
// kernels and the CPU restatement, so results agree bit for bit after the
// same number of sweeps.
#include "msq_internal.cuh"
#include "msq_jacobi_device.cuh"
#include "msq_jacobi_grid.cuh"

#include <cmath>
#include <cstring>

namespace msq {
namespace {

constexpr int kGridThreads = 256;

struct GridArgs {
  float *tiles;  // packed tiles of A
  float *v;      // V, row-major n x m
  const float *v_in;  // column-major starting V (null: the identity)
  float *q;      // this round's rotations, P x 64 (row-major 8x8 each)
  double *acc;   // off2, diag2 accumulators
  int n, m, nb, P;
  int round;
  int super_items;  // 2 x folded super-tile items, rounded up to 32
};

// A (column-major, n x n) -> symmetrised tiles (the same averaged load as
// the batched kernel); V = I, or the given starting V (a continued solve).
// grid.y = column block J.
__global__ void gridLoadKernel(const float *a, GridArgs g) {
  const int J = blockIdx.y;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < (J + 1) * kTileF;
       idx += gridDim.x * blockDim.x) {
    const int I = idx / kTileF, e = idx % kTileF;
    const int gi = 4 * I + e / 4, gj = 4 * J + e % 4;
    float val = 0.0f;
    if (gi < g.n && gj < g.n) {
      val = 0.5f * (a[gi + static_cast<int64_t>(gj) * g.n] + a[gj + static_cast<int64_t>(gi) * g.n]);
    }
    g.tiles[tileElement(triTile(I, J), e / 4, e % 4)] = val;
  }
  // V rows 4J .. 4J + 3
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 4 * g.m; idx += gridDim.x * blockDim.x) {
    const int r = 4 * J + idx / g.m, c = idx % g.m;
    if (r < g.n) {
      g.v[static_cast<int64_t>(r) * g.m + c] =
          g.v_in == nullptr ? (r == c ? 1.0f : 0.0f)
                            : (c < g.n ? g.v_in[r + static_cast<int64_t>(c) * g.n] : 0.0f);
    }
  }
}

// off2 (strictly off-diagonal) and diag2, FP64, as the batched kernel.
__global__ void gridNormKernel(GridArgs g) {
  __shared__ double red[2][kGridThreads / 32];
  const int64_t tiles = static_cast<int64_t>(g.nb) * (g.nb + 1) / 2;
  double off2 = 0.0, diag2 = 0.0;
  for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < tiles * kTileF;
       idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t t = idx / kTileF;
    const int e = static_cast<int>(idx % kTileF);
    // t = J (J + 1) / 2 + I, I <= J
    int J = static_cast<int>((sqrt(8.0 * static_cast<double>(t) + 1.0) - 1.0) / 2.0);
    while (static_cast<int64_t>(J) * (J + 1) / 2 > t) --J;
    while (static_cast<int64_t>(J + 1) * (J + 2) / 2 <= t) ++J;
    const int I = static_cast<int>(t - static_cast<int64_t>(J) * (J + 1) / 2);
    const double v = g.tiles[idx];  // any element of tile t (rows are only permuted)
    if (I < J) {
      off2 += 2.0 * v * v;
    } else {
      const int phys = e / 4, col = e % 4;
      const int row = phys ^ static_cast<int>(t & 3);
      if (row == col) diag2 += v * v;
      else off2 += v * v;
    }
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    off2 += __shfl_xor_sync(0xffffffffu, off2, s);
    diag2 += __shfl_xor_sync(0xffffffffu, diag2, s);
  }
  if (threadIdx.x % 32 == 0) {
    red[0][threadIdx.x / 32] = off2;
    red[1][threadIdx.x / 32] = diag2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kGridThreads / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    atomicAdd(&g.acc[0], a);
    atomicAdd(&g.acc[1], b);
  }
}

// The P pivots of one round: a quad of lanes per pivot (pivotSweep), the
// rotations written row-major to g.q.  Warp-uniform: every lane of a warp
// takes part in the quad shuffles.
__global__ void __launch_bounds__(kGridThreads) gridPivotKernel(GridArgs g) {
  __shared__ __align__(16) float qcol[kGridThreads / 4][kQS];
  const int t4 = threadIdx.x & 3;
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const bool active = k < g.P;
  float ra[8], rb[8];
  int tII = 0, tIJ = 0, tJJ = 0;
  if (active) {
    int I, J;
    rrPair(k, g.round, g.nb, I, J);
    tII = triTile(I, I);
    tIJ = triTile(I, J);
    tJJ = triTile(J, J);
    const float4 *sII = reinterpret_cast<const float4 *>(g.tiles + static_cast<int64_t>(tII) * kTileF);
    const float4 *sIJ = reinterpret_cast<const float4 *>(g.tiles + static_cast<int64_t>(tIJ) * kTileF);
    const float4 *sJJ = reinterpret_cast<const float4 *>(g.tiles + static_cast<int64_t>(tJJ) * kTileF);
    const int jr = 3 - t4;
    const float4 v0 = sII[t4 ^ (tII & 3)], v1 = sIJ[t4 ^ (tIJ & 3)], v2 = sJJ[jr ^ (tJJ & 3)];
    ra[0] = v0.x; ra[1] = v0.y; ra[2] = v0.z; ra[3] = v0.w;
    ra[4] = v1.x; ra[5] = v1.y; ra[6] = v1.z; ra[7] = v1.w;
#pragma unroll
    for (int i = 0; i < 4; ++i) rb[i] = g.tiles[tileElement(tIJ, i, jr)];
    rb[4] = v2.x; rb[5] = v2.y; rb[6] = v2.z; rb[7] = v2.w;
  } else {
#pragma unroll
    for (int y = 0; y < 8; ++y) ra[y] = rb[y] = 0.0f;
  }
  float *qs = qcol[threadIdx.x >> 2];
  pivotSweep(ra, rb, qs, t4, active);
  if (active) {
    float4 *sII = reinterpret_cast<float4 *>(g.tiles + static_cast<int64_t>(tII) * kTileF);
    float4 *sIJ = reinterpret_cast<float4 *>(g.tiles + static_cast<int64_t>(tIJ) * kTileF);
    float4 *sJJ = reinterpret_cast<float4 *>(g.tiles + static_cast<int64_t>(tJJ) * kTileF);
    sII[t4 ^ (tII & 3)] = make_float4(ra[0], ra[1], ra[2], ra[3]);
    sIJ[t4 ^ (tIJ & 3)] = make_float4(ra[4], ra[5], ra[6], ra[7]);
    sJJ[t4 ^ (tJJ & 3)] = make_float4(rb[4], rb[5], rb[6], rb[7]);
    // the quad's Q (row-major in qs) -> g.q[k]: lane t copies rows 2t, 2t+1
    const float4 *src = reinterpret_cast<const float4 *>(qs);
    float4 *dst = reinterpret_cast<float4 *>(g.q + static_cast<int64_t>(k) * kQF);
#pragma unroll
    for (int x = 0; x < 4; ++x) dst[4 * t4 + x] = src[4 * t4 + x];
  }
}

// Super-tile updates (items [0, super_items)) and the V update (items
// beyond: row fastest, then pair) of one round.
__global__ void __launch_bounds__(kGridThreads) gridUpdateKernel(GridArgs g) {
  const int64_t total = g.super_items + static_cast<int64_t>(g.n) * g.P;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t base = blockIdx.x * static_cast<int64_t>(blockDim.x) + (threadIdx.x & ~31); base < total;
       base += stride) {
    const int64_t w = base + (threadIdx.x & 31);
    if (base < g.super_items) {
      // warp-uniform branch: super_items is a multiple of 32
      const int w2 = static_cast<int>(w);
      const int h = w2 & 1;
      int k = 0, l = 0;
      const bool valid = foldedBlock(w2 >> 1, g.P, k, l) && k != l && (w2 >> 1) < ((g.P + 1) / 2) * (g.P + 1);
      if (!valid) k = l = 0;
      int rb0, rb1, cb0, cb1;
      rrPair(k, g.round, g.nb, rb0, rb1);
      rrPair(l, g.round, g.nb, cb0, cb1);
      const float4 *qk = reinterpret_cast<const float4 *>(g.q + static_cast<int64_t>(k) * kQF);
      const float4 *ql = reinterpret_cast<const float4 *>(g.q + static_cast<int64_t>(l) * kQF);
      superTileHalf(g.tiles, ComputedTri{}, qk, ql, rb0, rb1, cb0, cb1, h, valid);
    } else {
      const int64_t idx = w - g.super_items;
      if (idx >= static_cast<int64_t>(g.n) * g.P) continue;
      const int row = static_cast<int>(idx % g.n), k = static_cast<int>(idx / g.n);
      int I, J;
      rrPair(k, g.round, g.nb, I, J);
      const float4 *qk = reinterpret_cast<const float4 *>(g.q + static_cast<int64_t>(k) * kQF);
      float *vrow = g.v + static_cast<int64_t>(row) * g.m;
      const float4 a = *reinterpret_cast<const float4 *>(vrow + 4 * I);
      const float4 b = *reinterpret_cast<const float4 *>(vrow + 4 * J);
      const float x[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
      float o[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) o[c] = 0.0f;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 lo = qk[2 * j], hi = qk[2 * j + 1];
        o[0] = fmaf(x[j], lo.x, o[0]); o[1] = fmaf(x[j], lo.y, o[1]);
        o[2] = fmaf(x[j], lo.z, o[2]); o[3] = fmaf(x[j], lo.w, o[3]);
        o[4] = fmaf(x[j], hi.x, o[4]); o[5] = fmaf(x[j], hi.y, o[5]);
        o[6] = fmaf(x[j], hi.z, o[6]); o[7] = fmaf(x[j], hi.w, o[7]);
      }
      *reinterpret_cast<float4 *>(vrow + 4 * I) = make_float4(o[0], o[1], o[2], o[3]);
      *reinterpret_cast<float4 *>(vrow + 4 * J) = make_float4(o[4], o[5], o[6], o[7]);
    }
  }
}

// Eigenvalues (the diagonal), the rotated matrix written back in full
// (column-major) and V transposed into the caller's column-major vectors.
// grid.y = column block J of the output.
__global__ void gridFinishKernel(GridArgs g, float *a, float *vectors, float *eigenvalues) {
  __shared__ float tile[32][33];
  const int c0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
  // A write-back and eigenvalues
  for (int idx = threadIdx.x; idx < 32 * 32; idx += blockDim.x) {
    const int r = r0 + idx % 32, c = c0 + idx / 32;
    if (r < g.n && c < g.n) {
      const int I = r / 4, J = c / 4;
      const float val = I <= J ? g.tiles[tileElement(triTile(I, J), r % 4, c % 4)]
                               : g.tiles[tileElement(triTile(J, I), c % 4, r % 4)];
      a[r + static_cast<int64_t>(c) * g.n] = val;
      if (r == c) eigenvalues[r] = val;
    }
  }
  // vectors[r + c n] = V[r][c]: stage a 32 x 32 block of V (rows r0.., columns c0..)
  for (int idx = threadIdx.x; idx < 32 * 32; idx += blockDim.x) {
    const int rr = idx / 32, cc = idx % 32;
    const int r = r0 + rr, c = c0 + cc;
    tile[rr][cc] = (r < g.n && c < g.n) ? g.v[static_cast<int64_t>(r) * g.m + c] : 0.0f;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 32 * 32; idx += blockDim.x) {
    const int cc = idx / 32, rr = idx % 32;
    const int r = r0 + rr, c = c0 + cc;
    if (r < g.n && c < g.n) vectors[r + static_cast<int64_t>(c) * g.n] = tile[rr][cc];
  }
}

}  // namespace

int gridJacobiSolve(msq_ctx *ctx, float *matrix, float *vectors, float *eigenvalues, int n,
                    double tolerance, int max_sweeps, int *sweeps_out, double *off_ratio_out,
                    double *norm2_out, bool keep_vectors) {
  const int m = padded8(n), nb = m / 4, P = nb / 2;
  const int64_t tile_floats = static_cast<int64_t>(nb) * (nb + 1) / 2 * kTileF;
  const int64_t v_floats = static_cast<int64_t>(n) * m;
  const size_t bytes = 256 + ((tile_floats + v_floats + static_cast<int64_t>(P) * kQF) * sizeof(float) + 255) / 256 * 256;
  char *work = static_cast<char *>(scratch(ctx, bytes, kScratchGrid));
  if (work == nullptr) return MSQ_ERR_CUDA;
  if (ctx->grid_host == nullptr &&
      cudaCheck(ctx, cudaMallocHost(reinterpret_cast<void **>(&ctx->grid_host), 2 * sizeof(double)),
                "grid pinned") != MSQ_OK) {
    return MSQ_ERR_CUDA;
  }
  GridArgs g{};
  g.acc = reinterpret_cast<double *>(work);
  g.tiles = reinterpret_cast<float *>(work + 256);
  g.v = g.tiles + tile_floats;
  g.q = g.v + v_floats;
  g.v_in = keep_vectors ? vectors : nullptr;
  g.n = n;
  g.m = m;
  g.nb = nb;
  g.P = P;
  g.super_items = (2 * ((P + 1) / 2) * (P + 1) + 31) / 32 * 32;
  cudaStream_t s = ctx->stream;
  {
    dim3 grid(std::max(1, std::min(64, (nb * kTileF + 255) / 256)), nb);
    gridLoadKernel<<<grid, 256, 0, s>>>(matrix, g);
    MSQ_TRY(launched(ctx, "jacobi grid load"));
  }
  const int pivot_ctas = (4 * P + kGridThreads - 1) / kGridThreads;
  const int64_t update_items = g.super_items + static_cast<int64_t>(n) * P;
  const int update_ctas = static_cast<int>(std::min<int64_t>((update_items + kGridThreads - 1) / kGridThreads,
                                                             static_cast<int64_t>(kSmCount) * 16));
  // One sweep = nb - 1 rounds of (pivots, updates).  Captured into a graph
  // once per (order, buffers); launched directly while the launch timer runs.
  auto enqueueSweep = [&](cudaStream_t st) -> int {
    for (int r = 0; r < nb - 1; ++r) {
      g.round = r;
      gridPivotKernel<<<pivot_ctas, kGridThreads, 0, st>>>(g);
      MSQ_TRY(st == s ? launched(ctx, "jacobi grid pivots") : cudaCheck(ctx, cudaGetLastError(), "grid pivots"));
      gridUpdateKernel<<<update_ctas, kGridThreads, 0, st>>>(g);
      MSQ_TRY(st == s ? launched(ctx, "jacobi grid updates") : cudaCheck(ctx, cudaGetLastError(), "grid updates"));
    }
    return MSQ_OK;
  };
  const bool use_graph = !ctx->timing;
  if (use_graph && (ctx->grid_exec == nullptr || ctx->grid_n != n || ctx->grid_work != work)) {
    if (ctx->grid_exec != nullptr) {
      cudaGraphExecDestroy(ctx->grid_exec);
      ctx->grid_exec = nullptr;
    }
    cudaStream_t cs = auxStream(ctx, 4);
    if (cs == s) return setError(ctx, MSQ_ERR_CUDA, "grid jacobi: no capture stream");
    MSQ_TRY(cudaCheck(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "graph capture"));
    const int status = enqueueSweep(cs);
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(cs, &graph);
    if (status != MSQ_OK) {
      if (graph != nullptr) cudaGraphDestroy(graph);
      return status;
    }
    MSQ_TRY(cudaCheck(ctx, end, "graph capture end"));
    const cudaError_t inst = cudaGraphInstantiate(&ctx->grid_exec, graph, 0);
    cudaGraphDestroy(graph);
    MSQ_TRY(cudaCheck(ctx, inst, "graph instantiate"));
    ctx->grid_n = n;
    ctx->grid_work = work;
  }
  double norm2 = 0.0, ratio = 0.0;
  int sweeps = 0;
  const int norm_ctas = static_cast<int>(std::min<int64_t>((tile_floats + kGridThreads - 1) / kGridThreads,
                                                           static_cast<int64_t>(kSmCount) * 8));
  for (;;) {
    MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(g.acc, 0, 2 * sizeof(double), s), "grid norm reset"));
    gridNormKernel<<<norm_ctas, kGridThreads, 0, s>>>(g);
    MSQ_TRY(launched(ctx, "jacobi grid norm"));
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(ctx->grid_host, g.acc, 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
                      "grid norm read"));
    MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(s), "grid norm sync"));
    const double off2 = ctx->grid_host[0], diag2 = ctx->grid_host[1];
    if (sweeps == 0) norm2 = off2 + diag2;
    ratio = norm2 > 0.0 ? std::sqrt(off2 / norm2) : 0.0;
    if (ratio <= tolerance || sweeps >= max_sweeps) break;
    if (use_graph) {
      MSQ_TRY(cudaCheck(ctx, cudaGraphLaunch(ctx->grid_exec, s), "graph launch"));
      ++ctx->graph_launches;
      ctx->launches += 2 * static_cast<uint64_t>(nb - 1);
    } else {
      MSQ_TRY(enqueueSweep(s));
    }
    ++sweeps;
  }
  {
    dim3 grid((n + 31) / 32, (n + 31) / 32);
    gridFinishKernel<<<grid, 256, 0, s>>>(g, matrix, vectors, eigenvalues);
    MSQ_TRY(launched(ctx, "jacobi grid finish"));
  }
  if (sweeps_out) *sweeps_out = sweeps;
  if (off_ratio_out) *off_ratio_out = ratio;
  if (norm2_out) *norm2_out = norm2;
  return MSQ_OK;
}

}  // namespace msq
