// Batched blocked parallel-order two-sided Jacobi eigensolver.
//
// Replaces MetalRuntime::symmetricJacobi (src/metal_runtime.cpp:584-646),
// its kernels jacobi_rotations_f32 / jacobi_similarity_vectors_f32 /
// jacobi_root_eigenvalues_f32 (metal_mixed_sqrt.metal:1319-1444) and the
// host-built schedule makeJacobiSchedule (src/metal_solver.cpp:50-79).
//
// The reference sweeps all n(n-1)/2 index pairs with a round-robin order,
// one 2x2 rotation per pair, a full matrix pass per round.  Here the same
// rotation (tau = (a_qq - a_pp) / (2 a_pq), t = sign(tau) / (|tau| +
// sqrt(1 + tau^2)), c = 1/sqrt(1 + t^2), s = t c; pivot element set to zero)
// is applied in a blocked order laid out for GB300:
//  * indices are grouped in blocks of 4; the blocks are paired by the same
//    round-robin ("chess tournament") rule, computed arithmetically, so a
//    sweep has m/4 - 1 rounds instead of m - 1;
//  * each block pair is an 8x8 pivot that one thread holds in registers and
//    sweeps once over its 28 index pairs (7 inner round-robin rounds),
//    accumulating the rotations into an 8x8 orthogonal Q_k;
//  * every other 8x8 super-tile of A is then updated as T' = Q_k^T T Q_l, a
//    pair of small dense products held in registers (1024 FMA per 64
//    elements), so a round is FMA-bound instead of latency-bound;
//  * the upper triangle of A is stored as packed 4x4 tiles, in shared memory
//    when it fits (n <= 328) and in an L2-resident global workspace beyond;
//  * each round's Q_k are logged and a row-parallel kernel replays the sweep
//    onto V (rows of V evolve independently under V <- V Q), so V never
//    competes with A for shared memory;
//  * rotation angles are FP32 (as in the reference's kernel); the off-norm
//    that ends the sweeps is accumulated in FP64 — sweeps stop once
//    off(A) <= tol * ||A||_F instead of after a fixed 8;
//  * launches are size-bucketed (threads per CTA grow with n), largest first.
#include "msq_internal.cuh"

#include <algorithm>
#include <vector>

namespace msq {
namespace {

constexpr int kTileF = 16;      // floats per 4x4 tile
constexpr int kQF = 64;         // floats per 8x8 rotation
constexpr size_t kSmemLimit = 227 * 1024;
constexpr int kMaxOrder = 2048;
constexpr int kSweepThreadsMax = 256;
constexpr int kReplayThreads = 256;

struct JacobiState {
  double norm2;       // ||A||_F^2
  double off_ratio;   // off(A) / ||A||_F when the sweeps stopped
  int sweeps;         // sweeps applied
  int done;           // 1 once converged or out of budget
  // logged[p]: 1 if log buffer p holds a sweep not yet applied to V.  The
  // log is double-buffered by sweep parity so sweep k+1 can run while the
  // replay of sweep k reads the other buffer.
  int logged[2];
};

struct JacobiArgs {
  float *a;                  // user matrices (full, column-major)
  float *tiles;              // packed 4x4 tiles (global workspace)
  const int64_t *a_offset;   // element offset of matrix i in a
  const int64_t *t_offset;   // float offset of matrix i's tiles
  const int64_t *log_offset; // float offset of matrix i's rotation log
  const int64_t *eig_offset;
  const int32_t *n;
  float *log;
  float *eigenvalues;
  JacobiState *state;
  const int32_t *order;      // matrix ids of this launch, largest first
  double tol;
  int max_sweeps;
  int first;                 // 1 on the first launch (load A, set norm)
  int parity;                // log buffer of this sweep (log points at it)
};

__host__ __device__ constexpr int padded8(int n) { return (n + 7) & ~7; }

// Slot -> participant of round r (participants 1..m-1 rotate right by one
// per round, slot 0 fixed): the closed form of the std::rotate step in
// makeJacobiSchedule (src/metal_solver.cpp:75-76).
__device__ __forceinline__ int rrSlot(int slot, int round, int m) {
  if (slot == 0) return 0;
  int k = slot - 1 - round % (m - 1);
  if (k < 0) k += m - 1;
  return 1 + k;
}

__device__ __forceinline__ void rrPair(int pair, int round, int m, int &p, int &q) {
  const int a = rrSlot(pair, round, m);
  const int b = rrSlot(m - 1 - pair, round, m);
  p = a < b ? a : b;
  q = a < b ? b : a;
}

// Folded enumeration of the upper triangle {(i, j): i <= j < P}: rows i and
// P-1-i share one folded row of P+1 items.
__device__ __forceinline__ bool foldedBlock(int w, int P, int &i, int &j) {
  const int r = w / (P + 1);
  const int c = w - r * (P + 1);
  if (c < P - r) {
    i = r;
    j = r + c;
    return true;
  }
  if ((P & 1) && r == P / 2) return false;
  i = P - 1 - r;
  j = c - 1;
  return true;
}

__device__ double blockReduceSum(double v, double *red) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  const int warps = blockDim.x / 32;
  v = threadIdx.x < warps ? red[threadIdx.x] : 0.0;
  if (warp == 0) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  const double total = red[0];
  __syncthreads();
  return total;
}

// Packed tile (I, J), I <= J, of a matrix's tile array: tile index
// tri[J] + I, 16 floats.  A 4x4 tile spans half the 32 shared-memory banks,
// so without care the rows of all tiles would fall on two bank groups; row
// i of tile t is stored at physical row i ^ (t & 3), which spreads the
// float4 rows a warp touches over all eight 4-bank groups.
__device__ __forceinline__ int tileIndex(const int *tri, int I, int J) { return tri[J] + I; }

__device__ __forceinline__ int64_t tileElement(int t, int i, int j) {
  return static_cast<int64_t>(t) * kTileF + (((i ^ (t & 3)) << 2) | j);
}

// Loads block (R, C) of A (4x4, row-major in t) from the packed tiles.
__device__ __forceinline__ void loadBlock(float *tiles, const int *tri, int R, int C, float (&t)[4][4]) {
  if (R <= C) {
    const int ti = tileIndex(tri, R, C);
    const float4 *src = reinterpret_cast<const float4 *>(tiles + static_cast<int64_t>(ti) * kTileF);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 v = src[i ^ (ti & 3)];
      t[i][0] = v.x; t[i][1] = v.y; t[i][2] = v.z; t[i][3] = v.w;
    }
  } else {
    const int ti = tileIndex(tri, C, R);
    const float4 *src = reinterpret_cast<const float4 *>(tiles + static_cast<int64_t>(ti) * kTileF);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 v = src[i ^ (ti & 3)];
      t[0][i] = v.x; t[1][i] = v.y; t[2][i] = v.z; t[3][i] = v.w;
    }
  }
}

__device__ __forceinline__ void storeBlock(float *tiles, const int *tri, int R, int C, const float (&t)[4][4]) {
  if (R <= C) {
    const int ti = tileIndex(tri, R, C);
    float4 *dst = reinterpret_cast<float4 *>(tiles + static_cast<int64_t>(ti) * kTileF);
#pragma unroll
    for (int i = 0; i < 4; ++i) dst[i ^ (ti & 3)] = make_float4(t[i][0], t[i][1], t[i][2], t[i][3]);
  } else {
    const int ti = tileIndex(tri, C, R);
    float4 *dst = reinterpret_cast<float4 *>(tiles + static_cast<int64_t>(ti) * kTileF);
#pragma unroll
    for (int i = 0; i < 4; ++i) dst[i ^ (ti & 3)] = make_float4(t[0][i], t[1][i], t[2][i], t[3][i]);
  }
}

// One Jacobi rotation of the 8x8 pivot p on the index pair (a, b), the
// reference's angle formula (metal_mixed_sqrt.metal:1347-1357), accumulated
// into q (q <- q J).  J = [c s; -s c] on (a, b): column a' = c a - s b,
// column b' = s a + c b; p <- J^T p J with the pivot element set to zero.
// Every operation is an explicitly rounded one (no contraction into FMA, no
// approximate reciprocal square root), so the rotation is the same bit for
// bit as the C restatement compiled with -ffp-contract=off.
template <int a, int b>
__device__ __forceinline__ void rotatePivot(float (&p)[8][8], float (&q)[8][8]) {
  const float apq = p[a][b];
  if (apq == 0.0f) return;
  const float tau = __fdiv_rn(__fsub_rn(p[b][b], p[a][a]), __fmul_rn(2.0f, apq));
  const float root = __fsqrt_rn(__fadd_rn(__fmul_rn(tau, tau), 1.0f));
  const float t = copysignf(__fdiv_rn(1.0f, __fadd_rn(fabsf(tau), root)), tau);
  float c = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fmul_rn(t, t), 1.0f)));
  float s = __fmul_rn(t, c);
  // FP32 (c, s) carry a one-signed error in c^2 + s^2 - 1 that compounds
  // over the thousands of rotations applied to each row of V.  Evaluate
  // e = c^2 + s^2 - 1 exactly (two-product: each square split by an FMA;
  // c^2 >= 1/2 so c^2 - 1 is exact) and pull (c, s) back by (1 - e/2): the
  // rotation is then as orthogonal as one computed in FP64 and rounded.
  {
    const float cc = __fmul_rn(c, c), cce = fmaf(c, c, -cc);
    const float ss = __fmul_rn(s, s), sse = fmaf(s, s, -ss);
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(cc, 1.0f), ss), __fadd_rn(cce, sse));
    const float h = __fmul_rn(-0.5f, e);
    c = fmaf(h, c, c);
    s = fmaf(h, s, s);
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float pa = p[i][a], pb = p[i][b];
    p[i][a] = __fsub_rn(__fmul_rn(c, pa), __fmul_rn(s, pb));
    p[i][b] = __fadd_rn(__fmul_rn(s, pa), __fmul_rn(c, pb));
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float pa = p[a][j], pb = p[b][j];
    p[a][j] = __fsub_rn(__fmul_rn(c, pa), __fmul_rn(s, pb));
    p[b][j] = __fadd_rn(__fmul_rn(s, pa), __fmul_rn(c, pb));
  }
  p[a][b] = 0.0f;
  p[b][a] = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float qa = q[i][a], qb = q[i][b];
    q[i][a] = __fsub_rn(__fmul_rn(c, qa), __fmul_rn(s, qb));
    q[i][b] = __fadd_rn(__fmul_rn(s, qa), __fmul_rn(c, qb));
  }
}

// One cyclic sweep over the 28 pairs of the pivot in round-robin order
// (7 rounds of 4 disjoint pairs; disjoint rotations commute).
__device__ __forceinline__ void sweepPivot(float (&p)[8][8], float (&q)[8][8]) {
  rotatePivot<0, 7>(p, q); rotatePivot<1, 6>(p, q); rotatePivot<2, 5>(p, q); rotatePivot<3, 4>(p, q);
  rotatePivot<0, 6>(p, q); rotatePivot<5, 7>(p, q); rotatePivot<1, 4>(p, q); rotatePivot<2, 3>(p, q);
  rotatePivot<0, 5>(p, q); rotatePivot<4, 6>(p, q); rotatePivot<3, 7>(p, q); rotatePivot<1, 2>(p, q);
  rotatePivot<0, 4>(p, q); rotatePivot<3, 5>(p, q); rotatePivot<2, 6>(p, q); rotatePivot<1, 7>(p, q);
  rotatePivot<0, 3>(p, q); rotatePivot<2, 4>(p, q); rotatePivot<1, 5>(p, q); rotatePivot<6, 7>(p, q);
  rotatePivot<0, 2>(p, q); rotatePivot<1, 3>(p, q); rotatePivot<4, 7>(p, q); rotatePivot<5, 6>(p, q);
  rotatePivot<0, 1>(p, q); rotatePivot<2, 7>(p, q); rotatePivot<3, 6>(p, q); rotatePivot<4, 5>(p, q);
}

struct SweepSmem {
  double *red;
  int *tri;
  int *pair_i;
  int *pair_j;
  float *q;
  float *tiles;
};

__host__ __device__ __forceinline__ size_t sweepSmemLayout(int n, bool with_tiles, size_t *q_off,
                                                           size_t *tile_off) {
  const int m = padded8(n), nb = m / 4, P = nb / 2;
  size_t bytes = 32 * sizeof(double) + (nb + 1 + 2 * P) * sizeof(int);
  bytes = (bytes + 15) & ~static_cast<size_t>(15);
  *q_off = bytes;
  bytes += static_cast<size_t>(P) * kQF * sizeof(float);
  *tile_off = bytes;
  if (with_tiles) bytes += static_cast<size_t>(nb) * (nb + 1) / 2 * kTileF * sizeof(float);
  return bytes;
}

// One sweep (or the convergence check / write-back) for one matrix per CTA.
template <bool kSmem>
__global__ void __launch_bounds__(kSweepThreadsMax)
jacobiSweepKernel(JacobiArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mi = args.order[blockIdx.x];
  const int n = args.n[mi];
  const int m = padded8(n), nb = m / 4, P = nb / 2;
  JacobiState &st = args.state[mi];
  // Snapshot of the state before any thread writes it (the barriers below
  // keep thread 0's final update after every warp's snapshot).
  const JacobiState s0 = st;
  if (!args.first && s0.done) {
    if (threadIdx.x == 0) st.logged[args.parity] = 0;
    return;
  }
  size_t q_off, tile_off;
  sweepSmemLayout(n, kSmem, &q_off, &tile_off);
  double *red = reinterpret_cast<double *>(smem_raw);
  int *tri = reinterpret_cast<int *>(red + 32);
  int *pair_i = tri + nb + 1;
  int *pair_j = pair_i + P;
  float *qs = reinterpret_cast<float *>(smem_raw + q_off);
  float *gtiles = args.tiles + args.t_offset[mi];
  float *tiles = kSmem ? reinterpret_cast<float *>(smem_raw + tile_off) : gtiles;
  const int tile_floats = nb * (nb + 1) / 2 * kTileF;
  const float *full = args.a + args.a_offset[mi];

  for (int k = threadIdx.x; k <= nb; k += blockDim.x) tri[k] = k * (k + 1) / 2;
  __syncthreads();

  if (args.first) {
    // Symmetrised load, as working_from_symmetric_f32 and the averaged a_pq
    // of jacobi_rotations_f32 do (metal_mixed_sqrt.metal:1349-1350, 1922).
    for (int J = 0; J < nb; ++J) {
      for (int idx = threadIdx.x; idx < (J + 1) * kTileF; idx += blockDim.x) {
        const int I = idx / kTileF, e = idx % kTileF;
        const int gi = 4 * I + e / 4, gj = 4 * J + e % 4;
        float v = 0.0f;
        if (gi < n && gj < n) {
          v = 0.5f * (full[gi + static_cast<int64_t>(gj) * n] + full[gj + static_cast<int64_t>(gi) * n]);
        }
        tiles[tileElement(tri[J] + I, e / 4, e % 4)] = v;
      }
    }
  } else if (kSmem) {
    for (int k = threadIdx.x; k < tile_floats / 4; k += blockDim.x) {
      reinterpret_cast<float4 *>(tiles)[k] = reinterpret_cast<const float4 *>(gtiles)[k];
    }
  }
  __syncthreads();

  // Off-norm and norm in FP64.
  double off2 = 0.0, diag2 = 0.0;
  for (int J = 0; J < nb; ++J) {
    for (int idx = threadIdx.x; idx < (J + 1) * kTileF; idx += blockDim.x) {
      const int I = idx / kTileF, e = idx % kTileF;
      const double v = tiles[tileElement(tri[J] + I, e / 4, e % 4)];
      if (I < J) off2 += 2.0 * v * v;
      else if (e / 4 == e % 4) diag2 += v * v;
      else off2 += v * v;
    }
  }
  off2 = blockReduceSum(off2, red);
  diag2 = blockReduceSum(diag2, red);
  const double norm2 = args.first ? off2 + diag2 : s0.norm2;
  const int sweeps = args.first ? 0 : s0.sweeps;
  const double ratio = norm2 > 0.0 ? sqrt(off2 / norm2) : 0.0;

  if (ratio <= args.tol || sweeps >= args.max_sweeps) {
    // Eigenvalues = diagonal (jacobi_root_eigenvalues_f32 takes the sqrt
    // later, :1436-1444); full symmetric write-back of the matrix.
    float *eig = args.eigenvalues + args.eig_offset[mi];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      eig[k] = tiles[tileElement(tri[k / 4] + k / 4, k % 4, k % 4)];
    }
    float *out = args.a + args.a_offset[mi];
    for (int c = 0; c < n; ++c) {
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        const int I = r / 4, J = c / 4;
        const float v = I <= J ? tiles[tileElement(tri[J] + I, r % 4, c % 4)]
                               : tiles[tileElement(tri[I] + J, c % 4, r % 4)];
        out[r + static_cast<int64_t>(c) * n] = v;
      }
    }
    if (threadIdx.x == 0) {
      st.norm2 = norm2;
      st.sweeps = sweeps;
      st.off_ratio = ratio;
      st.done = 1;
      st.logged[args.parity] = 0;
    }
    return;
  }

  float *log = args.log + args.log_offset[mi];
  const int items = ((P + 1) / 2) * (P + 1);
  for (int round = 0; round < nb - 1; ++round) {
    // Pivots: one thread per block pair sweeps its 8x8 pivot in registers.
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
      int I, J;
      rrPair(k, round, nb, I, J);
      pair_i[k] = I;
      pair_j[k] = J;
      float p[8][8], q[8][8];
      {
        float t[4][4];
        loadBlock(tiles, tri, I, I, t);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) p[i][j] = t[i][j];
        loadBlock(tiles, tri, I, J, t);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            p[i][4 + j] = t[i][j];
            p[4 + j][i] = t[i][j];
          }
        loadBlock(tiles, tri, J, J, t);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) p[4 + i][4 + j] = t[i][j];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) q[i][j] = i == j ? 1.0f : 0.0f;
      sweepPivot(p, q);
      {
        float t[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) t[i][j] = p[i][j];
        storeBlock(tiles, tri, I, I, t);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) t[i][j] = p[i][4 + j];
        storeBlock(tiles, tri, I, J, t);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) t[i][j] = p[4 + i][4 + j];
        storeBlock(tiles, tri, J, J, t);
      }
      float4 *qdst = reinterpret_cast<float4 *>(qs + k * kQF);
      float4 *ldst = reinterpret_cast<float4 *>(log + (static_cast<int64_t>(round) * P + k) * kQF);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float4 lo = make_float4(q[i][0], q[i][1], q[i][2], q[i][3]);
        const float4 hi = make_float4(q[i][4], q[i][5], q[i][6], q[i][7]);
        qdst[2 * i] = lo;
        qdst[2 * i + 1] = hi;
        ldst[2 * i] = lo;
        ldst[2 * i + 1] = hi;
      }
    }
    __syncthreads();
    // Off-pivot super-tiles: T' = Q_k^T T Q_l for every k < l.
    for (int w = threadIdx.x; w < items; w += blockDim.x) {
      int k, l;
      if (!foldedBlock(w, P, k, l) || k == l) continue;
      const int rb[2] = {pair_i[k], pair_j[k]};
      const int cb[2] = {pair_i[l], pair_j[l]};
      float t[8][8];
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          float b4[4][4];
          loadBlock(tiles, tri, rb[x], cb[y], b4);
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) t[4 * x + i][4 * y + j] = b4[i][j];
        }
      float u[8][8];
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 8; ++c) u[a][c] = 0.0f;
      const float4 *qk = reinterpret_cast<const float4 *>(qs + k * kQF);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float4 lo = qk[2 * i], hi = qk[2 * i + 1];
        const float qr[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int c = 0; c < 8; ++c) u[a][c] = fmaf(qr[a], t[i][c], u[a][c]);
      }
      const float4 *ql = reinterpret_cast<const float4 *>(qs + l * kQF);
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 8; ++c) t[a][c] = 0.0f;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 lo = ql[2 * j], hi = ql[2 * j + 1];
        const float qr[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int c = 0; c < 8; ++c) t[a][c] = fmaf(u[a][j], qr[c], t[a][c]);
      }
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          float b4[4][4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) b4[i][j] = t[4 * x + i][4 * y + j];
          storeBlock(tiles, tri, rb[x], cb[y], b4);
        }
    }
    __syncthreads();
  }
  if (kSmem) {
    for (int k = threadIdx.x; k < tile_floats / 4; k += blockDim.x) {
      reinterpret_cast<float4 *>(gtiles)[k] = reinterpret_cast<const float4 *>(tiles)[k];
    }
  }
  if (threadIdx.x == 0) {
    st.norm2 = norm2;
    st.off_ratio = ratio;
    st.sweeps = sweeps + 1;
    st.done = 0;
    st.logged[args.parity] = 1;
  }
}

struct VArgs {
  float *v;
  const int64_t *a_offset;
  const int64_t *log_offset;
  const int32_t *n;
  const float *log;
  const JacobiState *state;
  const int32_t *work_matrix;  // per CTA: matrix id
  const int32_t *work_row;     // per CTA: first row
  int rows_per_cta;            // multiple of 8
  int parity;                  // log buffer to replay (log points at it)
};

__host__ __device__ __forceinline__ size_t replaySmemBytes(int max_n, int rows) {
  const int m = padded8(max_n), P = m / 8;
  return static_cast<size_t>(rows) * (m + 4) * sizeof(float) + static_cast<size_t>(P) * kQF * sizeof(float);
}

// Replays one logged sweep onto `rows` rows of V: V <- V Q_k on the column
// blocks (I_k, J_k) of every pair, round by round (the V update of
// jacobi_similarity_vectors_f32 z = 1, metal_mixed_sqrt.metal:1380-1390,
// with 8x8 rotations).  A thread applies one Q_k (held in registers) to 8
// rows.
__global__ void __launch_bounds__(kReplayThreads)
jacobiReplayKernel(VArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mi = args.work_matrix[blockIdx.x];
  if (!args.state[mi].logged[args.parity]) return;
  const int r0 = args.work_row[blockIdx.x];
  const int n = args.n[mi];
  const int m = padded8(n), nb = m / 4, P = nb / 2;
  const int R = args.rows_per_cta, ld = m + 4;
  float *vs = reinterpret_cast<float *>(smem_raw);    // [R][ld]
  float *qs = vs + static_cast<size_t>(R) * ld;       // [P][64]
  float *v = args.v + args.a_offset[mi];
  const int rows = min(R, n - r0);
  for (int k = threadIdx.x; k < m * R; k += blockDim.x) {
    const int c = k / R, r = k % R;
    vs[r * ld + c] = (c < n && r < rows) ? v[r0 + r + static_cast<int64_t>(c) * n] : 0.0f;
  }
  const float *log = args.log + args.log_offset[mi];
  const int groups = R / 8;
  for (int round = 0; round < nb - 1; ++round) {
    __syncthreads();
    const float4 *src = reinterpret_cast<const float4 *>(log + static_cast<int64_t>(round) * P * kQF);
    for (int k = threadIdx.x; k < P * kQF / 4; k += blockDim.x) reinterpret_cast<float4 *>(qs)[k] = src[k];
    __syncthreads();
    for (int item = threadIdx.x; item < P * groups; item += blockDim.x) {
      const int k = item % P, g = item / P;
      int I, J;
      rrPair(k, round, nb, I, J);
      float q[8][8];
      const float4 *qk = reinterpret_cast<const float4 *>(qs + k * kQF);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float4 lo = qk[2 * i], hi = qk[2 * i + 1];
        q[i][0] = lo.x; q[i][1] = lo.y; q[i][2] = lo.z; q[i][3] = lo.w;
        q[i][4] = hi.x; q[i][5] = hi.y; q[i][6] = hi.z; q[i][7] = hi.w;
      }
#pragma unroll 2
      for (int rr = 0; rr < 8; ++rr) {
        float *row = vs + (g * 8 + rr) * ld;
        const float4 a = *reinterpret_cast<const float4 *>(row + 4 * I);
        const float4 b = *reinterpret_cast<const float4 *>(row + 4 * J);
        const float x[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        float o[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float s = 0.0f;
#pragma unroll
          for (int j = 0; j < 8; ++j) s = fmaf(x[j], q[j][c], s);
          o[c] = s;
        }
        *reinterpret_cast<float4 *>(row + 4 * I) = make_float4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<float4 *>(row + 4 * J) = make_float4(o[4], o[5], o[6], o[7]);
      }
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n * R; k += blockDim.x) {
    const int c = k / R, r = k % R;
    if (r < rows) v[r0 + r + static_cast<int64_t>(c) * n] = vs[r * ld + c];
  }
}

__global__ void identityKernel(float *v, const int64_t *a_offset, const int32_t *n, int count) {
  for (int mi = blockIdx.y; mi < count; mi += gridDim.y) {
    const int64_t nn = static_cast<int64_t>(n[mi]) * n[mi];
    float *out = v + a_offset[mi];
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
      const int64_t r = k % n[mi], c = k / n[mi];
      out[k] = r == c ? 1.0f : 0.0f;
    }
  }
}

__global__ void jacobiReportKernel(const JacobiState *state, int count, int32_t *sweeps,
                                   float *off_ratio) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    if (sweeps) sweeps[i] = state[i].sweeps;
    if (off_ratio) off_ratio[i] = static_cast<float>(state[i].off_ratio);
  }
}

int threadsFor(int n) {
  if (n <= 16) return 32;
  if (n <= 32) return 64;
  if (n <= 64) return 128;
  return kSweepThreadsMax;
}

bool fitsSmem(int n) {
  size_t q_off, tile_off;
  return sweepSmemLayout(n, true, &q_off, &tile_off) <= kSmemLimit;
}

int replayRows(int max_n) {
  for (int rows = 32; rows >= 8; rows -= 8)
    if (replaySmemBytes(max_n, rows) <= kSmemLimit) return rows;
  return 0;
}

// Per-layout launch plan, kept per batch layout and device.
struct JacobiPlan {
  uint64_t key = 0;
  int count = 0;
  int device_id = 0;
  int64_t tile_total = 0, log_total = 0;
  int64_t *t_offset = nullptr, *log_offset = nullptr;
  int32_t *order = nullptr;  // ids grouped by bucket, largest first
  struct Bucket { int threads; bool smem; int first; int count; size_t smem_bytes; };
  std::vector<Bucket> buckets;
  int32_t *work_matrix = nullptr, *work_row = nullptr;
  int work_count = 0;
  int rows_per_cta = 0;
  size_t v_smem = 0;
  void *device = nullptr;
};

std::vector<JacobiPlan *> g_plans;

JacobiPlan *planFor(msq_ctx *ctx, const DeviceBatch *b) {
  for (JacobiPlan *p : g_plans)
    if (p->key == b->key && p->count == b->count && p->device_id == ctx->device) return p;
  auto *plan = new JacobiPlan;
  plan->device_id = ctx->device;
  plan->key = b->key;
  plan->count = b->count;
  const int count = b->count;
  std::vector<int64_t> t_off(count), l_off(count);
  for (int i = 0; i < count; ++i) {
    const int m = padded8(b->host_n[i]), nb = m / 4, P = nb / 2;
    t_off[i] = plan->tile_total;
    plan->tile_total += static_cast<int64_t>(nb) * (nb + 1) / 2 * kTileF;
    l_off[i] = plan->log_total;
    plan->log_total += static_cast<int64_t>(nb - 1) * P * kQF;
  }
  std::vector<int32_t> ids(count);
  for (int i = 0; i < count; ++i) ids[i] = i;
  auto key = [&](int i) { return threadsFor(b->host_n[i]) * (fitsSmem(b->host_n[i]) ? 1 : 2); };
  std::stable_sort(ids.begin(), ids.end(), [&](int x, int y) {
    if (key(x) != key(y)) return key(x) > key(y);
    return b->host_n[x] > b->host_n[y];
  });
  for (int i = 0; i < count;) {
    const int n0 = b->host_n[ids[i]];
    const int t = threadsFor(n0);
    const bool smem = fitsSmem(n0);
    int j = i;
    size_t bytes = 0;
    while (j < count && threadsFor(b->host_n[ids[j]]) == t && fitsSmem(b->host_n[ids[j]]) == smem) {
      size_t q_off, tile_off;
      bytes = std::max(bytes, sweepSmemLayout(b->host_n[ids[j]], smem, &q_off, &tile_off));
      ++j;
    }
    plan->buckets.push_back({t, smem, i, j - i, bytes});
    i = j;
  }
  plan->rows_per_cta = replayRows(b->max_n);
  plan->v_smem = replaySmemBytes(b->max_n, plan->rows_per_cta);
  std::vector<int32_t> wm, wr;
  for (int i = 0; i < count; ++i) {
    const int n = b->host_n[ids[i]];
    for (int r = 0; r < n; r += plan->rows_per_cta) {
      wm.push_back(ids[i]);
      wr.push_back(r);
    }
  }
  plan->work_count = static_cast<int>(wm.size());
  const size_t bytes = 2 * count * sizeof(int64_t) + count * sizeof(int32_t) +
                       2 * wm.size() * sizeof(int32_t) + 64;
  char *dev = nullptr;
  if (cudaCheck(ctx, cudaMalloc(&dev, bytes), "jacobi plan alloc") != MSQ_OK) {
    delete plan;
    return nullptr;
  }
  plan->device = dev;
  plan->t_offset = reinterpret_cast<int64_t *>(dev);
  plan->log_offset = plan->t_offset + count;
  plan->order = reinterpret_cast<int32_t *>(plan->log_offset + count);
  plan->work_matrix = plan->order + count;
  plan->work_row = plan->work_matrix + wm.size();
  cudaMemcpy(plan->t_offset, t_off.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->log_offset, l_off.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->order, ids.data(), count * sizeof(int32_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->work_matrix, wm.data(), wm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->work_row, wr.data(), wr.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (g_plans.size() >= 8) {
    cudaFree(g_plans.front()->device);
    delete g_plans.front();
    g_plans.erase(g_plans.begin());
  }
  g_plans.push_back(plan);
  return plan;
}

int setKernelAttributes() {
  static bool done = false;
  if (done) return MSQ_OK;
  if (cudaFuncSetAttribute(jacobiSweepKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kSmemLimit)) != cudaSuccess ||
      cudaFuncSetAttribute(jacobiSweepKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kSmemLimit)) != cudaSuccess ||
      cudaFuncSetAttribute(jacobiReplayKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kSmemLimit)) != cudaSuccess) {
    return MSQ_ERR_CUDA;
  }
  done = true;
  return MSQ_OK;
}

}  // namespace

// Enqueues the whole solve on ctx->stream (Jacobi scratch arena).
int jacobiEnqueue(msq_ctx *ctx, const DeviceBatch *b, float *matrices, float *vectors,
                  float *eigenvalues, double tolerance, int max_sweeps, int32_t *sweeps_done,
                  float *off_ratio) {
  if (b->max_n > kMaxOrder) {
    return setError(ctx, MSQ_ERR_UNSUPPORTED, "jacobi: order above 2048 is not supported");
  }
  JacobiPlan *plan = planFor(ctx, b);
  if (plan == nullptr) return MSQ_ERR_CUDA;
  if (plan->buckets.empty()) return MSQ_OK;
  const size_t state_bytes = (b->count * sizeof(JacobiState) + 255) & ~size_t(255);
  const size_t tile_bytes = (plan->tile_total * sizeof(float) + 255) & ~size_t(255);
  // Two log buffers (sweep parity) so sweep k+1 overlaps the replay of k.
  const size_t log_bytes = 2 * plan->log_total * sizeof(float);
  char *work = static_cast<char *>(scratch(ctx, state_bytes + tile_bytes + log_bytes, kScratchJacobi));
  if (work == nullptr) return MSQ_ERR_CUDA;
  if (setKernelAttributes() != MSQ_OK) return cudaCheck(ctx, cudaGetLastError(), "jacobi attributes");
  JacobiArgs args{};
  args.a = matrices;
  args.state = reinterpret_cast<JacobiState *>(work);
  args.tiles = reinterpret_cast<float *>(work + state_bytes);
  float *log_base = reinterpret_cast<float *>(work + state_bytes + tile_bytes);
  args.a_offset = b->offset;
  args.t_offset = plan->t_offset;
  args.log_offset = plan->log_offset;
  args.eig_offset = b->eig_offset;
  args.n = b->n;
  args.eigenvalues = eigenvalues;
  args.tol = tolerance;
  args.max_sweeps = max_sweeps;
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(args.state, 0, state_bytes, ctx->stream), "state reset"));
  {
    dim3 grid(64, std::min(b->count, 65535));
    identityKernel<<<grid, 256, 0, ctx->stream>>>(vectors, b->offset, b->n, b->count);
    MSQ_TRY(launched(ctx, "jacobi identity"));
  }
  VArgs vargs{vectors, b->offset, plan->log_offset, b->n, log_base, args.state,
              plan->work_matrix, plan->work_row, plan->rows_per_cta, 0};
  // Streams: size buckets round-robin over three sweep streams, the replay
  // on a fourth.  Order: sweep k of a bucket follows sweep k-1 (same
  // stream) and the replay of k-2 (which read the log buffer sweep k
  // overwrites); the replay of k follows every bucket's sweep k.
  syncReset(ctx);
  const int sweep_streams = std::min<int>(3, static_cast<int>(plan->buckets.size()));
  cudaStream_t ss[3];
  for (int i = 0; i < sweep_streams; ++i) {
    ss[i] = auxStream(ctx, 1 + i);
    MSQ_TRY(streamWait(ctx, ss[i], ctx->stream));
  }
  cudaStream_t rs = auxStream(ctx, 0);
  MSQ_TRY(streamWait(ctx, rs, ctx->stream));
  cudaEvent_t replay_done[2] = {nullptr, nullptr};  // by parity
  for (int launch = 0; launch <= max_sweeps; ++launch) {
    const int parity = launch & 1;
    args.first = launch == 0;
    args.parity = parity;
    args.log = log_base + parity * plan->log_total;
    if (replay_done[parity] != nullptr) {
      for (int i = 0; i < sweep_streams; ++i) {
        MSQ_TRY(cudaCheck(ctx, cudaStreamWaitEvent(ss[i], replay_done[parity], 0), "stream wait"));
      }
    }
    for (size_t k = 0; k < plan->buckets.size(); ++k) {
      const auto &bucket = plan->buckets[k];
      cudaStream_t s = ss[k % sweep_streams];
      args.order = plan->order + bucket.first;
      launchBegin(ctx, s);
      if (bucket.smem) {
        jacobiSweepKernel<true><<<bucket.count, bucket.threads, bucket.smem_bytes, s>>>(args);
      } else {
        jacobiSweepKernel<false><<<bucket.count, bucket.threads, bucket.smem_bytes, s>>>(args);
      }
      MSQ_TRY(launchedOn(ctx, s, "jacobi sweep"));
    }
    if (launch < max_sweeps) {
      for (int i = 0; i < sweep_streams; ++i) MSQ_TRY(streamWait(ctx, rs, ss[i]));
      vargs.parity = parity;
      vargs.log = args.log;
      launchBegin(ctx, rs);
      jacobiReplayKernel<<<plan->work_count, kReplayThreads, plan->v_smem, rs>>>(vargs);
      MSQ_TRY(launchedOn(ctx, rs, "jacobi replay"));
      replay_done[parity] = syncEvent(ctx);
      MSQ_TRY(cudaCheck(ctx, cudaEventRecord(replay_done[parity], rs), "event record"));
    }
  }
  for (int i = 0; i < sweep_streams; ++i) MSQ_TRY(streamWait(ctx, ctx->stream, ss[i]));
  MSQ_TRY(streamWait(ctx, ctx->stream, rs));
  if (sweeps_done != nullptr || off_ratio != nullptr) {
    jacobiReportKernel<<<gridFor(b->count, 256), 256, 0, ctx->stream>>>(args.state, b->count,
                                                                       sweeps_done, off_ratio);
    MSQ_TRY(launched(ctx, "jacobi report"));
  }
  return MSQ_OK;
}

}  // namespace msq

using namespace msq;

extern "C" int msq_jacobi_batched(msq_ctx *ctx, float *matrices, float *vectors,
                                  float *eigenvalues, const int32_t *n,
                                  const int64_t *offset, int count,
                                  double tolerance, int max_sweeps,
                                  int32_t *sweeps_done, float *off_ratio) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  if (matrices == nullptr || vectors == nullptr || eigenvalues == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_jacobi_batched: null buffer");
  }
  if (!(tolerance >= 0.0) || max_sweeps < 0 || max_sweeps > 64) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_jacobi_batched: tolerance must be >= 0, max_sweeps in [0, 64]");
  }
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return jacobiEnqueue(ctx, b, matrices, vectors, eigenvalues, tolerance,
                       max_sweeps, sweeps_done, off_ratio);
}

// ---------------------------------------------------------------------------
// Jacobi for callers that must not allocate device memory.
//
// Latency-critical loops (cudaMalloc/cudaFree may synchronise the device and
// take unbounded time) and host applications that own all device memory
// cannot use the context's grow-only scratch.  msq_jacobi_noalloc solves one
// matrix with the same kernels as msq_jacobi_batched, but every piece of
// scratch (the packed tiles of A, the per-round rotation log, the sweep state
// and the small layout tables) lives in the file-scope array below, sized
// for one matrix of order up to MSQ_NOALLOC_MAX_ORDER: 130 KiB of tiles,
// 504 KiB of log and a few hundred bytes of tables, about 0.65 MB in all.
// The array is part of the loaded module, so every GPU that loads this
// library holds it until the process exits.  It uses one log buffer (parity
// 0): sweeps and replays alternate on the caller's stream.
namespace msq {
namespace {

constexpr int kNoAllocOrder = MSQ_NOALLOC_MAX_ORDER;
constexpr int kNoAllocBlocks = padded8(kNoAllocOrder) / 4;
constexpr int kNoAllocPairs = kNoAllocBlocks / 2;
constexpr int kNoAllocRowsPerCta = 32;
constexpr int kNoAllocCtas = (kNoAllocOrder + kNoAllocRowsPerCta - 1) / kNoAllocRowsPerCta;

struct NoAllocScratch {
  JacobiState state[1];
  int32_t n[1];
  int32_t order[1];
  int64_t a_offset[1];  // all offsets are zero: one matrix
  int64_t t_offset[1];
  int64_t log_offset[1];
  int64_t eig_offset[1];
  int32_t work_matrix[kNoAllocCtas];
  int32_t work_row[kNoAllocCtas];
  alignas(16) float tiles[kNoAllocBlocks * (kNoAllocBlocks + 1) / 2 * kTileF];
  alignas(16) float log[(kNoAllocBlocks - 1) * kNoAllocPairs * kQF];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// Device address of g_noalloc_scratch per device, looked up once per device
// (cudaGetSymbolAddress with that device current).  Host code must not use
// the symbol itself: on the host it names a stand-in, not device memory.
NoAllocScratch *g_noalloc_address[64] = {};

// Resets what must start at zero (the sweep state) and writes the one-matrix
// layout tables; the tiles and the log are fully written before being read.
__global__ void noAllocSetupKernel(NoAllocScratch *s, int n) {
  const int t = threadIdx.x;
  if (t == 0) {
    s->state[0] = JacobiState{};
    s->n[0] = n;
    s->order[0] = 0;
    s->a_offset[0] = 0;
    s->t_offset[0] = 0;
    s->log_offset[0] = 0;
    s->eig_offset[0] = 0;
  }
  for (int r = t; r < kNoAllocCtas; r += blockDim.x) {
    s->work_matrix[r] = 0;
    s->work_row[r] = r * kNoAllocRowsPerCta;
  }
}

}  // namespace
}  // namespace msq

extern "C" int msq_jacobi_noalloc(float *matrix, float *vectors, float *eigenvalues, int n,
                                  double tolerance, int max_sweeps, void *stream,
                                  int32_t *sweeps_done, float *off_ratio) {
  if (matrix == nullptr || vectors == nullptr || eigenvalues == nullptr) {
    return MSQ_ERR_INVALID_ARGUMENT;
  }
  if (n < 1 || n > kNoAllocOrder) return MSQ_ERR_INVALID_ARGUMENT;  // beyond the static scratch
  if (!(tolerance >= 0.0) || max_sweeps < 0 || max_sweeps > 64) return MSQ_ERR_INVALID_ARGUMENT;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MSQ_ERR_CUDA;
  NoAllocScratch *s = g_noalloc_address[device];
  if (s == nullptr) {
    // One-time set-up for this device (so the first call on a device should
    // come before any stream capture).
    void *address = nullptr;
    if (cudaGetSymbolAddress(&address, g_noalloc_scratch) != cudaSuccess || address == nullptr) {
      return MSQ_ERR_CUDA;
    }
    if (setKernelAttributes() != MSQ_OK) return MSQ_ERR_CUDA;
    s = static_cast<NoAllocScratch *>(address);
    g_noalloc_address[device] = s;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  noAllocSetupKernel<<<1, 128, 0, st>>>(s, n);
  JacobiArgs args{};
  args.a = matrix;
  args.tiles = s->tiles;
  args.a_offset = s->a_offset;
  args.t_offset = s->t_offset;
  args.log_offset = s->log_offset;
  args.eig_offset = s->eig_offset;
  args.n = s->n;
  args.log = s->log;
  args.eigenvalues = eigenvalues;
  args.state = s->state;
  args.order = s->order;
  args.tol = tolerance;
  args.max_sweeps = max_sweeps;
  const bool smem = fitsSmem(n);
  size_t q_off, tile_off;
  const size_t sweep_smem = sweepSmemLayout(n, smem, &q_off, &tile_off);
  const int rows = (n + kNoAllocRowsPerCta - 1) / kNoAllocRowsPerCta;
  VArgs vargs{vectors, s->a_offset, s->log_offset, s->n, s->log, s->state,
              s->work_matrix, s->work_row, kNoAllocRowsPerCta};
  const size_t v_smem = replaySmemBytes(n, kNoAllocRowsPerCta);
  identityKernel<<<dim3(64, 1), 256, 0, st>>>(vectors, s->a_offset, s->n, 1);
  for (int launch = 0; launch <= max_sweeps; ++launch) {
    args.first = launch == 0;
    if (smem) {
      jacobiSweepKernel<true><<<1, threadsFor(n), sweep_smem, st>>>(args);
    } else {
      jacobiSweepKernel<false><<<1, threadsFor(n), sweep_smem, st>>>(args);
    }
    if (launch < max_sweeps) jacobiReplayKernel<<<rows, kReplayThreads, v_smem, st>>>(vargs);
  }
  if (sweeps_done != nullptr || off_ratio != nullptr) {
    jacobiReportKernel<<<1, 32, 0, st>>>(s->state, 1, sweeps_done, off_ratio);
  }
  return cudaGetLastError() == cudaSuccess ? MSQ_OK : MSQ_ERR_CUDA;
}
