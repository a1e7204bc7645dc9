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
#include <array>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace msq {
namespace {

constexpr int kTileF = 16;      // floats per 4x4 tile
constexpr int kQF = 64;         // floats per 8x8 rotation
// Shared-memory stride of the rotations in the sweep kernel: 68 floats puts
// Q_l of different pivots on different banks (a 64-float stride would map
// every Q_l row to the same four banks).
constexpr int kQS = 68;
constexpr size_t kSmemLimit = 227 * 1024;
constexpr int kMaxOrder = 2048;
constexpr int kSweepThreadsMax = 512;
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

// ---------------------------------------------------------------------------
// Pivot sweep: the 28 index pairs of an 8x8 pivot in the round-robin order of
// 8 indices, 7 groups of 4 disjoint pairs, one rotation per pair with the
// reference's angle formula (metal_mixed_sqrt.metal:1347-1357):
// tau = (p_bb - p_aa) / (2 p_ab), t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
// c = 1 / sqrt(1 + t^2), s = t c; J = [c s; -s c] on (a, b): column
// a' = c a - s b, column b' = s a + c b; p <- J^T p J, p_ab = p_ba = 0;
// Q <- Q J.
//
// A quad of lanes sweeps one pivot.  In group g lane t owns the two rows
// (a_t, b_t) of its pair.  The four angles of a group depend only on the
// pair's own 2x2 block, which no other rotation of the group touches, so
// they are computed at once and shared with shuffles; each lane then
// updates its two rows.  Element (x, y) of a row pair t and column pair j is
// touched by the row rotation of t and the column rotation of j, applied in
// the order of the pairs in the group (the sequential order); the diagonal
// block (j = t) takes the column rotation first.  Every operation is an
// explicitly rounded one (no FMA contraction, no approximate reciprocal
// square root), so the sweep equals, bit for bit, the sequential sweep of
// the C restatement compiled with -ffp-contract=off.

// Pairs of group g packed as 4 x (a: 3 bits, b: 3 bits), a < b.
__host__ __device__ constexpr uint32_t groupWord(int g) {
  constexpr int pairs[8][8] = {{0, 7, 1, 6, 2, 5, 3, 4}, {0, 6, 5, 7, 1, 4, 2, 3},
                               {0, 5, 4, 6, 3, 7, 1, 2}, {0, 4, 3, 5, 2, 6, 1, 7},
                               {0, 3, 2, 4, 1, 5, 6, 7}, {0, 2, 1, 3, 4, 7, 5, 6},
                               {0, 1, 2, 7, 3, 6, 4, 5},
                               // layout used to store the pivot: rows (t, 4 + t)
                               {0, 4, 1, 5, 2, 6, 3, 7}};
  uint32_t w = 0;
  for (int t = 0; t < 4; ++t)
    w |= static_cast<uint32_t>(pairs[g][2 * t] | (pairs[g][2 * t + 1] << 3)) << (6 * t);
  return w;
}

// For each row r: owner lane (2 bits) and slot (1 bit, 1 = second row of
// the pair) in group g, packed 3 bits per row.
__host__ __device__ constexpr uint32_t ownerWord(int g) {
  uint32_t w = 0;
  for (int t = 0; t < 4; ++t) {
    const uint32_t a = (groupWord(g) >> (6 * t)) & 7, b = (groupWord(g) >> (6 * t + 3)) & 7;
    w |= static_cast<uint32_t>(t) << (3 * a);
    w |= static_cast<uint32_t>(t | 4) << (3 * b);
  }
  return w;
}

__device__ __forceinline__ float pick8(const float (&r)[8], int i) {
  float v = r[0];
#pragma unroll
  for (int k = 1; k < 8; ++k) v = i == k ? r[k] : v;
  return v;
}

// Rotation angle of one pair (explicitly rounded; renormalised so that
// c^2 + s^2 - 1, evaluated exactly with FMA two-products, is pulled back by
// (1 - e/2): FP32 (c, s) otherwise carry a one-signed error in c^2 + s^2
// that compounds over the thousands of rotations applied to each row of V).
__device__ __forceinline__ bool jacobiAngle(float paa, float pbb, float pab, float &c, float &s) {
  c = 1.0f;
  s = 0.0f;
  if (pab == 0.0f) return false;
  const float tau = __fdiv_rn(__fsub_rn(pbb, paa), __fmul_rn(2.0f, pab));
  const float root = __fsqrt_rn(__fadd_rn(__fmul_rn(tau, tau), 1.0f));
  const float t = copysignf(__fdiv_rn(1.0f, __fadd_rn(fabsf(tau), root)), tau);
  float cc0 = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fmul_rn(t, t), 1.0f)));
  float ss0 = __fmul_rn(t, cc0);
  const float cc = __fmul_rn(cc0, cc0), cce = fmaf(cc0, cc0, -cc);
  const float ss = __fmul_rn(ss0, ss0), sse = fmaf(ss0, ss0, -ss);
  const float e = __fadd_rn(__fadd_rn(__fsub_rn(cc, 1.0f), ss), __fadd_rn(cce, sse));
  const float h = __fmul_rn(-0.5f, e);
  c = fmaf(h, cc0, cc0);
  s = fmaf(h, ss0, ss0);
  return true;
}

// x' = c x - s y, y' = s x + c y (explicitly rounded); identity if !on.
__device__ __forceinline__ void rot2(float &x, float &y, float c, float s, bool on) {
  const float nx = __fsub_rn(__fmul_rn(c, x), __fmul_rn(s, y));
  const float ny = __fadd_rn(__fmul_rn(s, x), __fmul_rn(c, y));
  x = on ? nx : x;
  y = on ? ny : y;
}

// One group of 4 rotations on the quad.  ra / rb: this lane's rows a_t / b_t
// (all 8 columns); qcol: the pivot's Q, column-major (column x at qcol[8x]).
template <int G>
__device__ __forceinline__ void pivotGroup(float (&ra)[8], float (&rb)[8], float *qcol, int t,
                                           bool active) {
  constexpr uint32_t W = groupWord(G);
  const int a = (W >> (6 * t)) & 7, b = (W >> (6 * t + 3)) & 7;
  float c, s;
  const bool on = jacobiAngle(pick8(ra, a), pick8(rb, b), pick8(ra, b), c, s);
  float cj[4], sj[4];
  bool onj[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    cj[j] = __shfl_sync(0xffffffffu, c, j, 4);
    sj[j] = __shfl_sync(0xffffffffu, s, j, 4);
    onj[j] = __shfl_sync(0xffffffffu, static_cast<int>(on), j, 4) != 0;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int A = (W >> (6 * j)) & 7, B = (W >> (6 * j + 3)) & 7;
    // 2x2 block X: rows (a_t, b_t), columns (A, B) of pair j.  If j comes
    // first in the group (or j = t) the column rotation precedes the row
    // rotation: Y = (C_t(R_j(X^T)))^T, else Y = C_j(R_t(X)), where R mixes
    // rows and C mixes columns with the same two-term arithmetic.
    const bool swap = j <= t;
    float x00 = ra[A], x01 = swap ? rb[A] : ra[B];
    float x10 = swap ? ra[B] : rb[A], x11 = rb[B];
    const float c1 = swap ? cj[j] : c, s1 = swap ? sj[j] : s;
    const bool on1 = swap ? onj[j] : on;
    const float c2 = swap ? c : cj[j], s2 = swap ? s : sj[j];
    const bool on2 = swap ? on : onj[j];
    rot2(x00, x10, c1, s1, on1);  // rows of X'
    rot2(x01, x11, c1, s1, on1);
    rot2(x00, x01, c2, s2, on2);  // columns of X'
    rot2(x10, x11, c2, s2, on2);
    const bool diag = j == t && on;
    ra[A] = x00;
    rb[B] = x11;
    const float y01 = swap ? x10 : x01, y10 = swap ? x01 : x10;
    ra[B] = diag ? 0.0f : y01;
    rb[A] = diag ? 0.0f : y10;
  }
  if (active && on) {
    float4 *ca = reinterpret_cast<float4 *>(qcol + 8 * a);
    float4 *cb = reinterpret_cast<float4 *>(qcol + 8 * b);
    float4 x0 = ca[0], x1 = ca[1], y0 = cb[0], y1 = cb[1];
    rot2(x0.x, y0.x, c, s, true); rot2(x0.y, y0.y, c, s, true);
    rot2(x0.z, y0.z, c, s, true); rot2(x0.w, y0.w, c, s, true);
    rot2(x1.x, y1.x, c, s, true); rot2(x1.y, y1.y, c, s, true);
    rot2(x1.z, y1.z, c, s, true); rot2(x1.w, y1.w, c, s, true);
    ca[0] = x0; ca[1] = x1; cb[0] = y0; cb[1] = y1;
  }
  __syncwarp();
}

// Moves the rows from the ownership of group G to that of group G + 1.
template <int G>
__device__ __forceinline__ void pivotExchange(float (&ra)[8], float (&rb)[8], int t) {
  constexpr uint32_t O = ownerWord(G), W1 = groupWord(G + 1);
  const int a1 = (W1 >> (6 * t)) & 7, b1 = (W1 >> (6 * t + 3)) & 7;
  const int src_a = (O >> (3 * a1)) & 3, slot_a = (O >> (3 * a1 + 2)) & 1;
  const int src_b = (O >> (3 * b1)) & 3, slot_b = (O >> (3 * b1 + 2)) & 1;
  float na[8], nb[8];
#pragma unroll
  for (int y = 0; y < 8; ++y) {
    const float u0 = __shfl_sync(0xffffffffu, ra[y], src_a, 4);
    const float u1 = __shfl_sync(0xffffffffu, rb[y], src_a, 4);
    const float v0 = __shfl_sync(0xffffffffu, ra[y], src_b, 4);
    const float v1 = __shfl_sync(0xffffffffu, rb[y], src_b, 4);
    na[y] = slot_a ? u1 : u0;
    nb[y] = slot_b ? v1 : v0;
  }
#pragma unroll
  for (int y = 0; y < 8; ++y) {
    ra[y] = na[y];
    rb[y] = nb[y];
  }
}

// Full pivot sweep on the quad; on return ra / rb hold rows (t, 4 + t) and
// qcol holds Q row-major.
__device__ __forceinline__ void pivotSweep(float (&ra)[8], float (&rb)[8], float *qcol, int t,
                                           bool active) {
  if (active) {
    // Q = I, column-major: lane t writes columns 2t and 2t + 1.
    float4 *q4 = reinterpret_cast<float4 *>(qcol);
#pragma unroll
    for (int x = 0; x < 2; ++x) {
      const int col = 2 * t + x;
      q4[2 * col] = make_float4(col == 0, col == 1, col == 2, col == 3);
      q4[2 * col + 1] = make_float4(col == 4, col == 5, col == 6, col == 7);
    }
  }
  __syncwarp();
  pivotGroup<0>(ra, rb, qcol, t, active); pivotExchange<0>(ra, rb, t);
  pivotGroup<1>(ra, rb, qcol, t, active); pivotExchange<1>(ra, rb, t);
  pivotGroup<2>(ra, rb, qcol, t, active); pivotExchange<2>(ra, rb, t);
  pivotGroup<3>(ra, rb, qcol, t, active); pivotExchange<3>(ra, rb, t);
  pivotGroup<4>(ra, rb, qcol, t, active); pivotExchange<4>(ra, rb, t);
  pivotGroup<5>(ra, rb, qcol, t, active); pivotExchange<5>(ra, rb, t);
  pivotGroup<6>(ra, rb, qcol, t, active); pivotExchange<6>(ra, rb, t);
  // Q column-major -> row-major in place: lane t gathers rows 2t, 2t + 1.
  float2 r2[8];
  if (active) {
#pragma unroll
    for (int col = 0; col < 8; ++col) r2[col] = reinterpret_cast<const float2 *>(qcol + 8 * col)[t];
  }
  __syncwarp();
  if (active) {
    float4 *q4 = reinterpret_cast<float4 *>(qcol);
    q4[4 * t + 0] = make_float4(r2[0].x, r2[1].x, r2[2].x, r2[3].x);
    q4[4 * t + 1] = make_float4(r2[4].x, r2[5].x, r2[6].x, r2[7].x);
    q4[4 * t + 2] = make_float4(r2[0].y, r2[1].y, r2[2].y, r2[3].y);
    q4[4 * t + 3] = make_float4(r2[4].y, r2[5].y, r2[6].y, r2[7].y);
  }
}

__host__ __device__ __forceinline__ size_t sweepSmemLayout(int n, bool with_tiles, size_t *q_off,
                                                           size_t *tile_off) {
  const int m = padded8(n), nb = m / 4, P = nb / 2;
  size_t bytes = 32 * sizeof(double) + (nb + 1 + 2 * P) * sizeof(int);
  bytes = (bytes + 15) & ~static_cast<size_t>(15);
  *q_off = bytes;
  bytes += static_cast<size_t>(P) * kQS * sizeof(float);
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
    // Pivots: a quad of lanes per block pair.  The loop is warp-uniform (all
    // lanes of a warp take part in the quad shuffles; lanes past P idle).
    const int quads = blockDim.x >> 2, t4 = threadIdx.x & 3;
    for (int base = 0; base < P; base += quads) {
      const int k = base + (threadIdx.x >> 2);
      const bool active = k < P;
      float ra[8], rb[8];
      int tII = 0, tIJ = 0, tJJ = 0;
      if (active) {
        int I, J;
        rrPair(k, round, nb, I, J);
        if (t4 == 0) {
          pair_i[k] = I;
          pair_j[k] = J;
        }
        tII = tileIndex(tri, I, I);
        tIJ = tileIndex(tri, I, J);
        tJJ = tileIndex(tri, J, J);
        // lane t starts with rows t (block I) and 7 - t (block J row 3 - t;
        // its left half is the mirror of tile (I, J))
        const float4 *sII = reinterpret_cast<const float4 *>(tiles + static_cast<int64_t>(tII) * kTileF);
        const float4 *sIJ = reinterpret_cast<const float4 *>(tiles + static_cast<int64_t>(tIJ) * kTileF);
        const float4 *sJJ = reinterpret_cast<const float4 *>(tiles + static_cast<int64_t>(tJJ) * kTileF);
        const int jr = 3 - t4;
        const float4 v0 = sII[t4 ^ (tII & 3)], v1 = sIJ[t4 ^ (tIJ & 3)], v2 = sJJ[jr ^ (tJJ & 3)];
        ra[0] = v0.x; ra[1] = v0.y; ra[2] = v0.z; ra[3] = v0.w;
        ra[4] = v1.x; ra[5] = v1.y; ra[6] = v1.z; ra[7] = v1.w;
#pragma unroll
        for (int i = 0; i < 4; ++i) rb[i] = tiles[tileElement(tIJ, i, jr)];
        rb[4] = v2.x; rb[5] = v2.y; rb[6] = v2.z; rb[7] = v2.w;
      } else {
#pragma unroll
        for (int y = 0; y < 8; ++y) ra[y] = rb[y] = 0.0f;
      }
      pivotSweep(ra, rb, qs + (active ? k : 0) * kQS, t4, active);
      if (active) {
        // rows t (tiles (I, I), (I, J)) and 4 + t (tile (J, J)); the lower
        // left block is the mirror of tile (I, J) and is not stored
        float4 *sII = reinterpret_cast<float4 *>(tiles + static_cast<int64_t>(tII) * kTileF);
        float4 *sIJ = reinterpret_cast<float4 *>(tiles + static_cast<int64_t>(tIJ) * kTileF);
        float4 *sJJ = reinterpret_cast<float4 *>(tiles + static_cast<int64_t>(tJJ) * kTileF);
        sII[t4 ^ (tII & 3)] = make_float4(ra[0], ra[1], ra[2], ra[3]);
        sIJ[t4 ^ (tIJ & 3)] = make_float4(ra[4], ra[5], ra[6], ra[7]);
        sJJ[t4 ^ (tJJ & 3)] = make_float4(rb[4], rb[5], rb[6], rb[7]);
      }
    }
    __syncthreads();
    {
      // this round's rotations, logged for the V replay (coalesced copy)
      const float4 *src = reinterpret_cast<const float4 *>(qs);
      float4 *dst = reinterpret_cast<float4 *>(log + static_cast<int64_t>(round) * P * kQF);
      for (int x = threadIdx.x; x < P * kQF / 4; x += blockDim.x) {
        dst[x] = src[(x >> 4) * (kQS / 4) + (x & 15)];
      }
    }
    // Off-pivot super-tiles: T' = Q_k^T T Q_l for every k < l, two lanes per
    // super-tile.  Lane h forms U[:, 4h:4h+4] = Q_k^T T[:, 4h:4h+4] from the
    // two 4x4 blocks of column block h, the pair swaps the halves of U each
    // needs, and lane h forms rows 4h..4h+3 of T' = U Q_l.  Every element is
    // the same ordered FMA chain as in one-lane form (u over i, t' over j).
    // The loop is warp-uniform so the pair shuffle has all lanes present.
    for (int base = threadIdx.x & ~31; base < 2 * items; base += blockDim.x) {
      const int w2 = base + (threadIdx.x & 31);
      const int h = w2 & 1;
      int k = 0, l = 0;
      const bool valid = w2 < 2 * items && foldedBlock(w2 >> 1, P, k, l) && k != l;
      if (!valid) k = l = 0;
      const int rb0 = pair_i[k], rb1 = pair_j[k];
      const int cbh = h ? pair_j[l] : pair_i[l];
      const float4 *qk = reinterpret_cast<const float4 *>(qs + k * kQS);
      const float4 *ql = reinterpret_cast<const float4 *>(qs + l * kQS);
      float u[8][4];
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) u[a][c] = 0.0f;
#pragma unroll
      for (int x = 0; x < 2; ++x) {
        float b4[4][4];
        if (valid) {
          loadBlock(tiles, tri, x ? rb1 : rb0, cbh, b4);
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int c = 0; c < 4; ++c) b4[i][c] = 0.0f;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 lo = qk[2 * (4 * x + i)], hi = qk[2 * (4 * x + i) + 1];
          const float qr[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
          for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) u[a][c] = fmaf(qr[a], b4[i][c], u[a][c]);
        }
      }
      // U rows of this lane's half: own columns, and the partner's columns
      // for these rows (the partner sends the rows of the other half).
      float ur[4][8];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float mine = h ? u[4 + r][c] : u[r][c];
          const float send = h ? u[r][c] : u[4 + r][c];
          const float got = __shfl_xor_sync(0xffffffffu, send, 1);
          ur[r][c] = h ? got : mine;
          ur[r][4 + c] = h ? mine : got;
        }
      float o[4][8];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) o[r][c] = 0.0f;
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const float4 lo = ql[2 * jj], hi = ql[2 * jj + 1];
        const float qr[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 8; ++c) o[r][c] = fmaf(ur[r][jj], qr[c], o[r][c]);
      }
      if (valid) {
        const int rbh = h ? rb1 : rb0;
        const int cb0 = pair_i[l], cb1 = pair_j[l];
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          float b4[4][4];
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) b4[r][c] = o[r][4 * y + c];
          storeBlock(tiles, tri, rbh, y ? cb1 : cb0, b4);
        }
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

// Replay shared memory: `rows` rows of V (stride m + 4) and two rounds of
// rotations (the next round's are copied in while the current one runs).
__host__ __device__ __forceinline__ size_t replaySmemBytes(int max_n, int rows) {
  const int m = padded8(max_n), P = m / 8;
  return static_cast<size_t>(rows) * (m + 4) * sizeof(float) +
         2 * static_cast<size_t>(P) * kQF * sizeof(float);
}

// 16-byte asynchronous global -> shared copies (cp.async, L2 only).
__device__ __forceinline__ void copyAsync16(void *smem, const void *gmem) {
  const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem) : "memory");
}
__device__ __forceinline__ void copyAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void copyAsyncWaitAll() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Replays one logged sweep onto `rows` rows of V: V <- V Q_k on the column
// blocks (I_k, J_k) of every pair, round by round (the V update of
// jacobi_similarity_vectors_f32 z = 1, metal_mixed_sqrt.metal:1380-1390,
// with 8x8 rotations).  Rows are the fast thread index: the 32 lanes of a
// warp update 32 rows with the same Q_k, so Q_k is read from shared memory
// as a broadcast, and the row stride (m + 4 floats, 4 mod 8) keeps the
// lanes' float4 row accesses free of bank conflicts.  The next round's
// rotations are copied from the log with cp.async while the current round
// runs, so a round costs one barrier.  Each element is the ordered chain
// o_c = sum_j x_j q_jc in FP32 FMA, as the CPU restatement.
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
  float *qbuf = vs + static_cast<size_t>(R) * ld;     // [2][P][64]
  float *v = args.v + args.a_offset[mi];
  const int rows = min(R, n - r0);
  const float *log = args.log + args.log_offset[mi];
  const int chunks = P * kQF / 4;  // 16-byte pieces of one round's rotations
  for (int x = threadIdx.x; x < chunks; x += blockDim.x) copyAsync16(qbuf + 4 * x, log + 4 * x);
  copyAsyncCommit();
  for (int k = threadIdx.x; k < m * R; k += blockDim.x) {
    const int c = k / R, r = k % R;
    vs[r * ld + c] = (c < n && r < rows) ? v[r0 + r + static_cast<int64_t>(c) * n] : 0.0f;
  }
  // item -> (pair k, slice of up to 32 rows); a lane takes row r_in of the
  // slice and, when R > 32, rows r_in + 32, r_in + 64, ... with the same Q_k
  const int lanes_r = R < 32 ? R : 32;
  const int per_lane = R < 32 ? 1 : R / 32;
  for (int round = 0; round < nb - 1; ++round) {
    copyAsyncWaitAll();
    __syncthreads();  // this round's rotations landed; last round's rows written
    if (round + 1 < nb - 1) {
      float *next = qbuf + ((round + 1) & 1) * P * kQF;
      const float *src = log + static_cast<int64_t>(round + 1) * P * kQF;
      for (int x = threadIdx.x; x < chunks; x += blockDim.x) copyAsync16(next + 4 * x, src + 4 * x);
      copyAsyncCommit();
    }
    const float *qs = qbuf + (round & 1) * P * kQF;
    for (int item = threadIdx.x; item < P * lanes_r; item += blockDim.x) {
      const int k = item / lanes_r, r_in = item % lanes_r;
      int I, J;
      rrPair(k, round, nb, I, J);
      const float4 *qk = reinterpret_cast<const float4 *>(qs + k * kQF);
      float q[8][8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 lo = qk[2 * j], hi = qk[2 * j + 1];
        q[j][0] = lo.x; q[j][1] = lo.y; q[j][2] = lo.z; q[j][3] = lo.w;
        q[j][4] = hi.x; q[j][5] = hi.y; q[j][6] = hi.z; q[j][7] = hi.w;
      }
      for (int e = 0; e < per_lane; ++e) {
        const int r = r_in + 32 * e;
        if (r >= rows) break;
        float *row = vs + r * ld;
        const float4 a = *reinterpret_cast<const float4 *>(row + 4 * I);
        const float4 b = *reinterpret_cast<const float4 *>(row + 4 * J);
        const float x[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        float o[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float acc = 0.0f;
#pragma unroll
          for (int j = 0; j < 8; ++j) acc = fmaf(x[j], q[j][c], acc);
          o[c] = acc;
        }
        *reinterpret_cast<float4 *>(row + 4 * I) = make_float4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<float4 *>(row + 4 * J) = make_float4(o[4], o[5], o[6], o[7]);
      }
    }
  }
  copyAsyncWaitAll();
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

// Threads of a sweep CTA: a quad per pivot and two lanes per super-tile
// (the kernel fits 128 registers, so 512 threads is one CTA per SM).
int threadsFor(int n) {
  if (n <= 16) return 32;
  if (n <= 32) return 64;
  if (n <= 64) return 128;
  if (n <= 256) return 256;
  return kSweepThreadsMax;
}

bool fitsSmem(int n) {
  size_t q_off, tile_off;
  return sweepSmemLayout(n, true, &q_off, &tile_off) <= kSmemLimit;
}

// Rows of V per replay CTA for matrices up to order max_n: the whole matrix
// when it is small, else the most rows (a multiple of 32) that keep two CTAs
// per SM (<= 112 KB of shared memory each), at least 8.
int replayRows(int max_n) {
  if (max_n <= 32) return padded8(max_n);
  int best = 0;
  const int cap = (max_n + 31) / 32 * 32;
  for (int rows = 32; rows <= cap; rows += 32)
    if (replaySmemBytes(max_n, rows) <= 112 * 1024) best = rows;
  if (best > 0) return best;
  for (int rows = 32; rows >= 8; rows -= 8)
    if (replaySmemBytes(max_n, rows) <= kSmemLimit) return rows;
  return 0;
}

// ---------------------------------------------------------------------------
// Size classes and the online autotuner of the sweep launch shape.
//
// Matrices are bucketed by size class; every class has a default CTA size
// and a short list of candidates.  All candidates compute the same bits (the
// CTA size only changes which thread runs which pivot quad and super-tile),
// so the tuner times them on live work: while a class is untuned, sweep
// launches 1..C of a call (full sweeps: every class needs more) each use the
// next candidate, bracketed by timing events; a later call reads the events
// and, once every candidate has a time, keeps the fastest for that device.
// The decisions are process-wide, like a benchmark cache, and
// msq_autotune_report prints them.
constexpr int kClasses = 9;

int sizeClass(int n) {
  if (n <= 16) return 0;
  if (n <= 32) return 1;
  if (n <= 64) return 2;
  if (n <= 128) return 3;
  if (n <= 256) return 4;
  if (fitsSmem(n)) return 5;
  if (n <= 512) return 6;
  if (n <= 1024) return 7;
  return 8;
}

const char *className(int c) {
  static const char *names[kClasses] = {"n<=16", "16<n<=32", "32<n<=64", "64<n<=128",
                                        "128<n<=256", "256<n<=328 (shared tiles)",
                                        "328<n<=512 (global tiles)", "512<n<=1024", "1024<n<=2048"};
  return names[c];
}

std::vector<int> classCandidates(int c) {
  switch (c) {
    case 0: return {32};
    case 1: return {64, 32};
    case 2: return {128, 64};
    case 3: return {256, 128};
    case 4: return {256, 512};
    default: return {512, 256};
  }
}

// Launch names per class (static strings for the launch timer).
const char *sweepName(int c) {
  static const char *names[kClasses] = {
      "jacobi sweep n<=16", "jacobi sweep n<=32", "jacobi sweep n<=64", "jacobi sweep n<=128",
      "jacobi sweep n<=256", "jacobi sweep n<=328", "jacobi sweep n<=512 (global)",
      "jacobi sweep n<=1024 (global)", "jacobi sweep n<=2048 (global)"};
  return names[c];
}

struct ClassTune {
  std::vector<int> cands;
  std::vector<double> ms;   // per candidate, < 0 until measured
  int best = -1;            // index into cands once tuned
  bool requested = false;   // a call is measuring this class
};

struct PendingTiming {
  int device, cls, cand;
  cudaEvent_t begin, end;
  int matrices;             // CTAs of the timed launch (for normalisation)
};

std::mutex g_tune_mutex;
std::map<int, std::array<ClassTune, kClasses>> g_tune;  // by device
std::vector<PendingTiming> g_pending;
bool g_tune_enabled = true;

std::array<ClassTune, kClasses> &tuneFor(int device) {
  auto it = g_tune.find(device);
  if (it == g_tune.end()) {
    std::array<ClassTune, kClasses> t;
    for (int c = 0; c < kClasses; ++c) {
      t[c].cands = classCandidates(c);
      t[c].ms.assign(t[c].cands.size(), -1.0);
      if (t[c].cands.size() == 1) t[c].best = 0;
    }
    it = g_tune.emplace(device, t).first;
  }
  return it->second;
}

// Reads finished measurements (no waiting); caller holds g_tune_mutex.
void harvestTimings() {
  for (size_t i = 0; i < g_pending.size();) {
    PendingTiming &p = g_pending[i];
    const cudaError_t q = cudaEventQuery(p.end);
    if (q == cudaErrorNotReady) {
      ++i;
      continue;
    }
    float ms = -1.0f;
    if (q == cudaSuccess) cudaEventElapsedTime(&ms, p.begin, p.end);
    cudaEventDestroy(p.begin);
    cudaEventDestroy(p.end);
    ClassTune &t = tuneFor(p.device)[p.cls];
    if (ms > 0.0f && t.best < 0) {
      const double per = ms / std::max(p.matrices, 1);
      if (t.ms[p.cand] < 0.0 || per < t.ms[p.cand]) t.ms[p.cand] = per;
      bool all = true;
      for (double v : t.ms) all = all && v > 0.0;
      if (all) {
        t.best = static_cast<int>(std::min_element(t.ms.begin(), t.ms.end()) - t.ms.begin());
      }
    }
    t.requested = false;
    g_pending.erase(g_pending.begin() + i);
  }
}

// Per-layout launch plan, kept per batch layout and device.
struct JacobiPlan {
  uint64_t key = 0;
  int count = 0;
  int device_id = 0;
  int64_t tile_total = 0, log_total = 0;
  int64_t *t_offset = nullptr, *log_offset = nullptr;
  int32_t *order = nullptr;  // ids grouped by bucket, largest first
  struct Bucket { int cls; bool smem; int first; int count; size_t smem_bytes; };
  std::vector<Bucket> buckets;
  int32_t *work_matrix = nullptr, *work_row = nullptr;
  int work_count = 0;
  // V replay launches, one per size class: CTAs [first, first + count) of
  // the work lists, `rows` rows each, `smem` bytes of shared memory.
  struct ReplayGroup { int first; int count; int rows; size_t smem; };
  std::vector<ReplayGroup> replays;
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
  // buckets by size class, largest class first
  std::stable_sort(ids.begin(), ids.end(), [&](int x, int y) {
    const int cx = sizeClass(b->host_n[x]), cy = sizeClass(b->host_n[y]);
    if (cx != cy) return cx > cy;
    return b->host_n[x] > b->host_n[y];
  });
  for (int i = 0; i < count;) {
    const int c = sizeClass(b->host_n[ids[i]]);
    const bool smem = fitsSmem(b->host_n[ids[i]]);
    int j = i;
    size_t bytes = 0;
    while (j < count && sizeClass(b->host_n[ids[j]]) == c) {
      size_t q_off, tile_off;
      bytes = std::max(bytes, sweepSmemLayout(b->host_n[ids[j]], smem, &q_off, &tile_off));
      ++j;
    }
    plan->buckets.push_back({c, smem, i, j - i, bytes});
    i = j;
  }
  std::vector<int32_t> wm, wr;
  for (const auto &bucket : plan->buckets) {
    int max_n = 0;
    for (int i = bucket.first; i < bucket.first + bucket.count; ++i) max_n = std::max(max_n, b->host_n[ids[i]]);
    const int rows = replayRows(max_n);
    const int first = static_cast<int>(wm.size());
    for (int i = bucket.first; i < bucket.first + bucket.count; ++i) {
      const int n = b->host_n[ids[i]];
      for (int r = 0; r < n; r += rows) {
        wm.push_back(ids[i]);
        wr.push_back(r);
      }
    }
    plan->replays.push_back({first, static_cast<int>(wm.size()) - first, rows,
                             replaySmemBytes(max_n, rows)});
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
              plan->work_matrix, plan->work_row, 0, 0};
  // Launch shape per bucket: the tuned CTA size, or (while its class is
  // being tuned) candidate c on sweep launch 1 + c with timing events.
  struct BucketLaunch { int threads; int measure; };  // measure: candidate or -1
  std::vector<std::vector<BucketLaunch>> shape(plan->buckets.size());
  bool measuring = false;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    harvestTimings();
    auto &tune = tuneFor(ctx->device);
    for (size_t k = 0; k < plan->buckets.size(); ++k) {
      ClassTune &t = tune[plan->buckets[k].cls];
      const bool measure = g_tune_enabled && t.best < 0 && !t.requested && max_sweeps >= 1;
      if (measure) t.requested = true;
      measuring = measuring || measure;
      for (int launch = 0; launch <= max_sweeps; ++launch) {
        const int c = launch - 1;
        if (measure && c >= 0 && c < static_cast<int>(t.cands.size())) {
          shape[k].push_back({t.cands[c], c});
        } else {
          shape[k].push_back({t.cands[t.best >= 0 ? t.best : 0], -1});
        }
      }
    }
  }
  // Streams: size buckets round-robin over three sweep streams, the replay
  // on a fourth.  Order: sweep k of a bucket follows sweep k-1 (same
  // stream) and the replay of k-2 (which read the log buffer sweep k
  // overwrites); the replay of k follows every bucket's sweep k.  A call
  // that measures candidate shapes runs serially so that each timed launch
  // has the GPU to itself.
  syncReset(ctx);
  const bool serial = !ctx->concurrent || measuring;
  const int sweep_streams = std::min<int>(3, static_cast<int>(plan->buckets.size()));
  cudaStream_t ss[3];
  for (int i = 0; i < sweep_streams; ++i) {
    ss[i] = serial ? ctx->stream : auxStream(ctx, 1 + i);
    MSQ_TRY(streamWait(ctx, ss[i], ctx->stream));
  }
  cudaStream_t rs = serial ? ctx->stream : auxStream(ctx, 0);
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
      const BucketLaunch how = shape[k][launch];
      cudaStream_t s = ss[k % sweep_streams];
      args.order = plan->order + bucket.first;
      cudaEvent_t t0 = nullptr, t1 = nullptr;
      if (how.measure >= 0) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, s);
      }
      launchBegin(ctx, s);
      if (bucket.smem) {
        jacobiSweepKernel<true><<<bucket.count, how.threads, bucket.smem_bytes, s>>>(args);
      } else {
        jacobiSweepKernel<false><<<bucket.count, how.threads, bucket.smem_bytes, s>>>(args);
      }
      MSQ_TRY(launchedOn(ctx, s, sweepName(bucket.cls)));
      if (how.measure >= 0) {
        cudaEventRecord(t1, s);
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_pending.push_back({ctx->device, bucket.cls, how.measure, t0, t1, bucket.count});
      }
    }
    if (launch < max_sweeps) {
      for (int i = 0; i < sweep_streams; ++i) MSQ_TRY(streamWait(ctx, rs, ss[i]));
      vargs.parity = parity;
      vargs.log = args.log;
      for (const auto &g : plan->replays) {
        vargs.work_matrix = plan->work_matrix + g.first;
        vargs.work_row = plan->work_row + g.first;
        vargs.rows_per_cta = g.rows;
        launchBegin(ctx, rs);
        jacobiReplayKernel<<<g.count, kReplayThreads, g.smem, rs>>>(vargs);
        MSQ_TRY(launchedOn(ctx, rs, "jacobi replay"));
      }
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

extern "C" int msq_autotune_report(int device, char *out, size_t capacity) {
  if (out == nullptr || capacity == 0) return MSQ_ERR_INVALID_ARGUMENT;
  std::string text;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    harvestTimings();
    auto &tune = tuneFor(device);
    for (int c = 0; c < kClasses; ++c) {
      const ClassTune &t = tune[c];
      text += std::string("jacobi sweep ") + className(c) + ": threads";
      for (size_t i = 0; i < t.cands.size(); ++i) {
        char buf[64];
        if (t.ms[i] > 0.0) {
          std::snprintf(buf, sizeof(buf), " %d=%.4fms", t.cands[i], t.ms[i]);
        } else {
          std::snprintf(buf, sizeof(buf), " %d=?", t.cands[i]);
        }
        text += buf;
      }
      text += t.best >= 0 ? " -> " + std::to_string(t.cands[t.best]) + "\n" : " -> untuned\n";
    }
  }
  std::strncpy(out, text.c_str(), capacity - 1);
  out[capacity - 1] = '\0';
  return MSQ_OK;
}

extern "C" int msq_autotune_reset(int enable) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  harvestTimings();
  g_tune.clear();
  g_tune_enabled = enable != 0;
  return MSQ_OK;
}

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
