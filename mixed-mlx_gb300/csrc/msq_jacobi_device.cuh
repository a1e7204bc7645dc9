// Device building blocks of the blocked Jacobi eigensolver, shared by the
// batched kernels (one CTA per matrix, msq_jacobi.cu) and the grid kernels
// (all SMs on one matrix, msq_jacobi_grid.cu): the round-robin schedule in
// closed form, the packed 4x4 tile layout of A, the quad-parallel 8x8 pivot
// sweep and asynchronous copies.  Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "msq_f32x2.cuh"
#include "msq_tcgen05.cuh"

namespace msq {
namespace {

constexpr int kTileF = 16;      // floats per 4x4 tile
constexpr int kQF = 64;         // floats per 8x8 rotation
// Shared-memory stride of the rotations in the sweep kernel: 68 floats puts
// Q_l of different pivots on different banks (a 64-float stride would map
// every Q_l row to the same four banks).
constexpr int kQS = 68;

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


__host__ __device__ constexpr int padded8(int n) { return (n + 7) & ~7; }

// Slot -> participant of round r (participants 1..m-1 rotate right by one
// per round, slot 0 fixed): the closed form of the std::rotate step in
// makeJacobiSchedule (src/metal_solver.cpp:75-76).
__host__ __device__ __forceinline__ int rrSlot(int slot, int round, int m) {
  if (slot == 0) return 0;
  int k = slot - 1 - round % (m - 1);
  if (k < 0) k += m - 1;
  return 1 + k;
}

__host__ __device__ __forceinline__ void rrPair(int pair, int round, int m, int &p, int &q) {
  const int a = rrSlot(pair, round, m);
  const int b = rrSlot(m - 1 - pair, round, m);
  p = a < b ? a : b;
  q = a < b ? b : a;
}

// Two-level pairing of nb blocks (the tensor-core eigenvector path): blocks
// form super-blocks of 8 (32 indices; the last may hold fewer, and a dummy
// empty one makes their count even).  Rounds 0..6 pair the blocks inside
// each super-block (round-robin over 8 slots); then an outer round-robin
// over super-blocks pairs them, and each outer round spends 8 rounds on the
// cross pairs (i of P with (i + t) mod 8 of Q in round t).  Every block pair
// meets once per sweep, and the rotations of rounds [0, 15) and of each
// later group of 8 stay inside the outer round's super-pairs, so their
// product is block diagonal with 64x64 blocks.  Blocks without a partner in
// a round are paired among themselves with the identity rotation (J stored
// as -1 - J in the schedule table).
constexpr int kSuperBlock = 8;
__host__ __device__ constexpr int twoLevelSupers(int nb) {
  return (nb + kSuperBlock - 1) / kSuperBlock + (((nb + kSuperBlock - 1) / kSuperBlock) & 1);
}
__host__ __device__ constexpr int twoLevelRounds(int nb) {
  return (kSuperBlock - 1) + kSuperBlock * (twoLevelSupers(nb) - 1);
}
// Stage s of the eigenvector update: rounds [first, first + count).
__host__ __device__ constexpr int twoLevelStageFirst(int s) {
  return s == 0 ? 0 : (kSuperBlock - 1) + kSuperBlock * s;
}
__host__ __device__ constexpr int twoLevelStageRounds(int s) {
  return s == 0 ? 2 * kSuperBlock - 1 : kSuperBlock;
}

// Pair k of a round from the two-level table (sched != nullptr) or the
// round-robin rule; *rotate is false for an identity pair.
__device__ __forceinline__ void roundPair(const int2 *sched, int k, int round, int nb, int &I,
                                          int &J, bool &rotate) {
  if (sched != nullptr) {
    const int2 ij = sched[round * (nb / 2) + k];
    I = ij.x;
    rotate = ij.y >= 0;
    J = rotate ? ij.y : -1 - ij.y;
  } else {
    rrPair(k, round, nb, I, J);
    rotate = true;
  }
}

// Folded enumeration of the upper triangle {(i, j): i <= j < P}: rows i and
// P-1-i share one folded row of P+1 items.
// The row w / (P + 1) is taken from a float reciprocal and corrected by one
// step either way (exact for every w < 2^22), instead of an integer divide.
__device__ __forceinline__ bool foldedBlock(int w, int P, int &i, int &j) {
  const int q = P + 1;
  int r = __float2int_rz(static_cast<float>(w) * __frcp_rn(static_cast<float>(q)));
  if ((r + 1) * q <= w) ++r;
  if (r * q > w) --r;
  const int c = w - r * q;
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

// Loads block (R, C) of A (4x4, row-major in t) from packed tile ti, which
// holds (min, max) of the two block indices (transposed when R > C).
// 16-byte asynchronous global -> shared copies (cp.async, L2 only).
__device__ __forceinline__ void copyAsync16(void *smem, const void *gmem) {
  const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem) : "memory");
}
__device__ __forceinline__ void copyAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void copyAsyncWaitAll() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ void loadTile(const float *tiles, int ti, bool transposed, float (&t)[4][4]) {
  const float4 *src = reinterpret_cast<const float4 *>(tiles + static_cast<int64_t>(ti) * kTileF);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 v = src[i ^ (ti & 3)];
    if (!transposed) {
      t[i][0] = v.x; t[i][1] = v.y; t[i][2] = v.z; t[i][3] = v.w;
    } else {
      t[0][i] = v.x; t[1][i] = v.y; t[2][i] = v.z; t[3][i] = v.w;
    }
  }
}

__device__ __forceinline__ void storeTile(float *tiles, int ti, bool transposed, const float (&t)[4][4]) {
  float4 *dst = reinterpret_cast<float4 *>(tiles + static_cast<int64_t>(ti) * kTileF);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    dst[i ^ (ti & 3)] = transposed ? make_float4(t[0][i], t[1][i], t[2][i], t[3][i])
                                   : make_float4(t[i][0], t[i][1], t[i][2], t[i][3]);
  }
}

// Block (R, C) through a table tri[J] = J (J + 1) / 2 (shared memory) ...
__device__ __forceinline__ void loadBlock(const float *tiles, const int *tri, int R, int C, float (&t)[4][4]) {
  if (R <= C) loadTile(tiles, tileIndex(tri, R, C), false, t);
  else loadTile(tiles, tileIndex(tri, C, R), true, t);
}

__device__ __forceinline__ void storeBlock(float *tiles, const int *tri, int R, int C, const float (&t)[4][4]) {
  if (R <= C) storeTile(tiles, tileIndex(tri, R, C), false, t);
  else storeTile(tiles, tileIndex(tri, C, R), true, t);
}

// ... or with the index computed (grid kernels).
__device__ __forceinline__ int triTile(int I, int J) { return J * (J + 1) / 2 + I; }

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
  // the IEEE quotients 1 / x (the shorter of the two correctly rounded
  // forms on this GPU: __fdiv_rn(1, x) ~51 cycles, __frcp_rn ~70)
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
// (all 8 columns); q: rows 2t and 2t + 1 of the pivot's Q, which every lane
// updates for all four rotations of the group (Q <- Q J touches columns a, b
// of each row; the group's pairs are disjoint, so their order is free).
template <int G>
__device__ __forceinline__ void pivotGroup(float (&ra)[8], float (&rb)[8], float (&q)[2][8], int t) {
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
    rot2(q[0][A], q[0][B], cj[j], sj[j], onj[j]);
    rot2(q[1][A], q[1][B], cj[j], sj[j], onj[j]);
  }
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

// Full pivot sweep on the quad; on return ra / rb hold rows (t, 4 + t) and,
// if active, qrow holds Q row-major (lane t writes rows 2t and 2t + 1).
__device__ __forceinline__ void pivotSweep(float (&ra)[8], float (&rb)[8], float *qrow, int t,
                                           bool active) {
  float q[2][8];
#pragma unroll
  for (int x = 0; x < 2; ++x)
#pragma unroll
    for (int y = 0; y < 8; ++y) q[x][y] = y == 2 * t + x ? 1.0f : 0.0f;
  pivotGroup<0>(ra, rb, q, t); pivotExchange<0>(ra, rb, t);
  pivotGroup<1>(ra, rb, q, t); pivotExchange<1>(ra, rb, t);
  pivotGroup<2>(ra, rb, q, t); pivotExchange<2>(ra, rb, t);
  pivotGroup<3>(ra, rb, q, t); pivotExchange<3>(ra, rb, t);
  pivotGroup<4>(ra, rb, q, t); pivotExchange<4>(ra, rb, t);
  pivotGroup<5>(ra, rb, q, t); pivotExchange<5>(ra, rb, t);
  pivotGroup<6>(ra, rb, q, t); pivotExchange<6>(ra, rb, t);
  if (active) {
    float4 *q4 = reinterpret_cast<float4 *>(qrow);
    q4[4 * t + 0] = make_float4(q[0][0], q[0][1], q[0][2], q[0][3]);
    q4[4 * t + 1] = make_float4(q[0][4], q[0][5], q[0][6], q[0][7]);
    q4[4 * t + 2] = make_float4(q[1][0], q[1][1], q[1][2], q[1][3]);
    q4[4 * t + 3] = make_float4(q[1][4], q[1][5], q[1][6], q[1][7]);
  }
}

// Tile lookup through the shared table tri[J] = J (J + 1) / 2 ...
struct SharedTri {
  const int *tri;
  __device__ __forceinline__ int operator()(int R, int C, bool &transposed) const {
    transposed = R > C;
    return transposed ? tri[R] + C : tri[C] + R;
  }
};
// ... or computed (grid kernels).
struct ComputedTri {
  __device__ __forceinline__ int operator()(int R, int C, bool &transposed) const {
    transposed = R > C;
    return transposed ? triTile(C, R) : triTile(R, C);
  }
};

// Where tile t lives: one flat array ...
struct FlatTiles {
  float *t;
  __device__ __forceinline__ float *base(int ti) const { return t + static_cast<int64_t>(ti) * kTileF; }
};
// ... or tiles [0, split) in shared memory and the rest in the global
// workspace (the global-tile sweep keeps what fits on chip).
struct SplitTiles {
  float *s;
  float *g;
  int split;
  __device__ __forceinline__ float *base(int ti) const {
    return ti < split ? s + ti * kTileF : g + static_cast<int64_t>(ti) * kTileF;
  }
};
// Element e = tileElement(t, i, j) of a tile store.
template <class Mem>
__device__ __forceinline__ float &tileAt(const Mem &mem, int64_t e) {
  return mem.base(static_cast<int>(e >> 4))[e & 15];
}

__device__ __forceinline__ void loadTileAt(const float *p, int ti, bool transposed, float (&t)[4][4]) {
  const float4 *src = reinterpret_cast<const float4 *>(p);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 v = src[i ^ (ti & 3)];
    if (!transposed) {
      t[i][0] = v.x; t[i][1] = v.y; t[i][2] = v.z; t[i][3] = v.w;
    } else {
      t[0][i] = v.x; t[1][i] = v.y; t[2][i] = v.z; t[3][i] = v.w;
    }
  }
}

__device__ __forceinline__ void storeTileAt(float *p, int ti, bool transposed, const float (&t)[4][4]) {
  float4 *dst = reinterpret_cast<float4 *>(p);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    dst[i ^ (ti & 3)] = transposed ? make_float4(t[0][i], t[1][i], t[2][i], t[3][i])
                                   : make_float4(t[i][0], t[i][1], t[i][2], t[i][3]);
  }
}

// Super-tile update T' = Q_k^T T Q_l on two lanes (h = 0, 1 of an adjacent
// pair; the warp's lanes must all call it).  T is the 8x8 block of A on row
// blocks (rb0, rb1) of pair k and column blocks (cb0, cb1) of pair l; qk, ql
// are the pair rotations (row-major 8x8).  Lane h forms
// U[:, 4h:4h+4] = Q_k^T T[:, 4h:4h+4] from the two 4x4 blocks of column
// block h, the pair swaps the halves of U each needs, and lane h forms rows
// 4h..4h+3 of T' = U Q_l.  Every element is the ordered FMA chain of the
// one-lane form (u over i, t' over j), as the CPU restatement.  Invalid
// lanes compute on zeros and store nothing.
template <class Mem, class TileOf>
__device__ __forceinline__ void superTileHalfMem(const Mem &mem, TileOf tileOf, const float4 *qk,
                                                 const float4 *ql, int rb0, int rb1, int cb0,
                                                 int cb1, int h, bool valid) {
  const int cbh = h ? cb1 : cb0;
  // u2[p][c] holds U rows 2p, 2p + 1 (lane-relative) of column c: the two
  // FMAs of a row pair are one fma.rn.f32x2 with the rotation row's
  // adjacent entries as one operand and the tile element broadcast
  f32x2 u2[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int c = 0; c < 4; ++c) u2[p][c] = f2zero();
  const ulonglong2 *qk2 = reinterpret_cast<const ulonglong2 *>(qk);
#pragma unroll
  for (int x = 0; x < 2; ++x) {
    float b4[4][4];
    if (valid) {
      bool tr;
      const int ti = tileOf(x ? rb1 : rb0, cbh, tr);
      loadTileAt(mem.base(ti), ti, tr, b4);
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) b4[i][c] = 0.0f;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      // U row a holds row (a + 4h) mod 8: lane h reads the two halves of the
      // rotation row in its own order (same FMA chains, no selects)
      const ulonglong2 first = qk2[2 * (4 * x + i) + h], second = qk2[2 * (4 * x + i) + 1 - h];
      const f32x2 qp[4] = {first.x, first.y, second.x, second.y};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const f32x2 bc = f2make(b4[i][c], b4[i][c]);
#pragma unroll
        for (int p = 0; p < 4; ++p) u2[p][c] = f2fma(qp[p], bc, u2[p][c]);
      }
    }
  }
  // T' = U Q_l for U rows 4h..4h+3: columns 0..3 of those rows come from
  // lane 0 of the pair and columns 4..7 from lane 1 (each lane keeps its own
  // rows 0..3 of u2 and sends rows 4..7).  o2[r][q] holds T' row r of this
  // lane's four, columns 2q, 2q + 1; the chain over U's columns runs 0..7
  // as in the one-lane form, the second half kept until the first is done.
  f32x2 o2[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 4; ++q) o2[r][q] = f2zero();
  const ulonglong2 *ql2 = reinterpret_cast<const ulonglong2 *>(ql);
  float later[4][4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float mine[4], send[4];
    f2split(u2[0][c], mine[0], mine[1]);
    f2split(u2[1][c], mine[2], mine[3]);
    f2split(u2[2][c], send[0], send[1]);
    f2split(u2[3][c], send[2], send[3]);
    const ulonglong2 lo = ql2[2 * c], hi = ql2[2 * c + 1];
    const f32x2 qp[4] = {lo.x, lo.y, hi.x, hi.y};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float got = __shfl_xor_sync(0xffffffffu, send[r], 1);
      const float now = h ? got : mine[r];
      later[r][c] = h ? mine[r] : got;
      const f32x2 ub = f2make(now, now);
#pragma unroll
      for (int q = 0; q < 4; ++q) o2[r][q] = f2fma(ub, qp[q], o2[r][q]);
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const ulonglong2 lo = ql2[2 * (4 + c)], hi = ql2[2 * (4 + c) + 1];
    const f32x2 qp[4] = {lo.x, lo.y, hi.x, hi.y};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const f32x2 ub = f2make(later[r][c], later[r][c]);
#pragma unroll
      for (int q = 0; q < 4; ++q) o2[r][q] = f2fma(ub, qp[q], o2[r][q]);
    }
  }
  if (valid) {
    const int rbh = h ? rb1 : rb0;
#pragma unroll
    for (int y = 0; y < 2; ++y) {
      float b4[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        f2split(o2[r][2 * y], b4[r][0], b4[r][1]);
        f2split(o2[r][2 * y + 1], b4[r][2], b4[r][3]);
      }
      bool tr;
      const int ti = tileOf(rbh, y ? cb1 : cb0, tr);
      storeTileAt(mem.base(ti), ti, tr, b4);
    }
  }
}

template <class TileOf>
__device__ __forceinline__ void superTileHalf(float *tiles, TileOf tileOf, const float4 *qk,
                                              const float4 *ql, int rb0, int rb1, int cb0, int cb1,
                                              int h, bool valid) {
  superTileHalfMem(FlatTiles{tiles}, tileOf, qk, ql, rb0, rb1, cb0, cb1, h, valid);
}


// TMA bulk copies (cp.async.bulk) of a contiguous block between global and
// shared memory; both addresses 16-byte aligned, size a multiple of 16.  The
// load completes on an mbarrier (expect_tx); the wait is bounded.
constexpr long long kTileWaitLimit = 1ll << 26;

__device__ __forceinline__ void bulkLoadTiles(void *smem, const void *gmem, uint32_t bytes,
                                              uint64_t *bar) {
  const uint32_t b = smemAddr(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smemAddr(smem)),
      "l"(gmem), "r"(bytes), "r"(b)
      : "memory");
}

// The barrier alone, with no copy behind it: phase 0 never completes (the
// failure-injection form of bulkLoadTiles).
__device__ __forceinline__ void barrierWithoutCopy(uint64_t *bar) {
  const uint32_t b = smemAddr(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// True once phase 0 of the barrier completed; false after `limit` polls.
__device__ __forceinline__ bool bulkWaitTiles(uint64_t *bar, long long limit = kTileWaitLimit) {
  const uint32_t b = smemAddr(bar);
  for (long long i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(b)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Store: every writer thread fences its shared writes to the async proxy and
// the CTA synchronises before one thread issues the copy and waits for it.
__device__ __forceinline__ void fenceSharedToAsync() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulkStoreTiles(void *gmem, const void *smem, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gmem),
               "r"(smemAddr(smem)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}


}  // namespace
}  // namespace msq
