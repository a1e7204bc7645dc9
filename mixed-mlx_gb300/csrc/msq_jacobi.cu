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
//    when it fits (n <= 320) and in an L2-resident global workspace beyond;
//  * each round's Q_k are logged and a row-parallel kernel replays the sweep
//    onto V (rows of V evolve independently under V <- V Q), so V never
//    competes with A for shared memory;
//  * rotation angles are FP32 (as in the reference's kernel); the off-norm
//    that ends the sweeps is accumulated in FP64 — sweeps stop once
//    off(A) <= tol * ||A||_F instead of after a fixed 8;
//  * launches are size-bucketed (threads per CTA grow with n), largest first.
#include "msq_internal.cuh"
#include "msq_jacobi_device.cuh"
#include "msq_jacobi_grid.cuh"
#include "msq_jacobi_tc.cuh"

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

namespace msq {
namespace {

constexpr size_t kSmemLimit = 227 * 1024;
// the sweep kernel also holds a small static shared block (its mbarrier)
constexpr size_t kSweepSmemLimit = kSmemLimit - 256;
// per CTA when two share an SM (228 KB per SM, 1 KB reserved per CTA)
constexpr size_t kSweepSmemHalf = 110 * 1024;
constexpr int kMaxOrder = 16384;    // grid kernels; the batched ones see n <= 1024
constexpr int kGridMinOrder = 1024;
constexpr int kGridFewLarge = 8;
// Routing cost model of the FP32 (round-robin) eigenvector mode, fitted to
// solves to 1e-7 on a GB300 (about ten sweeps; both paths scale alike with
// the sweep count): one matrix on one CTA takes about 3.8e-7 n^3 ms, and
// batched matrices above 256 saturate at about 40 in flight (their tiles
// stream from L2 / HBM), those up to 256 at about 300; the grid kernels take
// about 5 + 3.8e-5 n^2 ms per matrix, one matrix at a time.
constexpr double kCtaSolveMs = 3.8e-7;    // x n^3
constexpr double kGridSolveMs0 = 5.0;     // + kGridSolveMs2 x n^2
constexpr double kGridSolveMs2 = 3.8e-5;
constexpr double kLargeInFlight = 40.0;
constexpr double kSmallInFlight = 300.0;
constexpr int kGridCandidates = 16;

double ctaSolveMs(int n) { return kCtaSolveMs * n * static_cast<double>(n) * n; }
double gridSolveMs(int n) { return kGridSolveMs0 + kGridSolveMs2 * n * static_cast<double>(n); }

// The matrices of orders 257..1024 that go to the grid kernels: the p
// largest, p minimising the estimated time max(longest one-CTA solve left,
// batched work / matrices in flight, grid solves in sequence), and only
// where that beats the all-batched estimate by 10% (a batch without grid
// matrices runs without host synchronisation and can be captured).
std::vector<char> gridRouting(const int32_t *n, int count) {
  std::vector<char> grid(count, 0);
  std::vector<int> cand;
  double work = 0.0, small_max = 0.0;
  for (int i = 0; i < count; ++i) {
    if (n[i] > kGridMinOrder) {
      grid[i] = 1;
      continue;
    }
    if (n[i] > 256) {
      cand.push_back(i);
      work += ctaSolveMs(n[i]) / kLargeInFlight;
    } else {
      work += ctaSolveMs(n[i]) / kSmallInFlight;
      small_max = std::max(small_max, ctaSolveMs(n[i]));
    }
  }
  std::sort(cand.begin(), cand.end(), [&](int a, int b) { return n[a] > n[b] || (n[a] == n[b] && a < b); });
  const int limit = std::min<int>(kGridCandidates, static_cast<int>(cand.size()));
  auto estimate = [&](int p, double grid_ms, double batched_work) {
    const double longest = p < static_cast<int>(cand.size()) ? ctaSolveMs(n[cand[p]]) : small_max;
    return std::max({longest, batched_work, grid_ms});
  };
  const double all_batched = estimate(0, 0.0, work);
  double best = all_batched, grid_ms = 0.0;
  int best_p = 0;
  for (int p = 1; p <= limit; ++p) {
    const int i = cand[p - 1];
    grid_ms += gridSolveMs(n[i]);
    work -= ctaSolveMs(n[i]) / kLargeInFlight;
    const double t = estimate(p, grid_ms, work);
    if (t < best) {
      best = t;
      best_p = p;
    }
  }
  if (best_p > 0 && best < 0.9 * all_batched)
    for (int p = 0; p < best_p; ++p) grid[cand[p]] = 1;
  return grid;
}

// Routing: a matrix above kGridMinOrder is solved by the grid kernels with
// every SM, the rest by the batched kernels one CTA each, except: in the
// FP32 mode (0) the cost model picks the largest matrices to move to the grid
// kernels (a few large matrices whose one-CTA solves would outlast the
// batch); in the two-level modes (1-3, built for 256 < n <= 512) a matrix
// above 256 when at most kGridFewLarge such matrices are in the batch.
std::vector<char> routeToGrid(const int32_t *n, int count, int mode) {
  if (mode == 0) return gridRouting(n, count);
  int large = 0;
  for (int i = 0; i < count; ++i) large += n[i] > 256;
  std::vector<char> grid(count, 0);
  for (int i = 0; i < count; ++i)
    grid[i] = n[i] > kGridMinOrder || (n[i] > 256 && large <= kGridFewLarge);
  return grid;
}
constexpr int kSweepThreadsMax = 512;
constexpr int kReplayThreads = 256;

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
  const double *tols;        // per matrix (null: tol for all)
  int max_sweeps;
  int first;                 // 1 on the first launch (load A, set norm)
  int parity;                // log buffer of this sweep (log points at it)
  int *status;               // device status word (bounded waits)
  const int2 *sched;         // two-level pair tables (null: round-robin for all)
  const int32_t *sched_off;  // per matrix: its table in sched (int2 units), -1 = round-robin
  int smem_tiles;            // global-tile variant: tiles kept in shared memory
  int wait_test;             // 1: flag waits look for a value nothing writes and
                             //    the tile load's barrier gets no copy
};

__device__ __forceinline__ FlatTiles tileMem(std::true_type, float *s, float *, int) {
  return FlatTiles{s};
}
__device__ __forceinline__ SplitTiles tileMem(std::false_type, float *s, float *g, int split) {
  return SplitTiles{s, g, split};
}

// Entries (16-bit) of one round table of the sweep kernel: pairs (I, J),
// rotate flags, per block its pair and its partner (-1: not rotated).
__host__ __device__ constexpr int roundTableShorts(int nb) { return 3 * (nb / 2) + 2 * nb; }

// One round's table in shared memory and its P 8x8 rotations (kQS floats
// apart).
struct RoundTable {
  short *t;
  float *q;
  int P;
  __device__ short &pi(int k) const { return t[k]; }
  __device__ short &pj(int k) const { return t[P + k]; }
  __device__ short &on(int k) const { return t[2 * P + k]; }
  __device__ short &slot(int b) const { return t[3 * P + b]; }
  __device__ short &partner(int b) const { return t[5 * P + b]; }
};

// Polls of a done flag before the sweep kernel reports kStatusFlagTimeout
// (kFlagWaitTestLimit under the failure-injection mode).
constexpr int kFlagWaitLimit = 1 << 22;
constexpr int kFlagWaitTestLimit = 64;

// Shared memory of the sweep kernel: reduction scratch; the tile table, two
// work counters, P done flags and three round tables; the rotations of two
// rounds; then the packed tiles (with_tiles).
__host__ __device__ constexpr size_t sweepSmemLayout(int n, bool with_tiles, size_t *q_off,
                                                    size_t *tile_off) {
  const int m = padded8(n), nb = m / 4, P = nb / 2;
  size_t bytes = 32 * sizeof(double) + (nb + 1 + 2 + P) * sizeof(int) +
                 3 * roundTableShorts(nb) * sizeof(short);
  bytes = (bytes + 15) & ~static_cast<size_t>(15);
  *q_off = bytes;
  bytes += 2 * static_cast<size_t>(P) * kQS * sizeof(float);
  *tile_off = bytes;
  if (with_tiles) bytes += static_cast<size_t>(nb) * (nb + 1) / 2 * kTileF * sizeof(float);
  return bytes;
}

// One sweep (or the convergence check / write-back) for one matrix per CTA.
template <bool kSmem>
__global__ void __launch_bounds__(kSweepThreadsMax)
jacobiSweepKernel(JacobiArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t tile_bar;
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
  int *counters = tri + nb + 1;
  int *flags = counters + 2;
  short *tables = reinterpret_cast<short *>(flags + P);
  float *qs = reinterpret_cast<float *>(smem_raw + q_off);
  float *gtiles = args.tiles + args.t_offset[mi];
  float *stiles = reinterpret_cast<float *>(smem_raw + tile_off);
  const int tile_count = nb * (nb + 1) / 2;
  // the shared-tile variant holds every tile on chip; the global-tile one the
  // first smem_tiles (the rest stay in the L2-resident workspace)
  const int split = kSmem ? tile_count : min(args.smem_tiles, tile_count);
  const auto tiles = tileMem(std::integral_constant<bool, kSmem>{}, stiles, gtiles, split);
  const float *full = args.a + args.a_offset[mi];
  const int sched_at = args.sched_off != nullptr ? args.sched_off[mi] : -1;
  const int2 *sched = sched_at >= 0 ? args.sched + sched_at : nullptr;
  const int rounds = sched != nullptr ? twoLevelRounds(nb) : nb - 1;

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
        tileAt(tiles, tileElement(tri[J] + I, e / 4, e % 4)) = v;
      }
    }
  } else if (split > 0) {
    // the packed tiles kept between sweeps: one TMA bulk copy into shared
    // memory (bounded wait; on expiry the launch reports and does nothing).
    // Under failure injection no copy is issued, so nothing arrives.
    if (threadIdx.x == 0) {
      if (args.wait_test) barrierWithoutCopy(&tile_bar);
      else bulkLoadTiles(stiles, gtiles, split * kTileF * sizeof(float), &tile_bar);
    }
    __syncthreads();
    if (!bulkWaitTiles(&tile_bar, args.wait_test ? kFlagWaitTestLimit : kTileWaitLimit)) {
      if (threadIdx.x == 0) atomicExch(args.status, kStatusMbarrierTimeout);
      return;
    }
  }
  __syncthreads();

  // Off-norm and norm in FP64.
  double off2 = 0.0, diag2 = 0.0;
  for (int J = 0; J < nb; ++J) {
    for (int idx = threadIdx.x; idx < (J + 1) * kTileF; idx += blockDim.x) {
      const int I = idx / kTileF, e = idx % kTileF;
      const double v = tileAt(tiles, tileElement(tri[J] + I, e / 4, e % 4));
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

  if (ratio <= (args.tols ? args.tols[mi] : args.tol) || sweeps >= args.max_sweeps) {
    // Eigenvalues = diagonal (jacobi_root_eigenvalues_f32 takes the sqrt
    // later, :1436-1444); full symmetric write-back of the matrix.
    float *eig = args.eigenvalues + args.eig_offset[mi];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      eig[k] = tileAt(tiles, tileElement(tri[k / 4] + k / 4, k % 4, k % 4));
    }
    float *out = args.a + args.a_offset[mi];
    for (int c = 0; c < n; ++c) {
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        const int I = r / 4, J = c / 4;
        const float v = I <= J ? tileAt(tiles, tileElement(tri[J] + I, r % 4, c % 4))
                               : tileAt(tiles, tileElement(tri[I] + J, c % 4, r % 4));
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

  // The state after this sweep, written now (every thread took its snapshot
  // before the reductions' barriers; nothing below reads the state), so the
  // norms are not held in registers through the rounds.
  if (threadIdx.x == 0) {
    st.norm2 = norm2;
    st.off_ratio = ratio;
    st.sweeps = sweeps + 1;
    st.done = 0;
    st.logged[args.parity] = 1;
  }
  float *log = args.log + args.log_offset[mi];
  const int items = ((P + 1) / 2) * (P + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  // round r's table is buffer r % 3, its rotations buffer r & 1
  auto table = [&](int r) {
    return RoundTable{tables + (r % 3) * roundTableShorts(nb), qs + (r & 1) * P * kQS, P};
  };

  // Pairs of round r into its table (threads [first, blockDim) take part).
  auto stagePairs = [&](int r, int first) {
    const RoundTable t = table(r);
    for (int k = threadIdx.x - first; k < P; k += blockDim.x - first) {
      int I, J;
      bool on;
      roundPair(sched, k, r, nb, I, J, on);
      t.pi(k) = static_cast<short>(I);
      t.pj(k) = static_cast<short>(J);
      t.on(k) = static_cast<short>(on);
      t.slot(I) = static_cast<short>(k);
      t.slot(J) = static_cast<short>(k);
      t.partner(I) = static_cast<short>(on ? J : -1);
      t.partner(J) = static_cast<short>(on ? I : -1);
    }
  };

  // Pivots of a round: a quad of lanes per block pair, eight pairs per warp,
  // warps [0, pw) of the CTA.  The loop is warp-uniform (all lanes of a warp
  // take part in the quad shuffles; lanes past P idle).  An identity pair
  // keeps its blocks and logs Q = I.
  auto pivot = [&](const RoundTable &t, int k) {
    const int t4 = lane & 3;
    const bool present = k < P;
    const bool active = present && t.on(k);
    float ra[8], rb[8];
    int tII = 0, tIJ = 0, tJJ = 0;
    if (active) {
      const int I = t.pi(k), J = t.pj(k);
      tII = tileIndex(tri, I, I);
      tIJ = tileIndex(tri, I, J);
      tJJ = tileIndex(tri, J, J);
      // lane t starts with rows t (block I) and 7 - t (block J row 3 - t;
      // its left half is the mirror of tile (I, J))
      const float4 *sII = reinterpret_cast<const float4 *>(tiles.base(tII));
      const float4 *sIJ = reinterpret_cast<const float4 *>(tiles.base(tIJ));
      const float4 *sJJ = reinterpret_cast<const float4 *>(tiles.base(tJJ));
      const int jr = 3 - t4;
      const float4 v0 = sII[t4 ^ (tII & 3)], v1 = sIJ[t4 ^ (tIJ & 3)], v2 = sJJ[jr ^ (tJJ & 3)];
      ra[0] = v0.x; ra[1] = v0.y; ra[2] = v0.z; ra[3] = v0.w;
      ra[4] = v1.x; ra[5] = v1.y; ra[6] = v1.z; ra[7] = v1.w;
#pragma unroll
      for (int i = 0; i < 4; ++i) rb[i] = tileAt(tiles, tileElement(tIJ, i, jr));
      rb[4] = v2.x; rb[5] = v2.y; rb[6] = v2.z; rb[7] = v2.w;
    } else {
#pragma unroll
      for (int y = 0; y < 8; ++y) ra[y] = rb[y] = 0.0f;
    }
    pivotSweep(ra, rb, t.q + (active ? k : 0) * kQS, t4, active);
    if (active) {
      // rows t (tiles (I, I), (I, J)) and 4 + t (tile (J, J)); the lower
      // left block is the mirror of tile (I, J) and is not stored
      float4 *sII = reinterpret_cast<float4 *>(tiles.base(tII));
      float4 *sIJ = reinterpret_cast<float4 *>(tiles.base(tIJ));
      float4 *sJJ = reinterpret_cast<float4 *>(tiles.base(tJJ));
      sII[t4 ^ (tII & 3)] = make_float4(ra[0], ra[1], ra[2], ra[3]);
      sIJ[t4 ^ (tIJ & 3)] = make_float4(ra[4], ra[5], ra[6], ra[7]);
      sJJ[t4 ^ (tJJ & 3)] = make_float4(rb[4], rb[5], rb[6], rb[7]);
    } else if (present) {
      // identity pair: Q = I (lane t writes rows 2t and 2t + 1)
      float4 *q4 = reinterpret_cast<float4 *>(t.q + k * kQS);
#pragma unroll
      for (int x = 0; x < 2; ++x) {
        const int row = 2 * t4 + x;
        q4[2 * row] = make_float4(row == 0, row == 1, row == 2, row == 3);
        q4[2 * row + 1] = make_float4(row == 4, row == 5, row == 6, row == 7);
      }
    }
  };

  // Off-pivot super-tiles: T' = Q_k^T T Q_l for pairs k < l of a round, two
  // lanes per super-tile (warp-uniform: the pair shuffle has all lanes).
  auto superTile = [&](const RoundTable &t, int k, int l, int h, bool valid) {
    superTileHalfMem(tiles, SharedTri{tri}, reinterpret_cast<const float4 *>(t.q + k * kQS),
                     reinterpret_cast<const float4 *>(t.q + l * kQS), t.pi(k), t.pj(k), t.pi(l),
                     t.pj(l), h, valid);
  };
  // The super-tile (k, l) of round `cur` holding the tile (x, y) that pivot
  // kk of round `nxt` reads (none when cur paired x and y: its pivot wrote
  // that tile).  Two pairs of nxt can meet the same super-tile; the one
  // holding the smaller block computes it (*owner = kk) and the other waits
  // for it (*owner = that pair).  Returns whether kk needs a super-tile.
  auto criticalItem = [&](const RoundTable &cur, const RoundTable &nxt, int kk, int &k, int &l,
                          int &owner) {
    owner = kk;
    if (kk >= P || !nxt.on(kk)) return false;
    const int x = nxt.pi(kk), y = nxt.pj(kk);
    k = cur.slot(x);
    l = cur.slot(y);
    if (k == l) return false;
    const int ox = cur.pi(k) + cur.pj(k) - x, oy = cur.pi(l) + cur.pj(l) - y;
    if (nxt.partner(ox) == oy && min(ox, oy) < min(x, y)) owner = nxt.slot(ox);
    if (k > l) {
      const int s = k;
      k = l;
      l = s;
    }
    return true;
  };
  // Whether super-tile (k, l) of cur is one of those.
  auto isCritical = [&](const RoundTable &cur, const RoundTable &nxt, int k, int l) {
    const int p1 = nxt.partner(cur.pi(k)), p2 = nxt.partner(cur.pj(k));
    return (p1 >= 0 && cur.slot(p1) == l) || (p2 >= 0 && cur.slot(p2) == l);
  };
  // The other super-tiles of cur (all of them without a next round), taken
  // by warps 32 lanes (16 super-tiles) at a time from a shared counter.
  auto otherItems = [&](const RoundTable &cur, const RoundTable &nxt, bool more, int *counter) {
    for (;;) {
      int base = 0;
      if (lane == 0) base = atomicAdd(counter, 32);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= 2 * items) break;
      const int w2 = base + lane;
      int k = 0, l = 0;
      bool valid = w2 < 2 * items && foldedBlock(w2 >> 1, P, k, l) && k != l;
      if (valid && more && isCritical(cur, nxt, k, l)) valid = false;
      if (!valid) k = l = 0;
      superTile(cur, k, l, w2 & 1, valid);
    }
  };

  // Round r+1's pivots need only round r's pivots and, of r's super-tiles,
  // the one holding each pivot's cross tile.  So while the CTA updates
  // round r's other super-tiles, warps [0, pw) compute those super-tiles
  // (two lanes of each pivot's quad) and run round r+1's pivots: one barrier
  // per round.  Every tile sees the same operations in the same order as in
  // the plain round order (pivots, then all super-tiles, round by round).
  const int pw = min(warps, (P + 7) / 8);
  const int stage_first = pw < warps ? 32 * pw : 0;  // threads that stage tables and log
  stagePairs(0, 0);
  if (rounds > 1) stagePairs(1, 0);
  if (threadIdx.x == 0) counters[0] = counters[1] = 0;
  for (int k = threadIdx.x; k < P; k += blockDim.x) flags[k] = 0;
  __syncthreads();
  for (int base = 8 * warp; base < P; base += 8 * warps) pivot(table(0), base + (lane >> 2));
  __syncthreads();
  for (int round = 0; round < rounds; ++round) {
    const RoundTable cur = table(round), nxt = table(round + 1);
    const bool more = round + 1 < rounds;
    const bool pivot_warp = more && warp < pw;
    if (pivot_warp) {
      // round r's super-tiles under round r+1's pivots (all of this warp's
      // first, then their done flags, so no warp waits before it has set its own)
      for (int base = 8 * warp; base < P; base += 8 * pw) {
        const int kk = base + (lane >> 2);
        int k = 0, l = 0, owner = kk;
        const bool own = (lane & 2) == 0 && criticalItem(cur, nxt, kk, k, l, owner) && owner == kk;
        if (!own) k = l = 0;
        superTile(cur, k, l, lane & 1, own);
        __syncwarp();
        if (own && (lane & 3) == 0) {
          __threadfence_block();
          atomicExch(&flags[kk], round + 1);
        }
      }
      for (int base = 8 * warp; base < P; base += 8 * pw) {
        const int kk = base + (lane >> 2);
        int k = 0, l = 0, owner = kk;
        const bool wait = criticalItem(cur, nxt, kk, k, l, owner) && owner != kk;
        if (wait && (lane & 3) == 0) {
          // bounded: on expiry the launch reports and goes on
          int spins = 0;
          const int target = round + 1 + (args.wait_test ? (1 << 29) : 0);
          const int limit = args.wait_test ? kFlagWaitTestLimit : kFlagWaitLimit;
          while (atomicAdd(&flags[owner], 0) != target) {
            if (++spins > limit) {
              atomicExch(args.status, kStatusFlagTimeout);
              break;
            }
            __nanosleep(32);
          }
          __threadfence_block();
        }
        __syncwarp();
        pivot(nxt, kk);
      }
    }
    if (static_cast<int>(threadIdx.x) >= stage_first) {
      if (round + 2 < rounds) stagePairs(round + 2, stage_first);
      if (threadIdx.x == stage_first) counters[(round + 1) & 1] = 0;
      // this round's rotations, logged for the V replay (coalesced copy)
      const float4 *src = reinterpret_cast<const float4 *>(cur.q);
      float4 *dst = reinterpret_cast<float4 *>(log + static_cast<int64_t>(round) * P * kQF);
      for (int x = threadIdx.x - stage_first; x < P * kQF / 4; x += blockDim.x - stage_first) {
        dst[x] = src[(x >> 4) * (kQS / 4) + (x & 15)];
      }
    }
    otherItems(cur, nxt, more, counters + (round & 1));
    __syncthreads();
  }
  if (split > 0) {
    // the shared tiles back to the workspace: one TMA bulk copy
    fenceSharedToAsync();
    __syncthreads();
    if (threadIdx.x == 0) bulkStoreTiles(gtiles, stiles, split * kTileF * sizeof(float));
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
  const int2 *sched;           // two-level pair tables, as JacobiArgs
  const int32_t *sched_off;
};

// Replay shared memory: `rows` rows of V (stride m + 4) and two rounds of
// rotations (the next round's are copied in while the current one runs).
__host__ __device__ __forceinline__ size_t replaySmemBytes(int max_n, int rows) {
  const int m = padded8(max_n), P = m / 8;
  return static_cast<size_t>(rows) * (m + 4) * sizeof(float) +
         2 * static_cast<size_t>(P) * kQF * sizeof(float) + 2 * static_cast<size_t>(P) * sizeof(int2);
}


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
  int2 *pairs = reinterpret_cast<int2 *>(qbuf + 2 * P * kQF);  // [2][P] (I, J) by round parity
  float *v = args.v + args.a_offset[mi];
  const int rows = min(R, n - r0);
  const float *log = args.log + args.log_offset[mi];
  const int sched_at = args.sched_off != nullptr ? args.sched_off[mi] : -1;
  const int2 *sched = sched_at >= 0 ? args.sched + sched_at : nullptr;
  const int rounds = sched != nullptr ? twoLevelRounds(nb) : nb - 1;
  const int chunks = P * kQF / 4;  // 16-byte pieces of one round's rotations
  for (int x = threadIdx.x; x < chunks; x += blockDim.x) copyAsync16(qbuf + 4 * x, log + 4 * x);
  copyAsyncCommit();
  for (int k = threadIdx.x; k < m * R; k += blockDim.x) {
    const int c = k / R, r = k % R;
    vs[r * ld + c] = (c < n && r < rows) ? v[r0 + r + static_cast<int64_t>(c) * n] : 0.0f;
  }
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    int I, J;
    bool rotate;
    roundPair(sched, k, 0, nb, I, J, rotate);
    pairs[k] = make_int2(I, J);
  }
  // item -> (pair k, slice of up to 32 rows); a lane takes row r_in of the
  // slice and, when R > 32, rows r_in + 32, r_in + 64, ... with the same Q_k
  const int lanes_r = R < 32 ? R : 32;
  const int lanes_shift = R < 32 ? -1 : 5;
  const int per_lane = R < 32 ? 1 : R / 32;
  for (int round = 0; round < rounds; ++round) {
    copyAsyncWaitAll();
    __syncthreads();  // this round's rotations and pairs ready; last round's rows written
    if (round + 1 < rounds) {
      float *next = qbuf + ((round + 1) & 1) * P * kQF;
      const float *src = log + static_cast<int64_t>(round + 1) * P * kQF;
      for (int x = threadIdx.x; x < chunks; x += blockDim.x) copyAsync16(next + 4 * x, src + 4 * x);
      copyAsyncCommit();
      for (int k = threadIdx.x; k < P; k += blockDim.x) {
        int I, J;
        bool rotate;
        roundPair(sched, k, round + 1, nb, I, J, rotate);
        pairs[((round + 1) & 1) * P + k] = make_int2(I, J);
      }
    }
    const float *qs = qbuf + (round & 1) * P * kQF;
    const int2 *pr = pairs + (round & 1) * P;
    for (int item = threadIdx.x; item < P * lanes_r; item += blockDim.x) {
      const int k = lanes_shift > 0 ? item >> lanes_shift : item / lanes_r;
      const int r_in = lanes_shift > 0 ? item & 31 : item % lanes_r;
      const int2 ij = pr[k];
      const int I = ij.x, J = ij.y;
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

// V = I per matrix (column-major): CTAs over columns, threads down a column
// (coalesced stores, no per-element division).
__global__ void identityKernel(float *v, const int64_t *a_offset, const int32_t *n, int count) {
  for (int mi = blockIdx.y; mi < count; mi += gridDim.y) {
    const int nn = n[mi];
    float *out = v + a_offset[mi];
    for (int c = blockIdx.x; c < nn; c += gridDim.x) {
      float *col = out + static_cast<int64_t>(c) * nn;
      for (int r = threadIdx.x; r < nn; r += blockDim.x) col[r] = r == c ? 1.0f : 0.0f;
    }
  }
}

// Final state of a matrix solved by the grid kernels.
__global__ void gridStateKernel(JacobiState *st, int sweeps, double ratio, double norm2) {
  st->norm2 = norm2;
  st->off_ratio = ratio;
  st->sweeps = sweeps;
  st->done = 1;
  st->logged[0] = 0;
  st->logged[1] = 0;
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
  return sweepSmemLayout(n, true, &q_off, &tile_off) <= kSweepSmemLimit;
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
// and, once every candidate has kTuneSamples times (from as many calls),
// keeps the fastest for that device.
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
                                        "128<n<=256", "256<n<=320 (shared tiles)",
                                        "320<n<=512 (global tiles)", "512<n<=1024", "1024<n<=2048"};
  return names[c];
}

// A candidate is a CTA size; a negative one runs a shared-tile class with
// the global-tile variant (as many tiles in shared memory as fit two CTAs
// per SM, the rest in the workspace), trading on-chip tiles for a second
// CTA that overlaps the other's pivot phase.
std::vector<int> classCandidates(int c) {
  switch (c) {
    case 0: return {32};
    case 1: return {64, 32};
    case 2: return {128, 64};
    case 3: return {256, 128};
    case 4: return {256, 512, -256};
    case 5: return {512, 256, -256};
    default: return {512, 256};
  }
}

// Launch names per class (static strings for the launch timer).
const char *sweepName(int c) {
  static const char *names[kClasses] = {
      "jacobi sweep n<=16", "jacobi sweep n<=32", "jacobi sweep n<=64", "jacobi sweep n<=128",
      "jacobi sweep n<=256", "jacobi sweep n<=320", "jacobi sweep n<=512 (global)",
      "jacobi sweep n<=1024 (global)", "jacobi sweep n<=2048 (global)"};
  return names[c];
}

// Timed launches per candidate before a class is decided (the fastest of
// them counts: a single launch shares the GPU with the other buckets'
// streams, and one sample can misorder candidates a few percent apart).
constexpr int kTuneSamples = 2;

struct ClassTune {
  std::vector<int> cands;
  std::vector<double> ms;   // per candidate: fastest sample, < 0 until measured
  std::vector<int> samples; // per candidate: timed launches so far
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
      t[c].samples.assign(t[c].cands.size(), 0);
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
      ++t.samples[p.cand];
      bool all = true;
      for (int v : t.samples) all = all && v >= kTuneSamples;
      if (all) {
        t.best = static_cast<int>(std::min_element(t.ms.begin(), t.ms.end()) - t.ms.begin());
      }
    }
    t.requested = false;
    g_pending.erase(g_pending.begin() + i);
  }
}

// Per-layout launch plan, kept per batch layout and device in the context.
struct JacobiPlan {
  uint64_t key = 0;
  uint64_t serial = 0;  // unique per plan ever built (keys captured graphs)
  int count = 0;
  int device_id = 0;
  int64_t tile_total = 0, log_total = 0;
  int64_t *t_offset = nullptr, *log_offset = nullptr;
  int32_t *order = nullptr;  // ids grouped by bucket, largest first
  // smem_bytes: the class's kernel layout; base_bytes: the layout without
  // tiles (the global-tile variant adds what it keeps on chip)
  struct Bucket { int cls; bool smem; int first; int count; size_t smem_bytes; size_t base_bytes; };
  std::vector<Bucket> buckets;
  int32_t *work_matrix = nullptr, *work_row = nullptr;
  int work_count = 0;
  // V replay launches, one per size class: CTAs [first, first + count) of
  // the work lists, `rows` rows each, `smem` bytes of shared memory.
  struct ReplayGroup { int first; int count; int rows; size_t smem; };
  std::vector<ReplayGroup> replays;
  std::vector<int> grid_ids;  // matrices solved by the grid kernels
  // Eigenvector mode (msq_set_jacobi_vectors, resolved): two-level pair
  // tables for 256 < n <= 512 in modes 1 and 2; in mode 2 those matrices'
  // V update runs on the tensor cores (tcv) instead of the FP32 replay.
  int mode = 0;
  const int2 *sched = nullptr;
  const int32_t *sched_off = nullptr;
  TcVectorsDevice tcv;
  int64_t tcv_images = 0;
  // mode 2: the two-level tensor-core Jacobi for 256 < n <= 512 (tl),
  // its B scratch (elements of the batch) and diagonal blocks
  TwoLevelDevice tl;
  int64_t batch_elements = 0, diag_blocks = 0;
  void *device = nullptr;
};

}  // namespace

// The context's Jacobi plans (at most 8 layouts, oldest evicted first).
struct JacobiPlanCache {
  std::vector<JacobiPlan *> plans;
};

void destroyJacobiPlans(JacobiPlanCache *cache) {
  if (cache == nullptr) return;
  for (JacobiPlan *p : cache->plans) {
    cudaFree(p->device);
    delete p;
  }
  delete cache;
}

namespace {


// Carves aligned arrays out of one device allocation.
struct Carve {
  size_t bytes = 0;
  template <typename T>
  size_t take(size_t count) {
    bytes = (bytes + 15) & ~static_cast<size_t>(15);
    const size_t at = bytes;
    bytes += count * sizeof(T);
    return at;
  }
};

JacobiPlan *planFor(msq_ctx *ctx, const DeviceBatch *b, int mode) {
  if (ctx->jacobi_plans == nullptr) ctx->jacobi_plans = new JacobiPlanCache;
  auto &plans = ctx->jacobi_plans->plans;
  for (JacobiPlan *p : plans)
    if (p->key == b->key && p->count == b->count && p->device_id == ctx->device && p->mode == mode)
      return p;
  static std::atomic<uint64_t> next_serial{1};
  auto *plan = new JacobiPlan;
  plan->serial = next_serial.fetch_add(1);
  plan->device_id = ctx->device;
  plan->key = b->key;
  plan->count = b->count;
  plan->mode = mode;
  const int total = b->count;
  const std::vector<char> routed = routeToGrid(b->host_n.data(), total, mode);
  std::vector<int32_t> ids;
  std::vector<int64_t> t_off(total, 0), l_off(total, 0);
  std::vector<int32_t> sched_off(total, -1), sched_host, table;
  std::map<int, int32_t> sched_at;  // block count -> table offset (int2 units)
  std::vector<int> tc_ids, tl_ids;  // V on the tensor cores; A too (mode 3)
  std::vector<char> on_tc(total, 0);
  for (int i = 0; i < total; ++i) {
    const int n = b->host_n[i];
    if (routed[i]) {
      plan->grid_ids.push_back(i);
      continue;
    }
    const int m = padded8(n), nb = m / 4, P = nb / 2;
    const bool two_level = mode != 0 && n >= kTwoLevelMinOrder && n <= kTwoLevelMaxOrder;
    if (two_level && mode == 3) {
      // the two-level Jacobi with tensor-core updates of A: no packed
      // tiles, no rotation log
      tc_ids.push_back(i);
      tl_ids.push_back(i);
      on_tc[i] = 1;
      continue;
    }
    ids.push_back(i);
    t_off[i] = plan->tile_total;
    plan->tile_total += static_cast<int64_t>(nb) * (nb + 1) / 2 * kTileF;
    l_off[i] = plan->log_total;
    plan->log_total += static_cast<int64_t>(two_level ? twoLevelRounds(nb) : nb - 1) * P * kQF;
    if (two_level) {
      auto at = sched_at.find(nb);
      if (at == sched_at.end()) {
        twoLevelSchedule(nb, table);
        at = sched_at.emplace(nb, static_cast<int32_t>(sched_host.size() / 2)).first;
        sched_host.insert(sched_host.end(), table.begin(), table.end());
      }
      sched_off[i] = at->second;
      if (mode == 2) {
        tc_ids.push_back(i);
        on_tc[i] = 1;
      }
    }
  }
  TcVectorsTables tcv;
  tcVectorsTables(b->host_n.data(), total, tc_ids, tcv);
  TwoLevelTables tlt;
  twoLevelTables(b->host_n.data(), total, tl_ids, tlt);
  for (int i = 0; i < total; ++i)
    plan->batch_elements = std::max<int64_t>(
        plan->batch_elements, b->host_offset[i] + static_cast<int64_t>(b->host_n[i]) * b->host_n[i]);
  const int count = static_cast<int>(ids.size());
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
    size_t bytes = 0, base = 0;
    while (j < count && sizeClass(b->host_n[ids[j]]) == c) {
      size_t q_off, tile_off;
      bytes = std::max(bytes, sweepSmemLayout(b->host_n[ids[j]], smem, &q_off, &tile_off));
      base = std::max(base, sweepSmemLayout(b->host_n[ids[j]], false, &q_off, &tile_off));
      ++j;
    }
    plan->buckets.push_back({c, smem, i, j - i, bytes, base});
    i = j;
  }
  std::vector<int32_t> wm, wr;
  for (const auto &bucket : plan->buckets) {
    int max_n = 0;
    for (int i = bucket.first; i < bucket.first + bucket.count; ++i) max_n = std::max(max_n, b->host_n[ids[i]]);
    const int rows = replayRows(max_n);
    const int first = static_cast<int>(wm.size());
    for (int i = bucket.first; i < bucket.first + bucket.count; ++i) {
      if (on_tc[ids[i]]) continue;  // V on the tensor cores
      const int n = b->host_n[ids[i]];
      for (int r = 0; r < n; r += rows) {
        wm.push_back(ids[i]);
        wr.push_back(r);
      }
    }
    if (static_cast<int>(wm.size()) > first) {
      plan->replays.push_back({first, static_cast<int>(wm.size()) - first, rows,
                               replaySmemBytes(max_n, rows)});
    }
  }
  plan->work_count = static_cast<int>(wm.size());
  Carve carve;
  const size_t at_t = carve.take<int64_t>(total), at_l = carve.take<int64_t>(total);
  const size_t at_img = carve.take<int64_t>(total);
  const size_t at_order = carve.take<int32_t>(total), at_wm = carve.take<int32_t>(wm.size());
  const size_t at_wr = carve.take<int32_t>(wr.size()), at_so = carve.take<int32_t>(total);
  const size_t at_sched = carve.take<int32_t>(sched_host.size());
  const size_t at_prog = carve.take<int32_t>(tcv.prog.size());
  const size_t at_po = carve.take<int32_t>(total);
  const size_t at_fw = carve.take<int32_t>(tcv.form_work.size());
  const size_t at_aw = carve.take<int32_t>(tcv.apply_work.size());
  const size_t at_tl_ids = carve.take<int32_t>(tlt.ids.size());
  const size_t at_tl_inner = carve.take<int32_t>(tlt.inner.size());
  const size_t at_tl_diag = carve.take<int64_t>(total);
  char *dev = nullptr;
  if (cudaCheck(ctx, cudaMalloc(&dev, carve.bytes + 16), "jacobi plan alloc") != MSQ_OK) {
    delete plan;
    return nullptr;
  }
  auto put = [&](size_t at, const void *src, size_t bytes) {
    if (bytes > 0) cudaMemcpy(dev + at, src, bytes, cudaMemcpyHostToDevice);
  };
  plan->device = dev;
  plan->t_offset = reinterpret_cast<int64_t *>(dev + at_t);
  plan->log_offset = reinterpret_cast<int64_t *>(dev + at_l);
  plan->order = reinterpret_cast<int32_t *>(dev + at_order);
  plan->work_matrix = reinterpret_cast<int32_t *>(dev + at_wm);
  plan->work_row = reinterpret_cast<int32_t *>(dev + at_wr);
  put(at_t, t_off.data(), total * sizeof(int64_t));
  put(at_l, l_off.data(), total * sizeof(int64_t));
  put(at_order, ids.data(), count * sizeof(int32_t));
  put(at_wm, wm.data(), wm.size() * sizeof(int32_t));
  put(at_wr, wr.data(), wr.size() * sizeof(int32_t));
  if (!sched_host.empty()) {
    plan->sched = reinterpret_cast<const int2 *>(dev + at_sched);
    plan->sched_off = reinterpret_cast<const int32_t *>(dev + at_so);
    put(at_sched, sched_host.data(), sched_host.size() * sizeof(int32_t));
    put(at_so, sched_off.data(), total * sizeof(int32_t));
  }
  if (!tc_ids.empty()) {
    plan->tcv.form_work = reinterpret_cast<const int2 *>(dev + at_fw);
    plan->tcv.form_items = static_cast<int>(tcv.form_work.size() / 2);
    plan->tcv.apply_work = reinterpret_cast<const int2 *>(dev + at_aw);
    plan->tcv.apply_items = static_cast<int>(tcv.apply_work.size() / 2);
    plan->tcv.prog = reinterpret_cast<const int32_t *>(dev + at_prog);
    plan->tcv.prog_off = reinterpret_cast<const int32_t *>(dev + at_po);
    plan->tcv.image_off = reinterpret_cast<const int64_t *>(dev + at_img);
    plan->tcv_images = tcv.images;
    put(at_fw, tcv.form_work.data(), tcv.form_work.size() * sizeof(int32_t));
    put(at_aw, tcv.apply_work.data(), tcv.apply_work.size() * sizeof(int32_t));
    put(at_prog, tcv.prog.data(), tcv.prog.size() * sizeof(int32_t));
    put(at_po, tcv.prog_off.data(), total * sizeof(int32_t));
    put(at_img, tcv.image_off.data(), total * sizeof(int64_t));
  }
  if (!tl_ids.empty()) {
    plan->tl.ids = reinterpret_cast<const int32_t *>(dev + at_tl_ids);
    plan->tl.count = static_cast<int>(tlt.ids.size());
    plan->tl.inner = reinterpret_cast<const int2 *>(dev + at_tl_inner);
    plan->tl.stage_first = tlt.stage_first;
    plan->tl.stage_count = tlt.stage_count;
    plan->tl.diag_off = reinterpret_cast<const int64_t *>(dev + at_tl_diag);
    plan->diag_blocks = tlt.diag_blocks;
    put(at_tl_ids, tlt.ids.data(), tlt.ids.size() * sizeof(int32_t));
    put(at_tl_inner, tlt.inner.data(), tlt.inner.size() * sizeof(int32_t));
    put(at_tl_diag, tlt.diag_off.data(), total * sizeof(int64_t));
  }
  if (plans.size() >= 8) {
    cudaFree(plans.front()->device);
    ++ctx->alloc_generation;
    delete plans.front();
    plans.erase(plans.begin());
  }
  plans.push_back(plan);
  return plan;
}

// Opt-in shared memory sizes, set once per device (a bit per device).
int setKernelAttributes() {
  static std::atomic<uint64_t> done_mask{0};
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MSQ_ERR_CUDA;
  const uint64_t bit = uint64_t{1} << device;
  if (done_mask.load() & bit) return MSQ_OK;
  if (cudaFuncSetAttribute(jacobiSweepKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kSweepSmemLimit)) != cudaSuccess ||
      cudaFuncSetAttribute(jacobiSweepKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kSweepSmemLimit)) != cudaSuccess ||
      cudaFuncSetAttribute(jacobiReplayKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kSmemLimit)) != cudaSuccess) {
    return MSQ_ERR_CUDA;
  }
  done_mask.fetch_or(bit);
  return MSQ_OK;
}

}  // namespace

// Enqueues the whole solve on ctx->stream (Jacobi scratch arena).
// Whether jacobiEnqueue on this batch can run inside a whole-solve capture:
// every matrix on the batched kernels (the grid path synchronises per
// sweep) and no size class still being timed by the launch-shape tuner.
bool jacobiCapturable(msq_ctx *ctx, const DeviceBatch *b, bool low_bit_basis) {
  if (b->max_n > kMaxOrder) return false;
  const int mode = ctx->jacobi_vectors >= 0 ? ctx->jacobi_vectors : (low_bit_basis ? 2 : 0);
  JacobiPlan *plan = planFor(ctx, b, mode);
  if (plan == nullptr || !plan->grid_ids.empty()) return false;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  harvestTimings();
  auto &tune = tuneFor(ctx->device);
  for (const auto &bucket : plan->buckets) {
    if (g_tune_enabled && tune[bucket.cls].best < 0) return false;
  }
  return true;
}

int jacobiEnqueue(msq_ctx *ctx, const DeviceBatch *b, float *matrices, float *vectors,
                  float *eigenvalues, double tolerance, int max_sweeps, int32_t *sweeps_done,
                  float *off_ratio, bool low_bit_basis, const double *tols_device,
                  const double *tols_host, bool keep_vectors) {
  if (b->max_n > kMaxOrder) {
    return setError(ctx, MSQ_ERR_UNSUPPORTED, "jacobi: order above 16384 is not supported");
  }
  const int mode = ctx->jacobi_vectors >= 0 ? ctx->jacobi_vectors : (low_bit_basis ? 2 : 0);
  JacobiPlan *plan = planFor(ctx, b, mode);
  if (plan == nullptr) return MSQ_ERR_CUDA;
  const size_t state_bytes = (b->count * sizeof(JacobiState) + 255) & ~size_t(255);
  const size_t tile_bytes = (plan->tile_total * sizeof(float) + 255) & ~size_t(255);
  // Two log buffers (sweep parity) so sweep k+1 overlaps the replay of k.
  const size_t log_bytes = (2 * plan->log_total * sizeof(float) + 1023) & ~size_t(1023);
  // rotation images double-buffered by sweep parity (the V update of sweep
  // k reads them while sweep k + 1 writes the other set); two-level B
  // scratch and diagonal blocks
  const size_t image_set = static_cast<size_t>(plan->tcv_images) * kRotationImageBytes;
  const size_t b_bytes = plan->tl.count > 0
                             ? (static_cast<size_t>(plan->batch_elements) * sizeof(float) + 255) & ~size_t(255)
                             : 0;
  const size_t diag_bytes = static_cast<size_t>(plan->diag_blocks) * 4096 * sizeof(float);
  char *work = static_cast<char *>(scratch(
      ctx, state_bytes + tile_bytes + log_bytes + 2 * image_set + b_bytes + diag_bytes, kScratchJacobi));
  if (work == nullptr) return MSQ_ERR_CUDA;
  uint8_t *images = reinterpret_cast<uint8_t *>(work + state_bytes + tile_bytes + log_bytes);
  float *b_scratch = reinterpret_cast<float *>(work + state_bytes + tile_bytes + log_bytes + 2 * image_set);
  float *diag = reinterpret_cast<float *>(work + state_bytes + tile_bytes + log_bytes + 2 * image_set + b_bytes);
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
  args.tols = tols_device;
  args.max_sweeps = max_sweeps;
  args.status = ctx->d_status;
  args.sched = plan->sched;
  args.sched_off = plan->sched_off;
  args.wait_test = waitTestMode() == kWaitTestFlag;
  VArgs vargs{vectors, b->offset, plan->log_offset, b->n, log_base, args.state,
              plan->work_matrix, plan->work_row, 0, 0, plan->sched, plan->sched_off};
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
  // The batched launch sequence (no host synchronisation, no allocation) is
  // captured once into a CUDA graph per (plan, buffers, tolerance, budget,
  // launch shapes, concurrency) and replayed on later calls.  Calls that
  // measure launch shapes, run the launch timer or solve a matrix on the grid
  // kernels (host-synchronised per sweep) are enqueued directly.
  uint64_t shape_hash = 1469598103934665603ull;
  for (const auto &per : shape)
    for (const auto &h : per) shape_hash = (shape_hash ^ static_cast<uint64_t>(h.threads)) * 1099511628211ull;
  shape_hash = (shape_hash ^ (keep_vectors ? 0x9e37u : 0u)) * 1099511628211ull;
  const bool graphable = !measuring && !ctx->timing && plan->grid_ids.empty() && ctx->graphs &&
                         waitTestMode() == kWaitTestOff && !ctx->capturing;
  const JacobiGraphKey key{plan->serial, b->key, b->offset, matrices, vectors, eigenvalues,
                           sweeps_done, off_ratio, work, tols_device, tolerance, max_sweeps,
                           ctx->concurrent, shape_hash};
  if (graphable) {
    for (auto &e : ctx->jacobi_graphs) {
      if (e.key == key) {
        MSQ_TRY(cudaCheck(ctx, cudaGraphLaunch(e.exec, ctx->stream), "jacobi graph launch"));
        ++ctx->graph_launches;
        ctx->launches += e.launches;
        return MSQ_OK;
      }
    }
  }
  cudaStream_t caller = ctx->stream;
  cudaStream_t capture = nullptr;
  const uint64_t launches0 = ctx->launches;
  if (graphable) {
    capture = auxStream(ctx, 4);
    if (capture == caller) return setError(ctx, MSQ_ERR_CUDA, "jacobi: no capture stream");
    MSQ_TRY(cudaCheck(ctx, cudaStreamBeginCapture(capture, cudaStreamCaptureModeThreadLocal),
                      "jacobi capture"));
    ctx->stream = capture;
  }
  auto body = [&]() -> int {
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(args.state, 0, state_bytes, ctx->stream), "state reset"));
  if (!keep_vectors) {
    // a few CTAs per matrix (most matrices of a batch are small: a wide grid
    // would be mostly empty CTAs)
    dim3 grid(std::max(1, std::min(8, b->max_n / 64)), std::min(b->count, 65535));
    identityKernel<<<grid, 256, 0, ctx->stream>>>(vectors, b->offset, b->n, b->count);
    MSQ_TRY(launched(ctx, "jacobi identity"));
  }
  // Streams: size buckets round-robin over three sweep streams, the replay
  // on a fourth.  Order: sweep k of a bucket follows sweep k-1 (same
  // stream) and the replay of k-2 (which read the log buffer sweep k
  // overwrites); the replay of k follows every bucket's sweep k.  A call
  // that measures candidate shapes runs serially so that each timed launch
  // has the GPU to itself.
  syncReset(ctx);
  const bool serial = !ctx->concurrent || measuring;
  // the two-level group takes the stream after the buckets'
  const int groups = static_cast<int>(plan->buckets.size()) + (plan->tl.count > 0 ? 1 : 0);
  const int sweep_streams = std::min<int>(3, groups);
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
      const int threads = how.threads < 0 ? -how.threads : how.threads;
      if (bucket.smem && how.threads > 0) {
        jacobiSweepKernel<true><<<bucket.count, threads, bucket.smem_bytes, s>>>(args);
      } else {
        // global-tile variant: what fits of the tiles in shared memory, one
        // CTA per SM at 512 threads, two at 256 (the register budget allows
        // two)
        const size_t limit = threads >= 512 ? kSweepSmemLimit : kSweepSmemHalf;
        const size_t room = limit > bucket.base_bytes ? limit - bucket.base_bytes : 0;
        args.smem_tiles = static_cast<int>(room / (kTileF * sizeof(float)));
        jacobiSweepKernel<false><<<bucket.count, threads,
                                   bucket.base_bytes + args.smem_tiles * kTileF * sizeof(float), s>>>(args);
        args.smem_tiles = 0;
      }
      MSQ_TRY(launchedOn(ctx, s, sweepName(bucket.cls)));
      if (how.measure >= 0) {
        cudaEventRecord(t1, s);
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_pending.push_back({ctx->device, bucket.cls, how.measure, t0, t1, bucket.count});
      }
    }
    if (plan->tl.count > 0) {
      cudaStream_t s = ss[plan->buckets.size() % sweep_streams];
      MSQ_TRY(twoLevelEnqueue(ctx, s, plan->tl, plan->tcv, matrices, b_scratch, diag,
                              images + parity * image_set, b->offset, b->n, b->eig_offset,
                              eigenvalues, args.state, tolerance, tols_device, max_sweeps,
                              launch == 0, launch < max_sweeps, parity));
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
      MSQ_TRY(tcVectorsEnqueue(ctx, rs, plan->tcv, vectors, b->offset, b->n, args.state, args.log,
                               plan->log_offset, images + parity * image_set, parity,
                               plan->tl.count == 0));
      replay_done[parity] = syncEvent(ctx);
      MSQ_TRY(cudaCheck(ctx, cudaEventRecord(replay_done[parity], rs), "event record"));
    }
  }
  // Large matrices: the grid kernels on the context's stream, overlapping the
  // batched sweeps still running on the internal streams.
  for (const int gi : plan->grid_ids) {
    int sweeps = 0;
    double ratio = 0.0, norm2 = 0.0;
    MSQ_TRY(gridJacobiSolve(ctx, matrices + b->host_offset[gi], vectors + b->host_offset[gi],
                            eigenvalues + b->host_eig_offset[gi], b->host_n[gi],
                            tols_host ? tols_host[gi] : tolerance, max_sweeps,
                            &sweeps, &ratio, &norm2, keep_vectors));
    gridStateKernel<<<1, 1, 0, ctx->stream>>>(args.state + gi, sweeps, ratio, norm2);
    MSQ_TRY(launched(ctx, "jacobi grid state"));
  }
  for (int i = 0; i < sweep_streams; ++i) MSQ_TRY(streamWait(ctx, ctx->stream, ss[i]));
  MSQ_TRY(streamWait(ctx, ctx->stream, rs));
  if (sweeps_done != nullptr || off_ratio != nullptr) {
    jacobiReportKernel<<<gridFor(b->count, 256), 256, 0, ctx->stream>>>(args.state, b->count,
                                                                       sweeps_done, off_ratio);
    MSQ_TRY(launched(ctx, "jacobi report"));
  }
  return MSQ_OK;
  };
  const int status = body();
  if (!graphable) return status;
  ctx->stream = caller;
  cudaGraph_t graph = nullptr;
  const cudaError_t end = cudaStreamEndCapture(capture, &graph);
  if (status != MSQ_OK) {
    if (graph != nullptr) cudaGraphDestroy(graph);
    return status;
  }
  MSQ_TRY(cudaCheck(ctx, end, "jacobi capture end"));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  MSQ_TRY(cudaCheck(ctx, inst, "jacobi graph instantiate"));
  const uint64_t captured = ctx->launches - launches0;
  ctx->launches = launches0;
  if (ctx->jacobi_graphs.size() >= 8) {
    cudaGraphExecDestroy(ctx->jacobi_graphs.front().exec);
    ctx->jacobi_graphs.erase(ctx->jacobi_graphs.begin());
  }
  ctx->jacobi_graphs.push_back({key, exec, captured});
  MSQ_TRY(cudaCheck(ctx, cudaGraphLaunch(exec, ctx->stream), "jacobi graph launch"));
  ++ctx->graph_launches;
  ctx->launches += captured;
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
        const int c = t.cands[i];
        if (t.ms[i] > 0.0) {
          std::snprintf(buf, sizeof(buf), " %d%s=%.4fms", c < 0 ? -c : c, c < 0 ? "(split)" : "", t.ms[i]);
        } else {
          std::snprintf(buf, sizeof(buf), " %d%s=?", c < 0 ? -c : c, c < 0 ? "(split)" : "");
        }
        text += buf;
      }
      if (t.best >= 0) {
        const int c = t.cands[t.best];
        text += " -> " + std::to_string(c < 0 ? -c : c) + (c < 0 ? "(split)\n" : "\n");
      } else {
        text += " -> untuned\n";
      }
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

extern "C" int msq_jacobi_route(const int32_t *n, int count, int mode, int32_t *grid) {
  if (n == nullptr || grid == nullptr || count < 0 || mode < MSQ_VECTORS_REPLAY ||
      mode > MSQ_VECTORS_TENSOR_A)
    return MSQ_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < count; ++i)
    if (n[i] < 1) return MSQ_ERR_INVALID_ARGUMENT;
  const std::vector<char> routed = routeToGrid(n, count, mode);
  for (int i = 0; i < count; ++i) grid[i] = routed[i];
  return MSQ_OK;
}

extern "C" int msq_jacobi_batched(msq_ctx *ctx, float *matrices, float *vectors,
                                  float *eigenvalues, const int32_t *n,
                                  const int64_t *offset, int count,
                                  double tolerance, int max_sweeps,
                                  int32_t *sweeps_done, float *off_ratio) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
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
                       max_sweeps, sweeps_done, off_ratio, false, nullptr, nullptr, false);
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
  int status[1];  // bounded-wait status word of the sweep kernel
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
// The entries are atomic and the one-time set-up is serialised, so two host
// threads making their first call on one device at once are safe.
std::atomic<NoAllocScratch *> g_noalloc_address[64] = {};
std::mutex g_noalloc_setup_mutex;

// Resets what must start at zero (the sweep state and the kernels' status
// word) and writes the one-matrix layout tables; the tiles and the log are
// fully written before being read.
__global__ void noAllocSetupKernel(NoAllocScratch *s, int n) {
  const int t = threadIdx.x;
  if (t == 0) {
    s->state[0] = JacobiState{};
    s->status[0] = 0;
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

// Writes the call's report and makes a bounded-wait expiry visible: with the
// status word set, the eigenvalues become NaN, sweeps_done -1 and off_ratio
// NaN, so a caller sees the failure even with NULL report pointers and
// without a host synchronisation.
__global__ void noAllocReportKernel(const NoAllocScratch *s, float *eigenvalues, int n,
                                    int32_t *sweeps_done, float *off_ratio) {
  const bool failed = s->status[0] != 0;
  if (failed) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) eigenvalues[i] = __int_as_float(0x7fc00000);
  }
  if (threadIdx.x == 0) {
    if (sweeps_done != nullptr) sweeps_done[0] = failed ? -1 : s->state[0].sweeps;
    if (off_ratio != nullptr) {
      off_ratio[0] = failed ? __int_as_float(0x7fc00000) : static_cast<float>(s->state[0].off_ratio);
    }
  }
}

// Every order the entry point accepts keeps its tiles in shared memory.
constexpr size_t sharedTileSweepBytes(int n) {
  size_t q_off = 0, tile_off = 0;
  return sweepSmemLayout(n, true, &q_off, &tile_off);
}
static_assert(sharedTileSweepBytes(kNoAllocOrder) <= kSweepSmemLimit,
              "orders up to MSQ_NOALLOC_MAX_ORDER use the shared-tile sweep");

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
  // An error already pending on this thread belongs to the caller's earlier
  // work: leave it in place for the caller and launch nothing.
  if (cudaPeekAtLastError() != cudaSuccess) return MSQ_ERR_CUDA;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MSQ_ERR_CUDA;
  NoAllocScratch *s = g_noalloc_address[device].load(std::memory_order_acquire);
  if (s == nullptr) {
    // One-time set-up for this device (so the first call on a device should
    // come before any stream capture).
    std::lock_guard<std::mutex> lock(g_noalloc_setup_mutex);
    s = g_noalloc_address[device].load(std::memory_order_acquire);
    if (s == nullptr) {
      void *address = nullptr;
      if (cudaGetSymbolAddress(&address, g_noalloc_scratch) != cudaSuccess || address == nullptr) {
        return MSQ_ERR_CUDA;
      }
      if (setKernelAttributes() != MSQ_OK) return MSQ_ERR_CUDA;
      s = static_cast<NoAllocScratch *>(address);
      g_noalloc_address[device].store(s, std::memory_order_release);
    }
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
  args.status = s->status;
  args.wait_test = waitTestMode() == kWaitTestFlag;
  size_t q_off, tile_off;
  const size_t sweep_smem = sweepSmemLayout(n, true, &q_off, &tile_off);
  const int rows = (n + kNoAllocRowsPerCta - 1) / kNoAllocRowsPerCta;
  VArgs vargs{vectors, s->a_offset, s->log_offset, s->n, s->log, s->state,
              s->work_matrix, s->work_row, kNoAllocRowsPerCta};
  const size_t v_smem = replaySmemBytes(n, kNoAllocRowsPerCta);
  identityKernel<<<dim3(64, 1), 256, 0, st>>>(vectors, s->a_offset, s->n, 1);
  for (int launch = 0; launch <= max_sweeps; ++launch) {
    args.first = launch == 0;
    jacobiSweepKernel<true><<<1, threadsFor(n), sweep_smem, st>>>(args);
    if (launch < max_sweeps) jacobiReplayKernel<<<rows, kReplayThreads, v_smem, st>>>(vargs);
  }
  noAllocReportKernel<<<1, 256, 0, st>>>(s, eigenvalues, n, sweeps_done, off_ratio);
  // nothing was pending on entry, so an error here comes from these launches
  return cudaGetLastError() == cudaSuccess ? MSQ_OK : MSQ_ERR_CUDA;
}
