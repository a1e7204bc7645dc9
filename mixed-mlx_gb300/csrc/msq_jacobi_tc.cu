// Eigenvectors of the batched Jacobi on the tensor cores.
//
// The reference accumulates V <- V J after every round on the CUDA-core
// equivalent of its GPU (jacobi_similarity_vectors_f32,
// metal_mixed_sqrt.metal:1380-1390); the round-robin order it uses
// (makeJacobiSchedule, src/metal_solver.cpp:50-79) mixes every column with
// every other within a few rounds, so no product of consecutive rounds is
// cheaper to apply than the rounds themselves.  For orders 257..512 the
// solver can instead pair blocks in two levels (twoLevelSchedule): the
// rotations of each group of rounds stay inside fixed 64-index super-pairs,
// so the group's product is block diagonal with 64x64 blocks Z, and
// V <- V Z is a GEMM.  Two kernels per sweep:
//  * tcvFormKernel (one CTA per matrix and stage, one warp per super-pair)
//    replays the stage's logged 8x8 rotations onto a 64x64 identity in
//    shared memory (the same ordered FP32 chains as the FP32 replay; each
//    round's rotations staged by cp.async while the previous round runs) and
//    writes Z^T split into BF16 hi + lo, in the SWIZZLE_128B K-major layout
//    of a tcgen05 B operand: one 16 KB image per super-pair;
//  * tcvApplyKernel (one CTA per 128 rows of V) keeps those rows in TMEM
//    (128 lanes x 512 FP32 columns) for the whole sweep.  For every stage
//    and super-pair, warps 0-7 read the pair's 64 columns from TMEM, split
//    them into BF16 hi + lo operand tiles in shared memory, and one thread
//    issues tcgen05.mma (kind::f16, M = 128, N = 32, K = 64) writing the
//    product back into the same TMEM columns: three products per half
//    (hi Z_hi + lo Z_hi + hi Z_lo, FP32 accumulation).  A warp bulk-copies
//    the rotation images ahead through an mbarrier ring.
// Each product carries a relative error of about 2^-16 (the dropped lo x lo
// term and the BF16 lo rounding), so V stays orthonormal to about 1e-5 per
// stage: the solver uses this path only for plans whose basis is then
// quantized to BF16 or fewer bits.  Every mbarrier wait is bounded.
#include "msq_jacobi_device.cuh"
#include "msq_jacobi_tc.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <map>

namespace msq {

void twoLevelSchedule(int nb, std::vector<int32_t> &out) {
  const int supers = twoLevelSupers(nb), rounds = twoLevelRounds(nb);
  auto size = [&](int S) { return std::max(0, std::min(kSuperBlock, nb - kSuperBlock * S)); };
  out.assign(static_cast<size_t>(rounds) * nb, 0);
  std::vector<char> used(nb);
  for (int r = 0; r < rounds; ++r) {
    std::fill(used.begin(), used.end(), 0);
    int32_t *row = out.data() + static_cast<size_t>(r) * nb;
    int k = 0;
    auto add = [&](int I, int J) {
      row[2 * k] = I;
      row[2 * k + 1] = J;
      used[I] = used[J] = 1;
      ++k;
    };
    if (r < kSuperBlock - 1) {
      for (int S = 0; kSuperBlock * S < nb; ++S)
        for (int x = 0; x < kSuperBlock / 2; ++x) {
          int a, b;
          rrPair(x, r, kSuperBlock, a, b);
          if (b < size(S)) add(kSuperBlock * S + a, kSuperBlock * S + b);
        }
    } else {
      const int o = (r - (kSuperBlock - 1)) / kSuperBlock, t = (r - (kSuperBlock - 1)) % kSuperBlock;
      for (int x = 0; x < supers / 2; ++x) {
        int Ps, Qs;
        rrPair(x, o, supers, Ps, Qs);
        for (int i = 0; i < kSuperBlock; ++i) {
          const int j = (i + t) % kSuperBlock;
          if (i < size(Ps) && j < size(Qs)) add(kSuperBlock * Ps + i, kSuperBlock * Qs + j);
        }
      }
    }
    int idle = -1;
    for (int blk = 0; blk < nb; ++blk) {
      if (used[blk]) continue;
      if (idle < 0) {
        idle = blk;
        continue;
      }
      row[2 * k] = idle;
      row[2 * k + 1] = -1 - blk;
      ++k;
      idle = -1;
    }
  }
}

namespace {

constexpr int kFormThreads = 256;    // one warp per super-pair (at most 8)
constexpr int kFormLd = 68;          // row stride of a 64x64 Z block in shared memory
constexpr int kApplyThreads = 320;   // warps 0-7 rows (two per TMEM lane quarter), 8 MMA, 9 copies
constexpr int kRowWarps = 8;
constexpr int kApplyRows = 128;
constexpr uint32_t kApplyTmemCols = 512;
constexpr int kOperandBytes = 16384; // one BF16 term of a 128 x 64 operand
constexpr int kImageStages = 4;
constexpr int kOperandBuffers = 3;
constexpr long long kApplyWaitLimit = 1ll << 26;
// eight 64x64 blocks and two rounds of rotations (at most 64 pairs)
constexpr size_t kFormSmem =
    (static_cast<size_t>(8) * 64 * kFormLd + 2 * static_cast<size_t>(64) * kQF) * sizeof(float);
// A operands (kOperandBuffers x hi, lo), image ring, barriers; 1 KB alignment slack
constexpr size_t kApplySmem =
    kOperandBuffers * 2 * kOperandBytes + kImageStages * kRotationImageBytes + 1024 + 256;

// Stage stage of matrix with `supers` super-blocks (`real` of them
// non-empty): its super-pair x and whether the stage changes it (after the
// first stage a pair with the empty super-block has Z = I).
__host__ __device__ __forceinline__ bool stagePair(int stage, int x, int supers, int real, int &Ps,
                                                   int &Qs) {
  rrPair(x, stage, supers, Ps, Qs);
  return stage == 0 || Qs < real;
}

struct FormArgs {
  const float *log;
  const int64_t *log_offset;
  const int32_t *n;
  const JacobiState *state;
  const int2 *work;
  const int32_t *prog;
  const int32_t *prog_off;
  const int64_t *image_off;
  uint8_t *images;
  int parity;
};

// x = hi + lo with hi = bf16(x), lo = bf16(x - hi), for two consecutive
// elements packed as BF16x2 words (element e0 in the low half).
__device__ __forceinline__ void splitPair(float e0, float e1, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(e0, e1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(e0 - hf.x, e1 - hf.y);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

__global__ void __launch_bounds__(kFormThreads) tcvFormKernel(FormArgs args) {
  extern __shared__ __align__(16) float zs[];
  const int2 w = args.work[blockIdx.x];
  const int mi = w.x, stage = w.y;
  if (!args.state[mi].logged[args.parity]) return;  // uniform: before any barrier
  const int n = args.n[mi], m = padded8(n), nb = m / 4, P = nb / 2;
  const int supers = twoLevelSupers(nb), pairs = supers / 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool owner = warp < pairs;  // warp x forms the block of super-pair x
  float *z = zs + warp * 64 * kFormLd;
  float *qbuf = zs + 8 * 64 * kFormLd;  // [2][P][64]: a round's rotations, double-buffered
  if (owner) {
    for (int i = lane; i < 64; i += 32)
      for (int c = 0; c < 64; c += 4)
        *reinterpret_cast<float4 *>(z + i * kFormLd + c) =
            make_float4(i == c, i == c + 1, i == c + 2, i == c + 3);
  }
  const float *log = args.log + args.log_offset[mi];
  const int32_t *prog = args.prog + args.prog_off[mi];
  const int r0 = twoLevelStageFirst(stage), rounds = twoLevelStageRounds(stage);
  const int chunks = P * kQF / 4;
  for (int x = threadIdx.x; x < chunks; x += blockDim.x)
    copyAsync16(qbuf + 4 * x, log + static_cast<int64_t>(r0) * P * kQF + 4 * x);
  copyAsyncCommit();
  for (int t = 0; t < rounds; ++t) {
    const int r = r0 + t;
    copyAsyncWaitAll();
    __syncthreads();  // round t's rotations landed; every warp is done with round t - 1
    if (t + 1 < rounds) {
      float *next = qbuf + ((t + 1) & 1) * P * kQF;
      const float *src = log + static_cast<int64_t>(r + 1) * P * kQF;
      for (int x = threadIdx.x; x < chunks; x += blockDim.x) copyAsync16(next + 4 * x, src + 4 * x);
      copyAsyncCommit();
    }
    if (!owner) continue;
    const float *qs = qbuf + (t & 1) * P * kQF;
    const int mine = lane < 8 ? prog[(r * pairs + warp) * 8 + lane] : -1;
    for (int e = 0; e < 8; ++e) {
      const int code = __shfl_sync(0xffffffffu, mine, e);
      if (code < 0) break;
      const int k = code & 255, la = (code >> 8) & 255, lb = code >> 16;
      const float4 *q4 = reinterpret_cast<const float4 *>(qs + k * kQF);
      float q[8][8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 lo = q4[2 * j], hi = q4[2 * j + 1];
        q[j][0] = lo.x; q[j][1] = lo.y; q[j][2] = lo.z; q[j][3] = lo.w;
        q[j][4] = hi.x; q[j][5] = hi.y; q[j][6] = hi.z; q[j][7] = hi.w;
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float *row = z + (lane + 32 * h) * kFormLd;
        const float4 a = *reinterpret_cast<const float4 *>(row + 4 * la);
        const float4 b = *reinterpret_cast<const float4 *>(row + 4 * lb);
        const float x[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        float o[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float acc = 0.0f;
#pragma unroll
          for (int j = 0; j < 8; ++j) acc = fmaf(x[j], q[j][c], acc);
          o[c] = acc;
        }
        *reinterpret_cast<float4 *>(row + 4 * la) = make_float4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<float4 *>(row + 4 * lb) = make_float4(o[4], o[5], o[6], o[7]);
      }
    }
  }
  copyAsyncWaitAll();
  __syncwarp();
  if (!owner) return;
  // B operand rows j (output columns), K = the 64 local indices: Z^T, as
  // hi rows 0..63 then lo rows 0..63 (rows 32..63, super-block Q, start
  // 4 KB into each term).
  uint8_t *img = args.images +
                 (args.image_off[mi] + static_cast<int64_t>(stage) * pairs + warp) * kRotationImageBytes;
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    const int j = lane + 32 * h;
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int p = 0; p < 4; ++p)
        splitPair(z[(8 * c + 2 * p) * kFormLd + j], z[(8 * c + 2 * p + 1) * kFormLd + j], hi[p], lo[p]);
      const uint32_t at = swizzle128(j, c);
      *reinterpret_cast<uint4 *>(img + at) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4 *>(img + kImageTermBytes + at) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
  }
}

struct ApplyArgs {
  float *v;
  const int64_t *a_offset;
  const int32_t *n;
  const JacobiState *state;
  const int2 *work;
  const int64_t *image_off;
  const uint8_t *images;
  int parity;
  int *status;
};

// Bounded wait: false (status word set, abort flag raised) if the phase
// never completes, or once another role has aborted.
__device__ __forceinline__ bool applyWait(uint32_t bar, uint32_t parity, int *status,
                                          volatile int *abort_flag) {
  for (long long i = 0; i < kApplyWaitLimit; ++i) {
    if (mbarTryWait(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  atomicExch(status, kStatusMbarrierTimeout);
  *abort_flag = 1;
  return false;
}

__global__ void __launch_bounds__(kApplyThreads, 1) tcvApplyKernel(ApplyArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int2 w = args.work[blockIdx.x];
  const int mi = w.x, r0 = w.y;
  if (!args.state[mi].logged[args.parity]) return;  // uniform: before any barrier
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char *ops = base;                               // [buffers][hi, lo][16 KB]
  unsigned char *ring = base + kOperandBuffers * 2 * kOperandBytes;  // [kImageStages][16 KB]
  uint64_t *bars = reinterpret_cast<uint64_t *>(ring + kImageStages * kRotationImageBytes);
  uint64_t *a_full = bars, *a_empty = bars + kOperandBuffers;
  uint64_t *z_full = bars + 2 * kOperandBuffers, *z_empty = z_full + kImageStages;
  uint64_t *stage_done = z_empty + kImageStages;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(stage_done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int n = args.n[mi], m = padded8(n), nb = m / 4;
  const int supers = twoLevelSupers(nb), pairs = supers / 2, stages = supers - 1;
  const int real = (nb + kSuperBlock - 1) / kSuperBlock;

  if (threadIdx.x == 0) {
    for (int b = 0; b < kOperandBuffers; ++b) {
      mbarInit(smemAddr(&a_full[b]), 32 * kRowWarps);
      mbarInit(smemAddr(&a_empty[b]), 1);
    }
    for (int s = 0; s < kImageStages; ++s) {
      mbarInit(smemAddr(&z_full[s]), 1);
      mbarInit(smemAddr(&z_empty[s]), 1);
    }
    mbarInit(smemAddr(stage_done), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kRowWarps) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smemAddr(tmem_slot)),
                 "r"(kApplyTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  const uint8_t *images = args.images + args.image_off[mi] * kRotationImageBytes;

  if (warp == kRowWarps + 1) {
    if (lane == 0) {
      int zi = 0;
      for (int s = 0; s < stages && !*abort_flag; ++s)
        for (int x = 0; x < pairs; ++x) {
          int Ps, Qs;
          if (!stagePair(s, x, supers, real, Ps, Qs)) continue;
          const int slot = zi % kImageStages;
          if (zi >= kImageStages &&
              !applyWait(smemAddr(&z_empty[slot]), ((zi / kImageStages) - 1) & 1, args.status,
                         abort_flag))
            break;
          const uint32_t bar = smemAddr(&z_full[slot]);
          mbarArriveExpectTx(bar, static_cast<uint32_t>(kRotationImageBytes));
          bulkLoad(smemAddr(ring + slot * kRotationImageBytes),
                   images + (static_cast<int64_t>(s) * pairs + x) * kRotationImageBytes,
                   static_cast<uint32_t>(kRotationImageBytes), bar);
          ++zi;
        }
    }
  } else if (warp == kRowWarps) {
    if (lane == 0) {
      constexpr uint32_t idesc = instrDescBf16(128, 32);
      int it = 0, zi = 0;
      for (int s = 0; s < stages && !*abort_flag; ++s) {
        int last = -1;
        for (int x = 0; x < pairs; ++x) {
          int Ps, Qs;
          if (stagePair(s, x, supers, real, Ps, Qs)) last = x;
        }
        for (int x = 0; x < pairs; ++x) {
          int Ps, Qs;
          if (!stagePair(s, x, supers, real, Ps, Qs)) continue;
          const int slot = zi % kImageStages, buf = it % kOperandBuffers;
          if (!applyWait(smemAddr(&z_full[slot]), (zi / kImageStages) & 1, args.status, abort_flag) ||
              !applyWait(smemAddr(&a_full[buf]), (it / kOperandBuffers) & 1, args.status, abort_flag))
            break;
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t a_hi = smemAddr(ops + buf * 2 * kOperandBytes);
          const uint32_t a_lo = a_hi + kOperandBytes;
          const uint32_t zimg = smemAddr(ring + slot * kRotationImageBytes);
#pragma unroll 1
          for (int h = 0; h < 2; ++h) {
            const int S = h ? Qs : Ps;
            if (S >= real) continue;
            const uint32_t d = tmem + 32 * S;
            const uint64_t ah = smemDesc(a_hi), al = smemDesc(a_lo);
            const uint64_t zh = smemDesc(zimg + h * 4096);
            const uint64_t zl = smemDesc(zimg + kImageTermBytes + h * 4096);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              mmaBf16(d, ah + 2 * kk, zh + 2 * kk, idesc, kk > 0);
              mmaBf16(d, al + 2 * kk, zh + 2 * kk, idesc, 1);
              mmaBf16(d, ah + 2 * kk, zl + 2 * kk, idesc, 1);
            }
          }
          mmaCommit(smemAddr(&a_empty[buf]));
          mmaCommit(smemAddr(&z_empty[slot]));
          if (x == last) mmaCommit(smemAddr(stage_done));
          ++it;
          ++zi;
        }
      }
    }
  } else {
    // Rows: warps w and w + 4 share TMEM lane quarter w (rows 32w .. 32w + 31
    // of the chunk); warp w handles the P half of every super-pair (operand
    // chunks 0-3), warp w + 4 the Q half (chunks 4-7).
    const int quarter = warp & 3, half = warp >> 2;
    const int lrow = 32 * quarter + lane;
    const int row = r0 + lrow;
    const uint32_t lanes = tmem + ((32u * quarter) << 16);
    float *V = args.v + args.a_offset[mi];
#pragma unroll 1
    for (int cb = half; cb < real; cb += 2) {
      float vals[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int c = 32 * cb + i;
        vals[i] = row < n && c < n ? V[row + static_cast<int64_t>(c) * n] : 0.0f;
      }
      tmemStore32(lanes + 32 * cb, vals);
    }
    // the other warp of the lane quarter reads columns this warp stored
    asm volatile("tcgen05.fence::before_thread_sync;");
    asm volatile("bar.sync 1, %0;" ::"n"(32 * kRowWarps) : "memory");
    asm volatile("tcgen05.fence::after_thread_sync;");
    int it = 0;
    bool ok = true;
    for (int s = 0; s < stages && ok; ++s) {
      bool first = true;
      for (int x = 0; x < pairs; ++x) {
        int Ps, Qs;
        if (!stagePair(s, x, supers, real, Ps, Qs)) continue;
        const int buf = it % kOperandBuffers;
        if (it >= kOperandBuffers &&
            !applyWait(smemAddr(&a_empty[buf]), ((it / kOperandBuffers) - 1) & 1, args.status,
                       abort_flag)) {
          ok = false;
          break;
        }
        if (first && s > 0 &&
            !applyWait(smemAddr(stage_done), (s - 1) & 1, args.status, abort_flag)) {
          ok = false;
          break;
        }
        first = false;
        asm volatile("tcgen05.fence::after_thread_sync;");
        float f[32];
        const int S = half ? Qs : Ps;
        if (S < real) {
          tmemLoad32(lanes + 32 * S, f);
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) f[i] = 0.0f;
        }
        unsigned char *hi_op = ops + buf * 2 * kOperandBytes;
        unsigned char *lo_op = hi_op + kOperandBytes;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint32_t hv[4], lv[4];
#pragma unroll
          for (int p = 0; p < 4; ++p) splitPair(f[8 * c + 2 * p], f[8 * c + 2 * p + 1], hv[p], lv[p]);
          const uint32_t at = swizzle128(lrow, 4 * half + c);
          *reinterpret_cast<uint4 *>(hi_op + at) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
          *reinterpret_cast<uint4 *>(lo_op + at) = make_uint4(lv[0], lv[1], lv[2], lv[3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbarArrive(smemAddr(&a_full[buf]));
        ++it;
      }
    }
    if (ok && applyWait(smemAddr(stage_done), (stages - 1) & 1, args.status, abort_flag)) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
      for (int cb = half; cb < real; cb += 2) {
        float vals[32];
        tmemLoad32(lanes + 32 * cb, vals);
        if (row < n) {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int c = 32 * cb + i;
            if (c < n) V[row + static_cast<int64_t>(c) * n] = vals[i];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == kRowWarps) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kApplyTmemCols));
  }
}

// ---------------------------------------------------------------------------
// Two-level Jacobi with the off-diagonal work on the tensor cores.
//
// With the two-level pairing, the rounds of a stage rotate only inside the
// stage's 64-index super-pairs.  So each stage can run its rounds on the
// 64x64 diagonal blocks alone (tlInnerKernel: the quad-pivot sweep and
// super-tile updates of the batched kernel on 16 local blocks, with the
// stage rotation Z of the block accumulated in shared memory as it goes),
// and bring the rest of A up to date once per stage: A' = Z^T A Z with
// block-diagonal Z, as two tcgen05 passes B = A Z and A' = B^T Z (A' is
// symmetric; tlPassKernel, split-BF16 operands, FP32 accumulation).  The
// second pass takes the diagonal blocks from the inner kernel.  The stage
// rotations are the operand images the V update applies after the sweep.

constexpr int kInnerThreads = 128;
constexpr int kLocalBlocks = 16;
constexpr int kLocalTiles = kLocalBlocks * (kLocalBlocks + 1) / 2;
constexpr int kPassRows = 128;
constexpr int kPassThreads = 160;        // warps 0-3 rows, warp 4 TMEM + MMA + copies
constexpr uint32_t kPassTmemCols = 128;  // two 64-column accumulators
constexpr int kStageLd = 65;

struct CheckArgs {
  float *a;
  const int64_t *a_offset;
  const int32_t *n;
  const int64_t *eig_offset;
  float *eigenvalues;
  JacobiState *state;
  const int32_t *ids;
  double tol;
  const double *tols;  // per matrix (null: tol for all)
  int max_sweeps;
  int first;
  int parity;
};

// Convergence check before a sweep (and, on the first launch, the symmetrised
// input and ||A||_F^2): the state and the eigenvalues of a converged matrix.
__global__ void __launch_bounds__(256) tlCheckKernel(CheckArgs args) {
  __shared__ double red[32];
  const int mi = args.ids[blockIdx.x];
  JacobiState &st = args.state[mi];
  const JacobiState s0 = st;
  if (!args.first && s0.done) {
    if (threadIdx.x == 0) st.logged[args.parity] = 0;
    return;
  }
  const int n = args.n[mi];
  float *A = args.a + args.a_offset[mi];
  if (args.first) {
    // A <- (A + A^T) / 2 (working_from_symmetric_f32, metal_mixed_sqrt.metal:1349-1350)
    const int64_t pairs = static_cast<int64_t>(n) * (n - 1) / 2;
    for (int64_t q = threadIdx.x; q < pairs; q += blockDim.x) {
      int j = static_cast<int>((1.0 + sqrt(1.0 + 8.0 * static_cast<double>(q))) / 2.0);
      while (static_cast<int64_t>(j) * (j - 1) / 2 > q) --j;
      while (static_cast<int64_t>(j + 1) * j / 2 <= q) ++j;
      const int i = static_cast<int>(q - static_cast<int64_t>(j) * (j - 1) / 2);
      const int64_t ij = i + static_cast<int64_t>(j) * n, ji = j + static_cast<int64_t>(i) * n;
      const float v = 0.5f * (A[ij] + A[ji]);
      A[ij] = v;
      A[ji] = v;
    }
    __syncthreads();
  }
  double off2 = 0.0, diag2 = 0.0;
  const int64_t nn = static_cast<int64_t>(n) * n;
  for (int64_t q = threadIdx.x; q < nn; q += blockDim.x) {
    const double v = A[q];
    if (q % (n + 1) == 0) diag2 += v * v;
    else off2 += v * v;
  }
  off2 = blockReduceSum(off2, red);
  diag2 = blockReduceSum(diag2, red);
  const double norm2 = args.first ? off2 + diag2 : s0.norm2;
  const int sweeps = args.first ? 0 : s0.sweeps;
  const double ratio = norm2 > 0.0 ? sqrt(off2 / norm2) : 0.0;
  const bool stop = ratio <= (args.tols ? args.tols[mi] : args.tol) || sweeps >= args.max_sweeps;
  if (stop) {
    float *eig = args.eigenvalues + args.eig_offset[mi];
    for (int k = threadIdx.x; k < n; k += blockDim.x) eig[k] = A[k + static_cast<int64_t>(k) * n];
  }
  if (threadIdx.x == 0) {
    st.norm2 = norm2;
    st.off_ratio = ratio;
    st.sweeps = stop ? sweeps : sweeps + 1;
    st.done = stop ? 1 : 0;
    st.logged[args.parity] = stop ? 0 : 1;
  }
}

struct InnerArgs {
  const float *a;
  const int64_t *a_offset;
  const int32_t *n;
  const JacobiState *state;
  const int2 *work;          // (matrix, super-pair) of this stage
  const int32_t *prog;
  const int32_t *prog_off;
  const int64_t *image_off;
  uint8_t *images;
  float *diag;               // rotated 64x64 diagonal blocks (row-major, local order)
  const int64_t *diag_off;   // per matrix: first block (one per super-pair)
  int stage;
};

// Local index li (0..63) of super-pair (P, Q) -> global index, -1 outside A.
__device__ __forceinline__ int localToGlobal(int li, int Ps, int Qs, int n) {
  const int g = li < 32 ? 32 * Ps + li : 32 * Qs + li - 32;
  return g < n ? g : -1;
}

__global__ void __launch_bounds__(kInnerThreads, 4) tlInnerKernel(InnerArgs args) {
  __shared__ __align__(16) float tiles[kLocalTiles * kTileF];
  __shared__ __align__(16) float z[64 * kFormLd];
  __shared__ __align__(16) float qs[8 * kQS];
  __shared__ int tri[kLocalBlocks + 1];
  // local pairs of every round of the stage: the rotating ones, then the
  // other local blocks paired in order with the identity
  __shared__ int pairs_i[2 * kSuperBlock - 1][8], pairs_j[2 * kSuperBlock - 1][8];
  __shared__ int pairs_on[2 * kSuperBlock - 1][8];
  const int2 w = args.work[blockIdx.x];
  const int mi = w.x, x = w.y;
  if (args.state[mi].done) return;
  const int n = args.n[mi], m = padded8(n), nb = m / 4;
  const int supers = twoLevelSupers(nb), pairs = supers / 2;
  int Ps, Qs;
  rrPair(x, args.stage, supers, Ps, Qs);
  const float *A = args.a + args.a_offset[mi];
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int k = tid; k <= kLocalBlocks; k += blockDim.x) tri[k] = k * (k + 1) / 2;
  for (int i = tid; i < 64; i += blockDim.x)
    for (int c = 0; c < 64; c += 4)
      *reinterpret_cast<float4 *>(z + i * kFormLd + c) =
          make_float4(i == c, i == c + 1, i == c + 2, i == c + 3);
  __syncthreads();
  // upper triangle of the 64x64 block: column lj, rows li <= (lj | 3);
  // consecutive threads read consecutive rows of a column
  for (int q = tid; q < 64 * 64; q += blockDim.x) {
    const int lj = q >> 6, li = q & 63, I = li >> 2, J = lj >> 2;
    if (I > J) continue;
    const int gi = localToGlobal(li, Ps, Qs, n), gj = localToGlobal(lj, Ps, Qs, n);
    tiles[tileElement(tri[J] + I, li & 3, lj & 3)] =
        gi >= 0 && gj >= 0 ? A[gi + static_cast<int64_t>(gj) * n] : 0.0f;
  }
  const int32_t *prog = args.prog + args.prog_off[mi];
  const int r0 = twoLevelStageFirst(args.stage), rounds = twoLevelStageRounds(args.stage);
  if (tid < rounds) {
    const int t = tid;
    const int32_t *entry = prog + ((r0 + t) * pairs + x) * 8;
    unsigned used = 0;
    int cnt = 0;
    for (int e = 0; e < 8; ++e) {
      const int code = entry[e];
      if (code < 0) break;
      const int la = (code >> 8) & 255, lb = code >> 16;
      pairs_i[t][cnt] = la;
      pairs_j[t][cnt] = lb;
      pairs_on[t][cnt] = 1;
      used |= (1u << la) | (1u << lb);
      ++cnt;
    }
    int idle = -1;
    for (int L = 0; L < kLocalBlocks; ++L) {
      if (used & (1u << L)) continue;
      if (idle < 0) {
        idle = L;
        continue;
      }
      pairs_i[t][cnt] = idle;
      pairs_j[t][cnt] = L;
      pairs_on[t][cnt] = 0;
      ++cnt;
      idle = -1;
    }
  }
  __syncthreads();
  for (int t = 0; t < rounds; ++t) {
    const int *pair_i = pairs_i[t], *pair_j = pairs_j[t], *pair_on = pairs_on[t];
    if (warp == 0) {
      // pivots: quad k of warp 0 sweeps local pair k
      const int k = tid >> 2, t4 = tid & 3;
      const bool active = pair_on[k] != 0;
      const int I = pair_i[k], J = pair_j[k];
      float ra[8], rb[8];
      int tII = 0, tIJ = 0, tJJ = 0;
      if (active) {
        tII = tileIndex(tri, I, I);
        tIJ = tileIndex(tri, I, J);
        tJJ = tileIndex(tri, J, J);
        const float4 *sII = reinterpret_cast<const float4 *>(tiles + tII * kTileF);
        const float4 *sIJ = reinterpret_cast<const float4 *>(tiles + tIJ * kTileF);
        const float4 *sJJ = reinterpret_cast<const float4 *>(tiles + tJJ * kTileF);
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
        float4 *sII = reinterpret_cast<float4 *>(tiles + tII * kTileF);
        float4 *sIJ = reinterpret_cast<float4 *>(tiles + tIJ * kTileF);
        float4 *sJJ = reinterpret_cast<float4 *>(tiles + tJJ * kTileF);
        sII[t4 ^ (tII & 3)] = make_float4(ra[0], ra[1], ra[2], ra[3]);
        sIJ[t4 ^ (tIJ & 3)] = make_float4(ra[4], ra[5], ra[6], ra[7]);
        sJJ[t4 ^ (tJJ & 3)] = make_float4(rb[4], rb[5], rb[6], rb[7]);
      } else {
        float4 *q4 = reinterpret_cast<float4 *>(qs + k * kQS);
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          const int row = 2 * t4 + y;
          q4[2 * row] = make_float4(row == 0, row == 1, row == 2, row == 3);
          q4[2 * row + 1] = make_float4(row == 4, row == 5, row == 6, row == 7);
        }
      }
    }
    __syncthreads();
    if (warp < 3) {
      // off-pivot super-tiles of the local pairs, two lanes each (warp-uniform)
      constexpr int kItems = ((8 + 1) / 2) * (8 + 1);
      const int h = tid & 1;
      int k = 0, l = 0;
      const bool valid = tid < 2 * kItems && foldedBlock(tid >> 1, 8, k, l) && k != l;
      if (!valid) k = l = 0;
      superTileHalf(tiles, SharedTri{tri}, reinterpret_cast<const float4 *>(qs + k * kQS),
                    reinterpret_cast<const float4 *>(qs + l * kQS), pair_i[k], pair_j[k],
                    pair_i[l], pair_j[l], h, valid);
    }
    {
      // Z <- Z Q of the rotating pairs (row = tid mod 64, pairs of one parity)
      const int row = tid & 63;
      float *zr = z + row * kFormLd;
      for (int pp = tid >> 6; pp < 8; pp += 2) {
        if (!pair_on[pp]) continue;
        const int I = pair_i[pp], J = pair_j[pp];
        const float4 *q4 = reinterpret_cast<const float4 *>(qs + pp * kQS);
        const float4 a = *reinterpret_cast<const float4 *>(zr + 4 * I);
        const float4 b = *reinterpret_cast<const float4 *>(zr + 4 * J);
        const float xv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        float o[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 lo = q4[2 * j], hi = q4[2 * j + 1];
          o[0] = fmaf(xv[j], lo.x, o[0]); o[1] = fmaf(xv[j], lo.y, o[1]);
          o[2] = fmaf(xv[j], lo.z, o[2]); o[3] = fmaf(xv[j], lo.w, o[3]);
          o[4] = fmaf(xv[j], hi.x, o[4]); o[5] = fmaf(xv[j], hi.y, o[5]);
          o[6] = fmaf(xv[j], hi.z, o[6]); o[7] = fmaf(xv[j], hi.w, o[7]);
        }
        *reinterpret_cast<float4 *>(zr + 4 * I) = make_float4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<float4 *>(zr + 4 * J) = make_float4(o[4], o[5], o[6], o[7]);
      }
    }
    __syncthreads();
  }
  // the rotated diagonal block, row-major in local order
  float *D = args.diag + (args.diag_off[mi] + x) * 4096;
  for (int idx = tid; idx < 4096; idx += blockDim.x) {
    const int li = idx >> 6, lj = idx & 63, I = li >> 2, J = lj >> 2;
    D[idx] = I <= J ? tiles[tileElement(tri[J] + I, li & 3, lj & 3)]
                    : tiles[tileElement(tri[I] + J, lj & 3, li & 3)];
  }
  // Z^T split into the tcgen05 operand image (rows j, K = local index k)
  uint8_t *img = args.images +
                 (args.image_off[mi] + static_cast<int64_t>(args.stage) * pairs + x) * kRotationImageBytes;
  const int j = tid & 63;
  for (int c = tid >> 6; c < 8; c += 2) {
    uint32_t hv[4], lv[4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
      splitPair(z[(8 * c + 2 * p) * kFormLd + j], z[(8 * c + 2 * p + 1) * kFormLd + j], hv[p], lv[p]);
    const uint32_t at = swizzle128(j, c);
    *reinterpret_cast<uint4 *>(img + at) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
    *reinterpret_cast<uint4 *>(img + kImageTermBytes + at) = make_uint4(lv[0], lv[1], lv[2], lv[3]);
  }
}

struct PassArgs {
  const float *src;
  float *dst;
  const int64_t *a_offset;
  const int32_t *n;
  const JacobiState *state;
  const int2 *work;          // (matrix, first row)
  const int64_t *image_off;
  const uint8_t *images;
  const float *diag;
  const int64_t *diag_off;
  int stage;
  int *status;
};

// One 128-row chunk times the stage's block-diagonal Z, super-pair by
// super-pair, software-pipelined: the row warps split the operand of
// super-pair x into BF16 hi + lo (buffer x mod 2) while the MMA of x - 1
// runs, then drain the accumulator of x - 1 (TMEM, two 64-column buffers);
// a thread of warp 4 issues 12 tcgen05.mma per super-pair (M = 128, N = 64,
// three split products) and another bulk-copies the rotation images.
// Pass 1 (kSecond false): operand rows are rows of A, B = A Z is stored
// row-major through a shared-memory transpose (coalesced), so pass 2 reads
// its operand rows, the columns of B, with coalesced loads: A' = B^T Z,
// with the diagonal blocks taken from the inner kernel.
constexpr int kPassBuffers = 2;
constexpr size_t kPassSmemFirst = kPassBuffers * (2 * kOperandBytes + kRotationImageBytes) +
                                  static_cast<size_t>(kPassRows) * kStageLd * sizeof(float) + 1024 + 256;
constexpr size_t kPassSmemSecond = kPassBuffers * (2 * kOperandBytes + kRotationImageBytes) + 1024 + 256;

template <bool kSecond>
__global__ void __launch_bounds__(kPassThreads, 1) tlPassKernel(PassArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int2 w = args.work[blockIdx.x];
  const int mi = w.x, r0 = w.y;
  if (args.state[mi].done) return;  // uniform: before any barrier
  const int n = args.n[mi], m = padded8(n), nb = m / 4;
  const int supers = twoLevelSupers(nb), pairs = supers / 2;
  if (args.stage >= supers - 1) return;
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char *ops = base;                                            // [2][hi, lo]
  unsigned char *ring = base + kPassBuffers * 2 * kOperandBytes;        // [2] images
  unsigned char *after = ring + kPassBuffers * kRotationImageBytes;
  float *stage = reinterpret_cast<float *>(after);                      // pass 1 only
  uint64_t *bars = reinterpret_cast<uint64_t *>(
      after + (kSecond ? 0 : static_cast<size_t>(kPassRows) * kStageLd * sizeof(float)));
  uint64_t *img_full = bars, *op_full = bars + 2, *d_full = bars + 4, *d_empty = bars + 6;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 8);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < kPassBuffers; ++b) {
      mbarInit(smemAddr(&img_full[b]), 1);
      mbarInit(smemAddr(&op_full[b]), kPassRows);
      mbarInit(smemAddr(&d_full[b]), 1);
      mbarInit(smemAddr(&d_empty[b]), kPassRows);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smemAddr(tmem_slot)),
                 "r"(kPassTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  const float *S = args.src + args.a_offset[mi];
  float *Dst = args.dst + args.a_offset[mi];
  const uint8_t *images = args.images +
                          (args.image_off[mi] + static_cast<int64_t>(args.stage) * pairs) * kRotationImageBytes;

  if (warp == 4) {
    if (lane == 0) {
      // rotation images, two ahead
      for (int x = 0; x < pairs && !*abort_flag; ++x) {
        const int b = x & 1, u = x >> 1;
        if (u >= 1 && !applyWait(smemAddr(&d_full[b]), (u - 1) & 1, args.status, abort_flag)) break;
        mbarArriveExpectTx(smemAddr(&img_full[b]), static_cast<uint32_t>(kRotationImageBytes));
        bulkLoad(smemAddr(ring + b * kRotationImageBytes),
                 images + static_cast<int64_t>(x) * kRotationImageBytes,
                 static_cast<uint32_t>(kRotationImageBytes), smemAddr(&img_full[b]));
      }
    } else if (lane == 1) {
      constexpr uint32_t idesc = instrDescBf16(128, 64);
      for (int x = 0; x < pairs && !*abort_flag; ++x) {
        const int b = x & 1, u = x >> 1;
        if (!applyWait(smemAddr(&img_full[b]), u & 1, args.status, abort_flag) ||
            !applyWait(smemAddr(&op_full[b]), u & 1, args.status, abort_flag) ||
            (u >= 1 && !applyWait(smemAddr(&d_empty[b]), (u - 1) & 1, args.status, abort_flag)))
          break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t hi = smemAddr(ops + b * 2 * kOperandBytes);
        const uint64_t ah = smemDesc(hi), al = smemDesc(hi + kOperandBytes);
        const uint32_t img = smemAddr(ring + b * kRotationImageBytes);
        const uint64_t zh = smemDesc(img), zl = smemDesc(img + kImageTermBytes);
        const uint32_t d = tmem + 64 * b;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          mmaBf16(d, ah + 2 * kk, zh + 2 * kk, idesc, kk > 0);
          mmaBf16(d, al + 2 * kk, zh + 2 * kk, idesc, 1);
          mmaBf16(d, ah + 2 * kk, zl + 2 * kk, idesc, 1);
        }
        mmaCommit(smemAddr(&d_full[b]));
      }
    }
  } else {
    const int row = r0 + tid;  // operand row: a row of A (pass 1) or a column of B (pass 2)
    const float *diag = kSecond ? args.diag + args.diag_off[mi] * 4096 : nullptr;
    bool ok = true;
    for (int x = 0; x <= pairs && ok; ++x) {
      if (x < pairs) {
        // operand of super-pair x (its buffer was freed by the MMA of x - 2,
        // whose completion the drain of x - 2 waited for)
        int Ps, Qs;
        rrPair(x, args.stage, supers, Ps, Qs);
        const int b = x & 1;
        unsigned char *op_hi = ops + b * 2 * kOperandBytes, *op_lo = op_hi + kOperandBytes;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          uint32_t hv[4], lv[4];
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            float e[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const int g = localToGlobal(8 * c + 2 * p + q, Ps, Qs, n);
              // pass 1: A[row, g] (A symmetric: read as A[g, row]... column-major
              // A[row + g n]); pass 2: B[g, row], B row-major: B[row + g n]
              e[q] = row < n && g >= 0 ? S[row + static_cast<int64_t>(g) * n] : 0.0f;
            }
            splitPair(e[0], e[1], hv[p], lv[p]);
          }
          const uint32_t at = swizzle128(tid, c);
          *reinterpret_cast<uint4 *>(op_hi + at) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
          *reinterpret_cast<uint4 *>(op_lo + at) = make_uint4(lv[0], lv[1], lv[2], lv[3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbarArrive(smemAddr(&op_full[b]));
      }
      if (x >= 1) {
        // drain the accumulator of super-pair x - 1
        const int y = x - 1, b = y & 1, u = y >> 1;
        int Ps, Qs;
        rrPair(y, args.stage, supers, Ps, Qs);
        if (!applyWait(smemAddr(&d_full[b]), u & 1, args.status, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        float d[64];
        tmemLoad32(tmem + ((32u * warp) << 16) + 64 * b, d);
        tmemLoad32(tmem + ((32u * warp) << 16) + 64 * b + 32, d + 32);
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbarArrive(smemAddr(&d_empty[b]));
        if (kSecond) {
          if (row < n) {
            const int sb = row >> 5;
            const int local = sb == Ps ? row - 32 * Ps : (sb == Qs ? 32 + row - 32 * Qs : -1);
            const float *drow = local >= 0 ? diag + (static_cast<int64_t>(y) * 64 + local) * 64 : nullptr;
#pragma unroll
            for (int j = 0; j < 64; ++j) {
              const int g = localToGlobal(j, Ps, Qs, n);
              if (g < 0) continue;
              Dst[row + static_cast<int64_t>(g) * n] = drow != nullptr ? drow[j] : d[j];
            }
          }
        } else {
          // B row-major through a transpose in shared memory: a warp writes
          // 32 consecutive columns of one row of B
#pragma unroll
          for (int j = 0; j < 64; ++j) stage[tid * kStageLd + j] = d[j];
          asm volatile("bar.sync 1, 128;" ::: "memory");
          for (int rr = warp; rr < kPassRows; rr += 4) {
            const int R = r0 + rr;
            if (R >= n) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int g = localToGlobal(32 * h + lane, Ps, Qs, n);
              if (g >= 0) Dst[g + static_cast<int64_t>(R) * n] = stage[rr * kStageLd + 32 * h + lane];
            }
          }
          asm volatile("bar.sync 1, 128;" ::: "memory");
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 4) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kPassTmemCols));
  }
}

int setAttributes() {
  static std::atomic<uint64_t> done_mask{0};
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MSQ_ERR_CUDA;
  const uint64_t bit = uint64_t{1} << device;
  if (done_mask.load() & bit) return MSQ_OK;
  if (cudaFuncSetAttribute(tcvFormKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kFormSmem)) != cudaSuccess ||
      cudaFuncSetAttribute(tcvApplyKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kApplySmem)) != cudaSuccess ||
      cudaFuncSetAttribute(tlPassKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kPassSmemFirst)) != cudaSuccess ||
      cudaFuncSetAttribute(tlPassKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kPassSmemSecond)) != cudaSuccess) {
    return MSQ_ERR_CUDA;
  }
  done_mask.fetch_or(bit);
  return MSQ_OK;
}

}  // namespace

void tcVectorsTables(const int *host_n, int count, const std::vector<int> &ids,
                     TcVectorsTables &out) {
  out = TcVectorsTables{};
  out.prog_off.assign(count, -1);
  out.image_off.assign(count, 0);
  std::map<int, int32_t> prog_at;  // block count -> program offset
  std::vector<int32_t> sched;
  for (const int i : ids) {
    const int n = host_n[i], m = padded8(n), nb = m / 4, P = nb / 2;
    const int supers = twoLevelSupers(nb), pairs = supers / 2, stages = supers - 1;
    auto found = prog_at.find(nb);
    if (found == prog_at.end()) {
      const int rounds = twoLevelRounds(nb);
      twoLevelSchedule(nb, sched);
      const int32_t at = static_cast<int32_t>(out.prog.size());
      out.prog.resize(out.prog.size() + static_cast<size_t>(rounds) * pairs * 8, -1);
      for (int r = 0; r < rounds; ++r) {
        const int s = r < twoLevelStageRounds(0) ? 0 : (r - (kSuperBlock - 1)) / kSuperBlock;
        for (int x = 0; x < pairs; ++x) {
          int Ps, Qs;
          rrPair(x, s, supers, Ps, Qs);
          int32_t *entry = out.prog.data() + at + (static_cast<size_t>(r) * pairs + x) * 8;
          int e = 0;
          for (int k = 0; k < P; ++k) {
            const int I = sched[static_cast<size_t>(r) * nb + 2 * k];
            const int J = sched[static_cast<size_t>(r) * nb + 2 * k + 1];
            if (J < 0) continue;
            const int SI = I / kSuperBlock;
            if (SI != Ps && SI != Qs) continue;
            auto local = [&](int blk) {
              return blk / kSuperBlock == Ps ? blk - kSuperBlock * Ps
                                             : kSuperBlock + blk - kSuperBlock * Qs;
            };
            if (e < 8) entry[e++] = k | (local(I) << 8) | (local(J) << 16);
          }
        }
      }
      found = prog_at.emplace(nb, at).first;
    }
    out.prog_off[i] = found->second;
    out.image_off[i] = out.images;
    out.images += static_cast<int64_t>(stages) * pairs;
    for (int s = 0; s < stages; ++s) {
      out.form_work.push_back(i);
      out.form_work.push_back(s);
    }
    for (int r = 0; r < n; r += kApplyRows) {
      out.apply_work.push_back(i);
      out.apply_work.push_back(r);
    }
  }
}

int tcVectorsEnqueue(msq_ctx *ctx, cudaStream_t stream, const TcVectorsDevice &d, float *vectors,
                     const int64_t *a_offset, const int32_t *n, const void *state,
                     const float *log, const int64_t *log_offset, uint8_t *images, int parity,
                     bool form) {
  if (d.apply_items == 0) return MSQ_OK;
  if (setAttributes() != MSQ_OK) return cudaCheck(ctx, cudaGetLastError(), "tensor-core vectors attributes");
  const auto *st = static_cast<const JacobiState *>(state);
  if (form) {
    FormArgs fa{log, log_offset, n, st, d.form_work, d.prog, d.prog_off, d.image_off, images, parity};
    launchBegin(ctx, stream);
    tcvFormKernel<<<d.form_items, kFormThreads, kFormSmem, stream>>>(fa);
    MSQ_TRY(launchedOn(ctx, stream, "jacobi stage rotations"));
  }
  ApplyArgs aa{vectors, a_offset, n, st, d.apply_work, d.image_off, images, parity, ctx->d_status};
  launchBegin(ctx, stream);
  tcvApplyKernel<<<d.apply_items, kApplyThreads, kApplySmem, stream>>>(aa);
  return launchedOn(ctx, stream, "jacobi vectors tcgen05");
}

void twoLevelTables(const int *host_n, int count, const std::vector<int> &ids, TwoLevelTables &out) {
  out = TwoLevelTables{};
  out.diag_off.assign(count, 0);
  int max_stages = 0;
  for (const int i : ids) {
    const int nb = padded8(host_n[i]) / 4;
    max_stages = std::max(max_stages, twoLevelSupers(nb) - 1);
  }
  out.stage_first.assign(max_stages, 0);
  out.stage_count.assign(max_stages, 0);
  for (int s = 0; s < max_stages; ++s) {
    out.stage_first[s] = static_cast<int>(out.inner.size() / 2);
    for (const int i : ids) {
      const int supers = twoLevelSupers(padded8(host_n[i]) / 4);
      if (s >= supers - 1) continue;
      for (int x = 0; x < supers / 2; ++x) {
        out.inner.push_back(i);
        out.inner.push_back(x);
      }
    }
    out.stage_count[s] = static_cast<int>(out.inner.size() / 2) - out.stage_first[s];
  }
  for (const int i : ids) {
    out.ids.push_back(i);
    out.diag_off[i] = out.diag_blocks;
    out.diag_blocks += twoLevelSupers(padded8(host_n[i]) / 4) / 2;
  }
}

int twoLevelEnqueue(msq_ctx *ctx, cudaStream_t stream, const TwoLevelDevice &t,
                    const TcVectorsDevice &v, float *matrices, float *b_scratch, float *diag,
                    uint8_t *images, const int64_t *a_offset, const int32_t *n,
                    const int64_t *eig_offset, float *eigenvalues, void *state, double tol,
                    const double *tols, int max_sweeps, bool first, bool sweep, int parity) {
  if (t.count == 0) return MSQ_OK;
  if (setAttributes() != MSQ_OK) return cudaCheck(ctx, cudaGetLastError(), "two-level attributes");
  auto *st = static_cast<JacobiState *>(state);
  CheckArgs ca{matrices, a_offset, n, eig_offset, eigenvalues, st, t.ids, tol, tols, max_sweeps,
               first ? 1 : 0, parity};
  launchBegin(ctx, stream);
  tlCheckKernel<<<t.count, 256, 0, stream>>>(ca);
  MSQ_TRY(launchedOn(ctx, stream, "jacobi two-level check"));
  if (!sweep) return MSQ_OK;
  for (size_t s = 0; s < t.stage_first.size(); ++s) {
    InnerArgs ia{matrices, a_offset, n, st, t.inner + t.stage_first[s], v.prog, v.prog_off,
                 v.image_off, images, diag, t.diag_off, static_cast<int>(s)};
    launchBegin(ctx, stream);
    tlInnerKernel<<<t.stage_count[s], kInnerThreads, 0, stream>>>(ia);
    MSQ_TRY(launchedOn(ctx, stream, "jacobi two-level blocks"));
    PassArgs pa{matrices, b_scratch, a_offset, n, st, v.apply_work, v.image_off, images,
                diag, t.diag_off, static_cast<int>(s), ctx->d_status};
    launchBegin(ctx, stream);
    tlPassKernel<false><<<v.apply_items, kPassThreads, kPassSmemFirst, stream>>>(pa);
    MSQ_TRY(launchedOn(ctx, stream, "jacobi two-level A Z tcgen05"));
    pa.src = b_scratch;
    pa.dst = matrices;
    launchBegin(ctx, stream);
    tlPassKernel<true><<<v.apply_items, kPassThreads, kPassSmemSecond, stream>>>(pa);
    MSQ_TRY(launchedOn(ctx, stream, "jacobi two-level Z^T A Z tcgen05"));
  }
  return MSQ_OK;
}

}  // namespace msq

using namespace msq;

extern "C" int msq_jacobi_schedule(int blocks, int32_t *pairs, size_t capacity, int *rounds) {
  if (blocks < 2 || blocks % 2 != 0 || blocks > 4096 || rounds == nullptr)
    return MSQ_ERR_INVALID_ARGUMENT;
  *rounds = twoLevelRounds(blocks);
  if (pairs == nullptr) return MSQ_OK;
  if (capacity < static_cast<size_t>(*rounds) * blocks) return MSQ_ERR_INVALID_ARGUMENT;
  std::vector<int32_t> table;
  twoLevelSchedule(blocks, table);
  std::copy(table.begin(), table.end(), pairs);
  return MSQ_OK;
}

extern "C" int msq_set_jacobi_vectors(msq_ctx *ctx, int mode) {
  if (ctx == nullptr || mode < -1 || mode > 3) return MSQ_ERR_INVALID_ARGUMENT;
  ctx->jacobi_vectors = mode;
  return MSQ_OK;
}
