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
  // B operand rows j (output columns), K = the 64 local indices: Z^T,
  // halves j < 32 (super-block P) and j >= 32 (super-block Q), hi and lo.
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
      const uint32_t at = swizzle128(lane, c);
      *reinterpret_cast<uint4 *>(img + (2 * h) * 4096 + at) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4 *>(img + (2 * h + 1) * 4096 + at) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
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
            const uint64_t zh = smemDesc(zimg + h * 8192), zl = smemDesc(zimg + h * 8192 + 4096);
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

int setAttributes() {
  static std::atomic<uint64_t> done_mask{0};
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) return MSQ_ERR_CUDA;
  const uint64_t bit = uint64_t{1} << device;
  if (done_mask.load() & bit) return MSQ_OK;
  if (cudaFuncSetAttribute(tcvFormKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kFormSmem)) != cudaSuccess ||
      cudaFuncSetAttribute(tcvApplyKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kApplySmem)) != cudaSuccess) {
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
                     const float *log, const int64_t *log_offset, uint8_t *images, int parity) {
  if (d.form_items == 0) return MSQ_OK;
  if (setAttributes() != MSQ_OK) return cudaCheck(ctx, cudaGetLastError(), "tensor-core vectors attributes");
  const auto *st = static_cast<const JacobiState *>(state);
  FormArgs fa{log, log_offset, n, st, d.form_work, d.prog, d.prog_off, d.image_off, images, parity};
  launchBegin(ctx, stream);
  tcvFormKernel<<<d.form_items, kFormThreads, kFormSmem, stream>>>(fa);
  MSQ_TRY(launchedOn(ctx, stream, "jacobi stage rotations"));
  ApplyArgs aa{vectors, a_offset, n, st, d.apply_work, d.image_off, images, parity, ctx->d_status};
  launchBegin(ctx, stream);
  tcvApplyKernel<<<d.apply_items, kApplyThreads, kApplySmem, stream>>>(aa);
  return launchedOn(ctx, stream, "jacobi vectors tcgen05");
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
  if (ctx == nullptr || mode < -1 || mode > 2) return MSQ_ERR_INVALID_ARGUMENT;
  ctx->jacobi_vectors = mode;
  return MSQ_OK;
}
