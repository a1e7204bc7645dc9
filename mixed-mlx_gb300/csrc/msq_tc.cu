// Low-bit reconstruction X = W W^T on the 5th-generation tensor cores.
//
// Replaces reconstructLowFactorTiled / matmul_f32_low_right_* of the
// reference (src/metal_runtime.cpp:500-534, metal_mixed_sqrt.metal:
// 1540-1600), which decode the low-bit factor to FP32 in threadgroup memory
// and run an FP32 FMA tile GEMM.  Here the factor stays low-bit all the way
// into the MMA:
//   * packOperand quantizes the K-major factor W^T straight into 128-row x
//     128-byte tiles laid out in the canonical SWIZZLE_128B K-major shape
//     (16-byte chunk index XOR row mod 8 inside each 1024-byte atom), so a
//     tile is one contiguous 16 KB block that a single TMA bulk copy
//     (cp.async.bulk) lands in shared memory ready for the MMA;
//   * tcGemmKernel is a persistent, warp-specialized kernel: warp 4 issues
//     the bulk copies into a 4-stage mbarrier ring, warp 5 owns TMEM (256
//     columns: two 128x128 FP32 accumulators) and issues tcgen05.mma
//     (kind::f16 for BF16, kind::f8f6f4 for FP8 E4M3) from one thread, and
//     warps 0-3 drain the other accumulator with tcgen05.ld while the next
//     tile accumulates, applying the per-row FP8 scales r_i r_j.
// MX factors (E2M1 or E4M3 with one UE8M0 scale per 32 along K of a row;
// the reference's K-major MX operand with scale stride ld / 32,
// 3_spectral/lowbit_matmul.cpp:240-299) stay in their codes: packMxKernel
// writes E2M1 (two per byte) or E4M3 tiles plus one scale-factor tile each,
// the producer bulk-copies both, and the MMA thread moves each stage's
// scale factors into TMEM with tcgen05.cp and issues tcgen05.mma
// kind::mxf4 / kind::mxf8f6f4 .block_scale, which applies 2^(s - 127) per
// 32-element block inside the tensor core (the reference's blockwise
// ue8m0 / 32 product, 3_spectral/lowbit_matmul.metal:33).  Flat MXFP4 codes
// whose blocks straddle rows (order not divisible by 32) are decoded exactly
// into BF16 tiles (E2M1 x 2^e has at most 2 significant bits) and use
// kind::f16.  Every mbarrier wait is bounded; on expiry the kernel records
// kStatusMbarrierTimeout in the context's status word and unwinds.
#include "msq_codec_device.cuh"
#include "msq_internal.cuh"
#include "msq_stages.cuh"
#include "msq_tcgen05.cuh"

#include <algorithm>
#include <atomic>
#include <vector>

namespace msq {
namespace {

constexpr int kTileRows = 128;
constexpr int kTileBytes = 16384;  // 128 rows x 128 bytes
constexpr int kStages = 4;
constexpr int kTcThreads = 192;    // warps 0-3 epilogue, 4 producer, 5 MMA
constexpr uint32_t kTmemCols = 256;
constexpr long long kWaitLimit = 1ll << 26;

// kOpMxf4 / kOpMxf8: block-scaled operands (E2M1 packed two per byte, or
// E4M3) with one UE8M0 scale factor per 32 consecutive K of a row, run as
// tcgen05.mma kind::mxf4 / kind::mxf8f6f4 .block_scale with the scale
// factors staged in TMEM.
enum OperandKind : int { kOpBf16 = 0, kOpFp8 = 1, kOpMxf4 = 2, kOpMxf8 = 3 };
constexpr bool isBlockScaled(int kind) { return kind == kOpMxf4 || kind == kOpMxf8; }
// Scale-factor tile of one operand tile: atoms of 128 rows x 4 K blocks,
// byte 16 (r mod 32) + 4 (r / 32) + b of an atom holding row r, block b (the
// 32-lane x 128-bit source of tcgen05.cp ... warpx4).  An E2M1 tile row (256
// K) has 8 blocks (two atoms), an E4M3 row (128 K) 4 (one atom).
constexpr int kScaleAtomBytes = 512;
constexpr int kScaleTileBytes = 2 * kScaleAtomBytes;
// TMEM: two 128-column accumulators, then per stage 16 scale-factor
// columns (A atoms at +0, +4, B atoms at +8, +12).
constexpr uint32_t kTmemColsMx = 512;
constexpr uint32_t kScaleCol0 = 256;
constexpr int kMaxSegments = 6;
enum Epilogue : int {
  kEpiStore = 0,     // X = acc
  kEpiRowScale = 1,  // X_ij = acc * r_i * r_j (FP8 row-scaled factor)
  kEpiInverseH = 2,  // X_ij = acc / (s_i + s_j), s = sqrt(lambda)
  kEpiResidual = 3,  // X = A - acc, FP64 ||X||^2 and ||A||^2 per matrix
};

// Bounded wait: false (and the status word set) if the phase never completes.
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity, int *status,
                                         volatile int *abort_flag, long long limit = kWaitLimit) {
  for (long long i = 0; i < limit; ++i) {
    if (mbarTryWait(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  atomicExch(status, kStatusMbarrierTimeout);
  *abort_flag = 1;
  return false;
}

// Instruction descriptor: D = F32, K-major A and B, M = 128, N = 128.
// A/B type field: BF16 = 1 for kind::f16, E4M3 = 0 for kind::f8f6f4.
__host__ __device__ constexpr uint32_t instrDesc(int kind) {
  return (1u << 4) | ((kind == kOpBf16 ? 1u : 0u) << 7) | ((kind == kOpBf16 ? 1u : 0u) << 10) |
         ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

template <int kKind>
__device__ __forceinline__ void mmaIssue(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accum) {
  if constexpr (kKind == kOpBf16) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(instrDesc(kOpBf16)), "r"(accum));
  } else {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(instrDesc(kOpFp8)), "r"(accum));
  }
}

struct TcArgs {
  const int4 *work;        // (matrix, tile_m, tile_n, k_tiles)
  int items;
  // The accumulator sums A_s B_s^T over `segments` operand pairs (split-BF16
  // products); every packed operand shares the plan's tile geometry.
  int segments;
  const uint8_t *tiles_a[kMaxSegments];
  const uint8_t *tiles_b[kMaxSegments];
  const uint8_t *scales_a; // block-scaled kinds: scale-factor tiles (one segment)
  const uint8_t *scales_b;
  const int64_t *tile_base;// per matrix: first tile index
  const int32_t *n;
  const int64_t *x_offset;
  const int64_t *eig_offset;
  const float *row_scale;  // kEpiRowScale: per matrix row scales at eig_offset
  const float *eigenvalues;// kEpiInverseH: lambda, s = sqrt(max(lambda, 0))
  const float *a_in;       // kEpiResidual: R = A - acc
  double *norms;           // kEpiResidual: ||R||^2, ||A||^2 per matrix
  float *x;
  int *status;
  int wait_test;           // 1: the producer first waits on a barrier nothing arrives at
};

template <int kKind, int kEpi>
__global__ void __launch_bounds__(kTcThreads, 1) tcGemmKernel(TcArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr bool kMx = isBlockScaled(kKind);
  constexpr uint32_t kCols = kMx ? kTmemColsMx : kTmemCols;
  unsigned char *stage_mem = base;  // kStages x (A 16 KB, B 16 KB)
  // block-scaled kinds: kStages x (SFA 1 KB, SFB 1 KB) after the operands
  unsigned char *scale_mem = base + kStages * 2 * kTileBytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + kStages * 2 * kTileBytes +
                                                (kMx ? kStages * 2 * kScaleTileBytes : 0));
  uint64_t *full = bars, *empty = bars + kStages;
  uint64_t *acc_full = bars + 2 * kStages, *acc_empty = acc_full + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbarInit(smemAddr(&full[s]), 1);
      mbarInit(smemAddr(&empty[s]), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbarInit(smemAddr(&acc_full[a]), 1);
      mbarInit(smemAddr(&acc_empty[a]), 128);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smemAddr(tmem_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 4) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      if (args.wait_test) {
        // failure injection: phase 0 of empty[0] completes only after an
        // MMA commit, which needs a copy this thread has not issued; the
        // wait expires, sets the status and the abort flag, and every role
        // unwinds with no copy or MMA in flight
        mbarWait(smemAddr(&empty[0]), 0, args.status, abort_flag, 4096);
      }
      for (int item = blockIdx.x; item < args.items && !*abort_flag; item += gridDim.x) {
        const int4 w = args.work[item];
        const int64_t base = args.tile_base[w.x] * kTileBytes;
        for (int seg = 0; seg < args.segments; ++seg) {
          const uint8_t *ta = args.tiles_a[seg] + base;
          const uint8_t *tb = args.tiles_b[seg] + base;
          for (int kt = 0; kt < w.w; ++kt) {
            if (!mbarWait(smemAddr(&empty[stage]), phase ^ 1, args.status, abort_flag)) break;
            const uint32_t bar = smemAddr(&full[stage]);
            mbarArriveExpectTx(bar, 2 * kTileBytes + (kMx ? 2 * kScaleTileBytes : 0));
            unsigned char *dst = stage_mem + stage * 2 * kTileBytes;
            const int64_t tile_a = args.tile_base[w.x] + static_cast<int64_t>(w.y) * w.w + kt;
            const int64_t tile_b = args.tile_base[w.x] + static_cast<int64_t>(w.z) * w.w + kt;
            bulkLoad(smemAddr(dst), ta + (static_cast<int64_t>(w.y) * w.w + kt) * kTileBytes,
                     kTileBytes, bar);
            bulkLoad(smemAddr(dst + kTileBytes),
                     tb + (static_cast<int64_t>(w.z) * w.w + kt) * kTileBytes, kTileBytes, bar);
            if constexpr (kMx) {
              unsigned char *sdst = scale_mem + stage * 2 * kScaleTileBytes;
              bulkLoad(smemAddr(sdst), args.scales_a + tile_a * kScaleTileBytes, kScaleTileBytes,
                       bar);
              bulkLoad(smemAddr(sdst + kScaleTileBytes), args.scales_b + tile_b * kScaleTileBytes,
                       kScaleTileBytes, bar);
            }
            if (++stage == kStages) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int acc = 0;
      uint32_t acc_phase = 0;
      for (int item = blockIdx.x; item < args.items && !*abort_flag; item += gridDim.x) {
        const int4 w = args.work[item];
        if (!mbarWait(smemAddr(&acc_empty[acc]), acc_phase ^ 1, args.status, abort_flag)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t d = tmem + acc * 128;
        const int steps = args.segments * w.w;
        for (int step = 0; step < steps; ++step) {
          if (!mbarWait(smemAddr(&full[stage]), phase, args.status, abort_flag)) break;
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t a_addr = smemAddr(stage_mem + stage * 2 * kTileBytes);
          const uint64_t adesc = smemDesc(a_addr);
          const uint64_t bdesc = smemDesc(a_addr + kTileBytes);
          // 128 bytes of K per stage: four MMAs of 32 bytes (K = 16 BF16, 32
          // FP8 or 64 E2M1); the start address advances inside the swizzle
          // atom.
          if constexpr (kMx) {
            // the stage's scale-factor atoms into TMEM, then the MMAs (the
            // copies and MMAs of this thread execute in issue order)
            const uint32_t s_addr = smemAddr(scale_mem + stage * 2 * kScaleTileBytes);
            const uint32_t sf = tmem + kScaleCol0 + 16u * stage;
            const int atoms = kKind == kOpMxf4 ? 2 : 1;
            for (int at = 0; at < atoms; ++at) {
              tmemCopyScales(sf + 4u * at, smemDescPlain(s_addr + at * kScaleAtomBytes));
              tmemCopyScales(sf + 8u + 4u * at,
                             smemDescPlain(s_addr + kScaleTileBytes + at * kScaleAtomBytes));
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint32_t acc_on = (step | kk) != 0;
              if constexpr (kKind == kOpMxf4) {
                // K blocks 2kk, 2kk+1: atom kk/2, bytes 2(kk mod 2) and +1
                const uint32_t id = 2u * (kk & 1);
                mmaMxf4(d, adesc + 2 * kk, bdesc + 2 * kk, instrDescBlockScaled(true, id, id),
                        sf + 4u * (kk >> 1), sf + 8u + 4u * (kk >> 1), acc_on);
              } else {
                // K block kk: byte kk of the one atom
                mmaMxf8(d, adesc + 2 * kk, bdesc + 2 * kk,
                        instrDescBlockScaled(false, kk, kk), sf, sf + 8u, acc_on);
              }
            }
          } else {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              mmaIssue<kKind>(d, adesc + 2 * kk, bdesc + 2 * kk, (step | kk) != 0);
            }
          }
          mmaCommit(smemAddr(&empty[stage]));
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1;
          }
        }
        mmaCommit(smemAddr(&acc_full[acc]));
        if (++acc == 2) {
          acc = 0;
          acc_phase ^= 1;
        }
      }
    }
  } else {
    // Epilogue: thread t owns accumulator row t (TMEM lane t).
    int acc = 0;
    uint32_t acc_phase = 0;
    for (int item = blockIdx.x; item < args.items; item += gridDim.x) {
      const int4 w = args.work[item];
      if (!mbarWait(smemAddr(&acc_full[acc]), acc_phase, args.status, abort_flag)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int mi = w.x;
      const int n = args.n[mi];
      const int i = w.y * kTileRows + threadIdx.x;
      const int j0 = w.z * kTileRows;
      float *X = args.x + args.x_offset[mi];
      float ri = 1.0f;
      const float *rs = nullptr;
      if (kEpi == kEpiRowScale) {
        rs = args.row_scale + args.eig_offset[mi];
        ri = i < n ? rs[i] : 0.0f;
      }
      const float *lam = kEpi == kEpiInverseH ? args.eigenvalues + args.eig_offset[mi] : nullptr;
      const float si = kEpi == kEpiInverseH && i < n ? sqrtf(fmaxf(lam[i], 0.0f)) : 0.0f;

      const float *A = kEpi == kEpiResidual ? args.a_in + args.x_offset[mi] : nullptr;
      double rn = 0.0, an = 0.0;
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        float v[32];
        tmemLoad32(tmem + ((32u * warp) << 16) + acc * 128 + c * 32, v);
        // s_j of this chunk's 32 columns: one square root per lane (not one
        // per element), spread over the warp by shuffles that every lane runs
        float sj[32];
        if (kEpi == kEpiInverseH) {
          const int jl = j0 + c * 32 + lane;
          const float mine = jl < n ? sqrtf(fmaxf(lam[jl], 0.0f)) : 0.0f;
#pragma unroll
          for (int q = 0; q < 32; ++q) sj[q] = __shfl_sync(0xffffffffu, mine, q);
        }
        if (i < n) {
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const int j = j0 + c * 32 + q;
            if (j < n) {
              const int64_t at = i + static_cast<int64_t>(j) * n;
              float val = v[q];
              // (r_i r_j) first: the product of the two scales is the same
              // for (i, j) and (j, i), so X stays exactly symmetric
              if (kEpi == kEpiRowScale) val = val * (ri * rs[j]);
              if (kEpi == kEpiInverseH) {
                const float d = si + sj[q];
                val = d > 0.0f ? val / d : 0.0f;  // both roots 0: no correction
              }
              if (kEpi == kEpiResidual) {
                const float a = A[at];
                val = a - val;
                rn += static_cast<double>(val) * val;
                an += static_cast<double>(a) * a;
              }
              X[at] = val;
            }
          }
        }
      }
      if (kEpi == kEpiResidual) {
        // epilogue warps 0-3 reduce, then one atomic per warp
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
          rn += __shfl_xor_sync(0xffffffffu, rn, s);
          an += __shfl_xor_sync(0xffffffffu, an, s);
        }
        if (lane == 0) {
          atomicAdd(&args.norms[2 * mi], rn);
          atomicAdd(&args.norms[2 * mi + 1], an);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbarArrive(smemAddr(&acc_empty[acc]));
      if (++acc == 2) {
        acc = 0;
        acc_phase ^= 1;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 5) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kCols));
  }
}

// ------------------------------------------------------------ packing

enum PackSource : int {
  kPackF32Bf16 = 0,     // FP32 factor -> BF16
  kPackF32Fp8Row = 1,   // FP32 factor / row scale -> E4M3
  kPackBf16Codes = 3,   // flat BF16 codes
  kPackFp8Codes = 4,    // flat E4M3 codes (row scales separate)
  kPackMxfp4Codes = 5,  // flat MXFP4 codes + E8M0 scales, decoded into BF16
};

struct PackArgs {
  const int4 *work;       // (matrix, tile_m, tile_k, k_tiles)
  int items;
  const float *f;         // FP32 factor, K-major (F[k + i*n] = W_ik)
  const uint8_t *codes;   // flat codes in the same layout
  const uint8_t *mx_scales;
  const float *row_scale;
  const int64_t *f_offset;
  const int64_t *eig_offset;
  const int64_t *tile_base;
  const int32_t *n;
  uint8_t *tiles;
};

// One CTA of 128 threads per tile; thread r packs row r (128 bytes).
template <int kSource>
__global__ void __launch_bounds__(128) packKernel(PackArgs args) {
  for (int item = blockIdx.x; item < args.items; item += gridDim.x) {
    const int4 w = args.work[item];
    const int mi = w.x, n = args.n[mi];
    const int r = threadIdx.x;
    const int i = w.y * kTileRows + r;
    constexpr bool kFp8 = kSource == kPackF32Fp8Row || kSource == kPackFp8Codes;
    constexpr int kElems = kFp8 ? 128 : 64;  // elements per 128-byte row
    const int k0 = w.z * kElems;
    const int64_t off = args.f_offset[mi];
    uint8_t *tile = args.tiles + (args.tile_base[mi] + static_cast<int64_t>(w.y) * w.w + w.z) *
                                     kTileBytes;
    const bool row_ok = i < n;
    float inv_scale_row = 1.0f;
    if (kSource == kPackF32Fp8Row && row_ok) inv_scale_row = args.row_scale[args.eig_offset[mi] + i];
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
      uint32_t word[4] = {0, 0, 0, 0};
      if (row_ok) {
        if constexpr (kFp8) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int k = k0 + c * 16 + e;
            uint32_t code = 0;
            if (k < n) {
              const int64_t at = off + k + static_cast<int64_t>(i) * n;
              code = kSource == kPackFp8Codes ? args.codes[at]
                                              : encodeE4M3(rowDivide(args.f[at], inv_scale_row));
            }
            word[e / 4] |= code << (8 * (e % 4));
          }
        } else {
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const int k = k0 + c * 8 + e;
            uint32_t h = 0;
            if (k < n) {
              const int64_t at = off + k + static_cast<int64_t>(i) * n;
              if (kSource == kPackF32Bf16) {
                h = encodeBf16(args.f[at]);
              } else if (kSource == kPackBf16Codes) {
                h = reinterpret_cast<const uint16_t *>(args.codes)[at];
              } else {  // kPackMxfp4Codes: exact, at most 2 significant bits
                const uint32_t byte = args.codes[at / 2];
                const float d = decodeE2M1((byte >> ((at & 1) * 4)) & 0xfu);
                h = encodeBf16(mxScale(d, args.mx_scales[at / 32]));
              }
            }
            word[e / 2] |= h << (16 * (e % 2));
          }
        }
      }
      *reinterpret_cast<uint4 *>(tile + swizzle128(r, c)) =
          make_uint4(word[0], word[1], word[2], word[3]);
    }
  }
}

// Block-scaled operand tiles: codes in the SWIZZLE_128B K-major tile (E2M1
// two per byte, the even K in the low nibble; or E4M3) and the tile's
// scale-factor bytes in the atom layout of kScaleTileBytes.  Sources:
//   kMxF32Fp4    FP32 factor -> E2M1 + UE8M0 per 32 K of a row (the
//                reference's mxScaleExponent / floatToFp4E2M1 per block)
//   kMxCodesFp4  flat MXFP4 codes and scales (order divisible by 32, so
//                the flat 32-element blocks are row blocks)
//   kMxCodesFp8  flat MXFP8 E4M3 codes and scales (same condition)
// One CTA of 128 threads per tile; thread r packs row r.  Blocks beyond the
// order get zero codes and the unit scale (byte 127).
enum MxSource : int { kMxF32Fp4 = 0, kMxCodesFp4 = 1, kMxCodesFp8 = 2 };

struct MxPackArgs {
  const int4 *work;       // (matrix, tile_m, tile_k, k_tiles)
  int items;
  const float *f;
  const uint8_t *codes;
  const uint8_t *mx_scales;
  const int64_t *f_offset;
  const int64_t *tile_base;
  const int32_t *n;
  uint8_t *tiles;
  uint8_t *scale_tiles;
};

template <int kSource>
__global__ void __launch_bounds__(128) packMxKernel(MxPackArgs args) {
  constexpr bool kFp4 = kSource != kMxCodesFp8;
  constexpr int kElems = kFp4 ? 256 : 128;  // K per 128-byte tile row
  constexpr int kBlocks = kElems / 32;
  for (int item = blockIdx.x; item < args.items; item += gridDim.x) {
    const int4 w = args.work[item];
    const int mi = w.x, n = args.n[mi];
    const int r = threadIdx.x;
    const int i = w.y * kTileRows + r;
    const int k0 = w.z * kElems;
    const int64_t off = args.f_offset[mi];
    const int64_t t = args.tile_base[mi] + static_cast<int64_t>(w.y) * w.w + w.z;
    uint8_t *tile = args.tiles + t * kTileBytes;
    uint8_t *sft = args.scale_tiles + t * kScaleTileBytes;
    uint32_t sf_word[2] = {0x7f7f7f7fu, 0x7f7f7f7fu};
#pragma unroll 1
    for (int blk = 0; blk < kBlocks; ++blk) {
      const int kb = k0 + 32 * blk;
      uint32_t words[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // 32 codes: 16 (E2M1) or 32 bytes
      uint32_t sf = 127;
      if (i < n && kb < n) {
        const int64_t at = off + kb + static_cast<int64_t>(i) * n;
        if constexpr (kSource == kMxF32Fp4) {
          float x[32];
          float m = 0.0f;
#pragma unroll
          for (int e = 0; e < 32; ++e) {
            x[e] = kb + e < n ? args.f[at + e] : 0.0f;
            const float a = fabsf(x[e]);
            if (a <= 3.402823466e38f) m = fmaxf(m, a);
          }
          const int ex = mxExponent(m, 2);
          sf = static_cast<uint32_t>(ex + 127);
#pragma unroll
          for (int e = 0; e < 32; ++e) {
            const uint32_t code = kb + e < n ? encodeE2M1(mxDivide(x[e], ex)) : 0u;
            words[e / 8] |= code << (4 * (e % 8));
          }
        } else if constexpr (kSource == kMxCodesFp4) {
          // 16 bytes of codes at byte at / 2 (a multiple of 16), one scale
          const uint4 c = *reinterpret_cast<const uint4 *>(args.codes + at / 2);
          words[0] = c.x;
          words[1] = c.y;
          words[2] = c.z;
          words[3] = c.w;
          sf = args.mx_scales[at / 32];
        } else {
          const uint4 c0 = *reinterpret_cast<const uint4 *>(args.codes + at);
          const uint4 c1 = *reinterpret_cast<const uint4 *>(args.codes + at + 16);
          words[0] = c0.x;
          words[1] = c0.y;
          words[2] = c0.z;
          words[3] = c0.w;
          words[4] = c1.x;
          words[5] = c1.y;
          words[6] = c1.z;
          words[7] = c1.w;
          sf = args.mx_scales[at / 32];
        }
      }
      if constexpr (kFp4) {
        *reinterpret_cast<uint4 *>(tile + swizzle128(r, blk)) =
            make_uint4(words[0], words[1], words[2], words[3]);
      } else {
        *reinterpret_cast<uint4 *>(tile + swizzle128(r, 2 * blk)) =
            make_uint4(words[0], words[1], words[2], words[3]);
        *reinterpret_cast<uint4 *>(tile + swizzle128(r, 2 * blk + 1)) =
            make_uint4(words[4], words[5], words[6], words[7]);
      }
      const int shift = 8 * (blk % 4);
      sf_word[blk / 4] = (sf_word[blk / 4] & ~(0xffu << shift)) | (sf << shift);
    }
    // row r of atom a: 4 bytes at 16 (r mod 32) + 4 (r / 32)
    const int at_row = 16 * (r % 32) + 4 * (r / 32);
#pragma unroll
    for (int a = 0; a < kBlocks / 4; ++a) {
      *reinterpret_cast<uint32_t *>(sft + a * kScaleAtomBytes + at_row) = sf_word[a];
    }
  }
}

// Split-BF16 packing of an FP32 (or float-float hi + lo) matrix M, n x n
// column-major, as the K-major MMA operand: operand row i is column i of M
// (kTranspose false) or row i of M (kTranspose true).  Piece p is the BF16
// rounding of what pieces 0..p-1 left over, so three pieces carry the FP32
// mantissa and the products p_a p_b (exact in FP32) sum to M_a M_b.
struct SplitArgs {
  const int4 *work;
  int items;
  const float *hi;
  const float *lo;  // may be null
  const int64_t *offset;
  const int64_t *tile_base;
  const int32_t *n;
  int pieces;
  uint8_t *out[3];
};

template <bool kTranspose, bool kLo>
__global__ void __launch_bounds__(128) packSplitKernel(SplitArgs args) {
  // kTranspose false reads operand row i from column i of M: the tile's 128
  // columns x 64 rows are staged in shared memory with coalesced loads (a
  // warp reads 32 consecutive elements of one column, eight columns in
  // flight), then each thread reads its row there (stride 65: no bank
  // conflicts).  kLo: M is float-float (hi + lo).
  constexpr int kLd = 65;
  constexpr int kStage = kTranspose ? 1 : kTileRows * kLd;
  __shared__ float stage_hi[kStage];
  __shared__ float stage_lo[kLo ? kStage : 1];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  for (int item = blockIdx.x; item < args.items; item += gridDim.x) {
    const int4 w = args.work[item];
    const int mi = w.x, n = args.n[mi];
    const int r = threadIdx.x;
    const int i = w.y * kTileRows + r;
    const int k0 = w.z * 64;
    const float *H = args.hi + args.offset[mi];
    const float *L = kLo ? args.lo + args.offset[mi] : nullptr;
    const int64_t tile = (args.tile_base[mi] + static_cast<int64_t>(w.y) * w.w + w.z) * kTileBytes;
    if (!kTranspose) {
      __syncthreads();  // the previous item's rows have been read
#pragma unroll 1
      for (int c0 = 8 * warp; c0 < kTileRows; c0 += 32) {
        float xh[8][2], xl[8][2];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int col = w.y * kTileRows + c0 + q;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int k = k0 + lane + 32 * h;
            const bool in = col < n && k < n;
            const int64_t at = k + static_cast<int64_t>(col) * n;
            xh[q][h] = in ? H[at] : 0.0f;
            xl[q][h] = kLo && in ? L[at] : 0.0f;
          }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            stage_hi[(c0 + q) * kLd + lane + 32 * h] = xh[q][h];
            if (kLo) stage_lo[(c0 + q) * kLd + lane + 32 * h] = xl[q][h];
          }
      }
      __syncthreads();
    }
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
      uint32_t word[3][4] = {};
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k = k0 + c * 8 + e;
        float x = 0.0f, xl = 0.0f;
        if (kTranspose) {
          if (i < n && k < n) {
            const int64_t at = i + static_cast<int64_t>(k) * n;
            x = H[at];
            xl = kLo ? L[at] : 0.0f;
          }
        } else {
          x = stage_hi[r * kLd + c * 8 + e];
          xl = kLo ? stage_lo[r * kLd + c * 8 + e] : 0.0f;
        }
        const uint32_t h0 = encodeBf16(x);
        const float rem = (x - decodeBf16(static_cast<uint16_t>(h0))) + xl;
        const uint32_t h1 = encodeBf16(rem);
        const uint32_t h2 = encodeBf16(rem - decodeBf16(static_cast<uint16_t>(h1)));
        word[0][e / 2] |= h0 << (16 * (e % 2));
        word[1][e / 2] |= h1 << (16 * (e % 2));
        word[2][e / 2] |= h2 << (16 * (e % 2));
      }
      for (int p = 0; p < args.pieces; ++p) {
        *reinterpret_cast<uint4 *>(args.out[p] + tile + swizzle128(r, c)) =
            make_uint4(word[p][0], word[p][1], word[p][2], word[p][3]);
      }
    }
  }
}

// Row scales of the FP8 factor: r_i = max_k |W_ik| / 448 (1 for a zero
// row), the MSQ_FMT_FP8_E4M3FN_ROWSCALE definition with rows of W^T's
// K-major storage.  One warp per row.
__global__ void rowScaleKernel(const float *__restrict__ f, const int32_t *__restrict__ nn,
                               const int64_t *__restrict__ off, const int64_t *__restrict__ eoff,
                               int count, int64_t total_rows, const int32_t *__restrict__ row_matrix,
                               float *__restrict__ out) {
  const int lane = threadIdx.x % 32;
  for (int64_t row = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / 32;
       row < total_rows; row += static_cast<int64_t>(gridDim.x) * blockDim.x / 32) {
    const int mi = row_matrix[row];
    const int n = nn[mi];
    const int i = static_cast<int>(row - eoff[mi]);
    const float *src = f + off[mi] + static_cast<int64_t>(i) * n;
    float m = 0.0f;
    for (int k = lane; k < n; k += 32) {
      const float a = fabsf(src[k]);
      if (a <= 3.402823466e38f) m = fmaxf(m, a);
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
    if (lane == 0) out[row] = m == 0.0f ? 1.0f : __fdiv_rn(m, 448.0f);
  }
}

// Per-layout tile plan (packing work, GEMM work, tile bases).
struct TcPlan {
  uint64_t key;
  int count;
  int kind;
  int device_id;
  int pack_items, gemm_items;
  int64_t total_tiles;
  int4 *pack_work, *gemm_work;
  int64_t *tile_base;
  int32_t *row_matrix;
  void *device;
};

}  // namespace

// The context's tile plans (at most 32 layouts and kinds, oldest evicted).
struct TcPlanCache {
  std::vector<TcPlan *> plans;
};

void destroyTcPlans(TcPlanCache *cache) {
  if (cache == nullptr) return;
  for (TcPlan *p : cache->plans) {
    cudaFree(p->device);
    delete p;
  }
  delete cache;
}

namespace {

TcPlan *tcPlan(msq_ctx *ctx, const DeviceBatch *b, int kind) {
  if (ctx->tc_plans == nullptr) ctx->tc_plans = new TcPlanCache;
  auto &plans = ctx->tc_plans->plans;
  for (TcPlan *p : plans)
    if (p->key == b->key && p->count == b->count && p->kind == kind && p->device_id == ctx->device)
      return p;
  // K per 128-byte tile row
  const int elems = kind == kOpMxf4 ? 256 : (kind == kOpFp8 || kind == kOpMxf8) ? 128 : 64;
  std::vector<int64_t> base(b->count);
  std::vector<int4> pack, gemm;
  std::vector<int32_t> row_matrix;
  int64_t tiles = 0;
  std::vector<int> ids(b->count);
  for (int i = 0; i < b->count; ++i) ids[i] = i;
  std::stable_sort(ids.begin(), ids.end(),
                   [&](int x, int y) { return b->host_n[x] > b->host_n[y]; });
  for (int mi = 0; mi < b->count; ++mi) {
    const int n = b->host_n[mi];
    const int mt = (n + kTileRows - 1) / kTileRows, kt = (n + elems - 1) / elems;
    base[mi] = tiles;
    tiles += static_cast<int64_t>(mt) * kt;
    for (int a = 0; a < mt; ++a)
      for (int k = 0; k < kt; ++k) pack.push_back(make_int4(mi, a, k, kt));
    for (int r = 0; r < n; ++r) row_matrix.push_back(mi);
  }
  for (int mi : ids) {
    const int n = b->host_n[mi];
    const int mt = (n + kTileRows - 1) / kTileRows, kt = (n + elems - 1) / elems;
    for (int a = 0; a < mt; ++a)
      for (int c = 0; c < mt; ++c) gemm.push_back(make_int4(mi, a, c, kt));
  }
  auto *p = new TcPlan{};
  p->key = b->key;
  p->count = b->count;
  p->kind = kind;
  p->device_id = ctx->device;
  p->pack_items = static_cast<int>(pack.size());
  p->gemm_items = static_cast<int>(gemm.size());
  p->total_tiles = tiles;
  const size_t bytes = (pack.size() + gemm.size()) * sizeof(int4) + base.size() * sizeof(int64_t) +
                       row_matrix.size() * sizeof(int32_t) + 64;
  char *dev = nullptr;
  if (cudaCheck(ctx, cudaMalloc(&dev, bytes), "tc plan alloc") != MSQ_OK) {
    delete p;
    return nullptr;
  }
  p->device = dev;
  p->pack_work = reinterpret_cast<int4 *>(dev);
  p->gemm_work = p->pack_work + pack.size();
  p->tile_base = reinterpret_cast<int64_t *>(p->gemm_work + gemm.size());
  p->row_matrix = reinterpret_cast<int32_t *>(p->tile_base + base.size());
  cudaMemcpy(p->pack_work, pack.data(), pack.size() * sizeof(int4), cudaMemcpyHostToDevice);
  cudaMemcpy(p->gemm_work, gemm.data(), gemm.size() * sizeof(int4), cudaMemcpyHostToDevice);
  cudaMemcpy(p->tile_base, base.data(), base.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(p->row_matrix, row_matrix.data(), row_matrix.size() * sizeof(int32_t),
             cudaMemcpyHostToDevice);
  if (plans.size() >= 32) {
    cudaFree(plans.front()->device);
    ++ctx->alloc_generation;
    delete plans.front();
    plans.erase(plans.begin());
  }
  plans.push_back(p);
  return p;
}

size_t tcSmemBytes(int kind = kOpBf16) {
  return kStages * 2 * kTileBytes + (isBlockScaled(kind) ? kStages * 2 * kScaleTileBytes : 0) +
         1024 + 256;
}

// Opt-in shared memory of the GEMM kernels, once per device.
int tcAttributes(msq_ctx *ctx) {
  static std::atomic<uint64_t> done_mask{0};
  const uint64_t bit = ctx->device >= 0 && ctx->device < 64 ? uint64_t{1} << ctx->device : 0;
  if (bit != 0 && (done_mask.load() & bit)) return MSQ_OK;
  const int bytes = static_cast<int>(tcSmemBytes());
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(tcGemmKernel<kOpBf16, kEpiStore>, a, bytes), "tc attr"));
  MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(tcGemmKernel<kOpFp8, kEpiRowScale>, a, bytes), "tc attr"));
  MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(tcGemmKernel<kOpBf16, kEpiInverseH>, a, bytes), "tc attr"));
  MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(tcGemmKernel<kOpBf16, kEpiResidual>, a, bytes), "tc attr"));
  const int mx_bytes = static_cast<int>(tcSmemBytes(kOpMxf4));
  MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(tcGemmKernel<kOpMxf4, kEpiStore>, a, mx_bytes), "tc attr"));
  MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(tcGemmKernel<kOpMxf8, kEpiStore>, a, mx_bytes), "tc attr"));
  done_mask.fetch_or(bit);
  return MSQ_OK;
}

// Launches the persistent tcgen05 GEMM over the plan's work list:
// X = sum_s A_s B_s^T per matrix with the given epilogue.
int launchTcGemm(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, int epilogue, int segments,
                 const uint8_t *const *a_tiles, const uint8_t *const *b_tiles,
                 const float *row_scale, const float *eigenvalues, const float *a_in,
                 double *norms, float *x, const char *what,
                 const uint8_t *scale_tiles = nullptr) {
  MSQ_TRY(tcAttributes(ctx));
  TcArgs args{};
  args.scales_a = scale_tiles;
  args.scales_b = scale_tiles;
  args.work = p->gemm_work;
  args.items = p->gemm_items;
  args.segments = segments;
  for (int s = 0; s < segments; ++s) {
    args.tiles_a[s] = a_tiles[s];
    args.tiles_b[s] = b_tiles[s];
  }
  args.tile_base = p->tile_base;
  args.n = b->n;
  args.x_offset = b->offset;
  args.eig_offset = b->eig_offset;
  args.row_scale = row_scale;
  args.eigenvalues = eigenvalues;
  args.a_in = a_in;
  args.norms = norms;
  args.x = x;
  args.status = ctx->d_status;
  args.wait_test = waitTestMode() == kWaitTestMbarrier;
  const unsigned grid = std::min(p->gemm_items, kSmCount);
  const size_t smem = tcSmemBytes(p->kind);
  if (isBlockScaled(p->kind)) {
    if (scale_tiles == nullptr || segments != 1 || epilogue != kEpiStore) {
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "block-scaled GEMM: one segment, store");
    }
    if (p->kind == kOpMxf4) {
      tcGemmKernel<kOpMxf4, kEpiStore><<<grid, kTcThreads, smem, ctx->stream>>>(args);
    } else {
      tcGemmKernel<kOpMxf8, kEpiStore><<<grid, kTcThreads, smem, ctx->stream>>>(args);
    }
    return launched(ctx, what);
  }
  switch (epilogue) {
    case kEpiRowScale:
      tcGemmKernel<kOpFp8, kEpiRowScale><<<grid, kTcThreads, smem, ctx->stream>>>(args);
      break;
    case kEpiInverseH:
      tcGemmKernel<kOpBf16, kEpiInverseH><<<grid, kTcThreads, smem, ctx->stream>>>(args);
      break;
    case kEpiResidual:
      tcGemmKernel<kOpBf16, kEpiResidual><<<grid, kTcThreads, smem, ctx->stream>>>(args);
      break;
    default:
      tcGemmKernel<kOpBf16, kEpiStore><<<grid, kTcThreads, smem, ctx->stream>>>(args);
      break;
  }
  return launched(ctx, what);
}

int runTcGemm(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, const uint8_t *tiles,
              const float *row_scale, float *x) {
  const uint8_t *t[1] = {tiles};
  return launchTcGemm(ctx, b, p, p->kind == kOpFp8 ? kEpiRowScale : kEpiStore, 1, t, t,
                      row_scale, nullptr, nullptr, nullptr, x, "tcgen05 reconstruction");
}

template <int kSource>
int launchPackMx(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, const float *f,
                 const uint8_t *codes, const uint8_t *mx_scales, uint8_t *tiles,
                 uint8_t *scale_tiles) {
  MxPackArgs args{};
  args.work = p->pack_work;
  args.items = p->pack_items;
  args.f = f;
  args.codes = codes;
  args.mx_scales = mx_scales;
  args.f_offset = b->offset;
  args.tile_base = p->tile_base;
  args.n = b->n;
  args.tiles = tiles;
  args.scale_tiles = scale_tiles;
  packMxKernel<kSource><<<std::min(p->pack_items, kSmCount * 16), 128, 0, ctx->stream>>>(args);
  return launched(ctx, "pack block-scaled operand");
}

// X = (A * SF)(A * SF)^T from block-scaled operand tiles.
int runMxGemm(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, const uint8_t *tiles,
              const uint8_t *scale_tiles, float *x) {
  const uint8_t *t[1] = {tiles};
  return launchTcGemm(ctx, b, p, kEpiStore, 1, t, t, nullptr, nullptr, nullptr, nullptr, x,
                      "tcgen05 reconstruction", scale_tiles);
}

// Every matrix of the batch starts a 32-element block and has an order
// divisible by 32: the flat MX blocks of its codes are then row blocks.
bool rowAlignedBlocks(const DeviceBatch *b) {
  for (int i = 0; i < b->count; ++i)
    if (b->host_n[i] % 32 != 0 || b->host_offset[i] % 32 != 0) return false;
  return true;
}

template <int kSource>
int launchPack(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, const float *f,
               const uint8_t *codes, const uint8_t *mx_scales, const float *row_scale,
               uint8_t *tiles) {
  PackArgs args{};
  args.work = p->pack_work;
  args.items = p->pack_items;
  args.f = f;
  args.codes = codes;
  args.mx_scales = mx_scales;
  args.row_scale = row_scale;
  args.f_offset = b->offset;
  args.eig_offset = b->eig_offset;
  args.tile_base = p->tile_base;
  args.n = b->n;
  args.tiles = tiles;
  packKernel<kSource><<<std::min(p->pack_items, kSmCount * 16), 128, 0, ctx->stream>>>(args);
  return launched(ctx, "pack operand");
}

}  // namespace

namespace {

int packSplit(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, const float *hi, const float *lo,
              bool transpose, int pieces, uint8_t *const *out) {
  SplitArgs args{};
  args.work = p->pack_work;
  args.items = p->pack_items;
  args.hi = hi;
  args.lo = lo;
  args.offset = b->offset;
  args.tile_base = p->tile_base;
  args.n = b->n;
  args.pieces = pieces;
  for (int q = 0; q < pieces; ++q) args.out[q] = out[q];
  const unsigned grid = std::min(p->pack_items, kSmCount * 16);
  if (transpose) {
    if (lo) packSplitKernel<true, true><<<grid, 128, 0, ctx->stream>>>(args);
    else packSplitKernel<true, false><<<grid, 128, 0, ctx->stream>>>(args);
  } else {
    if (lo) packSplitKernel<false, true><<<grid, 128, 0, ctx->stream>>>(args);
    else packSplitKernel<false, false><<<grid, 128, 0, ctx->stream>>>(args);
  }
  return launched(ctx, "pack split-BF16");
}

// Scratch for split operands: kBuffers tile buffers of the BF16 plan.
constexpr int kBuffers = 6;
uint8_t *splitBuffers(msq_ctx *ctx, TcPlan *p, uint8_t *bufs[kBuffers]) {
  const size_t one = static_cast<size_t>(p->total_tiles) * kTileBytes;
  uint8_t *mem = static_cast<uint8_t *>(scratch(ctx, one * kBuffers, kScratchGemm));
  if (mem == nullptr) return nullptr;
  for (int q = 0; q < kBuffers; ++q) bufs[q] = mem + q * one;
  return mem;
}

// C = A B^T with A, B each split in two BF16 pieces: a0 b0 + a0 b1 + a1 b0
// (the dropped a1 b1 term is ~2^-16 relative).
int gemmSplit2(msq_ctx *ctx, const DeviceBatch *b, TcPlan *p, uint8_t *const *a, uint8_t *const *bb,
               int epilogue, const float *eigenvalues, float *out, const char *what) {
  const uint8_t *sa[3] = {a[0], a[0], a[1]};
  const uint8_t *sb[3] = {bb[0], bb[1], bb[0]};
  return launchTcGemm(ctx, b, p, epilogue, 3, sa, sb, nullptr, eigenvalues, nullptr, nullptr, out,
                      what);
}

}  // namespace

// One frozen-basis Sylvester sweep with every GEMM on the tensor cores
// (split-BF16 operands, FP32 accumulation in TMEM):
//   G = R V, C = (V^T G) o H, Z^T = C V^T, E = Z V^T, X <- X + (E + E^T)/2.
// The correction is residual-sized, so the ~1e-5 relative error of the
// two-piece products is far below what the next sweep can see.
int sylvesterTc(msq_ctx *ctx, const DeviceBatch *b, const float *v, const float *lam,
                const float *r, float *ws0, float *ws1, float **correction, bool basis_packed) {
  TcPlan *p = tcPlan(ctx, b, kOpBf16);
  if (p == nullptr) return MSQ_ERR_CUDA;
  uint8_t *buf[kBuffers];
  if (splitBuffers(ctx, p, buf) == nullptr) return MSQ_ERR_CUDA;
  uint8_t *vn[2] = {buf[0], buf[1]}, *vt[2] = {buf[2], buf[3]}, *op[2] = {buf[4], buf[5]};
  if (!basis_packed) {
    MSQ_TRY(packSplit(ctx, b, p, v, nullptr, false, 2, vn));  // rows = columns of V
    MSQ_TRY(packSplit(ctx, b, p, v, nullptr, true, 2, vt));   // rows = rows of V
  }
  MSQ_TRY(packSplit(ctx, b, p, r, nullptr, false, 2, op));  // R (symmetric)
  MSQ_TRY(gemmSplit2(ctx, b, p, op, vn, kEpiStore, nullptr, ws0, "tc sylvester G=RV"));
  MSQ_TRY(packSplit(ctx, b, p, ws0, nullptr, false, 2, op));
  MSQ_TRY(gemmSplit2(ctx, b, p, vn, op, kEpiInverseH, lam, ws1, "tc sylvester C=V'G/H"));
  MSQ_TRY(packSplit(ctx, b, p, ws1, nullptr, false, 2, op));
  MSQ_TRY(gemmSplit2(ctx, b, p, op, vt, kEpiStore, nullptr, ws0, "tc sylvester Zt=CV'"));
  MSQ_TRY(packSplit(ctx, b, p, ws0, nullptr, false, 2, op));
  MSQ_TRY(gemmSplit2(ctx, b, p, op, vt, kEpiStore, nullptr, ws1, "tc sylvester E=ZV'"));
  *correction = ws1;
  return MSQ_OK;
}

// R = A - X X on the tensor cores: X = x0 + x1 + x2 (BF16 pieces of the
// float-float X), X X ~ x0x0 + x0x1 + x1x0 + x0x2 + x2x0 + x1x1 accumulated
// in FP32 in one TMEM accumulator; the epilogue forms R and the FP64 norms.
// About FP32 accuracy: used between sweeps; the accepting residual is the
// float-float one.
int residualTc(msq_ctx *ctx, const DeviceBatch *b, const float *a, const float *x_hi,
               const float *x_lo, float *r, double *norms) {
  TcPlan *p = tcPlan(ctx, b, kOpBf16);
  if (p == nullptr) return MSQ_ERR_CUDA;
  uint8_t *buf[kBuffers];
  if (splitBuffers(ctx, p, buf) == nullptr) return MSQ_ERR_CUDA;
  MSQ_TRY(packSplit(ctx, b, p, x_hi, x_lo, false, 3, buf));
  const uint8_t *sa[6] = {buf[0], buf[0], buf[1], buf[0], buf[2], buf[1]};
  const uint8_t *sb[6] = {buf[0], buf[1], buf[0], buf[2], buf[0], buf[1]};
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(norms, 0, 2 * b->count * sizeof(double), ctx->stream),
                    "norm reset"));
  return launchTcGemm(ctx, b, p, kEpiResidual, 6, sa, sb, nullptr, nullptr, a, norms, r,
                      "tc residual");
}

int reconstructLowBit(msq_ctx *ctx, const DeviceBatch *b, int format, const float *f, float *x) {
  if (format == MSQ_FMT_MXFP4_E2M1) {
    // E2M1 codes with one UE8M0 scale per 32 K of a row, block-scaled MMA
    TcPlan *p = tcPlan(ctx, b, kOpMxf4);
    if (p == nullptr) return MSQ_ERR_CUDA;
    const size_t tile_bytes = static_cast<size_t>(p->total_tiles) * kTileBytes;
    uint8_t *mem = static_cast<uint8_t *>(
        scratch(ctx, tile_bytes + static_cast<size_t>(p->total_tiles) * kScaleTileBytes,
                kScratchOperand));
    if (mem == nullptr) return MSQ_ERR_CUDA;
    MSQ_TRY(launchPackMx<kMxF32Fp4>(ctx, b, p, f, nullptr, nullptr, mem, mem + tile_bytes));
    return runMxGemm(ctx, b, p, mem, mem + tile_bytes, x);
  }
  const int kind = format == MSQ_FMT_FP8_E4M3FN_ROWSCALE ? kOpFp8 : kOpBf16;
  TcPlan *p = tcPlan(ctx, b, kind);
  if (p == nullptr) return MSQ_ERR_CUDA;
  const size_t tile_bytes = static_cast<size_t>(p->total_tiles) * kTileBytes;
  const size_t rs_bytes = (b->total_order * sizeof(float) + 255) & ~size_t(255);
  uint8_t *mem = static_cast<uint8_t *>(scratch(ctx, tile_bytes + rs_bytes, kScratchOperand));
  if (mem == nullptr) return MSQ_ERR_CUDA;
  float *row_scale = reinterpret_cast<float *>(mem + tile_bytes);
  switch (format) {
    case MSQ_FMT_BF16:
      MSQ_TRY(launchPack<kPackF32Bf16>(ctx, b, p, f, nullptr, nullptr, nullptr, mem));
      break;
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE:
      rowScaleKernel<<<gridFor(b->total_order * 32, 256), 256, 0, ctx->stream>>>(
          f, b->n, b->offset, b->eig_offset, b->count, b->total_order, p->row_matrix, row_scale);
      MSQ_TRY(launched(ctx, "row scales"));
      MSQ_TRY(launchPack<kPackF32Fp8Row>(ctx, b, p, f, nullptr, nullptr, row_scale, mem));
      break;
    default:
      return setError(ctx, MSQ_ERR_UNSUPPORTED, "reconstruction format not supported");
  }
  return runTcGemm(ctx, b, p, mem, row_scale, x);
}

int reconstructEncoded(msq_ctx *ctx, const DeviceBatch *b, int format, const void *values,
                       const void *scales, float *x) {
  const int kind = format == MSQ_FMT_FP8_E4M3FN_ROWSCALE ? kOpFp8 : kOpBf16;
  if (format != MSQ_FMT_BF16 && format != MSQ_FMT_FP8_E4M3FN_ROWSCALE &&
      format != MSQ_FMT_MXFP4_E2M1 && format != MSQ_FMT_MXFP8_E4M3FN) {
    return setError(ctx, MSQ_ERR_UNSUPPORTED, "msq_reconstruct: format not supported");
  }
  if (format != MSQ_FMT_BF16 && scales == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_reconstruct: scales required");
  }
  const bool aligned = rowAlignedBlocks(b);
  if (format == MSQ_FMT_MXFP8_E4M3FN && !aligned) {
    return setError(ctx, MSQ_ERR_UNSUPPORTED,
                    "msq_reconstruct: MXFP8 needs orders and offsets divisible by 32");
  }
  if ((format == MSQ_FMT_MXFP4_E2M1 || format == MSQ_FMT_MXFP8_E4M3FN) && aligned) {
    // block-scaled MMA straight from the codes and their scale bytes
    const bool fp4 = format == MSQ_FMT_MXFP4_E2M1;
    TcPlan *p = tcPlan(ctx, b, fp4 ? kOpMxf4 : kOpMxf8);
    if (p == nullptr) return MSQ_ERR_CUDA;
    const size_t tile_bytes = static_cast<size_t>(p->total_tiles) * kTileBytes;
    uint8_t *mem = static_cast<uint8_t *>(
        scratch(ctx, tile_bytes + static_cast<size_t>(p->total_tiles) * kScaleTileBytes,
                kScratchOperand));
    if (mem == nullptr) return MSQ_ERR_CUDA;
    const uint8_t *codes = static_cast<const uint8_t *>(values);
    const uint8_t *sf = static_cast<const uint8_t *>(scales);
    if (fp4) {
      MSQ_TRY(launchPackMx<kMxCodesFp4>(ctx, b, p, nullptr, codes, sf, mem, mem + tile_bytes));
    } else {
      MSQ_TRY(launchPackMx<kMxCodesFp8>(ctx, b, p, nullptr, codes, sf, mem, mem + tile_bytes));
    }
    return runMxGemm(ctx, b, p, mem, mem + tile_bytes, x);
  }
  TcPlan *p = tcPlan(ctx, b, kind);
  if (p == nullptr) return MSQ_ERR_CUDA;
  uint8_t *mem = static_cast<uint8_t *>(
      scratch(ctx, static_cast<size_t>(p->total_tiles) * kTileBytes, kScratchOperand));
  if (mem == nullptr) return MSQ_ERR_CUDA;
  const uint8_t *codes = static_cast<const uint8_t *>(values);
  switch (format) {
    case MSQ_FMT_BF16:
      MSQ_TRY(launchPack<kPackBf16Codes>(ctx, b, p, nullptr, codes, nullptr, nullptr, mem));
      break;
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE:
      MSQ_TRY(launchPack<kPackFp8Codes>(ctx, b, p, nullptr, codes, nullptr,
                                        static_cast<const float *>(scales), mem));
      break;
    default:
      MSQ_TRY(launchPack<kPackMxfp4Codes>(ctx, b, p, nullptr, codes,
                                          reinterpret_cast<const uint8_t *>(scales), nullptr, mem));
      break;
  }
  return runTcGemm(ctx, b, p, mem,
                   kind == kOpFp8 ? static_cast<const float *>(scales) : nullptr, x);
}

}  // namespace msq
