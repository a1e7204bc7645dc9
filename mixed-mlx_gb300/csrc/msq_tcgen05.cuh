// Inline-PTX building blocks for the tcgen05 / TMA kernels (sm_103a):
// mbarriers, bulk copies, shared-memory matrix descriptors, MMA issue and
// TMEM loads / stores.  Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace msq {
namespace {

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of 16-byte chunk `chunk` of row `row` in a SWIZZLE_128B K-major
// operand: 128-byte rows, 8-row (1024-byte) atoms, chunk index XOR row mod 8.
__host__ __device__ __forceinline__ uint32_t swizzle128(int row, int chunk) {
  return (row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4);
}

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ void mbarArriveExpectTx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbarArrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Global -> shared bulk copy completing on `bar` (16-byte aligned, size a
// multiple of 16).
__device__ __forceinline__ void bulkLoad(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, 1024-byte atoms.
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr) {
  return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) |
         (static_cast<uint64_t>(1) << 16) |            // LBO (unused for SW128 K-major)
         (static_cast<uint64_t>(1024 >> 4) << 32) |    // SBO: 8-row atom stride
         (static_cast<uint64_t>(1) << 46) |            // descriptor version
         (static_cast<uint64_t>(2) << 61);             // SWIZZLE_128B
}

// Shared-memory descriptor of a no-swizzle K-major matrix whose 8-row x
// 16-byte core matrices are stored back to back (128 bytes apart along M):
// the source of tcgen05.cp for a 32-row x 16-byte scale-factor atom.
__device__ __forceinline__ uint64_t smemDescPlain(uint32_t addr) {
  return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) |
         (static_cast<uint64_t>(128 >> 4) << 16) |     // LBO (one core matrix along K)
         (static_cast<uint64_t>(128 >> 4) << 32) |     // SBO: next 8 rows
         (static_cast<uint64_t>(1) << 46);             // descriptor version, no swizzle
}

// Copies a 32-row x 128-bit scale-factor atom from shared memory into four
// consecutive TMEM columns of lanes 0-31, replicated into the lanes of all
// four sub-partitions (lane l + 32q, q = 0..3).  Ordered with the issuing
// thread's later tcgen05.mma.
__device__ __forceinline__ void tmemCopyScales(uint32_t taddr, uint64_t sdesc) {
  asm volatile("tcgen05.cp.cta_group::1.32x128b.warpx4 [%0], %1;" ::"r"(taddr), "l"(sdesc)
               : "memory");
}

// Instruction descriptor of the block-scaled kinds (kind::mxf4 with E2M1
// A and B, or kind::mxf8f6f4 with E4M3 A and B), FP32 D, K-major operands,
// M = N = 128, UE8M0 scale factors; sf_a / sf_b pick the byte of each
// scale-factor word that holds this MMA's first K block.
__host__ __device__ constexpr uint32_t instrDescBlockScaled(bool fp4, uint32_t sf_a,
                                                            uint32_t sf_b) {
  return (sf_b << 4) | ((fp4 ? 1u : 0u) << 7) | ((fp4 ? 1u : 0u) << 10) | ((128u >> 3) << 17) |
         (1u << 23) | ((128u >> 4) << 24) | (sf_a << 29);
}

// D (TMEM) = (A * SFA)(B * SFB)^T (+ D): E2M1 operands, K = 64 per MMA, two
// UE8M0 scale factors per row (one per 32 K).
__device__ __forceinline__ void mmaMxf4(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t sfa, uint32_t sfb, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %6, 0;\n"
      " tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], %1, %2, %3, [%4], "
      "[%5], p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(sfa), "r"(sfb), "r"(accumulate));
}

// E4M3 operands, K = 32 per MMA, one UE8M0 scale factor per row.
__device__ __forceinline__ void mmaMxf8(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t sfa, uint32_t sfb, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %6, 0;\n"
      " tcgen05.mma.cta_group::1.kind::mxf8f6f4.block_scale.scale_vec::1X [%0], %1, %2, %3, "
      "[%4], [%5], p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(sfa), "r"(sfb), "r"(accumulate));
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both
// operands K-major, shape M x N.
__host__ __device__ constexpr uint32_t instrDescBf16(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// D (TMEM) = A B^T (+ D if accumulate) for smem operands A (M x K) and B
// (N x K), K = 16 BF16, one thread issues.
__device__ __forceinline__ void mmaBf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// Arrives on `bar` once every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void mmaCommit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

// 32 consecutive TMEM columns of this warp's 32 lanes (lane = row).
__device__ __forceinline__ void tmemLoad32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmemStore32(uint32_t taddr, const float *v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, "
      "%29, %30, %31, %32};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
      "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
      "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
      "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
      "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
      "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
      "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
      "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
      "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
      "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

}  // namespace
}  // namespace msq
