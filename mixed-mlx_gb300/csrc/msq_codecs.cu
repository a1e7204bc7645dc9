// Codec kernels: FP32 <-> BF16 / FP8 E4M3FN / FP8 E5M2 / MXFP8 / FP4 E2M1 /
// MXFP4 / FP8 E4M3FN with a per-row FP32 scale.
//
// Replaces the reference's per-element quantize/decode kernels
// (metal_mixed_sqrt.metal:384-1259, 1661-1909) and is bit-exact with its host
// codec copyToStorage / storageValueAt (src/storage_codecs.cpp:249-374).
// HBM-bound streaming work: every thread owns 8 consecutive elements
// (two 16-byte loads), an MX block of 32 elements is owned by 4 adjacent
// lanes that agree on the block maximum through two xor-shuffles, and grids
// are a multiple of the SM count with a grid-stride loop.
#include "msq_codec_device.cuh"
#include "msq_internal.cuh"

#include <algorithm>

namespace msq {
namespace {

constexpr int kThreads = 256;
constexpr int kGroup = 8;  // elements per thread

struct Group {
  float v[kGroup];
};

__device__ __forceinline__ Group loadGroup(const float *__restrict__ source,
                                           size_t base, size_t elements,
                                           bool vector_ok) {
  Group g;
  if (vector_ok && base + kGroup <= elements) {
    const float4 a = __ldcs(reinterpret_cast<const float4 *>(source + base));
    const float4 b = __ldcs(reinterpret_cast<const float4 *>(source + base + 4));
    g.v[0] = a.x; g.v[1] = a.y; g.v[2] = a.z; g.v[3] = a.w;
    g.v[4] = b.x; g.v[5] = b.y; g.v[6] = b.z; g.v[7] = b.w;
  } else {
#pragma unroll
    for (int i = 0; i < kGroup; ++i) {
      g.v[i] = base + i < elements ? source[base + i] : 0.0f;
    }
  }
  return g;
}

__device__ __forceinline__ void storeGroup(float *__restrict__ output,
                                           size_t base, size_t elements,
                                           bool vector_ok, const Group &g) {
  if (vector_ok && base + kGroup <= elements) {
    __stcs(reinterpret_cast<float4 *>(output + base),
           make_float4(g.v[0], g.v[1], g.v[2], g.v[3]));
    __stcs(reinterpret_cast<float4 *>(output + base + 4),
           make_float4(g.v[4], g.v[5], g.v[6], g.v[7]));
  } else {
#pragma unroll
    for (int i = 0; i < kGroup; ++i) {
      if (base + i < elements) output[base + i] = g.v[i];
    }
  }
}

__device__ __forceinline__ float groupMaxFinite(const Group &g) {
  float m = 0.0f;
#pragma unroll
  for (int i = 0; i < kGroup; ++i) {
    const float a = fabsf(g.v[i]);
    if (a <= 3.402823466e38f) m = fmaxf(m, a);  // finite only (NaN fails)
  }
  return m;
}

// Writes `count` bytes of `packed` (little-endian) at byte offset `at`.
__device__ __forceinline__ void storeBytes(uint8_t *__restrict__ out, size_t at,
                                           uint64_t packed, int count,
                                           bool vector_ok) {
  if (vector_ok && count == 8) {
    *reinterpret_cast<uint64_t *>(out + at) = packed;
  } else if (vector_ok && count == 4) {
    *reinterpret_cast<uint32_t *>(out + at) = static_cast<uint32_t>(packed);
  } else {
    for (int i = 0; i < count; ++i) {
      out[at + i] = static_cast<uint8_t>(packed >> (8 * i));
    }
  }
}

// ---------------------------------------------------------------- encoders

template <int kFormat>
__global__ void __launch_bounds__(kThreads)
encodeScalarKernel(const float *__restrict__ source, size_t elements,
                   uint8_t *__restrict__ values, uint8_t *__restrict__ scales,
                   bool vector_ok) {
  const size_t groups = (elements + kGroup - 1) / kGroup;
  for (size_t group = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
       group < groups; group += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t base = group * kGroup;
    const Group g = loadGroup(source, base, elements, vector_ok);
    const size_t valid = elements - base < kGroup ? elements - base : kGroup;
    if constexpr (kFormat == MSQ_FMT_BF16) {
      uint16_t h[kGroup];
#pragma unroll
      for (int i = 0; i < kGroup; ++i) h[i] = encodeBf16(g.v[i]);
      uint16_t *out = reinterpret_cast<uint16_t *>(values);
      if (vector_ok && valid == kGroup) {
        uint4 packed;
        packed.x = h[0] | (static_cast<uint32_t>(h[1]) << 16);
        packed.y = h[2] | (static_cast<uint32_t>(h[3]) << 16);
        packed.z = h[4] | (static_cast<uint32_t>(h[5]) << 16);
        packed.w = h[6] | (static_cast<uint32_t>(h[7]) << 16);
        __stcs(reinterpret_cast<uint4 *>(out + base), packed);
      } else {
        for (size_t i = 0; i < valid; ++i) out[base + i] = h[i];
      }
    } else if constexpr (kFormat == MSQ_FMT_FP8_E4M3FN ||
                         kFormat == MSQ_FMT_FP8_E5M2) {
      uint64_t packed = 0;
#pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const uint32_t code = kFormat == MSQ_FMT_FP8_E4M3FN ? encodeE4M3(g.v[i])
                                                           : encodeE5M2(g.v[i]);
        packed |= static_cast<uint64_t>(code) << (8 * i);
      }
      storeBytes(values, base, packed, static_cast<int>(valid), vector_ok);
    } else if constexpr (kFormat == MSQ_FMT_FP4_E2M1) {
      // packFp4 (src/storage_codecs.cpp:138-146): low nibble = even index,
      // the pad nibble of an odd tail is the code of +0 (= 0).
      uint64_t packed = 0;
#pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        packed |= static_cast<uint64_t>(encodeE2M1(g.v[i])) << (4 * i);
      }
      storeBytes(values, base / 2, packed, static_cast<int>((valid + 1) / 2),
                 vector_ok);
    }
    (void)scales;
  }
}

// MX formats: 4 lanes x 8 elements per 32-element scale block.
template <int kFormat>
__global__ void __launch_bounds__(kThreads)
encodeMxKernel(const float *__restrict__ source, size_t elements,
               uint8_t *__restrict__ values, uint8_t *__restrict__ scales,
               bool vector_ok) {
  constexpr int kEmax = kFormat == MSQ_FMT_MXFP8_E4M3FN ? 8
                        : kFormat == MSQ_FMT_MXFP8_E5M2 ? 15
                                                        : 2;
  const size_t blocks = (elements + 31) / 32;
  const size_t groups = blocks * 4;  // whole blocks; lanes 0-3 share one
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  // The loop condition is taken on the warp's first group so all 32 lanes
  // run the same iterations (the full-mask shuffles need every lane).
  const size_t first = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  const size_t lane = threadIdx.x % 32;
  for (size_t group = first; group - lane < groups; group += stride) {
    const bool active = group < groups;
    const size_t base = group * kGroup;
    Group g;
    if (active) {
      g = loadGroup(source, base, elements, vector_ok);
    } else {
#pragma unroll
      for (int i = 0; i < kGroup; ++i) g.v[i] = 0.0f;
    }
    float m = groupMaxFinite(g);
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
    if (!active || base >= elements) continue;
    const int e = mxExponent(m, kEmax);
    const size_t valid = elements - base < kGroup ? elements - base : kGroup;
    if (group % 4 == 0) scales[group / 4] = static_cast<uint8_t>(e + 127);
    if constexpr (kFormat == MSQ_FMT_MXFP4_E2M1) {
      uint64_t packed = 0;
      if (e >= -126 && e <= 126) {
        // x / 2^e is the exact product x * 2^-e; a NaN keeps the sign of x
        const float s = exp2Int(-e);
#pragma unroll
        for (int i = 0; i < kGroup; i += 2) {
          packed |= static_cast<uint64_t>(encodeE2M1Pair(g.v[i] * s, g.v[i + 1] * s, g.v[i], g.v[i + 1]))
                    << (4 * i);
        }
      } else {
#pragma unroll
        for (int i = 0; i < kGroup; i += 2) {
          const float a = mxDivide(g.v[i], e), b = mxDivide(g.v[i + 1], e);
          packed |= static_cast<uint64_t>(encodeE2M1Pair(a, b, a, b)) << (4 * i);
        }
      }
      storeBytes(values, base / 2, packed, static_cast<int>((valid + 1) / 2),
                 vector_ok);
    } else {
      uint64_t packed = 0;
#pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const float scaled = mxDivide(g.v[i], e);
        const uint32_t code = kFormat == MSQ_FMT_MXFP8_E4M3FN ? encodeE4M3(scaled)
                                                              : encodeE5M2(scaled);
        packed |= static_cast<uint64_t>(code) << (8 * i);
      }
      storeBytes(values, base, packed, static_cast<int>(valid), vector_ok);
    }
  }
}

constexpr int kDecodeStride = 9;  // float4 per staged block row (8 + 1 pad)

// MXFP4 encode, one 32-element block per lane: a warp loads its 32
// consecutive blocks as 512 contiguous bytes per instruction into shared
// memory (the decode kernel's padded layout), then each lane takes its
// block's maximum without shuffles, converts its 32 values with the
// hardware E2M1 conversion and stores 16 bytes of codes and its scale byte.
// Whole blocks only: the generic kernel encodes a ragged tail.
__global__ void __launch_bounds__(kThreads)
encodeMxfp4Kernel(const float *__restrict__ source, size_t blocks, uint8_t *__restrict__ values,
                  uint8_t *__restrict__ scales) {
  __shared__ float4 stage[kThreads / 32][32 * kDecodeStride];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  float4 *my = stage[warp];
  const size_t warps = static_cast<size_t>(gridDim.x) * (blockDim.x / 32);
  for (size_t first = (blockIdx.x * static_cast<size_t>(blockDim.x / 32) + warp) * 32; first < blocks;
       first += warps * 32) {
    const float4 *in = reinterpret_cast<const float4 *>(source + first * 32);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int f = 32 * q + lane;
      if (first + f / 8 < blocks) my[(f / 8) * kDecodeStride + f % 8] = __ldcs(in + f);
    }
    __syncwarp();
    const size_t blk = first + lane;
    if (blk < blocks) {
      float v[32];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 t = my[lane * kDecodeStride + j];
        v[4 * j] = t.x; v[4 * j + 1] = t.y; v[4 * j + 2] = t.z; v[4 * j + 3] = t.w;
      }
      float m = 0.0f;
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const float a = fabsf(v[i]);
        if (a <= 3.402823466e38f) m = fmaxf(m, a);  // finite only (NaN fails)
      }
      const int e = mxExponent(m, 2);
      scales[blk] = static_cast<uint8_t>(e + 127);
      uint32_t w[4] = {0u, 0u, 0u, 0u};
      if (e >= -126 && e <= 126) {
        const float s = exp2Int(-e);
#pragma unroll
        for (int i = 0; i < 32; i += 2)
          w[i / 8] |= encodeE2M1Pair(v[i] * s, v[i + 1] * s, v[i], v[i + 1]) << (4 * (i % 8));
      } else {
#pragma unroll
        for (int i = 0; i < 32; i += 2) {
          const float a = mxDivide(v[i], e), b = mxDivide(v[i + 1], e);
          w[i / 8] |= encodeE2M1Pair(a, b, a, b) << (4 * (i % 8));
        }
      }
      __stcs(reinterpret_cast<uint4 *>(values + blk * 16), make_uint4(w[0], w[1], w[2], w[3]));
    }
    __syncwarp();
  }
}

// FP8 E4M3FN with one FP32 scale per contiguous row: s = max|row| / 448
// (1 when the row has no nonzero finite value), code = E4M3(x / s).  One warp
// per row: a max pass, then an encode pass (the row is re-read from L1/L2).
__global__ void __launch_bounds__(kThreads)
encodeRowScaleKernel(const float *__restrict__ source, size_t rows,
                     size_t row_length, uint8_t *__restrict__ values,
                     float *__restrict__ scales) {
  const int lane = threadIdx.x % 32;
  const size_t warps = static_cast<size_t>(gridDim.x) * (blockDim.x / 32);
  for (size_t row = blockIdx.x * static_cast<size_t>(blockDim.x / 32) + threadIdx.x / 32;
       row < rows; row += warps) {
    const float *in = source + row * row_length;
    float m = 0.0f;
    for (size_t i = lane; i < row_length; i += 32) {
      const float a = fabsf(in[i]);
      if (a <= 3.402823466e38f) m = fmaxf(m, a);
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
    const float scale = m == 0.0f ? 1.0f : __fdiv_rn(m, 448.0f);
    if (lane == 0) scales[row] = scale;
    uint8_t *out = values + row * row_length;
    for (size_t i = lane; i < row_length; i += 32) {
      out[i] = encodeE4M3(rowDivide(in[i], scale));
    }
  }
}

// ---------------------------------------------------------------- decoders

// MXFP4 decode, one 32-element block per lane: one 16-byte load of its
// codes and its scale byte (four times the bytes in flight per thread of
// the generic kernel), the hardware E2M1 -> FP16 conversion, and one
// multiplication by 2^(scale - 127) — exact for the exponents of normal
// powers of two; the two-step product of mxScale otherwise.  A warp decodes
// 32 consecutive blocks into shared memory (row stride 9 float4: no bank
// conflicts) and stores them back as 512 contiguous bytes per instruction.
// Whole blocks only: the generic kernel decodes a ragged tail.
__global__ void __launch_bounds__(kThreads)
decodeMxfp4Kernel(const uint8_t *__restrict__ values, const uint8_t *__restrict__ scales,
                  size_t blocks, float *__restrict__ output) {
  __shared__ float4 stage[kThreads / 32][32 * kDecodeStride];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  float4 *my = stage[warp];
  const size_t warps = static_cast<size_t>(gridDim.x) * (blockDim.x / 32);
  for (size_t first = (blockIdx.x * static_cast<size_t>(blockDim.x / 32) + warp) * 32; first < blocks;
       first += warps * 32) {
    const size_t blk = first + lane;
    if (blk < blocks) {
      const uint4 p = __ldcs(reinterpret_cast<const uint4 *>(values + blk * 16));
      const uint32_t scale = scales[blk];
      const int k = static_cast<int>(scale) - 127;
      const uint32_t w[4] = {p.x, p.y, p.z, p.w};
      float4 *row = my + lane * kDecodeStride;
      if (k >= -126 && k <= 127) {
        const float s = exp2Int(k);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float2 a = decodeE2M1Pair(w[q] & 0xffu), b = decodeE2M1Pair((w[q] >> 8) & 0xffu);
          const float2 c = decodeE2M1Pair((w[q] >> 16) & 0xffu), d = decodeE2M1Pair(w[q] >> 24);
          row[2 * q] = make_float4(a.x * s, a.y * s, b.x * s, b.y * s);
          row[2 * q + 1] = make_float4(c.x * s, c.y * s, d.x * s, d.y * s);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float v[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = mxScale(decodeE2M1((w[q] >> (4 * i)) & 0xfu), scale);
          row[2 * q] = make_float4(v[0], v[1], v[2], v[3]);
          row[2 * q + 1] = make_float4(v[4], v[5], v[6], v[7]);
        }
      }
    }
    __syncwarp();
    float4 *out = reinterpret_cast<float4 *>(output + first * 32);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int f = 32 * q + lane;  // float4 index in the warp's 32 blocks
      if (first + f / 8 < blocks) __stcs(out + f, my[(f / 8) * kDecodeStride + f % 8]);
    }
    __syncwarp();
  }
}

template <int kFormat>
__global__ void __launch_bounds__(kThreads)
decodeKernel(const uint8_t *__restrict__ values, const uint8_t *__restrict__ scales,
             size_t elements, float *__restrict__ output, bool vector_ok) {
  const size_t groups = (elements + kGroup - 1) / kGroup;
  for (size_t group = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
       group < groups; group += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t base = group * kGroup;
    const size_t valid = elements - base < kGroup ? elements - base : kGroup;
    const bool full = vector_ok && valid == kGroup;
    Group g;
    if constexpr (kFormat == MSQ_FMT_BF16) {
      const uint16_t *in = reinterpret_cast<const uint16_t *>(values);
      if (full) {
        const uint4 p = __ldcs(reinterpret_cast<const uint4 *>(in + base));
        const uint32_t w[4] = {p.x, p.y, p.z, p.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          g.v[2 * i] = decodeBf16(static_cast<uint16_t>(w[i] & 0xffffu));
          g.v[2 * i + 1] = decodeBf16(static_cast<uint16_t>(w[i] >> 16));
        }
      } else {
        for (int i = 0; i < kGroup; ++i)
          g.v[i] = i < static_cast<int>(valid) ? decodeBf16(in[base + i]) : 0.0f;
      }
    } else if constexpr (kFormat == MSQ_FMT_FP4_E2M1 ||
                         kFormat == MSQ_FMT_MXFP4_E2M1) {
      uint32_t packed = 0;
      if (full) {
        packed = *reinterpret_cast<const uint32_t *>(values + base / 2);
      } else {
        for (size_t i = 0; i < (valid + 1) / 2; ++i)
          packed |= static_cast<uint32_t>(values[base / 2 + i]) << (8 * i);
      }
      const uint32_t scale = kFormat == MSQ_FMT_MXFP4_E2M1 ? scales[base / 32] : 127u;
#pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const float d = decodeE2M1((packed >> (4 * i)) & 0xfu);
        g.v[i] = kFormat == MSQ_FMT_MXFP4_E2M1 ? mxScale(d, scale) : d;
      }
    } else {
      uint64_t packed = 0;
      if (full) {
        packed = *reinterpret_cast<const uint64_t *>(values + base);
      } else {
        for (size_t i = 0; i < valid; ++i)
          packed |= static_cast<uint64_t>(values[base + i]) << (8 * i);
      }
      constexpr bool kMx = kFormat == MSQ_FMT_MXFP8_E4M3FN ||
                           kFormat == MSQ_FMT_MXFP8_E5M2;
      constexpr bool kE4M3 = kFormat == MSQ_FMT_FP8_E4M3FN ||
                             kFormat == MSQ_FMT_MXFP8_E4M3FN;
      const uint32_t scale = kMx ? scales[base / 32] : 127u;
#pragma unroll
      for (int i = 0; i < kGroup; ++i) {
        const uint32_t code = static_cast<uint32_t>(packed >> (8 * i)) & 0xffu;
        const float d = kE4M3 ? decodeE4M3(code) : decodeE5M2(code);
        g.v[i] = kMx ? mxScale(d, scale) : d;
      }
    }
    storeGroup(output, base, elements, vector_ok, g);
  }
}

__global__ void __launch_bounds__(kThreads)
decodeRowScaleKernel(const uint8_t *__restrict__ values,
                     const float *__restrict__ scales, size_t elements,
                     size_t row_length, float *__restrict__ output) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
       i < elements; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    output[i] = rowScaleDecode(decodeE4M3(values[i]), scales[i / row_length]);
  }
}

bool aligned16(const void *p) {
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// ------------------------------------------------- stochastic rounding

// Stochastic encoders (msq_encode_stochastic): one thread per element, the
// element's flat index feeding the hash; FP4 lanes pair up by shuffle (the
// even lane writes the byte); MX formats take one warp per 32-element block
// (the block's finite maximum by a warp reduction, then x / 2^e per lane as
// the nearest encoders compute it).  The loop is warp-uniform.
template <int kFormat>
__global__ void __launch_bounds__(kThreads)
encodeStochasticKernel(const float *__restrict__ source, size_t elements, uint32_t seed,
                       uint32_t stream, uint8_t *__restrict__ values,
                       uint8_t *__restrict__ scales) {
  constexpr bool kMx = kFormat == MSQ_FMT_MXFP8_E4M3FN || kFormat == MSQ_FMT_MXFP8_E5M2 ||
                       kFormat == MSQ_FMT_MXFP4_E2M1;
  constexpr bool kFp4 = kFormat == MSQ_FMT_FP4_E2M1 || kFormat == MSQ_FMT_MXFP4_E2M1;
  const int lane = threadIdx.x & 31;
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t base = blockIdx.x * static_cast<size_t>(blockDim.x) + (threadIdx.x & ~31u);
       base < elements; base += stride) {
    const size_t i = base + lane;
    const bool valid = i < elements;
    float x = valid ? source[i] : 0.0f;
    if constexpr (kMx) {
      constexpr int kEmax = kFormat == MSQ_FMT_MXFP8_E4M3FN ? 8 : (kFormat == MSQ_FMT_MXFP8_E5M2 ? 15 : 2);
      const float a = fabsf(x);
      // finite magnitudes order like their bits
      uint32_t m = valid && a <= 3.402823466e38f ? __float_as_uint(a) : 0u;
      m = __reduce_max_sync(0xffffffffu, m);
      const int e = mxExponent(__uint_as_float(m), kEmax);
      if (lane == 0) scales[base / 32] = static_cast<uint8_t>(e + 127);
      x = mxDivide(x, e);
    }
    const uint32_t index = static_cast<uint32_t>(i);
    if constexpr (kFormat == MSQ_FMT_BF16) {
      if (valid) reinterpret_cast<uint16_t *>(values)[i] = encodeBf16Stochastic(x, index, seed, stream);
    } else if constexpr (kFormat == MSQ_FMT_FP8_E4M3FN || kFormat == MSQ_FMT_MXFP8_E4M3FN) {
      if (valid) values[i] = encodeE4M3Stochastic(x, index, seed, stream);
    } else if constexpr (kFormat == MSQ_FMT_FP8_E5M2 || kFormat == MSQ_FMT_MXFP8_E5M2) {
      if (valid) values[i] = encodeE5M2Stochastic(x, index, seed, stream);
    } else {
      static_assert(kFp4, "format");
      const uint32_t code = valid ? encodeE2M1Stochastic(x, index, seed, stream) : 0u;
      const uint32_t next = __shfl_down_sync(0xffffffffu, code, 1);
      if (valid && (i & 1) == 0) {
        values[i / 2] = static_cast<uint8_t>(code | (i + 1 < elements ? next << 4 : 0u));
      }
    }
  }
}

// Row-scaled FP8 with stochastic rounding: one warp per row as the nearest
// row-scale encoder, each element rounded with its flat index.
__global__ void __launch_bounds__(kThreads)
encodeRowScaleStochasticKernel(const float *__restrict__ source, size_t rows, size_t row_length,
                               uint32_t seed, uint32_t stream, uint8_t *__restrict__ values,
                               float *__restrict__ scales) {
  const int lane = threadIdx.x % 32;
  const size_t warps = static_cast<size_t>(gridDim.x) * (blockDim.x / 32);
  for (size_t row = blockIdx.x * static_cast<size_t>(blockDim.x / 32) + threadIdx.x / 32;
       row < rows; row += warps) {
    const float *in = source + row * row_length;
    float m = 0.0f;
    for (size_t i = lane; i < row_length; i += 32) {
      const float a = fabsf(in[i]);
      if (a <= 3.402823466e38f) m = fmaxf(m, a);
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
    const float scale = m == 0.0f ? 1.0f : __fdiv_rn(m, 448.0f);
    if (lane == 0) scales[row] = scale;
    uint8_t *out = values + row * row_length;
    for (size_t i = lane; i < row_length; i += 32) {
      out[i] = encodeE4M3Stochastic(rowDivide(in[i], scale),
                                    static_cast<uint32_t>(row * row_length + i), seed, stream);
    }
  }
}

// ------------------------------------------------- log-spectrum storage

// fp8_e4m3fn_log_s / fp4_e2m1_log_s (src/precision.hpp:87-92) in the
// device form of metal_mixed_sqrt.metal:1689-1804: per block of 8 root
// eigenvalues (min, span) of log2 s, the span lowered by one ulp when
// min + span rounds above the block's maximum log (so the top code decodes
// at or below the largest input); codes of maximum * (log2 s - min) / span
// (maximum 448 or 6), nearest or stochastic; decode exp2(min + span *
// dec(code) / maximum).  A value that is not finite and positive sets
// kStatusBadSpectrum (the reference host codec fails on it).
constexpr int kSpectrumBlock = 8;

__global__ void __launch_bounds__(kThreads)
spectrumMetadataKernel(const float *__restrict__ spectrum, size_t elements,
                       float2 *__restrict__ metadata, int *status) {
  const size_t blocks = (elements + kSpectrumBlock - 1) / kSpectrumBlock;
  for (size_t b = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; b < blocks;
       b += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t begin = b * kSpectrumBlock;
    const size_t end = begin + kSpectrumBlock < elements ? begin + kSpectrumBlock : elements;
    float lo = __uint_as_float(0x7f800000u), hi = -lo;
    bool bad = false;
    for (size_t i = begin; i < end; ++i) {
      const float v = spectrum[i];
      bad = bad || !(v > 0.0f) || !(v <= 3.402823466e38f);
      const float l = log2f(v);
      lo = fminf(lo, l);
      hi = fmaxf(hi, l);
    }
    if (bad) {
      atomicExch(status, kStatusBadSpectrum);
      lo = hi = 0.0f;
    }
    float span = hi - lo;
    if (lo + span > hi) span = nextafterf(span, 0.0f);
    metadata[b] = make_float2(lo, span);
  }
}

template <int kFormat>
__device__ __forceinline__ float spectrumScaled(const float *spectrum, const float2 *metadata,
                                                size_t i) {
  constexpr float kMax = kFormat == MSQ_FMT_FP8_E4M3FN ? 448.0f : 6.0f;
  const float2 block = metadata[i / kSpectrumBlock];
  return block.y == 0.0f ? 0.0f : __fdiv_rn(kMax * (log2f(spectrum[i]) - block.x), block.y);
}

// One thread per element; FP4 lanes pair up by shuffle (warp-uniform loop).
template <int kFormat>
__global__ void __launch_bounds__(kThreads)
spectrumEncodeKernel(const float *__restrict__ spectrum, size_t elements,
                     const float2 *__restrict__ metadata, int stochastic, uint32_t seed,
                     uint32_t stream, uint8_t *__restrict__ values) {
  const int lane = threadIdx.x & 31;
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t base = blockIdx.x * static_cast<size_t>(blockDim.x) + (threadIdx.x & ~31u);
       base < elements; base += stride) {
    const size_t i = base + lane;
    const bool valid = i < elements;
    const float x = valid ? spectrumScaled<kFormat>(spectrum, metadata, i) : 0.0f;
    const uint32_t index = static_cast<uint32_t>(i);
    if constexpr (kFormat == MSQ_FMT_FP8_E4M3FN) {
      if (valid) values[i] = stochastic ? encodeE4M3Stochastic(x, index, seed, stream) : encodeE4M3(x);
    } else {
      const uint32_t code =
          valid ? (stochastic ? encodeE2M1Stochastic(x, index, seed, stream) : encodeE2M1(x)) : 0u;
      const uint32_t next = __shfl_down_sync(0xffffffffu, code, 1);
      if (valid && (i & 1) == 0) {
        values[i / 2] = static_cast<uint8_t>(code | (i + 1 < elements ? next << 4 : 0u));
      }
    }
  }
}

template <int kFormat>
__global__ void __launch_bounds__(kThreads)
spectrumDecodeKernel(const uint8_t *__restrict__ values, const float2 *__restrict__ metadata,
                     size_t elements, float *__restrict__ spectrum) {
  constexpr float kMax = kFormat == MSQ_FMT_FP8_E4M3FN ? 448.0f : 6.0f;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < elements;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const float2 block = metadata[i / kSpectrumBlock];
    const float d = kFormat == MSQ_FMT_FP8_E4M3FN ? decodeE4M3(values[i])
                                                 : decodeE2M1((values[i / 2] >> ((i & 1) * 4)) & 0xfu);
    spectrum[i] = exp2f(block.x + __fdiv_rn(block.y * d, kMax));
  }
}

// Q(x) = decode(encode(x)) in place for every matrix of a batch, one
// launch: the per-element steps of the encode and decode kernels above,
// with MX blocks of 32 consecutive elements and scale rows of n elements
// taken within each matrix (n^2 elements from its offset), so the result is
// the encode -> decode round trip of each matrix on its own.
template <int kFormat>
__global__ void __launch_bounds__(kThreads)
quantizeBatchKernel(float *__restrict__ x, const int64_t *__restrict__ offset,
                    const int32_t *__restrict__ n, int count) {
  constexpr bool kMx = kFormat == MSQ_FMT_MXFP8_E4M3FN || kFormat == MSQ_FMT_MXFP8_E5M2 ||
                       kFormat == MSQ_FMT_MXFP4_E2M1;
  constexpr int kEmax = kFormat == MSQ_FMT_MXFP8_E4M3FN ? 8 : kFormat == MSQ_FMT_MXFP8_E5M2 ? 15 : 2;
  for (int mi = blockIdx.y; mi < count; mi += gridDim.y) {
    const int nn = n[mi];
    const int64_t elements = static_cast<int64_t>(nn) * nn;
    float *p = x + offset[mi];
    if constexpr (kFormat == MSQ_FMT_FP8_E4M3FN_ROWSCALE) {
      // one warp per row of n consecutive elements (encodeRowScaleKernel)
      const int lane = threadIdx.x % 32;
      const int warps = gridDim.x * (blockDim.x / 32);
      for (int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; row < nn; row += warps) {
        float *in = p + static_cast<int64_t>(row) * nn;
        float m = 0.0f;
        for (int i = lane; i < nn; i += 32) {
          const float a = fabsf(in[i]);
          if (a <= 3.402823466e38f) m = fmaxf(m, a);
        }
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, sh));
        const float scale = m == 0.0f ? 1.0f : __fdiv_rn(m, 448.0f);
        for (int i = lane; i < nn; i += 32)
          in[i] = rowScaleDecode(decodeE4M3(encodeE4M3(rowDivide(in[i], scale))), scale);
      }
    } else if constexpr (kMx) {
      // one thread per 32-element block (encodeMxKernel / decodeKernel)
      const int64_t blocks = (elements + 31) / 32;
      for (int64_t blk = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; blk < blocks;
           blk += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t base = blk * 32;
        float v[32];
        float m = 0.0f;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          v[i] = base + i < elements ? p[base + i] : 0.0f;
          const float a = fabsf(v[i]);
          if (a <= 3.402823466e38f) m = fmaxf(m, a);  // finite only (NaN fails)
        }
        const int e = mxExponent(m, kEmax);
        const uint32_t scale = static_cast<uint32_t>(e + 127);
        if constexpr (kFormat == MSQ_FMT_MXFP4_E2M1) {
          const bool exact = e >= -126 && e <= 126;
          const float sc = exact ? exp2Int(-e) : 1.0f;
#pragma unroll
          for (int i = 0; i < 32; i += 2) {
            uint32_t pair;
            if (exact) {
              pair = encodeE2M1Pair(v[i] * sc, v[i + 1] * sc, v[i], v[i + 1]);
            } else {
              const float a = mxDivide(v[i], e), b = mxDivide(v[i + 1], e);
              pair = encodeE2M1Pair(a, b, a, b);
            }
            v[i] = mxScale(decodeE2M1(pair & 0xfu), scale);
            v[i + 1] = mxScale(decodeE2M1((pair >> 4) & 0xfu), scale);
          }
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const float scaled = mxDivide(v[i], e);
            const float d = kFormat == MSQ_FMT_MXFP8_E4M3FN ? decodeE4M3(encodeE4M3(scaled))
                                                            : decodeE5M2(encodeE5M2(scaled));
            v[i] = mxScale(d, scale);
          }
        }
#pragma unroll
        for (int i = 0; i < 32; ++i)
          if (base + i < elements) p[base + i] = v[i];
      }
    } else {
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < elements;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float y = p[i];
        if constexpr (kFormat == MSQ_FMT_BF16) p[i] = decodeBf16(encodeBf16(y));
        else if constexpr (kFormat == MSQ_FMT_FP8_E4M3FN) p[i] = decodeE4M3(encodeE4M3(y));
        else if constexpr (kFormat == MSQ_FMT_FP8_E5M2) p[i] = decodeE5M2(encodeE5M2(y));
        else p[i] = decodeE2M1(encodeE2M1(y));  // FP4 E2M1
      }
    }
  }
}

}  // namespace

int quantizeBatch(msq_ctx *ctx, int format, const DeviceBatch *b, float *x) {
  if (format == MSQ_FMT_FP32) return MSQ_OK;
  const int64_t nn = static_cast<int64_t>(b->max_n) * b->max_n;
  int64_t units = nn;                                               // elements
  if (format == MSQ_FMT_FP8_E4M3FN_ROWSCALE) units = static_cast<int64_t>(b->max_n) * 32;  // a warp per row
  else if (format == MSQ_FMT_MXFP8_E4M3FN || format == MSQ_FMT_MXFP8_E5M2 ||
           format == MSQ_FMT_MXFP4_E2M1) units = (nn + 31) / 32;   // a thread per block
  const dim3 grid(static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((units + kThreads - 1) / kThreads, 64))),
                  static_cast<unsigned>(std::min(b->count, 65535)));
  switch (format) {
#define MSQ_QUANTIZE_CASE(F)                                                                   \
    case F:                                                                                   \
      quantizeBatchKernel<F><<<grid, kThreads, 0, ctx->stream>>>(x, b->offset, b->n, b->count); \
      break;
    MSQ_QUANTIZE_CASE(MSQ_FMT_BF16)
    MSQ_QUANTIZE_CASE(MSQ_FMT_FP8_E4M3FN)
    MSQ_QUANTIZE_CASE(MSQ_FMT_FP8_E5M2)
    MSQ_QUANTIZE_CASE(MSQ_FMT_MXFP8_E4M3FN)
    MSQ_QUANTIZE_CASE(MSQ_FMT_MXFP8_E5M2)
    MSQ_QUANTIZE_CASE(MSQ_FMT_FP4_E2M1)
    MSQ_QUANTIZE_CASE(MSQ_FMT_MXFP4_E2M1)
    MSQ_QUANTIZE_CASE(MSQ_FMT_FP8_E4M3FN_ROWSCALE)
#undef MSQ_QUANTIZE_CASE
    default:
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "quantize: unknown format");
  }
  return launched(ctx, "quantize");
}

}  // namespace msq

using namespace msq;

extern "C" size_t msq_storage_bytes(int format, size_t elements) {
  switch (format) {
    case MSQ_FMT_FP32: return elements * 4;
    case MSQ_FMT_BF16: return elements * 2;
    case MSQ_FMT_FP8_E4M3FN:
    case MSQ_FMT_FP8_E5M2:
    case MSQ_FMT_MXFP8_E4M3FN:
    case MSQ_FMT_MXFP8_E5M2:
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE: return elements;
    case MSQ_FMT_FP4_E2M1:
    case MSQ_FMT_MXFP4_E2M1: return (elements * 4 + 7) / 8;
    default: return 0;
  }
}

extern "C" size_t msq_scale_bytes(int format, size_t elements, size_t row_length) {
  switch (format) {
    case MSQ_FMT_MXFP8_E4M3FN:
    case MSQ_FMT_MXFP8_E5M2:
    case MSQ_FMT_MXFP4_E2M1: return (elements + 31) / 32;
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE:
      return row_length == 0 ? 0 : (elements / row_length) * sizeof(float);
    default: return 0;
  }
}

extern "C" int msq_encode(msq_ctx *ctx, int format, const float *source,
                          size_t elements, size_t row_length, uint8_t *values,
                          uint8_t *scales) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (elements == 0) return MSQ_OK;
  if (source == nullptr || values == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_encode: null buffer");
  }
  const bool needs_scales = msq_scale_bytes(format, elements, row_length ? row_length : 1) != 0;
  if (needs_scales && scales == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_encode: this format requires a scale plane");
  }
  const bool vec = aligned16(source) && aligned16(values);
  const size_t groups = (elements + kGroup - 1) / kGroup;
  const unsigned grid = gridFor(groups, kThreads);
  cudaStream_t s = ctx->stream;
  switch (format) {
    case MSQ_FMT_FP32:
      return cudaCheck(ctx, cudaMemcpyAsync(values, source, elements * 4,
                                            cudaMemcpyDeviceToDevice, s),
                       "msq_encode fp32 copy");
    case MSQ_FMT_BF16:
      encodeScalarKernel<MSQ_FMT_BF16><<<grid, kThreads, 0, s>>>(source, elements, values, scales, vec);
      break;
    case MSQ_FMT_FP8_E4M3FN:
      encodeScalarKernel<MSQ_FMT_FP8_E4M3FN><<<grid, kThreads, 0, s>>>(source, elements, values, scales, vec);
      break;
    case MSQ_FMT_FP8_E5M2:
      encodeScalarKernel<MSQ_FMT_FP8_E5M2><<<grid, kThreads, 0, s>>>(source, elements, values, scales, vec);
      break;
    case MSQ_FMT_FP4_E2M1:
      encodeScalarKernel<MSQ_FMT_FP4_E2M1><<<grid, kThreads, 0, s>>>(source, elements, values, scales, vec);
      break;
    case MSQ_FMT_MXFP8_E4M3FN:
      encodeMxKernel<MSQ_FMT_MXFP8_E4M3FN><<<gridFor((elements + 31) / 32 * 4, kThreads), kThreads, 0, s>>>(source, elements, values, scales, vec);
      break;
    case MSQ_FMT_MXFP8_E5M2:
      encodeMxKernel<MSQ_FMT_MXFP8_E5M2><<<gridFor((elements + 31) / 32 * 4, kThreads), kThreads, 0, s>>>(source, elements, values, scales, vec);
      break;
    case MSQ_FMT_MXFP4_E2M1:
      if (vec && elements >= 32) {
        const size_t whole = elements / 32;
        encodeMxfp4Kernel<<<gridFor(whole, kThreads), kThreads, 0, s>>>(source, whole, values, scales);
        if (whole * 32 < elements) {
          MSQ_TRY(launched(ctx, "msq_encode"));
          const size_t rest = elements - whole * 32;
          encodeMxKernel<MSQ_FMT_MXFP4_E2M1><<<1, kThreads, 0, s>>>(
              source + whole * 32, rest, values + whole * 16, scales + whole, vec);
        }
      } else {
        encodeMxKernel<MSQ_FMT_MXFP4_E2M1><<<gridFor((elements + 31) / 32 * 4, kThreads), kThreads, 0, s>>>(source, elements, values, scales, vec);
      }
      break;
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE: {
      if (row_length == 0 || elements % row_length != 0) {
        return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                        "msq_encode: elements must be a multiple of row_length");
      }
      const size_t rows = elements / row_length;
      encodeRowScaleKernel<<<gridFor(rows * 32, kThreads), kThreads, 0, s>>>(
          source, rows, row_length, values, reinterpret_cast<float *>(scales));
      break;
    }
    default:
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_encode: unknown format");
  }
  return launched(ctx, "msq_encode");
}

extern "C" int msq_decode(msq_ctx *ctx, int format, const uint8_t *values,
                          const uint8_t *scales, size_t elements,
                          size_t row_length, float *output) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (elements == 0) return MSQ_OK;
  if (values == nullptr || output == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_decode: null buffer");
  }
  const bool needs_scales = msq_scale_bytes(format, elements, row_length ? row_length : 1) != 0;
  if (needs_scales && scales == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_decode: this format requires a scale plane");
  }
  const bool vec = aligned16(values) && aligned16(output);
  const size_t groups = (elements + kGroup - 1) / kGroup;
  const unsigned grid = gridFor(groups, kThreads);
  cudaStream_t s = ctx->stream;
  switch (format) {
    case MSQ_FMT_FP32:
      return cudaCheck(ctx, cudaMemcpyAsync(output, values, elements * 4,
                                            cudaMemcpyDeviceToDevice, s),
                       "msq_decode fp32 copy");
    case MSQ_FMT_MXFP4_E2M1:
      if (vec && elements >= 32) {
        const size_t whole = elements / 32;
        decodeMxfp4Kernel<<<gridFor(whole, kThreads), kThreads, 0, s>>>(values, scales, whole, output);
        if (whole * 32 < elements) {
          MSQ_TRY(launched(ctx, "msq_decode"));
          decodeKernel<MSQ_FMT_MXFP4_E2M1><<<1, kThreads, 0, s>>>(
              values + whole * 16, scales + whole, elements - whole * 32, output + whole * 32, vec);
        }
      } else {
        decodeKernel<MSQ_FMT_MXFP4_E2M1><<<grid, kThreads, 0, s>>>(values, scales, elements, output, vec);
      }
      break;
#define MSQ_DECODE_CASE(F) \
    case F: decodeKernel<F><<<grid, kThreads, 0, s>>>(values, scales, elements, output, vec); break;
    MSQ_DECODE_CASE(MSQ_FMT_BF16)
    MSQ_DECODE_CASE(MSQ_FMT_FP8_E4M3FN)
    MSQ_DECODE_CASE(MSQ_FMT_FP8_E5M2)
    MSQ_DECODE_CASE(MSQ_FMT_MXFP8_E4M3FN)
    MSQ_DECODE_CASE(MSQ_FMT_MXFP8_E5M2)
    MSQ_DECODE_CASE(MSQ_FMT_FP4_E2M1)
#undef MSQ_DECODE_CASE
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE:
      if (row_length == 0 || elements % row_length != 0) {
        return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                        "msq_decode: elements must be a multiple of row_length");
      }
      decodeRowScaleKernel<<<gridFor(elements, kThreads), kThreads, 0, s>>>(
          values, reinterpret_cast<const float *>(scales), elements, row_length, output);
      break;
    default:
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_decode: unknown format");
  }
  return launched(ctx, "msq_decode");
}

extern "C" int msq_encode_stochastic(msq_ctx *ctx, int format, const float *source,
                                     size_t elements, size_t row_length, uint32_t seed,
                                     uint32_t stream, uint8_t *values, uint8_t *scales) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (elements == 0) return MSQ_OK;
  if (source == nullptr || values == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_encode_stochastic: null buffer");
  }
  const bool needs_scales = msq_scale_bytes(format, elements, row_length ? row_length : 1) != 0;
  if (needs_scales && scales == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_encode_stochastic: this format requires a scale plane");
  }
  cudaStream_t s = ctx->stream;
  const unsigned grid = gridFor((elements + 31) / 32 * 32, kThreads);
  switch (format) {
    case MSQ_FMT_FP32:
      return cudaCheck(ctx, cudaMemcpyAsync(values, source, elements * 4,
                                            cudaMemcpyDeviceToDevice, s),
                       "msq_encode_stochastic fp32 copy");
    case MSQ_FMT_BF16:
      encodeStochasticKernel<MSQ_FMT_BF16><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_FP8_E4M3FN:
      encodeStochasticKernel<MSQ_FMT_FP8_E4M3FN><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_FP8_E5M2:
      encodeStochasticKernel<MSQ_FMT_FP8_E5M2><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_FP4_E2M1:
      encodeStochasticKernel<MSQ_FMT_FP4_E2M1><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_MXFP8_E4M3FN:
      encodeStochasticKernel<MSQ_FMT_MXFP8_E4M3FN><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_MXFP8_E5M2:
      encodeStochasticKernel<MSQ_FMT_MXFP8_E5M2><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_MXFP4_E2M1:
      encodeStochasticKernel<MSQ_FMT_MXFP4_E2M1><<<grid, kThreads, 0, s>>>(source, elements, seed, stream, values, scales);
      break;
    case MSQ_FMT_FP8_E4M3FN_ROWSCALE: {
      if (row_length == 0 || elements % row_length != 0) {
        return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                        "msq_encode_stochastic: elements must be a multiple of row_length");
      }
      const size_t rows = elements / row_length;
      encodeRowScaleStochasticKernel<<<gridFor(rows * 32, kThreads), kThreads, 0, s>>>(
          source, rows, row_length, seed, stream, values, reinterpret_cast<float *>(scales));
      break;
    }
    default:
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_encode_stochastic: unknown format");
  }
  return launched(ctx, "msq_encode_stochastic");
}

extern "C" size_t msq_spectrum_metadata_bytes(size_t elements) {
  return 2 * sizeof(float) * ((elements + kSpectrumBlock - 1) / kSpectrumBlock);
}

extern "C" int msq_spectrum_encode(msq_ctx *ctx, int format, const float *spectrum,
                                   size_t elements, int rounding, uint32_t seed, uint32_t stream,
                                   uint8_t *values, float *metadata) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (elements == 0) return MSQ_OK;
  if (spectrum == nullptr || values == nullptr || metadata == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_spectrum_encode: null buffer");
  }
  if (format != MSQ_FMT_FP8_E4M3FN && format != MSQ_FMT_FP4_E2M1) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_spectrum_encode: log-spectrum storage uses FP8-E4M3FN or FP4-E2M1 codes");
  }
  if (rounding != MSQ_ROUND_NEAREST && rounding != MSQ_ROUND_STOCHASTIC) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_spectrum_encode: unknown rounding mode");
  }
  if (reinterpret_cast<uintptr_t>(metadata) % 8 != 0) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_spectrum_encode: metadata not 8-byte aligned");
  }
  cudaStream_t s = ctx->stream;
  float2 *meta = reinterpret_cast<float2 *>(metadata);
  const size_t blocks = (elements + kSpectrumBlock - 1) / kSpectrumBlock;
  spectrumMetadataKernel<<<gridFor(blocks, kThreads), kThreads, 0, s>>>(spectrum, elements, meta,
                                                                       ctx->d_status);
  MSQ_TRY(launched(ctx, "msq_spectrum_encode"));
  const unsigned grid = gridFor((elements + 31) / 32 * 32, kThreads);
  const int stochastic = rounding == MSQ_ROUND_STOCHASTIC;
  if (format == MSQ_FMT_FP8_E4M3FN) {
    spectrumEncodeKernel<MSQ_FMT_FP8_E4M3FN><<<grid, kThreads, 0, s>>>(spectrum, elements, meta,
                                                                        stochastic, seed, stream, values);
  } else {
    spectrumEncodeKernel<MSQ_FMT_FP4_E2M1><<<grid, kThreads, 0, s>>>(spectrum, elements, meta,
                                                                      stochastic, seed, stream, values);
  }
  return launched(ctx, "msq_spectrum_encode");
}

extern "C" int msq_spectrum_decode(msq_ctx *ctx, int format, const uint8_t *values,
                                   const float *metadata, size_t elements, float *spectrum) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (elements == 0) return MSQ_OK;
  if (spectrum == nullptr || values == nullptr || metadata == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_spectrum_decode: null buffer");
  }
  if (format != MSQ_FMT_FP8_E4M3FN && format != MSQ_FMT_FP4_E2M1) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_spectrum_decode: log-spectrum storage uses FP8-E4M3FN or FP4-E2M1 codes");
  }
  if (reinterpret_cast<uintptr_t>(metadata) % 8 != 0) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_spectrum_decode: metadata not 8-byte aligned");
  }
  cudaStream_t s = ctx->stream;
  const float2 *meta = reinterpret_cast<const float2 *>(metadata);
  if (format == MSQ_FMT_FP8_E4M3FN) {
    spectrumDecodeKernel<MSQ_FMT_FP8_E4M3FN><<<gridFor(elements, kThreads), kThreads, 0, s>>>(
        values, meta, elements, spectrum);
  } else {
    spectrumDecodeKernel<MSQ_FMT_FP4_E2M1><<<gridFor(elements, kThreads), kThreads, 0, s>>>(
        values, meta, elements, spectrum);
  }
  return launched(ctx, "msq_spectrum_decode");
}
