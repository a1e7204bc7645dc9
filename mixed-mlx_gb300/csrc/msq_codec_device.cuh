// Device encoders/decoders for the storage formats of the reference's host
// codec (src/storage_codecs.cpp).  Each function is a bit-exact restatement:
//
//  * floatToBf16 (src/storage_codecs.cpp:16-28): round-half-even on the top
//    16 bits, quiet bit forced for NaN — the same integer steps.
//  * floatToFp8E4M3Fn / floatToFp8E5M2 / floatToFp4E2M1 (:96-136) pick the
//    nearest finite code by a linear scan with ties to the even code
//    (nearestFiniteCode :79-94).  Neighbouring codes are within a factor of
//    two, so the scan's FP32 distances are exact for the two candidates that
//    bracket the input and the scan equals round-to-nearest-even on the
//    value.  Here that rounding is done with integer arithmetic on the FP32
//    bits: exponent rebias plus RNE of the dropped mantissa bits, and
//    rint(x * 2^(M - emin)) below the smallest normal.  Saturation, infinity
//    and NaN rules are the reference's, branch for branch.
//  * MX scale (mxScaleExponent :148-162): e = clamp(ilogb(max finite |x|) -
//    emax, -127, 128), 0 for an all-zero block; elements are enc(x / 2^e).
//    x * 2^-e is computed as a multiplication by the normal float 2^-e,
//    which rounds exactly like the reference's division by 2^e.
//  * Decoders (:30-77, :323-374) build the FP32 bits directly; MX decode is
//    an exact ldexp (all products are representable).
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

namespace msq {

__device__ __forceinline__ uint16_t encodeBf16(float value) {
  const uint32_t bits = __float_as_uint(value);
  uint32_t rounded = bits >> 16;
  const uint32_t remainder = bits & 0xffffu;
  if (remainder > 0x8000u || (remainder == 0x8000u && (rounded & 1u) != 0)) {
    ++rounded;
  }
  if ((bits & 0x7f800000u) == 0x7f800000u && (bits & 0x007fffffu) != 0) {
    rounded |= 0x0040u;
  }
  return static_cast<uint16_t>(rounded);
}

__device__ __forceinline__ float decodeBf16(uint16_t value) {
  return __uint_as_float(static_cast<uint32_t>(value) << 16);
}

// Round a finite, positive magnitude that is not above the format's largest
// finite value to the nearest code (ties to even).  kMant = mantissa bits,
// kBias = exponent bias; codes are (exponent_field << kMant) | mantissa.
template <int kMant, int kBias>
__device__ __forceinline__ uint32_t roundMagnitude(float magnitude) {
  constexpr int kEmin = 1 - kBias;  // exponent of the smallest normal
  const uint32_t bits = __float_as_uint(magnitude);
  const int exponent = static_cast<int>(bits >> 23) - 127;
  if (exponent < kEmin) {
    // Subnormal region of the target: multiples of 2^(kEmin - kMant).
    // The scaling is exact; rint rounds half to even.
    const float scaled = magnitude * __uint_as_float(
                                         static_cast<uint32_t>(127 + kMant - kEmin) << 23);
    return static_cast<uint32_t>(rintf(scaled));
  }
  const uint32_t mantissa = bits & 0x007fffffu;
  constexpr int kDrop = 23 - kMant;
  uint32_t code = (static_cast<uint32_t>(exponent + kBias) << kMant) |
                  (mantissa >> kDrop);
  const uint32_t remainder = mantissa & ((1u << kDrop) - 1u);
  constexpr uint32_t kHalf = 1u << (kDrop - 1);
  if (remainder > kHalf || (remainder == kHalf && (code & 1u) != 0)) {
    ++code;  // carries into the exponent field, as the code order requires
  }
  return code;
}

// floatToFp8E4M3Fn (src/storage_codecs.cpp:96-108)
__device__ __forceinline__ uint8_t encodeE4M3(float value) {
  const uint32_t bits = __float_as_uint(value);
  const uint32_t sign = (bits >> 24) & 0x80u;
  const float magnitude = fabsf(value);
  if (magnitude != magnitude) return static_cast<uint8_t>(sign | 0x7fu);
  if (magnitude == 0.0f) return static_cast<uint8_t>(sign);
  if (magnitude > 448.0f) return static_cast<uint8_t>(sign | 0x7eu);  // incl. inf
  return static_cast<uint8_t>(sign | roundMagnitude<3, 7>(magnitude));
}

// floatToFp8E5M2 (src/storage_codecs.cpp:110-125)
__device__ __forceinline__ uint8_t encodeE5M2(float value) {
  const uint32_t bits = __float_as_uint(value);
  const uint32_t sign = (bits >> 24) & 0x80u;
  const float magnitude = fabsf(value);
  if (magnitude != magnitude) return static_cast<uint8_t>(sign | 0x7eu);
  if (magnitude == 0.0f) return static_cast<uint8_t>(sign);
  if (isinf(magnitude)) return static_cast<uint8_t>(sign | 0x7cu);
  if (magnitude > 57344.0f) return static_cast<uint8_t>(sign | 0x7bu);
  return static_cast<uint8_t>(sign | roundMagnitude<2, 15>(magnitude));
}

// floatToFp4E2M1 (src/storage_codecs.cpp:127-136); 4-bit code in the low nibble
__device__ __forceinline__ uint32_t encodeE2M1(float value) {
  const uint32_t bits = __float_as_uint(value);
  const uint32_t sign = (bits >> 28) & 0x8u;
  const float magnitude = fabsf(value);
  if (magnitude != magnitude || magnitude == 0.0f) return sign;
  if (magnitude > 6.0f) return sign | 0x7u;  // incl. inf
  return sign | roundMagnitude<1, 1>(magnitude);
}

// Two values to E2M1 with the hardware conversion (round to nearest even,
// saturating to +-6 for a larger magnitude or an infinity), packed with the
// even element in the low nibble.  The conversion has no NaN code; a NaN
// becomes +-0 with its sign, as floatToFp4E2M1 maps it
// (src/storage_codecs.cpp:457-466): nan_even / nan_odd are the values whose
// NaN-ness and sign decide that (the unscaled inputs, since a product may
// not keep a NaN's sign).  Same codes as encodeE2M1.
__device__ __forceinline__ uint32_t encodeE2M1Pair(float even, float odd, float nan_even,
                                                   float nan_odd) {
  uint16_t r;
  asm("{\n .reg .b8 t;\n cvt.rn.satfinite.e2m1x2.f32 t, %1, %2;\n cvt.u16.u8 %0, t;\n}"
      : "=h"(r)
      : "f"(odd), "f"(even));
  uint32_t code = r;
  if (nan_even != nan_even) code = (code & 0xf0u) | ((__float_as_uint(nan_even) >> 28) & 0x8u);
  if (nan_odd != nan_odd) code = (code & 0x0fu) | ((__float_as_uint(nan_odd) >> 24) & 0x80u);
  return code;
}

__device__ __forceinline__ float signedNan(uint32_t negative) {
  return __uint_as_float(0x7fc00000u | (negative ? 0x80000000u : 0u));
}

// fp8E4M3FnToFloat (src/storage_codecs.cpp:37-49)
__device__ __forceinline__ float decodeE4M3(uint32_t code) {
  const uint32_t sign = (code & 0x80u) << 24;
  const uint32_t exponent = (code >> 3) & 0xfu;
  const uint32_t fraction = code & 0x7u;
  if (exponent == 0xfu && fraction == 0x7u) return signedNan(sign);
  if (exponent == 0) {
    // fraction * 2^-9, exact
    return __uint_as_float(sign | __float_as_uint(static_cast<float>(fraction) *
                                                  0.001953125f));
  }
  return __uint_as_float(sign | ((exponent + 120u) << 23) | (fraction << 20));
}

// fp8E5M2ToFloat (src/storage_codecs.cpp:51-66)
__device__ __forceinline__ float decodeE5M2(uint32_t code) {
  const uint32_t sign = (code & 0x80u) << 24;
  const uint32_t exponent = (code >> 2) & 0x1fu;
  const uint32_t fraction = code & 0x3u;
  if (exponent == 0x1fu) {
    return fraction == 0 ? __uint_as_float(sign | 0x7f800000u) : signedNan(sign);
  }
  if (exponent == 0) {
    return __uint_as_float(sign | __float_as_uint(static_cast<float>(fraction) *
                                                  1.52587890625e-05f));
  }
  return __uint_as_float(sign | ((exponent + 112u) << 23) | (fraction << 21));
}

// fp4E2M1ToFloat (src/storage_codecs.cpp:68-77); code in the low nibble
__device__ __forceinline__ float decodeE2M1(uint32_t code) {
  const uint32_t sign = (code & 0x8u) << 28;
  const uint32_t exponent = (code >> 1) & 0x3u;
  const uint32_t fraction = code & 0x1u;
  if (exponent == 0) {
    return __uint_as_float(sign | (fraction ? 0x3f000000u : 0u));
  }
  return __uint_as_float(sign | ((exponent + 126u) << 23) | (fraction << 22));
}

// Two E2M1 codes (one byte, even element in the low nibble) to FP32 through
// the hardware E2M1 -> FP16 conversion, which is exact (E2M1 values have at
// most two significant bits).  Same values as decodeE2M1.
__device__ __forceinline__ float2 decodeE2M1Pair(uint32_t byte) {
  uint32_t h2;
  asm("{\n .reg .b8 t;\n cvt.u8.u32 t, %1;\n cvt.rn.f16x2.e2m1x2 %0, t;\n}" : "=r"(h2) : "r"(byte));
  return __half22float2(*reinterpret_cast<const __half2 *>(&h2));
}

// ilogb of a finite, nonzero magnitude (normal or subnormal FP32).
__device__ __forceinline__ int ilogbFinite(float magnitude) {
  const uint32_t bits = __float_as_uint(magnitude) & 0x7fffffffu;
  const int field = static_cast<int>(bits >> 23);
  if (field != 0) return field - 127;
  return (31 - __clz(static_cast<int>(bits))) - 149;
}

// mxScaleExponent (src/storage_codecs.cpp:148-162) from a block maximum of
// finite magnitudes (0 when the block holds no nonzero finite value).
__device__ __forceinline__ int mxExponent(float block_maximum, int emax) {
  if (block_maximum == 0.0f) return 0;
  int e = ilogbFinite(block_maximum) - emax;
  e = e < -127 ? -127 : e;
  e = e > 128 ? 128 : e;
  return e;
}

// 2^k as a float for k in [-126, 127].
__device__ __forceinline__ float exp2Int(int k) {
  return __uint_as_float(static_cast<uint32_t>(k + 127) << 23);
}

// x / 2^e as the reference computes it (value_at(index) / scale); e is in
// [-127, 125] for every finite block, so 2^-e is a normal float and one
// correctly rounded multiplication gives the same result as the division.
__device__ __forceinline__ float mxDivide(float x, int e) {
  // A NaN keeps its sign through the reference's host division (x86 and
  // Arm propagate the NaN operand); the GPU multiply would canonicalise it.
  if (x != x) return x;
  if (e >= -126 && e <= 126) return x * exp2Int(-e);
  // e == -127: 2^127 is normal;  e > 126 cannot come from a finite block.
  return e < 0 ? x * 1.7014118346046923e38f : __fdiv_rn(x, 8.507059173023462e37f);
}

// Row-scaled FP8 (no reference counterpart): x / s rounded once, NaN kept
// with its sign as a host division keeps it; decode is code * s.
__device__ __forceinline__ float rowDivide(float x, float s) {
  return x != x ? x : __fdiv_rn(x, s);
}
__device__ __forceinline__ float rowScaleDecode(float decoded, float s) {
  return decoded != decoded ? decoded : decoded * s;
}

// Exact ldexp of a decoded element (<= 4 significant bits) by scale - 127,
// the reference's std::ldexp(decoded, scale - 127).
__device__ __forceinline__ float mxScale(float decoded, uint32_t scale_byte) {
  if (decoded != decoded) return decoded;  // NaN bits already canonical
  const int k = static_cast<int>(scale_byte) - 127;  // [-127, 128]
  const int half = k / 2;
  return (decoded * exp2Int(half)) * exp2Int(k - half);
}

// ---- stochastic rounding ---------------------------------------------------
// The reference's device quantizers for --rounding stochastic
// (metal_mixed_sqrt.metal): stochastic_hash / stochastic_round_up :394-405,
// encode_fp8_e4m3fn_stochastic :462-484, encode_fp8_e5m2_stochastic
// :545-568, encode_fp4_e2m1_stochastic :740-763, quantize_bf16_stochastic
// :1888-1907.  A finite magnitude strictly between two codes rounds up with
// probability (|x| - lo) / (hi - lo) against a 24-bit sample of the hash of
// (element index, seed, stream); zero, NaN and magnitudes at or above the
// largest finite code take the nearest code.  Adjacent codes differ by a
// power of two, so the probability is an exact quotient.

__device__ __forceinline__ uint32_t stochasticHash(uint32_t index, uint32_t seed, uint32_t stream) {
  const uint32_t state = index * 747796405u + seed + stream * 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

__device__ __forceinline__ bool stochasticUp(float probability, uint32_t index, uint32_t seed,
                                             uint32_t stream) {
  // 24-bit sample times 2^-24 (exact)
  const float sample = static_cast<float>(stochasticHash(index, seed, stream) >> 8u) *
                       5.9604644775390625e-08f;
  return sample < probability;
}

// The code below or above a finite magnitude that lies between codes, from
// its nearest code (codes of one sign are ordered like their values).
template <class Decode>
__device__ __forceinline__ uint32_t stochasticCode(uint32_t nearest, float magnitude, Decode dec,
                                                   uint32_t index, uint32_t seed, uint32_t stream) {
  const float nearest_value = dec(nearest);
  if (nearest_value == magnitude) return nearest;
  const uint32_t lower = nearest_value < magnitude ? nearest : nearest - 1u;
  const float lo = dec(lower), hi = dec(lower + 1u);
  const float probability = __fdiv_rn(magnitude - lo, hi - lo);
  return stochasticUp(probability, index, seed, stream) ? lower + 1u : lower;
}

__device__ __forceinline__ uint8_t encodeE4M3Stochastic(float value, uint32_t index, uint32_t seed,
                                                        uint32_t stream) {
  const float magnitude = fabsf(value);
  if (value != value || magnitude == 0.0f || magnitude >= 448.0f) return encodeE4M3(value);
  const uint32_t sign = (__float_as_uint(value) >> 24) & 0x80u;
  return static_cast<uint8_t>(
      sign | stochasticCode(encodeE4M3(magnitude), magnitude,
                            [](uint32_t c) { return decodeE4M3(c); }, index, seed, stream));
}

__device__ __forceinline__ uint8_t encodeE5M2Stochastic(float value, uint32_t index, uint32_t seed,
                                                        uint32_t stream) {
  const float magnitude = fabsf(value);
  if (value != value || isinf(magnitude) || magnitude == 0.0f || magnitude >= 57344.0f) {
    return encodeE5M2(value);
  }
  const uint32_t sign = (__float_as_uint(value) >> 24) & 0x80u;
  return static_cast<uint8_t>(
      sign | stochasticCode(encodeE5M2(magnitude), magnitude,
                            [](uint32_t c) { return decodeE5M2(c); }, index, seed, stream));
}

// 4-bit code in the low nibble
__device__ __forceinline__ uint32_t encodeE2M1Stochastic(float value, uint32_t index, uint32_t seed,
                                                         uint32_t stream) {
  const float magnitude = fabsf(value);
  if (value != value || magnitude == 0.0f || magnitude >= 6.0f) return encodeE2M1(value);
  const uint32_t sign = (__float_as_uint(value) >> 28) & 0x8u;
  return sign | stochasticCode(encodeE2M1(magnitude), magnitude,
                               [](uint32_t c) { return decodeE2M1(c); }, index, seed, stream);
}

__device__ __forceinline__ uint16_t encodeBf16Stochastic(float value, uint32_t index, uint32_t seed,
                                                         uint32_t stream) {
  if (!isfinite(value) || value == 0.0f) return encodeBf16(value);
  const uint32_t bits = __float_as_uint(value);
  uint32_t rounded = bits & 0xffff0000u;
  if ((stochasticHash(index, seed, stream) & 0xffffu) < (bits & 0xffffu)) rounded += 0x00010000u;
  return static_cast<uint16_t>(rounded >> 16);
}

}  // namespace msq
