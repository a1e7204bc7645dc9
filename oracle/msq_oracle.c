/*
 * msq_oracle.c — CPU restatement of the reference's algorithms for the SPD
 * square-root hot path.  TEST INFRASTRUCTURE: only tests/, the smoke check
 * and bench.py's CPU-baseline leg load this library, and only as the checker
 * (or as the timed CPU baseline); the product path never calls it.
 *
 * Pinned against the reference itself: tests/golden holds vectors produced by
 * the reference's own host codec (oracle/_ref, compiled from the reference
 * sources) and tests/test_oracle.py checks this file against them.
 *
 * Contents
 *  - codecs: the reference host codec (src/storage_codecs.cpp) restated with
 *    its linear nearest-code scan, so it is independent of the integer
 *    rounding the CUDA kernels use;
 *  - the FP8-E4M3 per-row-scale format (no reference counterpart);
 *  - the device quantizers' stochastic rounding and the log-spectrum
 *    storage of the root eigenvalues (restated from the shader source);
 *  - one correction of the native-quantized mode;
 *  - the symmetric paper test sets V-VII (generator and Hilbert matrix);
 *  - the parallel-order two-sided Jacobi of metal_mixed_sqrt.metal:1319-1444
 *    with the round-robin schedule of src/metal_solver.cpp:50-79, angles in
 *    FP64, FP32 storage, convergence-tested;
 *  - the float-float ("WorkingFloat") residual of
 *    metal_mixed_sqrt.metal:1278-1317, 1927-1942.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ codecs */

/* floatToBf16, src/storage_codecs.cpp:16-28 */
uint16_t msqo_encode_bf16(float value) {
  uint32_t bits;
  memcpy(&bits, &value, 4);
  uint32_t rounded = bits >> 16;
  uint32_t remainder = bits & 0xffffu;
  if (remainder > 0x8000u || (remainder == 0x8000u && (rounded & 1u) != 0))
    ++rounded;
  if ((bits & 0x7f800000u) == 0x7f800000u && (bits & 0x007fffffu) != 0)
    rounded |= 0x0040u;
  return (uint16_t)rounded;
}

/* bf16ToFloat, :30-35 */
float msqo_decode_bf16(uint16_t value) {
  uint32_t bits = (uint32_t)value << 16;
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

/* fp8E4M3FnToFloat, :37-49 */
float msqo_decode_e4m3(uint8_t value) {
  float sign = (value & 0x80u) == 0 ? 1.0f : -1.0f;
  unsigned exponent = (value >> 3) & 0x0fu, fraction = value & 0x07u;
  if (exponent == 0x0fu && fraction == 0x07u) return copysignf(NAN, sign);
  float magnitude = exponent == 0
                        ? ldexpf((float)fraction, -9)
                        : ldexpf(1.0f + (float)fraction / 8.0f, (int)exponent - 7);
  return copysignf(magnitude, sign);
}

/* fp8E5M2ToFloat, :51-66 */
float msqo_decode_e5m2(uint8_t value) {
  float sign = (value & 0x80u) == 0 ? 1.0f : -1.0f;
  unsigned exponent = (value >> 2) & 0x1fu, fraction = value & 0x03u;
  if (exponent == 0x1fu)
    return fraction == 0 ? copysignf(INFINITY, sign) : copysignf(NAN, sign);
  float magnitude = exponent == 0
                        ? ldexpf((float)fraction, -16)
                        : ldexpf(1.0f + (float)fraction / 4.0f, (int)exponent - 15);
  return copysignf(magnitude, sign);
}

/* fp4E2M1ToFloat, :68-77 */
float msqo_decode_e2m1(uint8_t value) {
  float sign = (value & 0x08u) == 0 ? 1.0f : -1.0f;
  unsigned exponent = (value >> 1) & 0x03u, fraction = value & 0x01u;
  float magnitude = exponent == 0
                        ? (float)fraction * 0.5f
                        : ldexpf(1.0f + (float)fraction * 0.5f, (int)exponent - 1);
  return copysignf(magnitude, sign);
}

/* nearestFiniteCode, :79-94: scan all finite codes, ties to the even code */
static uint8_t nearest_code(float magnitude, unsigned maximum_code,
                            float (*decode)(uint8_t)) {
  uint8_t nearest = 0;
  float best = fabsf(magnitude - decode(0));
  for (unsigned code = 1; code <= maximum_code; ++code) {
    float distance = fabsf(magnitude - decode((uint8_t)code));
    if (distance < best || (distance == best && (code & 1u) == 0 && (nearest & 1u) != 0)) {
      nearest = (uint8_t)code;
      best = distance;
    }
  }
  return nearest;
}

/* floatToFp8E4M3Fn, :96-108 */
uint8_t msqo_encode_e4m3(float value) {
  uint8_t sign = signbit(value) ? 0x80u : 0u;
  if (isnan(value)) return sign | 0x7fu;
  if (value == 0.0f) return sign;
  if (isinf(value) || fabsf(value) > 448.0f) return sign | 0x7eu;
  return sign | nearest_code(fabsf(value), 0x7eu, msqo_decode_e4m3);
}

/* floatToFp8E5M2, :110-125 */
uint8_t msqo_encode_e5m2(float value) {
  uint8_t sign = signbit(value) ? 0x80u : 0u;
  if (isnan(value)) return sign | 0x7eu;
  if (value == 0.0f) return sign;
  if (isinf(value)) return sign | 0x7cu;
  if (fabsf(value) > 57344.0f) return sign | 0x7bu;
  return sign | nearest_code(fabsf(value), 0x7bu, msqo_decode_e5m2);
}

/* floatToFp4E2M1, :127-136 */
uint8_t msqo_encode_e2m1(float value) {
  uint8_t sign = signbit(value) ? 0x08u : 0u;
  if (isnan(value) || value == 0.0f) return sign;
  if (isinf(value) || fabsf(value) > 6.0f) return sign | 0x07u;
  return sign | nearest_code(fabsf(value), 0x07u, msqo_decode_e2m1);
}

/* mxScaleExponent, :148-162 */
static int mx_exponent(const float *v, size_t begin, size_t end, int emax) {
  float maximum = 0.0f;
  for (size_t i = begin; i < end; ++i)
    if (isfinite(v[i]) && fabsf(v[i]) > maximum) maximum = fabsf(v[i]);
  if (maximum == 0.0f) return 0;
  int e = ilogbf(maximum) - emax;
  return e < -127 ? -127 : (e > 128 ? 128 : e);
}

/* Format ids follow HostStorageCodec (src/precision.hpp:24-33) plus 8 =
 * FP8-E4M3 with a per-row FP32 scale. */
size_t msqo_storage_bytes(int format, size_t elements) {
  switch (format) {
    case 0: return elements * 4;
    case 1: return elements * 2;
    case 6: case 7: return (elements * 4 + 7) / 8;
    default: return elements;
  }
}

/* copyValuesToStorage + packFp4/packMxfp8/packMxfp4, :138-313.
 * row_length is used only by format 8. Returns 0 on success. */
int msqo_encode(int format, const float *src, size_t elements, size_t row_length,
                uint8_t *values, uint8_t *scales) {
  switch (format) {
    case 0: memcpy(values, src, elements * 4); return 0;
    case 1:
      for (size_t i = 0; i < elements; ++i) ((uint16_t *)values)[i] = msqo_encode_bf16(src[i]);
      return 0;
    case 2: for (size_t i = 0; i < elements; ++i) values[i] = msqo_encode_e4m3(src[i]); return 0;
    case 3: for (size_t i = 0; i < elements; ++i) values[i] = msqo_encode_e5m2(src[i]); return 0;
    case 4: case 5: {
      int emax = format == 4 ? 8 : 15;
      for (size_t b = 0, blk = 0; b < elements; b += 32, ++blk) {
        size_t end = b + 32 < elements ? b + 32 : elements;
        int e = mx_exponent(src, b, end, emax);
        scales[blk] = (uint8_t)(e + 127);
        float scale = ldexpf(1.0f, e);
        for (size_t i = b; i < end; ++i)
          values[i] = format == 4 ? msqo_encode_e4m3(src[i] / scale) : msqo_encode_e5m2(src[i] / scale);
      }
      return 0;
    }
    case 6:
      for (size_t i = 0; i < elements; i += 2) {
        uint8_t lo = msqo_encode_e2m1(src[i]);
        uint8_t hi = i + 1 < elements ? msqo_encode_e2m1(src[i + 1]) : 0u;
        values[i / 2] = (uint8_t)(lo | (hi << 4));
      }
      return 0;
    case 7:
      for (size_t b = 0, blk = 0; b < elements; b += 32, ++blk) {
        size_t end = b + 32 < elements ? b + 32 : elements;
        int e = mx_exponent(src, b, end, 2);
        scales[blk] = (uint8_t)(e + 127);
        float scale = ldexpf(1.0f, e);
        for (size_t i = b; i < end; i += 2) {
          uint8_t lo = msqo_encode_e2m1(src[i] / scale);
          uint8_t hi = i + 1 < end ? msqo_encode_e2m1(src[i + 1] / scale) : 0u;
          values[i / 2] = (uint8_t)(lo | (hi << 4));
        }
      }
      return 0;
    case 8: {
      if (row_length == 0 || elements % row_length) return 1;
      float *row_scales = (float *)scales;
      for (size_t r = 0; r < elements / row_length; ++r) {
        const float *row = src + r * row_length;
        float m = 0.0f;
        for (size_t i = 0; i < row_length; ++i)
          if (isfinite(row[i]) && fabsf(row[i]) > m) m = fabsf(row[i]);
        float s = m == 0.0f ? 1.0f : m / 448.0f;
        row_scales[r] = s;
        for (size_t i = 0; i < row_length; ++i) values[r * row_length + i] = msqo_encode_e4m3(row[i] / s);
      }
      return 0;
    }
    default: return 1;
  }
}

/* storageValueAt, :323-374, for every index */
int msqo_decode(int format, const uint8_t *values, const uint8_t *scales,
                size_t elements, size_t row_length, float *out) {
  for (size_t i = 0; i < elements; ++i) {
    switch (format) {
      case 0: memcpy(&out[i], values + 4 * i, 4); break;
      case 1: out[i] = msqo_decode_bf16(((const uint16_t *)values)[i]); break;
      case 2: out[i] = msqo_decode_e4m3(values[i]); break;
      case 3: out[i] = msqo_decode_e5m2(values[i]); break;
      case 4: out[i] = ldexpf(msqo_decode_e4m3(values[i]), (int)scales[i / 32] - 127); break;
      case 5: out[i] = ldexpf(msqo_decode_e5m2(values[i]), (int)scales[i / 32] - 127); break;
      case 6: out[i] = msqo_decode_e2m1((values[i / 2] >> ((i & 1u) * 4)) & 0x0fu); break;
      case 7:
        out[i] = ldexpf(msqo_decode_e2m1((values[i / 2] >> ((i & 1u) * 4)) & 0x0fu),
                        (int)scales[i / 32] - 127);
        break;
      case 8:
        if (row_length == 0) return 1;
        out[i] = msqo_decode_e4m3(values[i]) * ((const float *)scales)[i / row_length];
        break;
      default: return 1;
    }
  }
  return 0;
}

/* ------------------------------------------------- stochastic rounding */

/* The reference's device quantizers for --rounding stochastic
 * (metal_mixed_sqrt.metal): stochastic_hash / stochastic_round_up :394-405;
 * encode_fp8_e4m3fn_stochastic :462-484, encode_fp8_e5m2_stochastic
 * :545-568, encode_fp4_e2m1_stochastic :740-763 (bracketing codes lo < |x|
 * < hi; round up with probability (|x| - lo) / (hi - lo) against a 24-bit
 * sample of the hash of (element index, seed, stream); zero, NaN, and
 * magnitudes at or above the largest finite code take the nearest code);
 * quantize_bf16_stochastic :1888-1907 (add one BF16 ulp when the hash's low
 * 16 bits are below the 16 dropped bits).  The MX quantizers
 * (:971-1000, :1113-1140, :1232-1260) scale a block of 32 as the nearest
 * ones do and apply the element rule to x / 2^e with the global index.  No
 * host counterpart exists: these are restated from the shader source.
 * Adjacent codes differ by a power of two, so the probability is an exact
 * quotient whatever the division. */
uint32_t msqo_stochastic_hash(uint32_t index, uint32_t seed, uint32_t stream) {
  uint32_t state = index * 747796405u + seed + stream * 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

static int round_up(float probability, uint32_t index, uint32_t seed, uint32_t stream) {
  float sample = (float)(msqo_stochastic_hash(index, seed, stream) >> 8u) * 0x1.0p-24f;
  return sample < probability;
}

/* the bracketing codes of a finite magnitude below the largest code */
static uint8_t sr_code(uint8_t nearest, float magnitude, float (*dec)(uint8_t), uint32_t index,
                       uint32_t seed, uint32_t stream) {
  float nearest_value = dec(nearest);
  if (nearest_value == magnitude) return nearest;
  uint8_t lower = nearest_value < magnitude ? nearest : (uint8_t)(nearest - 1u);
  uint8_t upper = (uint8_t)(lower + 1u);
  float lo = dec(lower), hi = dec(upper);
  float p = (magnitude - lo) / (hi - lo);
  return round_up(p, index, seed, stream) ? upper : lower;
}

uint8_t msqo_encode_e4m3_sr(float value, uint32_t index, uint32_t seed, uint32_t stream) {
  float magnitude = fabsf(value);
  if (isnan(value) || magnitude == 0.0f || magnitude >= 448.0f) return msqo_encode_e4m3(value);
  uint8_t sign = signbit(value) ? 0x80u : 0u;
  return (uint8_t)(sign | sr_code(msqo_encode_e4m3(magnitude), magnitude, msqo_decode_e4m3,
                                  index, seed, stream));
}

uint8_t msqo_encode_e5m2_sr(float value, uint32_t index, uint32_t seed, uint32_t stream) {
  float magnitude = fabsf(value);
  if (isnan(value) || isinf(value) || magnitude == 0.0f || magnitude >= 57344.0f)
    return msqo_encode_e5m2(value);
  uint8_t sign = signbit(value) ? 0x80u : 0u;
  return (uint8_t)(sign | sr_code(msqo_encode_e5m2(magnitude), magnitude, msqo_decode_e5m2,
                                  index, seed, stream));
}

uint8_t msqo_encode_e2m1_sr(float value, uint32_t index, uint32_t seed, uint32_t stream) {
  float magnitude = fabsf(value);
  if (isnan(value) || magnitude == 0.0f || magnitude >= 6.0f) return msqo_encode_e2m1(value);
  uint8_t sign = signbit(value) ? 0x08u : 0u;
  /* the shader scans for the largest code not above the magnitude */
  uint8_t lower = 0;
  while (lower < 7u && msqo_decode_e2m1((uint8_t)(lower + 1u)) <= magnitude) ++lower;
  float lo = msqo_decode_e2m1(lower);
  if (lo == magnitude || lower == 7u) return (uint8_t)(sign | lower);
  uint8_t upper = (uint8_t)(lower + 1u);
  float p = (magnitude - lo) / (msqo_decode_e2m1(upper) - lo);
  return (uint8_t)(sign | (round_up(p, index, seed, stream) ? upper : lower));
}

uint16_t msqo_encode_bf16_sr(float value, uint32_t index, uint32_t seed, uint32_t stream) {
  if (!isfinite(value) || value == 0.0f) return msqo_encode_bf16(value);
  uint32_t bits;
  memcpy(&bits, &value, 4);
  uint32_t rounded = bits & 0xffff0000u;
  if ((msqo_stochastic_hash(index, seed, stream) & 0xffffu) < (bits & 0xffffu)) rounded += 0x00010000u;
  return (uint16_t)(rounded >> 16);
}

/* Stochastic counterpart of msqo_encode for every format (8: E4M3 of
 * x / s_row, s_row = max|row| / 448, with the element's flat index). */
int msqo_encode_stochastic(int format, const float *src, size_t elements, size_t row_length,
                           uint32_t seed, uint32_t stream, uint8_t *values, uint8_t *scales) {
  switch (format) {
    case 0: memcpy(values, src, elements * 4); return 0;
    case 1:
      for (size_t i = 0; i < elements; ++i)
        ((uint16_t *)values)[i] = msqo_encode_bf16_sr(src[i], (uint32_t)i, seed, stream);
      return 0;
    case 2:
      for (size_t i = 0; i < elements; ++i) values[i] = msqo_encode_e4m3_sr(src[i], (uint32_t)i, seed, stream);
      return 0;
    case 3:
      for (size_t i = 0; i < elements; ++i) values[i] = msqo_encode_e5m2_sr(src[i], (uint32_t)i, seed, stream);
      return 0;
    case 4: case 5: {
      int emax = format == 4 ? 8 : 15;
      for (size_t b = 0, blk = 0; b < elements; b += 32, ++blk) {
        size_t end = b + 32 < elements ? b + 32 : elements;
        int e = mx_exponent(src, b, end, emax);
        scales[blk] = (uint8_t)(e + 127);
        float scale = ldexpf(1.0f, e);
        for (size_t i = b; i < end; ++i)
          values[i] = format == 4 ? msqo_encode_e4m3_sr(src[i] / scale, (uint32_t)i, seed, stream)
                                  : msqo_encode_e5m2_sr(src[i] / scale, (uint32_t)i, seed, stream);
      }
      return 0;
    }
    case 6:
      for (size_t i = 0; i < elements; i += 2) {
        uint8_t lo = msqo_encode_e2m1_sr(src[i], (uint32_t)i, seed, stream);
        uint8_t hi = i + 1 < elements ? msqo_encode_e2m1_sr(src[i + 1], (uint32_t)(i + 1), seed, stream) : 0u;
        values[i / 2] = (uint8_t)(lo | (hi << 4));
      }
      return 0;
    case 7:
      for (size_t b = 0, blk = 0; b < elements; b += 32, ++blk) {
        size_t end = b + 32 < elements ? b + 32 : elements;
        int e = mx_exponent(src, b, end, 2);
        scales[blk] = (uint8_t)(e + 127);
        float scale = ldexpf(1.0f, e);
        for (size_t i = b; i < end; i += 2) {
          uint8_t lo = msqo_encode_e2m1_sr(src[i] / scale, (uint32_t)i, seed, stream);
          uint8_t hi = i + 1 < end ? msqo_encode_e2m1_sr(src[i + 1] / scale, (uint32_t)(i + 1), seed, stream) : 0u;
          values[i / 2] = (uint8_t)(lo | (hi << 4));
        }
      }
      return 0;
    case 8: {
      if (row_length == 0 || elements % row_length) return 1;
      float *row_scales = (float *)scales;
      for (size_t r = 0; r < elements / row_length; ++r) {
        const float *row = src + r * row_length;
        float m = 0.0f;
        for (size_t i = 0; i < row_length; ++i)
          if (isfinite(row[i]) && fabsf(row[i]) > m) m = fabsf(row[i]);
        float s = m == 0.0f ? 1.0f : m / 448.0f;
        row_scales[r] = s;
        for (size_t i = 0; i < row_length; ++i) {
          size_t k = r * row_length + i;
          values[k] = msqo_encode_e4m3_sr(row[i] / s, (uint32_t)k, seed, stream);
        }
      }
      return 0;
    }
    default: return 1;
  }
}

/* ------------------------------------------------- log-spectrum storage */

/* fp8_e4m3fn_log_s / fp4_e2m1_log_s (src/precision.hpp:87-92): root
 * eigenvalues in blocks of 8 stored as codes of maximum * (log2 s - min) /
 * span, metadata (min, span) of log2 s per block; decode exp2(min + span *
 * dec(code) / maximum), maximum = 448 (E4M3) or 6 (E2M1).  The device form
 * (metal_mixed_sqrt.metal:1689-1804): the span is lowered by one ulp when
 * min + span rounds above the block's maximum log, so the top code decodes
 * at or below the largest input.  The host form (copySpectrumToStorage,
 * src/storage_codecs.cpp:400-440) keeps the span; with that difference the
 * two agree (tests).  Inputs must be finite and positive.  Returns 0, or 1
 * for an unsupported format or an invalid input. */
int msqo_spectrum_encode(int format, const float *s, size_t elements, int stochastic,
                         uint32_t seed, uint32_t stream, uint8_t *values, float *metadata) {
  if (format != 2 && format != 6) return 1;
  const float maximum = format == 2 ? 448.0f : 6.0f;
  for (size_t b = 0, blk = 0; b < elements; b += 8, ++blk) {
    size_t end = b + 8 < elements ? b + 8 : elements;
    float lo = INFINITY, hi = -INFINITY;
    for (size_t i = b; i < end; ++i) {
      if (!(s[i] > 0.0f) || !isfinite(s[i])) return 1;
      float l = log2f(s[i]);
      lo = fminf(lo, l);
      hi = fmaxf(hi, l);
    }
    float span = hi - lo;
    if (lo + span > hi) span = nextafterf(span, 0.0f);
    metadata[2 * blk] = lo;
    metadata[2 * blk + 1] = span;
  }
  if (format == 6) memset(values, 0, (elements + 1) / 2);
  for (size_t i = 0; i < elements; ++i) {
    const float lo = metadata[2 * (i / 8)], span = metadata[2 * (i / 8) + 1];
    const float x = span == 0.0f ? 0.0f : maximum * (log2f(s[i]) - lo) / span;
    if (format == 2) {
      values[i] = stochastic ? msqo_encode_e4m3_sr(x, (uint32_t)i, seed, stream) : msqo_encode_e4m3(x);
    } else {
      uint8_t c = stochastic ? msqo_encode_e2m1_sr(x, (uint32_t)i, seed, stream) : msqo_encode_e2m1(x);
      values[i / 2] |= (uint8_t)(c << ((i & 1u) * 4));
    }
  }
  return 0;
}

int msqo_spectrum_decode(int format, const uint8_t *values, const float *metadata,
                         size_t elements, float *out) {
  if (format != 2 && format != 6) return 1;
  const float maximum = format == 2 ? 448.0f : 6.0f;
  for (size_t i = 0; i < elements; ++i) {
    const float lo = metadata[2 * (i / 8)], span = metadata[2 * (i / 8) + 1];
    const float d = format == 2 ? msqo_decode_e4m3(values[i])
                                : msqo_decode_e2m1((values[i / 2] >> ((i & 1u) * 4)) & 0x0fu);
    out[i] = exp2f(lo + span * d / maximum);
  }
  return 0;
}

/* ----------------------------------------- native-quantized correction */

/* C = A B (n x n, column-major), each element the FMA chain over the inner
 * index in order (matmul_f32 and the low-precision matmuls on decoded
 * operands, metal_mixed_sqrt.metal:39-56). */
static void matmul_fma(const float *a, const float *b, float *c, unsigned n) {
  for (unsigned col = 0; col < n; ++col)
    for (unsigned row = 0; row < n; ++row) {
      float sum = 0.0f;
      for (unsigned k = 0; k < n; ++k) sum = fmaf(a[row + (size_t)k * n], b[k + (size_t)col * n], sum);
      c[row + (size_t)col * n] = sum;
    }
}

/* x quantized to `format` (nearest; row length n for format 8) and decoded */
static int quantize_decode(int format, float *x, unsigned n, uint8_t *codes, uint8_t *scales) {
  if (format == 0) return 0;
  size_t e = (size_t)n * n, rl = format == 8 ? n : 0;
  if (msqo_encode(format, x, e, rl, codes, scales)) return 1;
  return msqo_decode(format, codes, scales, e, rl, x);
}

/* One correction of the native-quantized mode (refineNativeStaged,
 * src/metal_runtime.cpp:313-411; driven at src/metal_solver.cpp:829-848):
 * R_q = Q(R), W1 = Q(Vt R_q), W2 = Q(W1 V), C = Q(W2_ij / (s_i + s_j)),
 * W1 = Q(V C), E = Q(W1 Vt); e_out receives E.  v / vt are the decoded
 * stored basis and transposed basis, s the decoded root eigenvalues. */
int msqo_native_correction(int format, const float *v, const float *vt, const float *s,
                           const float *r, unsigned n, float *e_out) {
  size_t e = (size_t)n * n;
  float *rq = malloc(e * 4), *w1 = malloc(e * 4), *w2 = malloc(e * 4);
  uint8_t *codes = malloc(e * 4 + 16), *scales = malloc(e + 4 * (size_t)n + 16);
  int rc = 1;
  if (!rq || !w1 || !w2 || !codes || !scales) goto done;
  memcpy(rq, r, e * 4);
  if (quantize_decode(format, rq, n, codes, scales)) goto done;
  matmul_fma(vt, rq, w1, n);
  if (quantize_decode(format, w1, n, codes, scales)) goto done;
  matmul_fma(w1, v, w2, n);
  if (quantize_decode(format, w2, n, codes, scales)) goto done;
  for (unsigned j = 0; j < n; ++j)
    for (unsigned i = 0; i < n; ++i) w1[i + (size_t)j * n] = w2[i + (size_t)j * n] / (s[i] + s[j]);
  if (quantize_decode(format, w1, n, codes, scales)) goto done;
  matmul_fma(v, w1, w2, n);
  if (quantize_decode(format, w2, n, codes, scales)) goto done;
  matmul_fma(w2, vt, e_out, n);
  if (quantize_decode(format, e_out, n, codes, scales)) goto done;
  rc = 0;
done:
  free(rq); free(w1); free(w2); free(codes); free(scales);
  return rc;
}

/* -------------------------------------------------- paper test sets */

/* DeterministicGenerator (src/accelerate_backend.cpp:626-664): xorshift
 * state update, 53-bit uniform from a multiplied state, Box-Muller normals
 * (cosine first, sine kept as the spare). */
typedef struct { uint64_t state; double spare; int has_spare; } paper_rng;

static double rng_uniform(paper_rng *g) {
  uint64_t v = g->state;
  v ^= v >> 12;
  v ^= v << 25;
  v ^= v >> 27;
  g->state = v;
  return (double)((v * UINT64_C(2685821657736338717)) >> 11) * 0x1.0p-53;
}

static double rng_normal(paper_rng *g) {
  if (g->has_spare) { g->has_spare = 0; return g->spare; }
  double first = rng_uniform(g);
  if (first < 2.2250738585072014e-308) first = 2.2250738585072014e-308;
  double second = rng_uniform(g);
  double radius = sqrt(-2.0 * log(first)), angle = 6.283185307179586476925286766559 * second;
  g->spare = radius * sin(angle);
  g->has_spare = 1;
  return radius * cos(angle);
}

/* preparePaperMatrix (src/accelerate_backend.cpp:690-801) for the symmetric
 * sets V (uniform), VI (normal) and VII (Hilbert + 1e-6 I), before the
 * spectral shift of V and VI (which needs the FP64 extreme eigenvalues and
 * is applied by the caller).  *seed receives the generator seed (0 for VII).
 * Returns 0, or 1 for another set. */
int msqo_paper_matrix(int set, unsigned n, double *out, uint64_t *seed) {
  if (set == 7) {
    for (unsigned c = 0; c < n; ++c) {
      for (unsigned r = 0; r < n; ++r) out[r + (size_t)c * n] = 1.0 / (double)(r + c + 1);
      out[c + (size_t)c * n] += 1.0e-6;
    }
    *seed = 0;
    return 0;
  }
  if (set != 5 && set != 6) return 1;
  paper_rng g;
  g.state = UINT64_C(0x243f6a8885a308d3) ^ (UINT64_C(0x9e3779b97f4a7c15) * (uint64_t)set);
  *seed = g.state;
  if (g.state == 0) g.state = UINT64_C(0x9e3779b97f4a7c15);
  g.has_spare = 0;
  g.spare = 0.0;
  for (unsigned c = 0; c < n; ++c)
    for (unsigned r = c; r < n; ++r) {
      double v = set == 5 ? rng_uniform(&g) : rng_normal(&g);
      out[r + (size_t)c * n] = v;
      out[c + (size_t)r * n] = v;
    }
  return 0;
}

/* ---------------------------------------------------------------- Jacobi */

/* Round-robin ("chess tournament") pairing of makeJacobiSchedule
 * (src/metal_solver.cpp:50-79) computed arithmetically: participants are
 * rotated right by one (slot 0 fixed) after every round, so in round r slot k
 * (k >= 1) holds participant 1 + ((k - 1 - r) mod (m - 1)), m = padded order.
 * Pair j joins slots j and m-1-j. */
static unsigned rr_slot(unsigned slot, unsigned round, unsigned m) {
  if (slot == 0) return 0;
  unsigned k = (slot - 1 + (m - 1) - (round % (m - 1))) % (m - 1);
  return 1 + k;
}

void msqo_jacobi_pair(unsigned order, unsigned round, unsigned pair,
                      unsigned *p, unsigned *q) {
  unsigned m = order + (order & 1u);
  unsigned a = rr_slot(pair, round, m), b = rr_slot(m - 1 - pair, round, m);
  *p = a < b ? a : b;
  *q = a < b ? b : a;
}

/* Two-level pairing of nb blocks (nb even), the order the CUDA solver uses
 * for orders 257..512 when it accumulates eigenvectors on the tensor cores:
 * super-blocks of 8 blocks (the last holds nb mod 8 when that is nonzero; an
 * empty one is added when their count is odd).  Rounds 0..6: inside every
 * super-block, round r of the round-robin over its 8 slots (pairs whose
 * slots both exist).  Then for each outer round o of the round-robin over
 * super-blocks and t = 0..7: block i of P with block (i + t) mod 8 of Q for
 * every super-pair (P, Q), P < Q.  Blocks left without a partner are paired
 * in increasing order, as identity rotations (J stored as -1 - J).  out:
 * rounds x nb ints, pair k of round r at out[r * nb + 2k]. */
static unsigned tl_supers(unsigned nb) {
  unsigned s = (nb + 7u) / 8u;
  return s + (s & 1u);
}

int msqo_two_level_rounds(unsigned nb) { return (int)(7u + 8u * (tl_supers(nb) - 1u)); }

void msqo_two_level_schedule(unsigned nb, int *out) {
  unsigned supers = tl_supers(nb), rounds = (unsigned)msqo_two_level_rounds(nb);
  unsigned char *used = (unsigned char *)malloc(nb);
  for (unsigned r = 0; r < rounds; ++r) {
    int *row = out + (size_t)r * nb;
    unsigned k = 0;
    memset(used, 0, nb);
    if (r < 7) {
      for (unsigned S = 0; 8 * S < nb; ++S) {
        unsigned size = nb - 8 * S < 8 ? nb - 8 * S : 8;
        for (unsigned x = 0; x < 4; ++x) {
          unsigned a, b;
          msqo_jacobi_pair(8, r, x, &a, &b);
          if (b < size) {
            row[2 * k] = (int)(8 * S + a);
            row[2 * k + 1] = (int)(8 * S + b);
            used[8 * S + a] = used[8 * S + b] = 1;
            ++k;
          }
        }
      }
    } else {
      unsigned o = (r - 7) / 8, t = (r - 7) % 8;
      for (unsigned x = 0; x < supers / 2; ++x) {
        unsigned P, Q;
        msqo_jacobi_pair(supers, o, x, &P, &Q);
        unsigned sp = 8 * P >= nb ? 0 : (nb - 8 * P < 8 ? nb - 8 * P : 8);
        unsigned sq = 8 * Q >= nb ? 0 : (nb - 8 * Q < 8 ? nb - 8 * Q : 8);
        for (unsigned i = 0; i < 8; ++i) {
          unsigned j = (i + t) % 8;
          if (i < sp && j < sq) {
            row[2 * k] = (int)(8 * P + i);
            row[2 * k + 1] = (int)(8 * Q + j);
            used[8 * P + i] = used[8 * Q + j] = 1;
            ++k;
          }
        }
      }
    }
    int idle = -1;
    for (unsigned blk = 0; blk < nb; ++blk) {
      if (used[blk]) continue;
      if (idle < 0) { idle = (int)blk; continue; }
      row[2 * k] = idle;
      row[2 * k + 1] = -1 - (int)blk;
      ++k;
      idle = -1;
    }
  }
  free(used);
}

/* One parallel-order cyclic Jacobi solve of the symmetric FP32 matrix a
 * (n x n, column-major, overwritten), vectors v (n x n), eigenvalues w.
 * Per round: angles of all disjoint pairs from the round's start matrix in
 * FP64 (the reference computes them in FP32, metal_mixed_sqrt.metal:
 * 1331-1361: tau = (a_qq - a_pp) / (2 a_pq), t = sign(tau) / (|tau| +
 * sqrt(1 + tau^2)), c = 1/sqrt(1 + t^2), s = t c), then A <- J^T A J and
 * V <- V J with the 4-term update of :1363-1411.  Sweeps continue until
 * off(A) <= tol * ||A||_F (FP64) or max_sweeps.  Returns sweeps done. */
int msqo_jacobi(float *a, float *v, float *w, unsigned n, double tol,
                int max_sweeps, double *off_ratio) {
  unsigned m = n + (n & 1u);
  unsigned pairs = m / 2;
  float *next = (float *)malloc(sizeof(float) * n * n);
  float *vn = (float *)malloc(sizeof(float) * n * n);
  float *c = (float *)malloc(sizeof(float) * (m + 1));
  float *s = (float *)malloc(sizeof(float) * (m + 1));
  unsigned *partner = (unsigned *)malloc(sizeof(unsigned) * (m + 1));
  for (unsigned j = 0; j < n; ++j)
    for (unsigned i = 0; i < n; ++i) v[i + j * n] = i == j ? 1.0f : 0.0f;
  double norm2 = 0.0;
  for (size_t i = 0; i < (size_t)n * n; ++i) norm2 += (double)a[i] * a[i];
  double norm = sqrt(norm2);
  int sweeps = 0;
  double ratio = 0.0;
  for (;;) {
    double off2 = 0.0;
    for (unsigned j = 0; j < n; ++j)
      for (unsigned i = 0; i < n; ++i)
        if (i != j) off2 += (double)a[i + j * n] * a[i + j * n];
    ratio = norm > 0 ? sqrt(off2) / norm : 0.0;
    if (ratio <= tol || sweeps >= max_sweeps) break;
    for (unsigned round = 0; round + 1 < m; ++round) {
      for (unsigned k = 0; k < pairs; ++k) {
        unsigned p, q;
        msqo_jacobi_pair(n, round, k, &p, &q);
        partner[p] = q;
        partner[q] = p;
        double cs = 1.0, sn = 0.0;
        if (q < n) {
          double app = a[p + p * n], aqq = a[q + q * n];
          double apq = 0.5 * ((double)a[p + q * n] + (double)a[q + p * n]);
          if (apq != 0.0) {
            double tau = (aqq - app) / (2.0 * apq);
            double t = copysign(1.0 / (fabs(tau) + sqrt(1.0 + tau * tau)), tau);
            cs = 1.0 / sqrt(1.0 + t * t);
            sn = t * cs;
          }
        }
        /* rotation seen from p: (c, -s); from q: (c, +s) */
        c[p] = (float)cs; s[p] = (float)-sn;
        c[q] = (float)cs; s[q] = (float)sn;
      }
      for (unsigned col = 0; col < n; ++col) {
        unsigned cp = partner[col] < n ? partner[col] : col;
        float cc = c[col], cs_ = partner[col] < n ? s[col] : 0.0f;
        for (unsigned row = 0; row < n; ++row) {
          unsigned rp = partner[row] < n ? partner[row] : row;
          float rc = c[row], rs = partner[row] < n ? s[row] : 0.0f;
          next[row + col * n] = rc * cc * a[row + col * n] + rs * cc * a[rp + col * n] +
                                rc * cs_ * a[row + cp * n] + rs * cs_ * a[rp + cp * n];
          vn[row + col * n] = cc * v[row + col * n] + cs_ * v[row + cp * n];
        }
      }
      /* The pivot element of every rotated pair is annihilated exactly (the
       * classic Jacobi step; the CUDA kernel does the same).  The reference's
       * 4-term update leaves its FP32 rounding residue there instead, which
       * is harmless for its fixed 8 sweeps but would floor a convergence
       * test on off(A). */
      for (unsigned k = 0; k < pairs; ++k) {
        unsigned p, q;
        msqo_jacobi_pair(n, round, k, &p, &q);
        if (q < n) {
          next[p + q * n] = 0.0f;
          next[q + p * n] = 0.0f;
        }
      }
      memcpy(a, next, sizeof(float) * n * n);
      memcpy(v, vn, sizeof(float) * n * n);
    }
    ++sweeps;
  }
  for (unsigned i = 0; i < n; ++i) w[i] = a[i + i * n];
  if (off_ratio) *off_ratio = ratio;
  free(next); free(vn); free(c); free(s); free(partner);
  return sweeps;
}

/* Blocked ordering of the same rotations, as the CUDA eigensolver applies
 * them: indices in blocks of 4 (order padded to a multiple of 8 with zero
 * rows), block pairs by the round-robin rule over m/4 blocks; each 8x8
 * pivot gets one cyclic sweep of the scalar rotation above in the
 * round-robin order of 8 indices, accumulated into Q; every off-pivot 8x8
 * super-tile (k < l) is replaced by Q_k^T T Q_l and mirrored; V <- V Q.
 * FP32 storage and arithmetic (the pivot angles too) with the roundings the
 * CUDA kernels make, FP64 off-norm: after the same number of sweeps the
 * results agree bit for bit.  Returns sweeps; a_out (nullable) receives the
 * rotated matrix. */
static const int kInner[28][2] = {
    {0, 7}, {1, 6}, {2, 5}, {3, 4}, {0, 6}, {5, 7}, {1, 4}, {2, 3}, {0, 5}, {4, 6},
    {3, 7}, {1, 2}, {0, 4}, {3, 5}, {2, 6}, {1, 7}, {0, 3}, {2, 4}, {1, 5}, {6, 7},
    {0, 2}, {1, 3}, {4, 7}, {5, 6}, {0, 1}, {2, 7}, {3, 6}, {4, 5}};

static void pivot_sweep(float p[8][8], float q[8][8]) {
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < 8; ++c) q[r][c] = r == c ? 1.0f : 0.0f;
  for (int k = 0; k < 28; ++k) {
    int a = kInner[k][0], b = kInner[k][1];
    float apq = p[a][b];
    if (apq == 0.0f) continue;
    float tau = (p[b][b] - p[a][a]) / (2.0f * apq);
    float t = copysignf(1.0f / (fabsf(tau) + sqrtf(tau * tau + 1.0f)), tau);
    float c = 1.0f / sqrtf(t * t + 1.0f), s = t * c;
    /* exact e = c^2 + s^2 - 1 (FMA two-products), then (c, s) *= 1 - e/2 */
    float cc = c * c, cce = fmaf(c, c, -cc), ss = s * s, sse = fmaf(s, s, -ss);
    float e = ((cc - 1.0f) + ss) + (cce + sse);
    float h = -0.5f * e;
    c = fmaf(h, c, c);
    s = fmaf(h, s, s);
    for (int i = 0; i < 8; ++i) {
      float pa = p[i][a], pb = p[i][b];
      p[i][a] = c * pa - s * pb;
      p[i][b] = s * pa + c * pb;
    }
    for (int j = 0; j < 8; ++j) {
      float pa = p[a][j], pb = p[b][j];
      p[a][j] = c * pa - s * pb;
      p[b][j] = s * pa + c * pb;
    }
    p[a][b] = p[b][a] = 0.0f;
    for (int i = 0; i < 8; ++i) {
      float qa = q[i][a], qb = q[i][b];
      q[i][a] = c * qa - s * qb;
      q[i][b] = s * qa + c * qb;
    }
  }
}

int msqo_jacobi_blocked_order(const float *a_in, float *a_out, float *v_out, float *w,
                              unsigned n, double tol, int max_sweeps, double *off_ratio,
                              int two_level);

int msqo_jacobi_blocked(const float *a_in, float *a_out, float *v_out, float *w, unsigned n,
                        double tol, int max_sweeps, double *off_ratio) {
  return msqo_jacobi_blocked_order(a_in, a_out, v_out, w, n, tol, max_sweeps, off_ratio, 0);
}

/* two_level != 0: the two-level pairing above instead of the round-robin
 * rule (identity pairs keep their pivot blocks and use Q = I). */
int msqo_jacobi_blocked_order(const float *a_in, float *a_out, float *v_out, float *w,
                              unsigned n, double tol, int max_sweeps, double *off_ratio,
                              int two_level) {
  unsigned m = (n + 7u) & ~7u, nb = m / 4, P = nb / 2;
  unsigned rounds = two_level ? (unsigned)msqo_two_level_rounds(nb) : nb - 1;
  int *sched = NULL;
  if (two_level) {
    sched = (int *)malloc(sizeof(int) * (size_t)rounds * nb);
    msqo_two_level_schedule(nb, sched);
  }
  float *A = (float *)calloc((size_t)m * m, sizeof(float));
  float *V = (float *)calloc((size_t)m * m, sizeof(float));
  float (*Q)[8][8] = malloc(sizeof(float) * 64 * (P ? P : 1));
  unsigned *bi = malloc(sizeof(unsigned) * (P ? P : 1)), *bj = malloc(sizeof(unsigned) * (P ? P : 1));
  for (unsigned c = 0; c < n; ++c)
    for (unsigned r = 0; r < n; ++r)
      A[r + (size_t)c * m] = 0.5f * (a_in[r + (size_t)c * n] + a_in[c + (size_t)r * n]);
  for (unsigned i = 0; i < m; ++i) V[i + (size_t)i * m] = 1.0f;
  double norm2 = 0.0;
  for (size_t i = 0; i < (size_t)m * m; ++i) norm2 += (double)A[i] * A[i];
  int sweeps = 0;
  double ratio = 0.0;
  for (;;) {
    double off2 = 0.0;
    for (unsigned c = 0; c < m; ++c)
      for (unsigned r = 0; r < m; ++r)
        if (r != c) off2 += (double)A[r + (size_t)c * m] * A[r + (size_t)c * m];
    ratio = norm2 > 0 ? sqrt(off2 / norm2) : 0.0;
    if (ratio <= tol || sweeps >= max_sweeps) break;
    for (unsigned round = 0; round < rounds; ++round) {
      for (unsigned k = 0; k < P; ++k) {
        unsigned I, J;
        int rotate = 1;
        if (sched) {
          int sj = sched[(size_t)round * nb + 2 * k + 1];
          I = (unsigned)sched[(size_t)round * nb + 2 * k];
          rotate = sj >= 0;
          J = (unsigned)(rotate ? sj : -1 - sj);
        } else {
          msqo_jacobi_pair(nb, round, k, &I, &J);
        }
        bi[k] = I;
        bj[k] = J;
        if (!rotate) {
          for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) Q[k][r][c] = r == c ? 1.0f : 0.0f;
          continue;
        }
        float p[8][8];
        unsigned idx[8];
        for (int x = 0; x < 4; ++x) { idx[x] = 4 * I + x; idx[4 + x] = 4 * J + x; }
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) p[r][c] = A[idx[r] + (size_t)idx[c] * m];
        pivot_sweep(p, Q[k]);
        /* the two diagonal 4x4 blocks are kept whole; the off-diagonal
         * block is kept from the upper half and mirrored (the CUDA solver
         * stores only upper 4x4 tiles) */
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) {
            if ((r < 4) == (c < 4)) A[idx[r] + (size_t)idx[c] * m] = p[r][c];
            else if (r < 4) A[idx[r] + (size_t)idx[c] * m] = A[idx[c] + (size_t)idx[r] * m] = p[r][c];
          }
      }
      /* off-pivot super-tiles k < l, mirrored into the lower half */
      for (unsigned k = 0; k < P; ++k)
        for (unsigned l = k + 1; l < P; ++l) {
          unsigned ri[8], ci[8];
          for (int x = 0; x < 4; ++x) {
            ri[x] = 4 * bi[k] + x; ri[4 + x] = 4 * bj[k] + x;
            ci[x] = 4 * bi[l] + x; ci[4 + x] = 4 * bj[l] + x;
          }
          float t[8][8], u[8][8], o[8][8];
          for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) t[r][c] = A[ri[r] + (size_t)ci[c] * m];
          for (int a = 0; a < 8; ++a)
            for (int c = 0; c < 8; ++c) {
              float s = 0.0f;
              for (int i = 0; i < 8; ++i) s = fmaf(Q[k][i][a], t[i][c], s);
              u[a][c] = s;
            }
          for (int a = 0; a < 8; ++a)
            for (int c = 0; c < 8; ++c) {
              float s = 0.0f;
              for (int j = 0; j < 8; ++j) s = fmaf(u[a][j], Q[l][j][c], s);
              o[a][c] = s;
            }
          for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c)
              A[ri[r] + (size_t)ci[c] * m] = A[ci[c] + (size_t)ri[r] * m] = o[r][c];
        }
      for (unsigned row = 0; row < m; ++row)
        for (unsigned k = 0; k < P; ++k) {
          unsigned ci[8];
          for (int x = 0; x < 4; ++x) { ci[x] = 4 * bi[k] + x; ci[4 + x] = 4 * bj[k] + x; }
          float x8[8], o8[8];
          for (int j = 0; j < 8; ++j) x8[j] = V[row + (size_t)ci[j] * m];
          for (int c = 0; c < 8; ++c) {
            float s = 0.0f;
            for (int j = 0; j < 8; ++j) s = fmaf(x8[j], Q[k][j][c], s);
            o8[c] = s;
          }
          for (int c = 0; c < 8; ++c) V[row + (size_t)ci[c] * m] = o8[c];
        }
    }
    ++sweeps;
  }
  for (unsigned i = 0; i < n; ++i) w[i] = A[i + (size_t)i * m];
  for (unsigned c = 0; c < n; ++c)
    for (unsigned r = 0; r < n; ++r) {
      v_out[r + (size_t)c * n] = V[r + (size_t)c * m];
      if (a_out) a_out[r + (size_t)c * n] = A[r + (size_t)c * m];
    }
  if (off_ratio) *off_ratio = ratio;
  free(A); free(V); free(Q); free(bi); free(bj); free(sched);
  return sweeps;
}

/* --------------------------------------------------- float-float residual */

typedef struct { float hi, lo; } ff;

static ff ff_norm(float hi, float lo) { float s = hi + lo; ff r = {s, lo - (s - hi)}; return r; }

/* working_add, metal_mixed_sqrt.metal:1285-1291 */
static ff ff_add(ff a, ff b) {
  float s = a.hi + b.hi, vr = s - a.hi;
  float e = (a.hi - (s - vr)) + (b.hi - vr) + a.lo + b.lo;
  return ff_norm(s, e);
}

/* working_multiply, :1293-1299 */
static ff ff_mul(ff a, ff b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p) + a.hi * b.lo + a.lo * b.hi + a.lo * b.lo;
  return ff_norm(p, e);
}

/* working_residual, :1927-1942: R = A - X X in float-float; returns
 * ||R||_F / ||A||_F accumulated in FP64. */
double msqo_ff_residual(const float *a, const float *x_hi, const float *x_lo,
                        unsigned n, float *r_out) {
  double rn = 0.0, an = 0.0;
  for (unsigned col = 0; col < n; ++col)
    for (unsigned row = 0; row < n; ++row) {
      ff sum = {0.0f, 0.0f};
      for (unsigned k = 0; k < n; ++k) {
        ff l = {x_hi[row + k * n], x_lo ? x_lo[row + k * n] : 0.0f};
        ff r = {x_hi[k + col * n], x_lo ? x_lo[k + col * n] : 0.0f};
        sum = ff_add(sum, ff_mul(l, r));
      }
      ff m = {a[row + col * n], 0.0f};
      ff neg = {-sum.hi, -sum.lo};
      ff res = ff_add(m, neg);
      double rv = (double)res.hi + res.lo;
      if (r_out) r_out[row + col * n] = res.hi + res.lo;
      rn += rv * rv;
      an += (double)a[row + col * n] * a[row + col * n];
    }
  return sqrt(rn / an);
}
