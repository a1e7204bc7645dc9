// cuda_spectral — the stage-3 precision plans of the reference
// (run_spectral / precision_plans, 3_spectral/spectral.cpp:769-1385) on the
// CUDA solver, host code over the C ABI.
//
// A plan stores the FP32 eigenbasis and the root spectrum s = sqrt(lambda)
// in two formats.  The initial root is X0 = (Vq diag(sq)) Vinv with Vinv the
// transpose of the quantized basis, or, for an FP16 basis, the FP16
// quantization of the FP32 basis's explicit inverse (invert_basis,
// :600-637; rejected when its 1-norm condition is not below 1e4).  The
// corrections solve the Sylvester equation in the frozen basis,
// E = V ((Vinv R V) o H) Vinv with H_ij = 1 / (sq_i + sq_j), and add E to the
// float-float root.  A low-bit basis of a matrix with condition below 1000
// runs its products on low-bit operands (every operand re-encoded to the
// basis format, FP32 accumulation) while the residual is above 1e-3, and
// leaves them for FP32 products after two corrections in a row without a
// 2x drop of the residual (the stall fallback, :1225-1232, :1356-1363).  A
// correction that takes the residual above max(1, 1e4 x initial) stops the
// plan as divergent.
#include "cuda_backend.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <vector>

namespace mixed_sqrt {
namespace {

[[noreturn]] void failSpectral(const std::string &message) { throw std::runtime_error(message); }

class Buffer {
 public:
  explicit Buffer(size_t bytes) {
    if (bytes != 0 && cudaMalloc(&ptr_, bytes) != cudaSuccess)
      failSpectral("cuda_spectral: device allocation failed");
  }
  ~Buffer() {
    if (ptr_ != nullptr) cudaFree(ptr_);
  }
  Buffer(const Buffer &) = delete;
  Buffer &operator=(const Buffer &) = delete;
  template <typename T>
  T *as() const { return static_cast<T *>(ptr_); }

 private:
  void *ptr_ = nullptr;
};

void toDevice(void *dst, const void *src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    failSpectral("cuda_spectral: host to device copy failed");
}

void toHost(void *dst, const void *src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    failSpectral("cuda_spectral: device to host copy failed");
}

// The library's codec id of a stage-3 format (FP16 has none: it is
// converted on the host, IEEE binary16 with round-to-nearest-even).
int codecOf(CudaFactorFormat format) {
  switch (format) {
    case CudaFactorFormat::Bf16: return MSQ_FMT_BF16;
    case CudaFactorFormat::Fp8E4M3: return MSQ_FMT_FP8_E4M3FN;
    case CudaFactorFormat::Fp8E5M2: return MSQ_FMT_FP8_E5M2;
    case CudaFactorFormat::MxFp8E4M3: return MSQ_FMT_MXFP8_E4M3FN;
    case CudaFactorFormat::MxFp4E2M1: return MSQ_FMT_MXFP4_E2M1;
    default: return MSQ_FMT_FP32;
  }
}

// value_bytes / scale_bytes (:341-377) per stored value
double storageBits(CudaFactorFormat format, size_t values) {
  size_t bytes = 0;
  switch (format) {
    case CudaFactorFormat::Fp32: bytes = 4 * values; break;
    case CudaFactorFormat::Fp16:
    case CudaFactorFormat::Bf16: bytes = 2 * values; break;
    case CudaFactorFormat::Fp8E4M3:
    case CudaFactorFormat::Fp8E5M2:
    case CudaFactorFormat::MxFp8E4M3: bytes = values; break;
    case CudaFactorFormat::MxFp4E2M1: bytes = (values + 1) / 2; break;
  }
  if (format == CudaFactorFormat::MxFp8E4M3 || format == CudaFactorFormat::MxFp4E2M1)
    bytes += (values + 31) / 32;
  return 8.0 * static_cast<double>(bytes) / static_cast<double>(values);
}

// IEEE binary16, round to nearest even (subnormals kept, overflow to inf).
float toHalfAndBack(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  const uint32_t sign = (u >> 16) & 0x8000u;
  const uint32_t mag = u & 0x7fffffffu;
  uint16_t h;
  if (mag >= 0x7f800000u) {
    h = static_cast<uint16_t>(sign | 0x7c00u | (mag > 0x7f800000u ? 0x200u : 0u));
  } else if (mag >= 0x477ff000u) {  // rounds to 65520 or more: infinity
    h = static_cast<uint16_t>(sign | 0x7c00u);
  } else if (mag < 0x38800000u) {  // below 2^-14: subnormal half (or zero)
    // value = m * 2^-24 with m = |x| * 2^24 rounded half to even
    float ax;
    std::memcpy(&ax, &mag, 4);
    const float scaled = ax * 16777216.0f;  // exact: a power-of-two scaling
    const float rounded = std::nearbyint(scaled);  // round-half-even in the default mode
    h = static_cast<uint16_t>(sign | static_cast<uint32_t>(rounded));
  } else {
    const uint32_t e = (mag >> 23) - 112;  // rebias 127 -> 15
    uint32_t m = mag & 0x7fffffu;
    uint32_t r = (e << 10) | (m >> 13);
    const uint32_t rest = m & 0x1fffu;
    if (rest > 0x1000u || (rest == 0x1000u && (r & 1u))) ++r;
    h = static_cast<uint16_t>(sign | r);
  }
  // decode
  const uint32_t hs = (h & 0x8000u) << 16;
  const uint32_t he = (h >> 10) & 0x1fu, hm = h & 0x3ffu;
  uint32_t out;
  if (he == 0) {
    const float v = static_cast<float>(hm) * 5.9604644775390625e-8f;  // 2^-24
    std::memcpy(&out, &v, 4);
    out |= hs;
  } else if (he == 31) {
    out = hs | 0x7f800000u | (hm << 13);
  } else {
    out = hs | ((he + 112) << 23) | (hm << 13);
  }
  float f;
  std::memcpy(&f, &out, 4);
  return f;
}

// Quantize + decode `count` values in `format` (nearest rounding), on the
// device through the library's codecs (FP16 on the host).
std::vector<float> quantized(CudaRuntime &runtime, CudaFactorFormat format,
                             const std::vector<float> &values) {
  if (format == CudaFactorFormat::Fp32) return values;
  if (format == CudaFactorFormat::Fp16) {
    std::vector<float> out(values.size());
    for (size_t i = 0; i < values.size(); ++i) out[i] = toHalfAndBack(values[i]);
    return out;
  }
  msq_ctx *ctx = runtime.context();
  const int codec = codecOf(format);
  const size_t count = values.size();
  Buffer in(count * sizeof(float)), out(count * sizeof(float)),
      codes(msq_storage_bytes(codec, count) + 16), scales(msq_scale_bytes(codec, count, 0) + 16);
  toDevice(in.as<float>(), values.data(), count * sizeof(float));
  runtime.check(msq_encode(ctx, codec, in.as<float>(), count, 0, codes.as<uint8_t>(),
                           scales.as<uint8_t>()),
                "quantize");
  runtime.check(msq_decode(ctx, codec, codes.as<uint8_t>(), scales.as<uint8_t>(), count, 0,
                           out.as<float>()),
                "quantize");
  runtime.check(msq_synchronize(ctx), "quantize");
  std::vector<float> result(count);
  toHost(result.data(), out.as<float>(), count * sizeof(float));
  return result;
}

// relative_error (:270-280): ||value - reference|| / ||reference||
double relativeErrorF(const std::vector<float> &value, const std::vector<float> &reference) {
  double d = 0.0, r = 0.0;
  for (size_t i = 0; i < value.size(); ++i) {
    d = std::hypot(d, static_cast<double>(value[i]) - static_cast<double>(reference[i]));
    r = std::hypot(r, static_cast<double>(reference[i]));
  }
  return d / r;
}

double relativeErrorD(const std::vector<double> &x, const std::vector<double> &ref) {
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < x.size(); ++i) {
    num += (x[i] - ref[i]) * (x[i] - ref[i]);
    den += ref[i] * ref[i];
  }
  return std::sqrt(num / den);
}

// invert_basis (:600-637): the inverse of the FP32 basis by LU with partial
// pivoting (FP64 here) and its 1-norm condition ||V||_1 ||V^-1||_1 (the
// reference estimates the same quantity with sgecon).  False when singular.
bool invertBasis(const std::vector<float> &basis, size_t n, std::vector<float> &inverse,
                 double &condition) {
  std::vector<double> a(basis.begin(), basis.end()), inv(n * n, 0.0);
  for (size_t i = 0; i < n; ++i) inv[i + i * n] = 1.0;
  double norm = 0.0;
  for (size_t c = 0; c < n; ++c) {
    double sum = 0.0;
    for (size_t r = 0; r < n; ++r) sum += std::fabs(a[r + c * n]);
    norm = std::max(norm, sum);
  }
  for (size_t k = 0; k < n; ++k) {
    size_t p = k;
    for (size_t r = k + 1; r < n; ++r)
      if (std::fabs(a[r + k * n]) > std::fabs(a[p + k * n])) p = r;
    if (a[p + k * n] == 0.0) {
      condition = std::numeric_limits<double>::infinity();
      return false;
    }
    if (p != k)
      for (size_t c = 0; c < n; ++c) {
        std::swap(a[k + c * n], a[p + c * n]);
        std::swap(inv[k + c * n], inv[p + c * n]);
      }
    const double d = a[k + k * n];
    for (size_t c = 0; c < n; ++c) {
      a[k + c * n] /= d;
      inv[k + c * n] /= d;
    }
    for (size_t r = 0; r < n; ++r) {
      if (r == k) continue;
      const double f = a[r + k * n];
      if (f == 0.0) continue;
      for (size_t c = 0; c < n; ++c) {
        a[r + c * n] -= f * a[k + c * n];
        inv[r + c * n] -= f * inv[k + c * n];
      }
    }
  }
  double inv_norm = 0.0;
  for (size_t c = 0; c < n; ++c) {
    double sum = 0.0;
    for (size_t r = 0; r < n; ++r) sum += std::fabs(inv[r + c * n]);
    inv_norm = std::max(inv_norm, sum);
  }
  condition = norm * inv_norm;
  inverse.assign(inv.begin(), inv.end());
  return std::isfinite(condition);
}

bool lowBitBasis(CudaFactorFormat format) {
  return format == CudaFactorFormat::Fp8E4M3 || format == CudaFactorFormat::Fp8E5M2 ||
         format == CudaFactorFormat::MxFp8E4M3 || format == CudaFactorFormat::MxFp4E2M1;
}

}  // namespace

const char *cudaFactorFormatName(CudaFactorFormat format) {
  switch (format) {
    case CudaFactorFormat::Fp32: return "fp32";
    case CudaFactorFormat::Fp16: return "fp16";
    case CudaFactorFormat::Bf16: return "bf16";
    case CudaFactorFormat::Fp8E4M3: return "fp8_e4m3";
    case CudaFactorFormat::Fp8E5M2: return "fp8_e5m2";
    case CudaFactorFormat::MxFp8E4M3: return "mxfp8_e4m3";
    case CudaFactorFormat::MxFp4E2M1: return "mxfp4_e2m1";
  }
  return "unknown";
}

std::vector<CudaPrecisionPlan> cudaPrecisionPlans() {
  using F = CudaFactorFormat;
  return {{"fp32_baseline", F::Fp32, F::Fp32},     {"spectrum_fp16", F::Fp32, F::Fp16},
          {"spectrum_bf16", F::Fp32, F::Bf16},     {"spectrum_e4m3", F::Fp32, F::Fp8E4M3},
          {"spectrum_e5m2", F::Fp32, F::Fp8E5M2},  {"spectrum_mxfp8", F::Fp32, F::MxFp8E4M3},
          {"spectrum_mxfp4", F::Fp32, F::MxFp4E2M1}, {"basis_fp16", F::Fp16, F::Fp32},
          {"basis_bf16", F::Bf16, F::Fp32},        {"basis_e4m3", F::Fp8E4M3, F::Fp32},
          {"basis_e5m2", F::Fp8E5M2, F::Fp32},     {"basis_mxfp8", F::MxFp8E4M3, F::Fp32},
          {"basis_mxfp4", F::MxFp4E2M1, F::Fp32},  {"fp16_mxfp8", F::Fp16, F::MxFp8E4M3},
          {"bf16_mxfp8", F::Bf16, F::MxFp8E4M3},   {"e4m3_mxfp4", F::Fp8E4M3, F::MxFp4E2M1}};
}

CudaSpectralResult runCudaSpectral(CudaRuntime &runtime, const CudaProblem &problem,
                                   const CudaPrecisionPlan &plan, size_t max_corrections,
                                   double tolerance) {
  if (problem.prepared_matrix == nullptr || problem.order == 0)
    failSpectral("run_spectral: no matrix");
  const size_t n = problem.order;
  const size_t count = n * n;
  const std::vector<double> &matrix = problem.prepared_matrix->values;
  CudaSpectralResult result;
  result.plan = plan.name;
  result.basis_format = cudaFactorFormatName(plan.basis);
  result.spectrum_format = cudaFactorFormatName(plan.spectrum);
  result.order = n;
  result.condition = problem.condition;
  const double nan = std::numeric_limits<double>::quiet_NaN();
  result.basis_relative_error = result.spectrum_relative_error = result.basis_condition = nan;
  result.initial_error = result.final_error = result.final_residual = nan;
  result.basis_bits_per_value = storageBits(plan.basis, count);
  result.spectrum_bits_per_value = storageBits(plan.spectrum, n);
  result.weighted_factor_storage_bits =
      (result.basis_bits_per_value * count + result.spectrum_bits_per_value * n) /
      static_cast<double>(count + n);
  const bool fp16_basis = plan.basis == CudaFactorFormat::Fp16;
  const bool low = lowBitBasis(plan.basis) && problem.condition < 1000.0;
  result.product_backend = fp16_basis ? "fp16_products" : low ? "lowbit_products" : "fp32_gemm";
  result.arithmetic_format = fp16_basis ? "fp16_fp32_mixed_to_fp32"
                             : low      ? "adaptive_low_then_fp32"
                                        : "fp32";

  msq_ctx *ctx = runtime.context();
  const int32_t nn = static_cast<int32_t>(n);
  const int64_t off = 0;
  const size_t bytes = count * sizeof(float);

  // factor_float: FP32 eigendecomposition, root spectrum s = sqrt(lambda)
  Buffer a(bytes), a_lo(bytes), work(bytes), v(bytes), w(n * sizeof(float));
  std::vector<float> a_hi(count), a_low(count);
  for (size_t i = 0; i < count; ++i) {
    a_hi[i] = static_cast<float>(matrix[i]);
    a_low[i] = static_cast<float>(matrix[i] - a_hi[i]);
  }
  toDevice(a.as<float>(), a_hi.data(), bytes);
  toDevice(a_lo.as<float>(), a_low.data(), bytes);
  toDevice(work.as<float>(), a_hi.data(), bytes);
  runtime.check(msq_jacobi_batched(ctx, work.as<float>(), v.as<float>(), w.as<float>(), &nn, &off,
                                   1, 1.0e-7, 20, nullptr, nullptr),
                "factor_float");
  runtime.check(msq_synchronize(ctx), "factor_float");
  std::vector<float> basis(count), root_spectrum(n);
  toHost(basis.data(), v.as<float>(), bytes);
  toHost(root_spectrum.data(), w.as<float>(), n * sizeof(float));
  for (float &value : root_spectrum) {
    if (!(value > 0.0f) || !std::isfinite(value))
      failSpectral("The FP32 factor has an invalid spectrum.");
    value = std::sqrt(value);
  }

  // basis inverse: V^T of the quantized basis, or the FP16 quantization of
  // the FP32 basis's explicit inverse
  std::vector<float> inverse;
  if (fp16_basis) {
    if (!invertBasis(basis, n, inverse, result.basis_condition) ||
        !(result.basis_condition < 1.0e4)) {
      result.reason = "ill_conditioned_basis";
      return result;
    }
  } else {
    result.basis_condition = 1.0;
  }
  const std::vector<float> vq = quantized(runtime, plan.basis, basis);
  const std::vector<float> sq = quantized(runtime, plan.spectrum, root_spectrum);
  result.basis_relative_error = relativeErrorF(vq, basis);
  result.spectrum_relative_error = relativeErrorF(sq, root_spectrum);
  for (float value : sq) {
    if (!(value > 0.0f) || !std::isfinite(value)) {
      result.reason = "invalid_spectrum";
      return result;
    }
  }
  std::vector<float> vinv(count);
  if (fp16_basis) {
    vinv = quantized(runtime, CudaFactorFormat::Fp16, inverse);
    for (float value : vinv)
      if (!std::isfinite(value)) {
        result.reason = "ill_conditioned_basis";
        return result;
      }
  } else {
    for (size_t c = 0; c < n; ++c)
      for (size_t r = 0; r < n; ++r) vinv[r + c * n] = vq[c + r * n];
  }
  result.accepted = true;

  // device operands: V, V^-1, lambda_q = sq^2 (the GEMM epilogue divides by
  // sqrt(lambda_i) + sqrt(lambda_j) = sq_i + sq_j), diag(sq)-scaled V
  Buffer dv(bytes), dvinv(bytes), dlam(n * sizeof(float)), scaled(bytes), x_hi(bytes),
      x_lo(bytes), r(bytes), t0(bytes), t1(bytes), norms(2 * sizeof(double));
  std::vector<float> lam_q(n), vs(count);
  for (size_t i = 0; i < n; ++i) lam_q[i] = sq[i] * sq[i];
  for (size_t c = 0; c < n; ++c)
    for (size_t rr = 0; rr < n; ++rr) vs[rr + c * n] = vq[rr + c * n] * sq[c];
  // low-bit products: operands re-encoded to the basis format
  // (an FP16 basis scales in FP16: scale_columns_f16)
  const std::vector<float> vs_op =
      low ? quantized(runtime, plan.basis, vs)
          : fp16_basis ? quantized(runtime, CudaFactorFormat::Fp16, vs) : vs;
  const std::vector<float> vinv_op = low ? quantized(runtime, plan.basis, vinv) : vinv;
  toDevice(dv.as<float>(), vq.data(), bytes);
  toDevice(dvinv.as<float>(), vinv.data(), bytes);
  toDevice(dlam.as<float>(), lam_q.data(), n * sizeof(float));
  toDevice(scaled.as<float>(), vs_op.data(), bytes);
  toDevice(t1.as<float>(), vinv_op.data(), bytes);
  runtime.check(msq_gemm(ctx, 0, 0, scaled.as<float>(), t1.as<float>(), &nn, &off, 1, nullptr,
                         x_hi.as<float>()),
                "initial root");
  if (cudaMemset(x_lo.as<float>(), 0, bytes) != cudaSuccess) failSpectral("initial root");

  auto residual = [&]() {
    runtime.check(msq_residual_general(ctx, a.as<float>(), a_lo.as<float>(), x_hi.as<float>(),
                                       x_lo.as<float>(), &nn, &off, 1, r.as<float>(),
                                       norms.as<double>()),
                  "residual_and_norm");
    double host[2];
    toHost(host, norms.as<double>(), sizeof(host));
    if (!(host[1] > 0.0) || !std::isfinite(host[0])) return std::numeric_limits<double>::infinity();
    return std::sqrt(host[0] / host[1]);
  };
  auto forward = [&]() {
    if (problem.supplied_reference == nullptr) return nan;
    std::vector<float> hi(count), lo(count);
    toHost(hi.data(), x_hi.as<float>(), bytes);
    toHost(lo.data(), x_lo.as<float>(), bytes);
    std::vector<double> x(count);
    for (size_t i = 0; i < count; ++i) x[i] = static_cast<double>(hi[i]) + lo[i];
    return relativeErrorD(x, *problem.supplied_reference);
  };
  // one product on low-bit or FP32 operands: C = L R (L, R device)
  std::vector<float> host_tmp(count);
  auto lowOperand = [&](float *device) {
    toHost(host_tmp.data(), device, bytes);
    const std::vector<float> q = quantized(runtime, plan.basis, host_tmp);
    toDevice(device, q.data(), bytes);
  };

  double measured = residual();
  result.history.push_back({0, measured, forward(), false});
  result.initial_error = result.history.front().forward_error;
  const double divergence_limit = std::max(1.0, 1.0e4 * measured);
  bool low_on = true;
  double low_prev = measured;
  int low_stalls = 0;
  for (size_t iteration = 0;
       measured > tolerance && iteration < max_corrections && measured < divergence_limit;
       ++iteration) {
    const bool use_low = low && low_on && measured > 1.0e-3;
    // W = Vinv R; C = (W V) o H; W = V C; E = W Vinv
    float *R = r.as<float>();
    const float *Vinv = dvinv.as<float>();
    const float *V = dv.as<float>();
    if (use_low) {
      toDevice(t1.as<float>(), vinv_op.data(), bytes);
      lowOperand(R);
      runtime.check(msq_gemm(ctx, 0, 0, t1.as<float>(), R, &nn, &off, 1, nullptr, t0.as<float>()),
                    "correction");
      lowOperand(t0.as<float>());
      toDevice(t1.as<float>(), vq.data(), bytes);  // the basis is already in its format
      runtime.check(msq_gemm(ctx, 0, 0, t0.as<float>(), t1.as<float>(), &nn, &off, 1,
                             dlam.as<float>(), R),
                    "correction");
      lowOperand(R);
      runtime.check(msq_gemm(ctx, 0, 0, t1.as<float>(), R, &nn, &off, 1, nullptr, t0.as<float>()),
                    "correction");
      lowOperand(t0.as<float>());
      toDevice(t1.as<float>(), vinv_op.data(), bytes);
      runtime.check(msq_gemm(ctx, 0, 0, t0.as<float>(), t1.as<float>(), &nn, &off, 1, nullptr, R),
                    "correction");
    } else {
      runtime.check(msq_gemm(ctx, 0, 0, Vinv, R, &nn, &off, 1, nullptr, t0.as<float>()),
                    "correction");
      runtime.check(msq_gemm(ctx, 0, 0, t0.as<float>(), V, &nn, &off, 1, dlam.as<float>(),
                             t1.as<float>()),
                    "correction");
      runtime.check(msq_gemm(ctx, 0, 0, V, t1.as<float>(), &nn, &off, 1, nullptr, t0.as<float>()),
                    "correction");
      runtime.check(msq_gemm(ctx, 0, 0, t0.as<float>(), Vinv, &nn, &off, 1, nullptr, R),
                    "correction");
    }
    runtime.check(msq_working_add(ctx, x_hi.as<float>(), x_lo.as<float>(), R, &nn, &off, 1),
                  "working_add");
    measured = residual();
    result.history.push_back({iteration + 1, measured, forward(), use_low});
    if (use_low) ++result.low_product_corrections;
    if (low && low_on && measured > tolerance) {
      low_stalls = measured > low_prev * 0.5 ? low_stalls + 1 : 0;
      low_prev = measured;
      low_on = low_stalls < 2;
    }
  }
  result.iterations = result.correction_count = result.history.size() - 1;
  result.final_residual = result.history.back().residual;
  result.final_error = result.history.back().forward_error;
  result.converged = result.final_residual <= tolerance;
  if (result.converged) result.reason = "converged";
  else if (!std::isfinite(result.final_residual)) result.reason = "nonfinite_residual";
  else if (result.final_residual >= divergence_limit) result.reason = "divergent";
  else result.reason = "correction_limit";
  return result;
}

}  // namespace mixed_sqrt
