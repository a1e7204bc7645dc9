// cuda_backend: runCudaCase / runCuda over the C ABI (host code; the CUDA
// work is enqueued through msq_* entry points).  Follows runMetalCase's
// GPU-resident branch (src/metal_solver.cpp:477-604) and
// solveGpuResidentSpd (src/metal_solver.cpp:92-336).
#include "cuda_backend.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <utility>
#include <vector>
#include <stdexcept>

namespace mixed_sqrt {
namespace {

using Clock = std::chrono::steady_clock;

[[noreturn]] void failCuda(const std::string &message) { throw std::runtime_error(message); }

double since(Clock::time_point start) {
  return std::chrono::duration<double>(Clock::now() - start).count();
}

class DeviceBuffer {
 public:
  explicit DeviceBuffer(size_t bytes) : bytes_(bytes) {
    if (bytes_ != 0 && cudaMalloc(&ptr_, bytes_) != cudaSuccess) {
      failCuda("cuda_backend: device allocation failed");
    }
  }
  ~DeviceBuffer() {
    if (ptr_ != nullptr) cudaFree(ptr_);
  }
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  template <typename T>
  T *as() const { return static_cast<T *>(ptr_); }

 private:
  void *ptr_ = nullptr;
  size_t bytes_ = 0;
};

void copyIn(void *dst, const void *src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    failCuda("cuda_backend: host to device copy failed");
}

void copyOut(void *dst, const void *src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    failCuda("cuda_backend: device to host copy failed");
}

// relativeError (src/numerics.cpp:230-240)
double relativeErrorOf(const std::vector<double> &x, const std::vector<double> &ref) {
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < x.size(); ++i) {
    const double d = x[i] - ref[i];
    num += d * d;
    den += ref[i] * ref[i];
  }
  return std::sqrt(num / den);
}

// relativeSymmetryError (src/numerics.cpp:252-264)
double symmetryErrorOf(const std::vector<double> &x, size_t n) {
  double num = 0.0, den = 0.0;
  for (size_t c = 0; c < n; ++c)
    for (size_t r = 0; r < n; ++r) {
      const double v = x[r + c * n];
      const double d = v - x[c + r * n];
      num += d * d;
      den += v * v;
    }
  return den > 0.0 ? std::sqrt(num / den) : 0.0;
}

int codecFor(CudaBasisFormat format) {
  switch (format) {
    case CudaBasisFormat::Bf16: return MSQ_FMT_BF16;
    case CudaBasisFormat::Fp8E4M3FnRowScale: return MSQ_FMT_FP8_E4M3FN_ROWSCALE;
    case CudaBasisFormat::Mxfp4E2M1: return MSQ_FMT_MXFP4_E2M1;
    case CudaBasisFormat::Fp8E4M3Fn: return MSQ_FMT_FP8_E4M3FN;
    case CudaBasisFormat::Fp8E5M2: return MSQ_FMT_FP8_E5M2;
    case CudaBasisFormat::Mxfp8E4M3Fn: return MSQ_FMT_MXFP8_E4M3FN;
    case CudaBasisFormat::Mxfp8E5M2: return MSQ_FMT_MXFP8_E5M2;
    case CudaBasisFormat::Fp4E2M1: return MSQ_FMT_FP4_E2M1;
    default: return MSQ_FMT_FP32;
  }
}

constexpr CudaBasisFormat kBasisFormats[] = {
    CudaBasisFormat::Fp32,      CudaBasisFormat::Bf16,        CudaBasisFormat::Fp8E4M3FnRowScale,
    CudaBasisFormat::Mxfp4E2M1, CudaBasisFormat::Fp8E4M3Fn,   CudaBasisFormat::Fp8E5M2,
    CudaBasisFormat::Mxfp8E4M3Fn, CudaBasisFormat::Mxfp8E5M2, CudaBasisFormat::Fp4E2M1};

}  // namespace

const char *cudaBasisFormatName(CudaBasisFormat format) {
  switch (format) {
    case CudaBasisFormat::Fp32: return "fp32";
    case CudaBasisFormat::Bf16: return "bf16";
    case CudaBasisFormat::Fp8E4M3FnRowScale: return "fp8_e4m3fn_rowscale";
    case CudaBasisFormat::Mxfp4E2M1: return "mxfp4_e2m1";
    case CudaBasisFormat::Fp8E4M3Fn: return "fp8_e4m3fn";
    case CudaBasisFormat::Fp8E5M2: return "fp8_e5m2";
    case CudaBasisFormat::Mxfp8E4M3Fn: return "mxfp8_e4m3fn";
    case CudaBasisFormat::Mxfp8E5M2: return "mxfp8_e5m2";
    case CudaBasisFormat::Fp4E2M1: return "fp4_e2m1";
  }
  return "unknown";
}

CudaBasisFormat cudaBasisFormatForCliName(const std::string &name) {
  for (CudaBasisFormat f : kBasisFormats) {
    if (name == cudaBasisFormatName(f)) return f;
  }
  failCuda("Unsupported precision: " + name);
}

const char *cudaSpectrumFormatName(CudaSpectrumFormat format) {
  switch (format) {
    case CudaSpectrumFormat::Fp32: return "fp32";
    case CudaSpectrumFormat::Fp8E4M3FnLogS: return "fp8_e4m3fn_log_s";
    case CudaSpectrumFormat::Fp4E2M1LogS: return "fp4_e2m1_log_s";
  }
  return "unknown";
}

CudaSpectrumFormat cudaSpectrumFormatForCliName(const std::string &name) {
  for (CudaSpectrumFormat f : {CudaSpectrumFormat::Fp32, CudaSpectrumFormat::Fp8E4M3FnLogS,
                               CudaSpectrumFormat::Fp4E2M1LogS}) {
    if (name == cudaSpectrumFormatName(f)) return f;
  }
  failCuda("Unsupported spectrum precision: " + name);
}

const char *cudaRoundingModeName(CudaRoundingMode mode) {
  return mode == CudaRoundingMode::Stochastic ? "stochastic" : "nearest";
}

CudaRoundingMode cudaRoundingModeForCliName(const std::string &name) {
  if (name == "nearest") return CudaRoundingMode::Nearest;
  if (name == "stochastic") return CudaRoundingMode::Stochastic;
  failCuda("--rounding requires nearest or stochastic.");
}

double cudaBasisOrthogonalityTolerance(CudaBasisFormat format) {
  switch (format) {
    case CudaBasisFormat::Fp32: return 1.0e-3;
    case CudaBasisFormat::Bf16: return 5.0e-3;
    case CudaBasisFormat::Mxfp4E2M1:
    case CudaBasisFormat::Fp4E2M1: return 5.0e-1;  // 4-bit storage
    default: return 1.5e-1;                        // 8-bit storage
  }
}

CudaRuntime::CudaRuntime(int device) {
  if (msq_create(&ctx_, device) != MSQ_OK || ctx_ == nullptr) {
    failCuda("cuda_backend: could not create the CUDA context");
  }
}

CudaRuntime::~CudaRuntime() { msq_destroy(ctx_); }

void CudaRuntime::check(int status, const char *what) const {
  if (status != MSQ_OK) {
    failCuda(std::string(what) + ": " + msq_last_error(ctx_));
  }
}

CaseResult runCudaCase(CudaRuntime &runtime, const CudaSolverConfiguration &configuration,
                       const CudaProblem &problem) {
  if (problem.prepared_matrix == nullptr) failCuda("A prepared matrix is required.");
  const PreparedMatrix &prepared = *problem.prepared_matrix;
  const size_t n = problem.order;
  if (n < 1 || n > 2048 || prepared.values.size() != n * n) {
    failCuda("The GPU-resident matrix dimensions are invalid.");
  }
  if (!std::all_of(prepared.values.begin(), prepared.values.end(),
                   [](double v) { return std::isfinite(v); })) {
    failCuda("The prepared matrix is nonfinite.");
  }
  if (!std::isfinite(problem.tolerance) || !(problem.tolerance > 0.0)) {
    failCuda("The residual tolerance must be positive and finite.");
  }
  msq_ctx *ctx = runtime.context();
  const size_t elements = n * n;
  const int32_t nn = static_cast<int32_t>(n);
  const int64_t off = 0;

  CaseResult result;
  result.paper_test_set = prepared.paper_test_set;
  result.matrix_family = prepared.matrix_family;
  result.matrix_type = prepared.matrix_type;
  result.solver_backend = "cuda";
  result.order = n;
  result.condition = prepared.condition;
  result.precision = cudaBasisFormatName(configuration.basis_format);
  result.basis_precision = result.precision;
  result.spectrum_precision = "fp32";
  result.correction_mode =
      configuration.native_correction ? "native_quantized" : "fp32_reorthogonalized";
  result.kernel_path = "tiled";
  result.rounding_mode = cudaRoundingModeName(configuration.rounding_mode);
  result.rounding_seed = configuration.rounding_seed;
  result.stopping_policy =
      configuration.native_correction && configuration.stop_on_stagnation ? "stagnation" : "fixed_budget";
  result.dispatch_policy = configuration.native_correction ? "fused" : "not_applicable";
  result.precision_policy = configuration.basis_format == CudaBasisFormat::Fp32 ||
                                    configuration.basis_format == CudaBasisFormat::Bf16
                                ? "required_full_accuracy"
                                : "measured_controlled";
  result.execution_model = configuration.basis_format == CudaBasisFormat::Fp32
                               ? "native_low_correction"
                               : "quantized_factor_reorthogonalized_fp32_correction";
  std::ostringstream name;
  name << "spd_n" << n << "_cuda_" << result.precision;
  result.name = name.str();
  result.fp32_basis_bytes = elements * sizeof(float);

  // Host -> device: the FP64 input as an FP32 high word (the eigensolver's
  // input) plus its low word, so the residual sees the full matrix, as
  // solveGpuResidentSpd keeps A as a WorkingFloat (src/metal_solver.cpp:186-196).
  std::vector<float> a32(elements), a32_lo(elements);
  for (size_t i = 0; i < elements; ++i) {
    a32[i] = static_cast<float>(prepared.values[i]);
    a32_lo[i] = static_cast<float>(prepared.values[i] - static_cast<double>(a32[i]));
  }
  DeviceBuffer a_lo(elements * sizeof(float));
  copyIn(a_lo.as<float>(), a32_lo.data(), elements * sizeof(float));
  DeviceBuffer a(elements * sizeof(float)), work(elements * sizeof(float)),
      v(elements * sizeof(float)), lam(n * sizeof(float)), f(elements * sizeof(float)),
      fq(elements * sizeof(float)), x_hi(elements * sizeof(float)), x_lo(elements * sizeof(float)),
      r(elements * sizeof(float)), ws(2 * elements * sizeof(float)), gram(elements * sizeof(float)),
      codes(elements * 4 + 64), scales(elements + 4 * n + 64), norms(2 * sizeof(double)),
      ones(n * sizeof(float));
  copyIn(a.as<float>(), a32.data(), elements * sizeof(float));
  copyIn(work.as<float>(), a32.data(), elements * sizeof(float));
  const std::vector<float> unit(n, 1.0f);
  copyIn(ones.as<float>(), unit.data(), n * sizeof(float));

  const auto mixed_start = Clock::now();
  runtime.check(msq_jacobi_batched(ctx, work.as<float>(), v.as<float>(), lam.as<float>(), &nn, &off,
                                   1, configuration.jacobi_tolerance,
                                   configuration.jacobi_max_sweeps, nullptr, nullptr),
                "symmetricJacobi");
  runtime.check(msq_synchronize(ctx), "symmetricJacobi");
  result.times.low_eigen_seconds = since(mixed_start);
  std::vector<float> eig(n);
  copyOut(eig.data(), lam.as<float>(), n * sizeof(float));
  for (float value : eig) {
    if (!(value > 0.0f) || !std::isfinite(value)) {
      failCuda("The frozen GPU spectrum contains an invalid value.");
    }
  }

  // Orthogonality of a basis (quantized or not): ||V V^T - I||_F / sqrt(n)
  // from the FP32 Gram product, summed on the host as
  // measureF32Orthogonality does (src/metal_runtime.cpp:742-776).
  auto orthogonality = [&](const float *basis_t) {
    runtime.check(msq_reconstruct(ctx, MSQ_FMT_FP32, basis_t, nullptr, &nn, &off, 1,
                                  gram.as<float>()),
                  "measureF32Orthogonality");
    std::vector<float> g(elements);
    copyOut(g.data(), gram.as<float>(), elements * sizeof(float));
    double sum = 0.0;
    for (size_t c = 0; c < n; ++c)
      for (size_t rr = 0; rr < n; ++rr) {
        const double d = static_cast<double>(g[rr + c * n]) - (rr == c ? 1.0 : 0.0);
        sum += d * d;
      }
    return std::sqrt(sum / static_cast<double>(n));
  };
  // V^T in K-major order: the factor with lambda = 1.
  runtime.check(msq_make_factor(ctx, v.as<float>(), ones.as<float>(), &nn, &off, 1, f.as<float>()),
                "transpose basis");
  result.frozen_basis_orthogonality = orthogonality(f.as<float>());

  // Quantization of the basis (and of the factor built on it): nearest, or
  // the device quantizers' stochastic rounding with the run's seed on
  // stream 0, as the reference quantizes its basis (src/metal_solver.cpp:219).
  const bool stochastic = configuration.rounding_mode == CudaRoundingMode::Stochastic;
  auto encode_basis = [&](int c, const float *src, size_t rl) {
    return stochastic ? msq_encode_stochastic(ctx, c, src, elements, rl, configuration.rounding_seed,
                                              0u, codes.as<uint8_t>(), scales.as<uint8_t>())
                      : msq_encode(ctx, c, src, elements, rl, codes.as<uint8_t>(),
                                   scales.as<uint8_t>());
  };
  CudaBasisFormat format = configuration.basis_format;
  const int codec = codecFor(format);
  const size_t row_length = codec == MSQ_FMT_FP8_E4M3FN_ROWSCALE ? n : 0;
  if (format != CudaBasisFormat::Fp32) {
    const auto quantize_start = Clock::now();
    runtime.check(encode_basis(codec, f.as<float>(), row_length), "quantizeAndDecode");
    runtime.check(msq_decode(ctx, codec, codes.as<uint8_t>(), scales.as<uint8_t>(), elements,
                             row_length, fq.as<float>()),
                  "quantizeAndDecode");
    result.quantized_basis_orthogonality = orthogonality(fq.as<float>());
    result.low_factor_basis_bytes =
        msq_storage_bytes(codec, elements) + msq_scale_bytes(codec, elements, row_length ? row_length : 1);
    const bool usable = std::isfinite(result.quantized_basis_orthogonality) &&
                        result.quantized_basis_orthogonality <=
                            cudaBasisOrthogonalityTolerance(format);
    if (usable || !configuration.orthogonality_gate) {
      result.selected_basis_stage = cudaBasisFormatName(format);
    } else {
      // Escalation of a rejected low-precision basis (src/metal_solver.cpp:225-235).
      result.selected_basis_stage = std::string(cudaBasisFormatName(format)) + "_rejected_to_fp32";
      ++result.precision_escalations;
      format = CudaBasisFormat::Fp32;
    }
    result.factor_quantization_seconds += since(quantize_start);
  } else {
    result.selected_basis_stage = "fp32";
  }
  // The root eigenvalues s = sqrt(lambda) of the initial root, optionally in
  // log-affine storage: quantizeAndDecode of the spectrum on stream 1 and the
  // reference's validity check (src/metal_solver.cpp:241-263).  The
  // corrections below use the FP32 spectrum, as the reference returns to
  // the stable roots for them (:304-310).
  result.spectrum_precision = cudaSpectrumFormatName(configuration.spectrum_format);
  DeviceBuffer lam0(n * sizeof(float));
  bool quantized_spectrum = false;
  if (configuration.spectrum_format != CudaSpectrumFormat::Fp32) {
    const auto spectrum_start = Clock::now();
    const int sfmt = configuration.spectrum_format == CudaSpectrumFormat::Fp8E4M3FnLogS
                         ? MSQ_FMT_FP8_E4M3FN
                         : MSQ_FMT_FP4_E2M1;
    std::vector<float> roots(n);
    for (size_t i = 0; i < n; ++i) roots[i] = std::sqrt(eig[i]);
    DeviceBuffer s_in(n * sizeof(float)), s_out(n * sizeof(float)), s_codes(n + 16),
        s_meta(msq_spectrum_metadata_bytes(n) + 16);
    copyIn(s_in.as<float>(), roots.data(), n * sizeof(float));
    runtime.check(msq_spectrum_encode(ctx, sfmt, s_in.as<float>(), n,
                                      stochastic ? MSQ_ROUND_STOCHASTIC : MSQ_ROUND_NEAREST,
                                      configuration.rounding_seed, 1u, s_codes.as<uint8_t>(),
                                      s_meta.as<float>()),
                  "quantizeAndDecode spectrum");
    runtime.check(msq_spectrum_decode(ctx, sfmt, s_codes.as<uint8_t>(), s_meta.as<float>(), n,
                                      s_out.as<float>()),
                  "quantizeAndDecode spectrum");
    runtime.check(msq_synchronize(ctx), "quantizeAndDecode spectrum");
    std::vector<float> quantized(n);
    copyOut(quantized.data(), s_out.as<float>(), n * sizeof(float));
    result.factor_quantization_seconds += since(spectrum_start);
    bool usable = true;
    for (float value : quantized) usable = usable && value > 0.0f && std::isfinite(value);
    if (usable) {
      for (size_t i = 0; i < n; ++i) quantized[i] *= quantized[i];  // lambda = s^2
      copyIn(lam0.as<float>(), quantized.data(), n * sizeof(float));
      quantized_spectrum = true;
      result.selected_spectrum_stage = cudaSpectrumFormatName(configuration.spectrum_format);
    } else {
      result.selected_spectrum_stage =
          std::string(cudaSpectrumFormatName(configuration.spectrum_format)) + "_rejected_to_fp32";
      ++result.precision_escalations;
    }
  } else {
    result.selected_spectrum_stage = "fp32";
  }

  // Initial root X0 = W W^T, W = V diag(lambda^(1/4)).
  const auto initial_start = Clock::now();
  runtime.check(msq_make_factor(ctx, v.as<float>(), quantized_spectrum ? lam0.as<float>() : lam.as<float>(),
                                &nn, &off, 1, f.as<float>()),
                "prepareFrozenSpectralFactor");
  if (format == CudaBasisFormat::Fp32) {
    runtime.check(msq_reconstruct(ctx, MSQ_FMT_FP32, f.as<float>(), nullptr, &nn, &off, 1,
                                  x_hi.as<float>()),
                  "reconstructTiled");
  } else {
    const int fcodec = codecFor(format);
    const size_t frow = fcodec == MSQ_FMT_FP8_E4M3FN_ROWSCALE ? n : 0;
    runtime.check(encode_basis(fcodec, f.as<float>(), frow), "quantize factor");
    // Tensor-core paths straight from the codes: BF16, per-row FP8, MXFP4 and
    // (row-aligned blocks) MXFP8.  The other reference formats decode to
    // FP32 and run the FP32 GEMM, as reconstructLowFactorTiled does.
    const bool tensor = fcodec == MSQ_FMT_BF16 || fcodec == MSQ_FMT_FP8_E4M3FN_ROWSCALE ||
                        fcodec == MSQ_FMT_MXFP4_E2M1 ||
                        (fcodec == MSQ_FMT_MXFP8_E4M3FN && n % 32 == 0);
    if (tensor) {
      runtime.check(msq_reconstruct(ctx, fcodec, codes.as<uint8_t>(), scales.as<float>(), &nn,
                                    &off, 1, x_hi.as<float>()),
                    "reconstructLowFactorTiled");
    } else {
      runtime.check(msq_decode(ctx, fcodec, codes.as<uint8_t>(), scales.as<uint8_t>(), elements,
                               0, fq.as<float>()),
                    "reconstructLowFactorTiled");
      runtime.check(msq_reconstruct(ctx, MSQ_FMT_FP32, fq.as<float>(), nullptr, &nn, &off, 1,
                                    x_hi.as<float>()),
                    "reconstructLowFactorTiled");
    }
  }
  if (cudaMemset(x_lo.as<float>(), 0, elements * sizeof(float)) != cudaSuccess)
    failCuda("initializeWorkingRoot failed");
  runtime.check(msq_synchronize(ctx), "initial root");
  result.times.initial_gpu_seconds = since(initial_start);

  auto residual = [&]() {
    const auto t0 = Clock::now();
    runtime.check(msq_residual(ctx, a.as<float>(), a_lo.as<float>(), x_hi.as<float>(),
                               x_lo.as<float>(), &nn, &off, 1,
                               r.as<float>(), norms.as<double>()),
                  "computeWorkingResidual");
    double host[2];
    copyOut(host, norms.as<double>(), sizeof(host));
    result.times.residual_fp64_seconds += since(t0);
    if (!(host[1] > 0.0) || !std::isfinite(host[0]) || !std::isfinite(host[1]))
      return std::numeric_limits<double>::infinity();
    return std::sqrt(host[0] / host[1]);
  };
  auto root_now = [&]() {
    std::vector<float> hi(elements), lo(elements);
    copyOut(hi.data(), x_hi.as<float>(), elements * sizeof(float));
    copyOut(lo.data(), x_lo.as<float>(), elements * sizeof(float));
    std::vector<double> root(elements);
    for (size_t i = 0; i < elements; ++i) root[i] = static_cast<double>(hi[i]) + lo[i];
    return root;
  };
  auto forward_error = [&](const std::vector<double> &root) {
    if (problem.supplied_reference == nullptr ||
        problem.supplied_reference->size() != elements) {
      return std::numeric_limits<double>::quiet_NaN();
    }
    return relativeErrorOf(root, *problem.supplied_reference);
  };

  // Native-quantized corrections (refineNativeStaged, the frozen-factor loop
  // of src/metal_solver.cpp:829-915): the stored basis V and V^T and the
  // stored spectrum in the selected formats (nearest, as copyToStorage /
  // copySpectrumToStorage store them), every stage of the correction in the
  // basis format.
  const bool native = configuration.native_correction;
  const int ncodec = codecFor(format);
  DeviceBuffer nv(native ? elements * sizeof(float) : 0), nvt(native ? elements * sizeof(float) : 0),
      ns(native ? n * sizeof(float) : 0), nws(native ? 3 * elements * sizeof(float) : 0),
      best_hi(native ? elements * sizeof(float) : 0), best_lo(native ? elements * sizeof(float) : 0);
  if (native) {
    runtime.check(msq_make_factor(ctx, v.as<float>(), ones.as<float>(), &nn, &off, 1, nvt.as<float>()),
                  "transpose basis");
    const size_t nrow = ncodec == MSQ_FMT_FP8_E4M3FN_ROWSCALE ? n : 0;
    auto store = [&](const float *src, float *dst) {
      if (ncodec == MSQ_FMT_FP32) {
        // the context's stream is idle here (synchronised above)
        if (src != dst &&
            cudaMemcpy(dst, src, elements * sizeof(float), cudaMemcpyDeviceToDevice) != cudaSuccess)
          failCuda("copyToStorage failed");
        return;
      }
      runtime.check(msq_encode(ctx, ncodec, src, elements, nrow, codes.as<uint8_t>(), scales.as<uint8_t>()),
                    "copyToStorage");
      runtime.check(msq_decode(ctx, ncodec, codes.as<uint8_t>(), scales.as<uint8_t>(), elements, nrow, dst),
                    "unpackFromStorage");
    };
    runtime.check(msq_synchronize(ctx), "transpose basis");
    store(v.as<float>(), nv.as<float>());
    store(nvt.as<float>(), nvt.as<float>());
    std::vector<float> roots(n);
    if (quantized_spectrum) {
      copyOut(roots.data(), lam0.as<float>(), n * sizeof(float));
      for (float &x : roots) x = std::sqrt(x);  // lambda0 = s_q^2 holds the stored roots squared
    } else {
      for (size_t i = 0; i < n; ++i) roots[i] = std::sqrt(eig[i]);
    }
    copyIn(ns.as<float>(), roots.data(), n * sizeof(float));
    runtime.check(msq_synchronize(ctx), "native correction operands");
  }

  double res = residual();
  result.history.push_back({0, res, forward_error(root_now())});
  double best = res;
  bool best_saved = false;
  size_t iteration = 0, flat_steps = 0;
  std::string stages;
  uint64_t correction_launches = 0;
  while (res > problem.tolerance && iteration < problem.max_iterations && std::isfinite(res)) {
    const auto t0 = Clock::now();
    const uint64_t launches_before = msq_launch_count(ctx);
    if (native) {
      runtime.check(msq_native_sylvester_sweep(ctx, ncodec, nv.as<float>(), nvt.as<float>(),
                                               ns.as<float>(), r.as<float>(), &nn, &off, 1,
                                               x_hi.as<float>(), x_lo.as<float>(), nws.as<float>(),
                                               codes.as<uint8_t>(), scales.as<uint8_t>()),
                    "refineNativeStaged");
    } else {
      runtime.check(msq_sylvester_sweep(ctx, MSQ_FMT_FP32, v.as<float>(), lam.as<float>(),
                                        r.as<float>(), &nn, &off, 1, x_hi.as<float>(),
                                        x_lo.as<float>(), ws.as<float>()),
                    "refineUpdateAndMeasure");
    }
    correction_launches += msq_launch_count(ctx) - launches_before;
    stages += (stages.empty() ? "" : ";") +
              std::string(native ? "native_quantized" : "fp32_frozen");
    const double previous_best = best;
    res = residual();
    result.times.correction_gpu_seconds += since(t0);
    ++iteration;
    result.history.push_back({iteration, res, forward_error(root_now())});
    if (!std::isfinite(res)) break;
    if (native && res < best) {
      best = res;
      // keep the best root (the stagnation policy returns it)
      if (cudaMemcpy(best_hi.as<float>(), x_hi.as<float>(), elements * sizeof(float),
                     cudaMemcpyDeviceToDevice) != cudaSuccess ||
          cudaMemcpy(best_lo.as<float>(), x_lo.as<float>(), elements * sizeof(float),
                     cudaMemcpyDeviceToDevice) != cudaSuccess)
        failCuda("best root copy failed");
      best_saved = true;
    }
    if (native && configuration.stop_on_stagnation && res > problem.tolerance) {
      const double improvement = previous_best > 0.0 ? (previous_best - res) / previous_best : 0.0;
      flat_steps = improvement > configuration.min_relative_improvement ? 0 : flat_steps + 1;
      result.stagnation_steps = flat_steps;
      if (flat_steps >= configuration.stagnation_window) break;
    }
  }
  if (native && configuration.stop_on_stagnation && best_saved &&
      best < result.history.back().residual) {
    // the stagnation policy reports the best root (src/metal_solver.cpp:905-915)
    if (cudaMemcpy(x_hi.as<float>(), best_hi.as<float>(), elements * sizeof(float),
                   cudaMemcpyDeviceToDevice) != cudaSuccess ||
        cudaMemcpy(x_lo.as<float>(), best_lo.as<float>(), elements * sizeof(float),
                   cudaMemcpyDeviceToDevice) != cudaSuccess)
      failCuda("best root copy failed");
    res = best;
    result.history.push_back({iteration, best, forward_error(root_now())});
  }
  result.times.mixed_total_seconds = since(mixed_start);
  if (!stages.empty()) result.correction_stage_history = stages;
  if (iteration > 0) result.kernel_dispatches_per_correction = correction_launches / iteration;
  result.low_factor_corrections = native && ncodec != MSQ_FMT_FP32 ? iteration : 0;
  const std::vector<double> root = root_now();
  if (problem.supplied_reference != nullptr && problem.supplied_reference->size() == elements &&
      n <= 1024) {
    // the FP64 residual of the supplied reference root (runMetalCase reports it)
    const std::vector<double> &ref = *problem.supplied_reference;
    double num = 0.0, den = 0.0;
    std::vector<double> column(n);
    for (size_t c = 0; c < n; ++c) {
      std::fill(column.begin(), column.end(), 0.0);
      for (size_t k = 0; k < n; ++k) {
        const double b = ref[k + c * n];
        for (size_t r2 = 0; r2 < n; ++r2) column[r2] += ref[r2 + k * n] * b;
      }
      for (size_t r2 = 0; r2 < n; ++r2) {
        const double a = prepared.values[r2 + c * n];
        num += (a - column[r2]) * (a - column[r2]);
        den += a * a;
      }
    }
    result.reference_residual = den > 0.0 ? std::sqrt(num / den) : 0.0;
  }

  result.best_residual = result.history.front().residual;
  result.best_forward_error = result.history.front().forward_error;
  result.best_iteration = 0;
  for (const auto &h : result.history) {
    if (std::isfinite(h.residual) && h.residual < result.best_residual) {
      result.best_residual = h.residual;
      result.best_forward_error = h.forward_error;
      result.best_iteration = h.iteration;
    }
  }
  result.final_residual = result.history.back().residual;
  result.final_forward_error = result.history.back().forward_error;
  result.converged = std::isfinite(res) && res <= problem.tolerance;
  result.finite = std::isfinite(res) &&
                  std::all_of(root.begin(), root.end(), [](double x) { return std::isfinite(x); });
  // termination reasons of the reference (src/metal_solver.cpp:550-564)
  if (!result.finite) {
    result.termination_reason = "nonfinite";
  } else if (result.converged) {
    result.termination_reason = "converged";
  } else if (result.history.back().residual > result.history.front().residual) {
    result.termination_reason = "diverged";
  } else {
    result.termination_reason = "budget_exhausted";
  }
  result.status = result.termination_reason;
  result.symmetry_error = symmetryErrorOf(root, n);
  if (problem.enforce_policy) {
    // Contract enforcement (src/metal_solver.cpp:583-602).
    if (!result.finite) failCuda("The GPU-resident solver produced a nonfinite result.");
    if (!result.converged) {
      std::ostringstream message;
      message << std::setprecision(17)
              << "The GPU-resident solver did not reach the residual tolerance. Residual: "
              << result.final_residual;
      failCuda(message.str());
    }
    if (result.symmetry_error > 1.0e-12) failCuda("The GPU-resident result lost symmetric structure.");
  }
  return result;
}

int runCuda(const CudaRunOptions &options, const PreparedMatrix &matrix) {
  CudaRuntime runtime(options.device);
  CudaSolverConfiguration configuration;
  configuration.basis_format = options.basis_format;
  configuration.spectrum_format = options.spectrum_format;
  configuration.rounding_mode = options.rounding_mode;
  configuration.rounding_seed = options.rounding_seed;
  configuration.native_correction = options.native_correction;
  configuration.stop_on_stagnation = options.stop_on_stagnation;
  configuration.stagnation_window = options.stagnation_window;
  configuration.min_relative_improvement = options.min_relative_improvement;
  CudaProblem problem;
  problem.order = matrix.order;
  problem.condition = matrix.condition;
  problem.max_iterations = options.max_iterations;
  problem.tolerance = options.tolerance;
  problem.enforce_policy = false;
  problem.prepared_matrix = &matrix;
  const CaseResult result = runCudaCase(runtime, configuration, problem);
  // key=value report in the style of printResult (src/reporting.cpp:22-122)
  std::cout << std::setprecision(6) << "case=" << result.name
            << " solver_backend=" << result.solver_backend << " n=" << result.order
            << " basis=" << result.selected_basis_stage
            << " spectrum=" << result.selected_spectrum_stage
            << " status=" << result.status << " iterations=" << (result.history.size() - 1)
            << std::scientific << " final_residual=" << result.final_residual
            << " basis_orthogonality=" << result.frozen_basis_orthogonality
            << " quantized_basis_orthogonality=" << result.quantized_basis_orthogonality
            << " symmetry_error=" << result.symmetry_error
            << " mixed_seconds=" << result.times.mixed_total_seconds << '\n';
  return options.enforce_policy && !result.converged ? 1 : 0;
}

}  // namespace mixed_sqrt

namespace mixed_sqrt {
namespace {

// One row of a schema: (column, formatted value) in column order.
using Row = std::vector<std::pair<const char *, std::string>>;

template <typename T>
std::string text(const T &value) {
  std::ostringstream out;
  out << std::setprecision(17) << value;
  return out.str();
}

double basisStorageRatio(const CaseResult &r) {
  return r.fp32_basis_bytes > 0 ? static_cast<double>(r.low_factor_basis_bytes) /
                                      static_cast<double>(r.fp32_basis_bytes)
                                : 0.0;
}

double otherSeconds(const CaseResult &r) {
  const double accounted = r.times.low_eigen_seconds + r.times.initial_gpu_seconds +
                           r.times.residual_fp64_seconds + r.times.correction_gpu_seconds;
  return std::max(0.0, r.times.mixed_total_seconds - accounted);
}

// The columns both files begin with (through kernel_path).
void leadingColumns(const CaseResult &r, Row &row) {
  row.insert(row.end(), {
      {"paper_test_set", r.paper_test_set}, {"matrix_family", r.matrix_family},
      {"matrix_type", r.matrix_type}, {"solver_backend", r.solver_backend},
      {"rng_seed", text(r.rng_seed)}, {"rounding_mode", r.rounding_mode},
      {"rounding_seed", text(r.rounding_seed)}, {"diagonal_shift", text(r.diagonal_shift)},
      {"shift_rule", r.shift_rule}, {"case", r.name}, {"precision", r.precision},
      {"basis_precision", r.basis_precision}, {"spectrum_precision", r.spectrum_precision},
      {"correction_mode", r.correction_mode}, {"precision_policy", r.precision_policy},
      {"stopping_policy", r.stopping_policy}, {"dispatch_policy", r.dispatch_policy},
      {"termination_reason", r.termination_reason}, {"selection_policy", r.selection_policy},
      {"precision_attempts", text(r.precision_attempts)}, {"execution_model", r.execution_model},
      {"kernel_path", r.kernel_path}});
}

// Basis stages through basis_reorthogonalization_seconds.
void stageColumns(const CaseResult &r, Row &row) {
  row.insert(row.end(), {
      {"selected_basis_stage", r.selected_basis_stage},
      {"selected_spectrum_stage", r.selected_spectrum_stage},
      {"correction_stage_history", r.correction_stage_history},
      {"precision_escalations", text(r.precision_escalations)},
      {"low_factor_corrections", text(r.low_factor_corrections)},
      {"low_factor_basis_bytes", text(r.low_factor_basis_bytes)},
      {"fp32_basis_bytes", text(r.fp32_basis_bytes)},
      {"basis_storage_ratio", text(basisStorageRatio(r))},
      {"quantized_basis_orthogonality", text(r.quantized_basis_orthogonality)},
      {"factor_quantization_seconds", text(r.factor_quantization_seconds)},
      {"basis_reorthogonalization_seconds", text(r.basis_reorthogonalization_seconds)}});
}

void referenceTimingColumns(const CaseResult &r, Row &row) {
  row.insert(row.end(), {
      {"reference_timing_min_seconds", text(r.reference_timing.minimum_seconds)},
      {"reference_timing_max_seconds", text(r.reference_timing.maximum_seconds)},
      {"reference_timing_median_seconds", text(r.reference_timing.median_seconds)},
      {"reference_timing_mean_seconds", text(r.reference_timing.mean_seconds)},
      {"reference_timing_variance_seconds2", text(r.reference_timing.variance_seconds2)}});
}

void pairedRatioColumns(const CaseResult &r, Row &row) {
  row.insert(row.end(), {
      {"paired_ratio_mean", text(r.paired_ratio_summary.mean)},
      {"paired_ratio_variance", text(r.paired_ratio_summary.variance)},
      {"paired_ratio_min", text(r.paired_ratio_summary.minimum)},
      {"paired_ratio_max", text(r.paired_ratio_summary.maximum)},
      {"paired_ratio_median", text(r.paired_ratio_summary.median)}});
}

// The phase columns factorization_seconds .. mixed_total_seconds.
void phaseColumns(const CaseResult &r, Row &row) {
  const PhaseTimes &t = r.times;
  row.insert(row.end(), {
      {"factorization_seconds", text(t.low_eigen_seconds)},
      {"initial_root_seconds", text(t.initial_gpu_seconds)},
      {"single_seconds", text(t.low_eigen_seconds + t.initial_gpu_seconds)},
      {"residual_seconds", text(t.residual_fp64_seconds)},
      {"correction_system_seconds", text(t.correction_gpu_seconds)},
      {"updates_and_others_seconds", text(otherSeconds(r))},
      {"mixed_total_seconds", text(t.mixed_total_seconds)}});
}

Row summaryRow(const CaseResult &r) {
  static const IterationMeasurement kEmpty{0, std::numeric_limits<double>::quiet_NaN(),
                                           std::numeric_limits<double>::quiet_NaN()};
  const IterationMeasurement &first = r.history.empty() ? kEmpty : r.history.front();
  const IterationMeasurement &last = r.history.empty() ? kEmpty : r.history.back();
  const double total = r.times.mixed_total_seconds;
  auto fraction = [total](double seconds) { return text(total > 0.0 ? seconds / total : 0.0); };
  Row row;
  leadingColumns(r, row);
  row.insert(row.end(), {
      {"command_buffers_per_correction", text(r.command_buffers_per_correction)},
      {"kernel_dispatches_per_correction", text(r.kernel_dispatches_per_correction)}});
  stageColumns(r, row);
  row.insert(row.end(), {
      {"warmups", text(r.timing.warmups)}, {"evaluations", text(r.timing.evaluations)},
      {"timing_evaluations", text(r.timing.evaluations)},
      {"timing_min_seconds", text(r.timing.minimum_seconds)},
      {"timing_max_seconds", text(r.timing.maximum_seconds)},
      {"timing_median_seconds", text(r.timing.median_seconds)},
      {"timing_mean_seconds", text(r.timing.mean_seconds)},
      {"timing_variance_seconds2", text(r.timing.variance_seconds2)}});
  referenceTimingColumns(r, row);
  row.insert(row.end(), {
      {"order", text(r.order)}, {"condition", text(r.condition)},
      {"iterations", text(last.iteration)}, {"best_iteration", text(r.best_iteration)},
      {"best_residual", text(r.best_residual)}, {"best_forward_error", text(r.best_forward_error)},
      {"stagnation_steps", text(r.stagnation_steps)}, {"converged", text(r.converged)},
      {"finite", text(r.finite)}, {"status", r.status},
      {"initial_residual", text(first.residual)}, {"final_residual", text(r.final_residual)},
      {"initial_forward_error", text(first.forward_error)},
      {"final_forward_error", text(r.final_forward_error)},
      {"symmetry_error", text(r.symmetry_error)}, {"reference_residual", text(r.reference_residual)},
      {"frozen_factor_error", text(r.frozen_factor_error)},
      {"frozen_factor_relative_error", text(r.frozen_factor_relative_error)},
      {"frozen_basis_orthogonality", text(r.frozen_basis_orthogonality)},
      {"frozen_sylvester_inverse_norm", text(r.frozen_sylvester_inverse_norm)},
      {"frozen_contraction_bound", text(r.frozen_contraction_bound)},
      {"certificate_usable", text(r.certificate_usable)},
      {"reference_seconds", text(r.times.reference_seconds)},
      {"low_eigen_seconds", text(r.times.low_eigen_seconds)},
      {"initial_gpu_seconds", text(r.times.initial_gpu_seconds)},
      {"residual_fp64_seconds", text(r.times.residual_fp64_seconds)},
      {"correction_gpu_seconds", text(r.times.correction_gpu_seconds)},
      {"update_fp64_seconds", text(r.times.update_fp64_seconds)}});
  phaseColumns(r, row);
  row.insert(row.end(), {
      {"low_eigen_fraction", fraction(r.times.low_eigen_seconds)},
      {"initial_gpu_fraction", fraction(r.times.initial_gpu_seconds)},
      {"residual_fraction", fraction(r.times.residual_fp64_seconds)},
      {"correction_gpu_fraction", fraction(r.times.correction_gpu_seconds)},
      {"update_fraction", fraction(r.times.update_fp64_seconds)}});
  pairedRatioColumns(r, row);
  row.push_back({"mixed_to_reference",
                 text(r.reference_timing.mean_seconds > 0.0
                          ? r.timing.mean_seconds / r.reference_timing.mean_seconds
                          : 0.0)});
  return row;
}

Row iterationRow(const CaseResult &r, const IterationMeasurement &record) {
  Row row;
  leadingColumns(r, row);
  stageColumns(r, row);
  row.insert(row.end(), {
      {"order", text(r.order)}, {"condition", text(r.condition)},
      {"warmups", text(r.timing.warmups)}, {"evaluations", text(r.timing.evaluations)},
      {"timing_evaluations", text(r.timing.evaluations)}});
  referenceTimingColumns(r, row);
  pairedRatioColumns(r, row);
  phaseColumns(r, row);
  row.insert(row.end(), {{"iteration", text(record.iteration)},
                         {"residual", text(record.residual)},
                         {"forward_error", text(record.forward_error)}});
  return row;
}

void writeNames(std::ostream &out, const Row &row) {
  for (size_t i = 0; i < row.size(); ++i) out << (i ? "," : "") << row[i].first;
  out << '\n';
}

void writeValues(std::ostream &out, const Row &row) {
  for (size_t i = 0; i < row.size(); ++i) out << (i ? "," : "") << row[i].second;
  out << '\n';
}

}  // namespace

void writeCudaSummaryHeader(std::ostream &output) { writeNames(output, summaryRow(CaseResult{})); }

void writeCudaIterationsHeader(std::ostream &output) {
  writeNames(output, iterationRow(CaseResult{}, IterationMeasurement{0, 0.0, 0.0}));
}

void writeCudaCaseCsv(const CaseResult &result, std::ostream &summary, std::ostream &iterations) {
  writeValues(summary, summaryRow(result));
  for (const IterationMeasurement &record : result.history) {
    writeValues(iterations, iterationRow(result, record));
  }
}

}  // namespace mixed_sqrt

extern "C" int msq_csv_headers(char *summary, size_t summary_capacity, char *iterations,
                               size_t iterations_capacity) {
  std::ostringstream s, i;
  mixed_sqrt::writeCudaSummaryHeader(s);
  mixed_sqrt::writeCudaIterationsHeader(i);
  const std::string a = s.str(), b = i.str();
  if (summary == nullptr || iterations == nullptr || a.size() + 1 > summary_capacity ||
      b.size() + 1 > iterations_capacity) {
    return MSQ_ERR_INVALID_ARGUMENT;
  }
  std::copy(a.begin(), a.end(), summary);
  summary[a.size()] = '\0';
  std::copy(b.begin(), b.end(), iterations);
  iterations[b.size()] = '\0';
  return MSQ_OK;
}
