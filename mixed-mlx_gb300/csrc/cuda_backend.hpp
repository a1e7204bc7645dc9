// cuda_backend — the C++ host side of the CUDA solver, mirroring the
// reference's backend contract so it drops in beside metal_backend and
// accelerate_backend:
//
//   reference                                     here
//   MetalRuntime (src/metal_runtime.hpp:69-76)    CudaRuntime (RAII msq_ctx)
//   MetalSolverConfiguration / MetalProblem       CudaSolverConfiguration /
//     (src/metal_solver.hpp:12-25)                  CudaProblem
//   runMetalCase (src/metal_solver.cpp:338-604)   runCudaCase
//   MetalRunOptions / runMetal                    CudaRunOptions / runCuda
//     (src/metal_backend.hpp:13-36)
//
// Errors follow the reference: fail() -> std::runtime_error for invalid
// input or a failing CUDA call; numerical outcomes (not converged, rejected
// low-precision basis, diverged) are reported in CaseResult.status and
// termination_reason.  Built inside the reference tree (define
// MSQ_WITH_REFERENCE_CONTRACT and put src/ on the include path) the
// reference's own experiment.hpp types are used; standalone, the subset of
// PreparedMatrix / CaseResult fields this backend fills is declared here
// with the same names and meanings.
#pragma once

#include <cstddef>
#include <cstdint>
#include <limits>
#include <ostream>
#include <string>
#include <vector>

#include "../../include/msq_cuda.h"

#ifdef MSQ_WITH_REFERENCE_CONTRACT
#include "experiment.hpp"
#else
namespace mixed_sqrt {

struct PreparedMatrix {
  std::vector<double> values;  // column-major, order x order
  size_t order = 0;
  double condition = 0.0;
  std::string paper_test_set = "controlled";
  std::string matrix_family = "conditioned_spd";
  std::string matrix_type = "symmetric";
  uint64_t rng_seed = 0;
};

struct IterationMeasurement {
  size_t iteration;
  double residual;
  double forward_error;
};

struct PhaseTimes {
  double reference_seconds = 0.0;
  double low_eigen_seconds = 0.0;
  double initial_gpu_seconds = 0.0;
  double residual_fp64_seconds = 0.0;
  double correction_gpu_seconds = 0.0;
  double update_fp64_seconds = 0.0;
  double mixed_total_seconds = 0.0;
};

struct TimingSummary {
  size_t warmups = 0;
  size_t evaluations = 1;
  double minimum_seconds = 0.0;
  double maximum_seconds = 0.0;
  double median_seconds = 0.0;
  double mean_seconds = 0.0;
  double variance_seconds2 = 0.0;
};

struct PairedRatioSummary {
  double mean = 0.0;
  double variance = 0.0;
  double minimum = 0.0;
  double maximum = 0.0;
  double median = 0.0;
};

// The fields of the reference's CaseResult (src/experiment.hpp:64-125), with
// its names and defaults, so that results report in its schema.
struct CaseResult {
  std::string name;
  std::string paper_test_set = "controlled";
  std::string matrix_family = "conditioned_spd";
  std::string matrix_type = "symmetric";
  std::string solver_backend = "cuda";
  uint64_t rng_seed = 0;
  double diagonal_shift = 0.0;
  std::string shift_rule = "not_applicable";
  std::string precision;
  std::string basis_precision;
  std::string correction_mode;
  std::string spectrum_precision;
  std::string precision_policy;
  std::string rounding_mode = "nearest";
  uint32_t rounding_seed = 0;
  std::string execution_model;
  std::string kernel_path;
  std::string status;
  std::string stopping_policy = "fixed_budget";
  std::string dispatch_policy = "not_applicable";
  std::string termination_reason;
  std::string selection_policy = "fixed";
  std::string selected_basis_stage = "not_applicable";
  std::string selected_spectrum_stage = "not_applicable";
  std::string correction_stage_history = "not_applicable";
  size_t precision_attempts = 1;
  size_t order = 0;
  size_t low_factor_basis_bytes = 0;
  size_t fp32_basis_bytes = 0;
  size_t best_iteration = 0;
  size_t stagnation_steps = 0;
  size_t command_buffers_per_correction = 0;
  size_t kernel_dispatches_per_correction = 0;
  size_t precision_escalations = 0;
  size_t low_factor_corrections = 0;
  TimingSummary timing;
  TimingSummary reference_timing;
  std::vector<double> paired_ratios;
  PairedRatioSummary paired_ratio_summary;
  double condition = 0.0;
  bool converged = false;
  bool finite = false;
  double symmetry_error = 0.0;
  double reference_residual = 0.0;
  double frozen_factor_relative_error = 0.0;
  double frozen_factor_error = 0.0;
  double frozen_basis_orthogonality = 0.0;
  double quantized_basis_orthogonality = std::numeric_limits<double>::quiet_NaN();
  double factor_quantization_seconds = 0.0;
  double basis_reorthogonalization_seconds = 0.0;
  double frozen_sylvester_inverse_norm = 0.0;
  double frozen_contraction_bound = 0.0;
  bool certificate_usable = false;
  double best_residual = std::numeric_limits<double>::quiet_NaN();
  double best_forward_error = std::numeric_limits<double>::quiet_NaN();
  double final_residual = std::numeric_limits<double>::quiet_NaN();
  double final_forward_error = std::numeric_limits<double>::quiet_NaN();
  std::vector<IterationMeasurement> history;
  PhaseTimes times;
};

}  // namespace mixed_sqrt
#endif

namespace mixed_sqrt {

// Basis storage of the frozen factor (the reference's Precision subset this
// backend implements; FP8 is the per-row-scaled E4M3 format).
// The reference's basis precisions (kPrecisionSpecs, src/precision.hpp:64-90)
// plus the per-row-scaled FP8 format, which has no reference counterpart.
enum class CudaBasisFormat {
  Fp32, Bf16, Fp8E4M3FnRowScale, Mxfp4E2M1,
  Fp8E4M3Fn, Fp8E5M2, Mxfp8E4M3Fn, Mxfp8E5M2, Fp4E2M1
};

const char *cudaBasisFormatName(CudaBasisFormat format);
CudaBasisFormat cudaBasisFormatForCliName(const std::string &name);
// basisOrthogonalityTolerance (src/configuration.cpp:109-118) per format.
double cudaBasisOrthogonalityTolerance(CudaBasisFormat format);

// Storage of the root eigenvalues used by the initial root: FP32, or the
// log-affine formats of the reference's fp8_e4m3fn_log_s / fp4_e2m1_log_s
// spectrum precisions (src/precision.hpp:87-92).
enum class CudaSpectrumFormat { Fp32, Fp8E4M3FnLogS, Fp4E2M1LogS };

const char *cudaSpectrumFormatName(CudaSpectrumFormat format);
CudaSpectrumFormat cudaSpectrumFormatForCliName(const std::string &name);

// --rounding nearest|stochastic (RoundingMode, src/precision.hpp:22): how the
// basis and the spectrum are quantized.
enum class CudaRoundingMode { Nearest, Stochastic };

const char *cudaRoundingModeName(CudaRoundingMode mode);
CudaRoundingMode cudaRoundingModeForCliName(const std::string &name);

class CudaRuntime {
 public:
  explicit CudaRuntime(int device = 0);
  ~CudaRuntime();
  CudaRuntime(const CudaRuntime &) = delete;
  CudaRuntime &operator=(const CudaRuntime &) = delete;
  msq_ctx *context() const { return ctx_; }
  // Throws (fail) with msq_last_error() when status != MSQ_OK.
  void check(int status, const char *what) const;

 private:
  msq_ctx *ctx_ = nullptr;
};

struct CudaSolverConfiguration {
  CudaBasisFormat basis_format = CudaBasisFormat::Fp32;
  CudaSpectrumFormat spectrum_format = CudaSpectrumFormat::Fp32;
  CudaRoundingMode rounding_mode = CudaRoundingMode::Nearest;
  uint32_t rounding_seed = 0;        // --rounding-seed (stochastic rounding)
  // --correction native_quantized (CorrectionMode): corrections with every
  // operand and intermediate stored in the basis format (refineNativeStaged),
  // and its stopping policy: a fixed budget, or --native-stopping stagnation
  // (stop after `stagnation_window` corrections in a row that improve the best
  // residual by no more than `min_relative_improvement`, keep the best root).
  bool native_correction = false;
  bool stop_on_stagnation = false;
  size_t stagnation_window = 4;              // the reference's defaults
  double min_relative_improvement = 1.0e-3;
  double jacobi_tolerance = 1.0e-7;  // off(A) <= tol * ||A||_F
  int jacobi_max_sweeps = 15;
  bool orthogonality_gate = true;    // reject a basis that fails the tolerance
};

struct CudaProblem {
  size_t order = 0;
  double condition = 0.0;
  size_t max_iterations = 8;
  double tolerance = 1.0e-12;
  bool enforce_policy = false;
  const PreparedMatrix *prepared_matrix = nullptr;
  const std::vector<double> *supplied_reference = nullptr;  // FP64 root
};

// The GPU-resident solve of one matrix: Jacobi eigensolver, quantized
// frozen factor with the orthogonality gate (escalation to FP32 on failure),
// tensor-core reconstruction, float-float residual, frozen-basis Sylvester
// corrections while residual > tolerance and iterations < max_iterations.
CaseResult runCudaCase(CudaRuntime &runtime, const CudaSolverConfiguration &configuration,
                       const CudaProblem &problem);

struct CudaRunOptions {
  CudaBasisFormat basis_format = CudaBasisFormat::Fp32;
  CudaSpectrumFormat spectrum_format = CudaSpectrumFormat::Fp32;
  CudaRoundingMode rounding_mode = CudaRoundingMode::Nearest;
  uint32_t rounding_seed = 0;
  bool native_correction = false;
  bool stop_on_stagnation = false;
  size_t stagnation_window = 4;
  double min_relative_improvement = 1.0e-3;
  size_t max_iterations = 8;
  double tolerance = 1.0e-12;
  bool enforce_policy = true;
  int device = 0;
};

// ---- stage-3 precision plans (3_spectral/spectral.cpp:769-1385) ----------
// The factor formats of FactorFormat (3_spectral/spectral.hpp); names as
// format_name (:321-339).
enum class CudaFactorFormat { Fp32, Fp16, Bf16, Fp8E4M3, Fp8E5M2, MxFp8E4M3, MxFp4E2M1 };
const char *cudaFactorFormatName(CudaFactorFormat format);

struct CudaPrecisionPlan {
  std::string name;
  CudaFactorFormat basis;
  CudaFactorFormat spectrum;
};
// precision_plans() (:769-786): the same 16 plans in the same order.
std::vector<CudaPrecisionPlan> cudaPrecisionPlans();

struct CudaSpectralIteration {
  size_t iteration;
  double residual;
  double forward_error;
  bool low_product;  // the correction ran on low-bit operands
};

// SpectralResult's fields that have a CUDA meaning.
struct CudaSpectralResult {
  std::string plan, basis_format, spectrum_format, product_backend, arithmetic_format;
  std::string reason;  // converged, correction_limit, divergent, nonfinite_residual,
                       // ill_conditioned_basis, invalid_spectrum
  size_t order = 0;
  double condition = 0.0;
  bool accepted = false;
  bool converged = false;
  size_t iterations = 0;
  size_t correction_count = 0;
  size_t low_product_corrections = 0;
  double basis_bits_per_value = 0.0;
  double spectrum_bits_per_value = 0.0;
  double weighted_factor_storage_bits = 0.0;
  double basis_relative_error = 0.0;
  double spectrum_relative_error = 0.0;
  double basis_condition = 0.0;
  double initial_error = 0.0;
  double final_error = 0.0;
  double final_residual = 0.0;
  std::vector<CudaSpectralIteration> history;
};

// run_spectral's counterpart: the plan's factor formats, the initial root,
// frozen-basis corrections (low-bit products with the stall fallback for a
// low-bit basis below condition 1000) until `tolerance`, `max_corrections`
// or divergence.  problem.condition selects the low-bit products as the
// reference's problem.condition does; problem.supplied_reference (FP64
// root) gives the forward errors.
CudaSpectralResult runCudaSpectral(CudaRuntime &runtime, const CudaProblem &problem,
                                   const CudaPrecisionPlan &plan, size_t max_corrections = 30,
                                   double tolerance = 1.0e-12);

// The reference's CSV schema (writeSummaryHeader / writeCaseCsv /
// writeIterationsHeader, src/reporting.cpp:124-330): the same columns in the
// same order, so analysis written for the reference's summary and
// per-iteration files reads these unchanged.
void writeCudaSummaryHeader(std::ostream &output);
void writeCudaIterationsHeader(std::ostream &output);
void writeCudaCaseCsv(const CaseResult &result, std::ostream &summary, std::ostream &iterations);

// runMetal's counterpart for a prepared matrix: solves, prints the result in
// the reference's key=value style and returns 0, or 1 when enforce_policy
// is set and the case missed its tolerance.
int runCuda(const CudaRunOptions &options, const PreparedMatrix &matrix);

}  // namespace mixed_sqrt
