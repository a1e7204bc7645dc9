// Drives the C++ host mirror (runCudaCase) on one matrix, the way the
// reference's CLI drives runMetalCase.  Input file: int32 n, n*n FP64 A
// (column-major), optionally n*n FP64 reference root.  Prints key=value.
// Usage: cuda_backend_check <matrix.bin> spectral <plan> <tolerance> <max_corrections> [condition]
//        (a stage-3 precision plan through runCudaSpectral), or
//        cuda_backend_check <matrix.bin> <basis: fp32|bf16|fp8_e4m3fn_rowscale|mxfp4_e2m1|...>
//                           <tolerance> <max_iterations>
//                           [spectrum: fp32|fp8_e4m3fn_log_s|fp4_e2m1_log_s]
//                           [rounding: nearest|stochastic] [rounding seed]
//                           [correction: fp32_reorthogonalized|native_quantized]
//                           [native stopping: fixed_budget|stagnation] [csv prefix]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "cuda_backend.hpp"

int main(int argc, char **argv) {
  if (argc < 5) {
    std::cerr << "usage: cuda_backend_check matrix.bin basis tolerance max_iterations\n";
    return 2;
  }
  try {
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) throw std::runtime_error("cannot open input");
    int32_t n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1) throw std::runtime_error("bad input");
    mixed_sqrt::PreparedMatrix m;
    m.order = static_cast<size_t>(n);
    m.values.resize(m.order * m.order);
    if (std::fread(m.values.data(), sizeof(double), m.values.size(), f) != m.values.size())
      throw std::runtime_error("bad input");
    std::vector<double> ref(m.values.size());
    const bool have_ref = std::fread(ref.data(), sizeof(double), ref.size(), f) == ref.size();
    std::fclose(f);
    mixed_sqrt::CudaRuntime runtime(0);
    if (std::string(argv[2]) == "spectral") {
      // cuda_backend_check <matrix.bin> spectral <plan> <tolerance> <max_corrections> <condition>
      mixed_sqrt::CudaProblem problem;
      problem.order = m.order;
      problem.condition = argc > 6 ? std::atof(argv[6]) : 0.0;
      problem.prepared_matrix = &m;
      problem.supplied_reference = have_ref ? &ref : nullptr;
      const std::string name = argv[3];
      for (const auto &plan : mixed_sqrt::cudaPrecisionPlans()) {
        if (plan.name != name) continue;
        const auto r = mixed_sqrt::runCudaSpectral(runtime, problem, plan,
                                                   static_cast<size_t>(std::atoi(argv[5])),
                                                   std::atof(argv[4]));
        std::cout << std::setprecision(17) << "plan=" << r.plan << " accepted=" << r.accepted
                  << " converged=" << r.converged << " reason=" << r.reason
                  << " iterations=" << r.iterations
                  << " low_product_corrections=" << r.low_product_corrections
                  << " product_backend=" << r.product_backend
                  << " basis_error=" << r.basis_relative_error
                  << " spectrum_error=" << r.spectrum_relative_error
                  << " basis_condition=" << r.basis_condition
                  << " basis_bits=" << r.basis_bits_per_value
                  << " spectrum_bits=" << r.spectrum_bits_per_value
                  << " weighted_bits=" << r.weighted_factor_storage_bits
                  << " initial_error=" << r.initial_error << " final_error=" << r.final_error
                  << " final_residual=" << r.final_residual << " residuals=";
        for (size_t k = 0; k < r.history.size(); ++k)
          std::cout << (k ? "," : "") << r.history[k].residual;
        std::cout << "\n";
        return 0;
      }
      throw std::runtime_error("unknown plan " + name);
    }
    mixed_sqrt::CudaSolverConfiguration config;
    config.basis_format = mixed_sqrt::cudaBasisFormatForCliName(argv[2]);
    // optional: spectrum precision, rounding mode, rounding seed
    if (argc > 5) config.spectrum_format = mixed_sqrt::cudaSpectrumFormatForCliName(argv[5]);
    if (argc > 6) config.rounding_mode = mixed_sqrt::cudaRoundingModeForCliName(argv[6]);
    if (argc > 7) config.rounding_seed = static_cast<uint32_t>(std::strtoul(argv[7], nullptr, 0));
    // optional: correction mode (fp32_reorthogonalized | native_quantized) and
    // native stopping policy (fixed_budget | stagnation)
    if (argc > 8) config.native_correction = std::string(argv[8]) == "native_quantized";
    if (argc > 9) config.stop_on_stagnation = std::string(argv[9]) == "stagnation";
    // optional: write the reference's CSV schema to <prefix>_summary.csv and
    // <prefix>_iterations.csv
    const std::string csv_prefix = argc > 10 ? argv[10] : "";
    mixed_sqrt::CudaProblem problem;
    problem.order = m.order;
    problem.tolerance = std::atof(argv[3]);
    problem.max_iterations = static_cast<size_t>(std::atoi(argv[4]));
    problem.prepared_matrix = &m;
    problem.supplied_reference = have_ref ? &ref : nullptr;
    const mixed_sqrt::CaseResult r = mixed_sqrt::runCudaCase(runtime, config, problem);
    if (!csv_prefix.empty()) {
      std::ofstream summary(csv_prefix + "_summary.csv"), iterations(csv_prefix + "_iterations.csv");
      mixed_sqrt::writeCudaSummaryHeader(summary);
      mixed_sqrt::writeCudaIterationsHeader(iterations);
      mixed_sqrt::writeCudaCaseCsv(r, summary, iterations);
    }
    std::cout << std::setprecision(17) << "status=" << r.status
              << " iterations=" << (r.history.size() - 1)
              << " final_residual=" << r.final_residual
              << " final_forward_error=" << r.final_forward_error
              << " initial_residual=" << r.history.front().residual
              << " selected_basis_stage=" << r.selected_basis_stage
              << " selected_spectrum_stage=" << r.selected_spectrum_stage
              << " correction_mode=" << r.correction_mode
              << " stagnation_steps=" << r.stagnation_steps
              << " best_residual=" << r.best_residual
              << " precision_escalations=" << r.precision_escalations
              << " basis_orthogonality=" << r.frozen_basis_orthogonality
              << " quantized_basis_orthogonality=" << r.quantized_basis_orthogonality
              << " symmetry_error=" << r.symmetry_error << "\n";
    return 0;
  } catch (const std::exception &error) {
    // the reference's main(): report and exit nonzero (src/main.cpp:12-16)
    std::cerr << "error: " << error.what() << "\n";
    return 1;
  }
}
