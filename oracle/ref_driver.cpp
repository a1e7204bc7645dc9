// extern "C" entry points over the reference's own CPU code, compiled
// unmodified from the reference tree (src/storage_codecs.cpp,
// src/configuration.cpp, src/numerics.cpp, src/accelerate_backend.cpp, ...).
//
// TEST INFRASTRUCTURE ONLY. This file is part of the oracle: it is built into
// oracle/_ref/libmsq_ref.so where the reference sources are present and is
// loaded only by tests and by the generator of tests/golden fixtures. The
// product never links or calls it.
#include "accelerate_backend.hpp"
#include "numerics.hpp"
#include "precision.hpp"
#include "reporting.hpp"
#include "storage_codecs.hpp"

#include <Metal/Metal.hpp>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <exception>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

using namespace mixed_sqrt;

namespace {

std::string g_error;

// Codec ids follow HostStorageCodec (src/precision.hpp:24-33).
const PrecisionSpec *specForCodec(int codec) {
  for (const PrecisionSpec &spec : kPrecisionSpecs) {
    if (static_cast<int>(spec.host_storage) == codec &&
        !spec.usesLogSpectrum()) {
      return &spec;
    }
  }
  return nullptr;
}

template <typename F>
int guarded(F &&body) {
  try {
    body();
    return 0;
  } catch (const std::exception &error) {
    g_error = error.what();
    return 1;
  }
}

}  // namespace

extern "C" {

const char *ref_last_error() { return g_error.c_str(); }

int ref_check_codecs() { return guarded([] { checkLowPrecisionCodecs(); }); }

size_t ref_storage_bytes(int codec, size_t elements) {
  const PrecisionSpec *spec = specForCodec(codec);
  return spec == nullptr ? 0 : storageBytes(*spec, elements);
}

size_t ref_scale_bytes(int codec, size_t elements) {
  const PrecisionSpec *spec = specForCodec(codec);
  return spec == nullptr ? 0 : scaleBytes(*spec, elements);
}

// copyToStorage (src/storage_codecs.cpp:315-321).
int ref_encode(int codec, const float *source, size_t elements,
               uint8_t *values, uint8_t *scales) {
  return guarded([&] {
    const PrecisionSpec *spec = specForCodec(codec);
    if (spec == nullptr) throw std::runtime_error("unknown codec");
    std::vector<float> input(source, source + elements);
    MTL::Buffer value_buffer(values, storageBytes(*spec, elements));
    MTL::Buffer scale_buffer(scales, scaleBytes(*spec, elements));
    copyToStorage(*spec, input, &value_buffer,
                  scales == nullptr ? nullptr : &scale_buffer);
  });
}

// storageValueAt (src/storage_codecs.cpp:323-374) for every index.
int ref_decode(int codec, const uint8_t *values, const uint8_t *scales,
               size_t elements, float *output) {
  return guarded([&] {
    const PrecisionSpec *spec = specForCodec(codec);
    if (spec == nullptr) throw std::runtime_error("unknown codec");
    MTL::Buffer value_buffer(const_cast<uint8_t *>(values),
                             storageBytes(*spec, elements));
    MTL::Buffer scale_buffer(const_cast<uint8_t *>(scales),
                             scaleBytes(*spec, elements));
    for (size_t index = 0; index < elements; ++index) {
      output[index] = storageValueAt(
          *spec, &value_buffer, scales == nullptr ? nullptr : &scale_buffer,
          index);
    }
  });
}

// The log-spectrum precision whose scalar codec is `codec` (2 = FP8-E4M3FN,
// 6 = FP4-E2M1: fp8_e4m3fn_log_s / fp4_e2m1_log_s of kPrecisionSpecs).
const PrecisionSpec *logSpecForCodec(int codec) {
  for (const PrecisionSpec &spec : kPrecisionSpecs) {
    if (static_cast<int>(spec.host_storage) == codec && spec.usesLogSpectrum()) {
      return &spec;
    }
  }
  return nullptr;
}

// copySpectrumToStorage (src/storage_codecs.cpp:400-440): codes and two
// floats (min, span) per block of spectral_block_elements.
int ref_spectrum_encode(int codec, const float *source, size_t elements,
                        uint8_t *values, float *metadata) {
  return guarded([&] {
    const PrecisionSpec *spec = logSpecForCodec(codec);
    if (spec == nullptr) throw std::runtime_error("no log-spectrum precision for codec");
    std::vector<float> input(source, source + elements);
    MTL::Buffer value_buffer(values, storageBytes(*spec, elements));
    MTL::Buffer metadata_buffer(metadata, spectrumMetadataBytes(*spec, elements));
    copySpectrumToStorage(*spec, input, &value_buffer, &metadata_buffer);
  });
}

// spectrumValueAt (src/storage_codecs.cpp:442-460) for every index.
int ref_spectrum_decode(int codec, const uint8_t *values, const float *metadata,
                        size_t elements, float *output) {
  return guarded([&] {
    const PrecisionSpec *spec = logSpecForCodec(codec);
    if (spec == nullptr) throw std::runtime_error("no log-spectrum precision for codec");
    MTL::Buffer value_buffer(const_cast<uint8_t *>(values), storageBytes(*spec, elements));
    MTL::Buffer metadata_buffer(const_cast<float *>(metadata),
                                spectrumMetadataBytes(*spec, elements));
    for (size_t index = 0; index < elements; ++index) {
      output[index] = spectrumValueAt(*spec, &value_buffer, &metadata_buffer, index);
    }
  });
}

// writeSummaryHeader / writeIterationsHeader (src/reporting.cpp:124-166,
// 305-327) into the files `summary_path` and `iterations_path`.
int ref_csv_headers(const char *summary_path, const char *iterations_path) {
  return guarded([&] {
    std::ofstream summary(summary_path), iterations(iterations_path);
    writeSummaryHeader(summary);
    writeIterationsHeader(iterations);
  });
}

// preparePaperMatrix (src/accelerate_backend.cpp:690-801) for set
// I..VII = 1..7: values and (diagonal_shift, condition, rng_seed).
int ref_paper_matrix(int set, size_t order, double *output, double *meta) {
  return guarded([&] {
    const PreparedMatrix m = preparePaperMatrix(static_cast<PaperTestSet>(set), order);
    std::copy(m.values.begin(), m.values.end(), output);
    meta[0] = m.diagonal_shift;
    meta[1] = m.condition;
    meta[2] = static_cast<double>(m.rng_seed);
  });
}

// makeSpdMatrix (src/numerics.cpp:175-195).
int ref_make_spd(size_t order, double condition, double *output) {
  return guarded([&] {
    const std::vector<double> matrix = makeSpdMatrix(order, condition);
    std::memcpy(output, matrix.data(), matrix.size() * sizeof(double));
  });
}

// symmetricReferenceRoot (src/accelerate_backend.cpp:594-607).
int ref_reference_root(const double *matrix, size_t order, double *root) {
  return guarded([&] {
    std::vector<double> input(matrix, matrix + order * order);
    const std::vector<double> result = symmetricReferenceRoot(input, order);
    std::memcpy(root, result.data(), result.size() * sizeof(double));
  });
}

// relativeResidual / relativeError (src/numerics.cpp:213-240).
double ref_relative_residual(const double *matrix, const double *root,
                             size_t order) {
  std::vector<double> a(matrix, matrix + order * order);
  std::vector<double> x(root, root + order * order);
  return relativeResidual(a, x, order);
}

double ref_relative_error(const double *root, const double *reference,
                          size_t elements) {
  std::vector<double> x(root, root + elements);
  std::vector<double> r(reference, reference + elements);
  return relativeError(x, r);
}

// runAccelerateCase (src/accelerate_backend.cpp:803-1091), symmetric branch.
// summary = {final_residual, final_forward_error, iterations, converged,
//            reference_residual, frozen_factor_relative_error,
//            mixed_total_seconds}
int ref_run_accelerate(const double *matrix, size_t order, double condition,
                       size_t max_corrections, double tolerance,
                       double *summary, double *history, size_t history_cap) {
  return guarded([&] {
    PreparedMatrix prepared;
    prepared.values.assign(matrix, matrix + order * order);
    prepared.order = order;
    prepared.condition = condition;
    const CaseResult result =
        runAccelerateCase(prepared, max_corrections, tolerance);
    summary[0] = result.final_residual;
    summary[1] = result.final_forward_error;
    summary[2] = static_cast<double>(result.history.size() - 1);
    summary[3] = result.converged ? 1.0 : 0.0;
    summary[4] = result.reference_residual;
    summary[5] = result.frozen_factor_relative_error;
    summary[6] = result.times.mixed_total_seconds;
    for (size_t i = 0; i < result.history.size() && i < history_cap; ++i) {
      history[2 * i] = result.history[i].residual;
      history[2 * i + 1] = result.history[i].forward_error;
    }
  });
}

}  // extern "C"
