// Pipeline stages behind the C ABI and the batched solve.
//
// msq_solve_batched is the batched form of solveGpuResidentSpd
// (src/metal_solver.cpp:92-336): Jacobi -> factor W = V diag(lambda^(1/4))
// -> (quantize W) -> reconstruction X0 = W W^T -> float-float residual ->
// frozen-basis Sylvester sweeps (refineUpdateAndMeasure,
// src/metal_runtime.cpp:847-966) -> final float-float residual.  Matrices
// are grouped by plan; a matrix whose final residual misses the tolerance is
// re-solved by the plain FP32 plan (the reference escalates a rejected
// low-precision factor to FP32 the same way, src/metal_solver.cpp:225-235).
// Corrections always use the FP32 stable basis, as the reference does
// (:304-310).
#include "msq_dense.cuh"
#include "msq_internal.cuh"
#include "msq_stages.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

namespace msq {
namespace {

size_t alignUp(size_t bytes) { return (bytes + 255) & ~static_cast<size_t>(255); }

// One Sylvester sweep on a batch, FP32 GEMMs on the CUDA cores:
//   G = R V, C = (V^T G) o H, Z = V C, E = Z V^T, X <- X + (E + E^T)/2.
int sylvesterFp32(msq_ctx *ctx, const DeviceBatch *b, const float *v, const float *lam,
                  const float *r, float *x_hi, float *x_lo, float *ws0, float *ws1) {
  MSQ_TRY(gemmTN(ctx, b, r, v, ws0, kEpilogueStore, nullptr));           // G = R V
  MSQ_TRY(gemmTN(ctx, b, v, ws0, ws1, kEpilogueInverseH, lam));          // C = V^T G o H
  MSQ_TRY(gemmTN(ctx, b, v, ws1, ws0, kEpilogueStore, nullptr, true));   // Z = V C
  MSQ_TRY(gemmTN(ctx, b, ws0, v, ws1, kEpilogueStore, nullptr, true, true));  // E = Z V^T
  return symmetricAdd(ctx, b, x_hi, x_lo, ws1);
}

}  // namespace

int sylvesterSweep(msq_ctx *ctx, const DeviceBatch *b, int gemm_format, const float *v,
                   const float *lam, const float *r, float *x_hi, float *x_lo, float *ws0,
                   float *ws1, bool basis_packed) {
  if (gemm_format == MSQ_FMT_BF16) {
    float *e = nullptr;
    MSQ_TRY(sylvesterTc(ctx, b, v, lam, r, ws0, ws1, &e, basis_packed));
    return symmetricAdd(ctx, b, x_hi, x_lo, e);
  }
  return sylvesterFp32(ctx, b, v, lam, r, x_hi, x_lo, ws0, ws1);
}

// X0 = F^T F from the FP32 factor F (K-major W^T) in the plan's format.
int reconstructFromFactor(msq_ctx *ctx, const DeviceBatch *b, int plan_format, const float *f,
                          float *x) {
  switch (plan_format) {
    case MSQ_PLAN_FP32:
      return gemmTN(ctx, b, f, f, x, kEpilogueStore, nullptr);
    case MSQ_PLAN_BF16:
      return reconstructLowBit(ctx, b, MSQ_FMT_BF16, f, x);
    case MSQ_PLAN_FP8:
      return reconstructLowBit(ctx, b, MSQ_FMT_FP8_E4M3FN_ROWSCALE, f, x);
    case MSQ_PLAN_MXFP4:
      return reconstructLowBit(ctx, b, MSQ_FMT_MXFP4_E2M1, f, x);
    default:
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "unknown plan format");
  }
}

}  // namespace msq

using namespace msq;

extern "C" int msq_make_factor(msq_ctx *ctx, const float *vectors, const float *eigenvalues,
                               const int32_t *n, const int64_t *offset, int count,
                               float *factor_t) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!vectors || !eigenvalues || !factor_t)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_make_factor: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return makeFactor(ctx, b, vectors, eigenvalues, factor_t);
}

extern "C" int msq_reconstruct(msq_ctx *ctx, int format, const void *values, const void *scales,
                               const int32_t *n, const int64_t *offset, int count, float *root) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!values || !root) return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_reconstruct: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  if (format == MSQ_FMT_FP32) {
    const float *f = static_cast<const float *>(values);
    return gemmTN(ctx, b, f, f, root, kEpilogueStore, nullptr);
  }
  return reconstructEncoded(ctx, b, format, values, scales, root);
}

extern "C" int msq_reconstruct_factor(msq_ctx *ctx, int plan_format, const float *factor_t,
                                      const int32_t *n, const int64_t *offset, int count,
                                      float *root) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!factor_t || !root)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_reconstruct_factor: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return reconstructFromFactor(ctx, b, plan_format, factor_t, root);
}

extern "C" int msq_gemm(msq_ctx *ctx, int trans_a, int trans_b, const float *a, const float *b,
                        const int32_t *n, const int64_t *offset, int count,
                        const float *eigenvalues, float *c) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!a || !b || !c) return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_gemm: null buffer");
  const DeviceBatch *batch = prepareBatch(ctx, n, offset, count);
  if (batch == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  // gemmTN reads A(i,k) at i + k n when M-major (op(A) = A) and at k + i n
  // otherwise (op(A) = A^T); B(k,j) at k + j n (op(B) = B) or j + k n (B^T)
  return gemmTN(ctx, batch, a, b, c, eigenvalues ? kEpilogueInverseH : kEpilogueStore,
                eigenvalues, trans_a == 0, trans_b != 0);
}

extern "C" int msq_working_add(msq_ctx *ctx, float *x_hi, float *x_lo, const float *e,
                               const int32_t *n, const int64_t *offset, int count) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!x_hi || !x_lo || !e)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_working_add: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return workingAdd(ctx, b, x_hi, x_lo, e);
}

extern "C" int msq_residual_general(msq_ctx *ctx, const float *a, const float *a_lo,
                                    const float *x_hi, const float *x_lo, const int32_t *n,
                                    const int64_t *offset, int count, float *residual,
                                    double *norms) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!a || !x_hi || !norms)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_residual_general: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return residualFFGeneral(ctx, b, a, x_hi, x_lo, residual, norms, a_lo);
}

extern "C" int msq_residual(msq_ctx *ctx, const float *a, const float *a_lo, const float *x_hi,
                            const float *x_lo, const int32_t *n, const int64_t *offset, int count,
                            float *residual, double *norms) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!a || !x_hi || !norms) return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_residual: null buffer");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return residualFF(ctx, b, a, x_hi, x_lo, residual, norms, a_lo);
}

extern "C" int msq_sylvester_sweep(msq_ctx *ctx, int gemm_format, const float *vectors,
                                   const float *eigenvalues, const float *residual,
                                   const int32_t *n, const int64_t *offset, int count,
                                   float *x_hi, float *x_lo, float *workspace) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!vectors || !eigenvalues || !residual || !x_hi || !x_lo || !workspace)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_sylvester_sweep: null buffer");
  if (gemm_format != MSQ_FMT_FP32 && gemm_format != MSQ_FMT_BF16)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_sylvester_sweep: gemm_format must be FP32 or BF16");
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  float *ws0 = workspace;
  float *ws1 = workspace + b->host_offset.back() + static_cast<int64_t>(b->host_n.back()) * b->host_n.back();
  return sylvesterSweep(ctx, b, gemm_format, vectors, eigenvalues, residual, x_hi, x_lo, ws0, ws1);
}

extern "C" int msq_native_sylvester_sweep(msq_ctx *ctx, int format, const float *vectors,
                                          const float *vectors_t, const float *spectrum,
                                          const float *residual, const int32_t *n,
                                          const int64_t *offset, int count, float *x_hi,
                                          float *x_lo, float *workspace, uint8_t *codes,
                                          uint8_t *scales) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (!vectors || !vectors_t || !spectrum || !residual || !x_hi || !x_lo || !workspace)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_native_sylvester_sweep: null buffer");
  if (format < MSQ_FMT_FP32 || format > MSQ_FMT_FP8_E4M3FN_ROWSCALE)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_native_sylvester_sweep: unknown format");
  (void)codes;  // the quantizer round-trips in place; no code buffers needed
  (void)scales;
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  int64_t extent = 0;
  for (int i = 0; i < b->count; ++i)
    extent = std::max(extent, b->host_offset[i] + static_cast<int64_t>(b->host_n[i]) * b->host_n[i]);
  float *rq = workspace, *w1 = workspace + extent, *w2 = workspace + 2 * extent;
  // Every matrix of the batch per launch; Q(x) quantizes each matrix to
  // `format` (nearest, per matrix; row length n for the row-scaled format)
  // and decodes it in place.
  MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(rq, residual, extent * sizeof(float),
                                         cudaMemcpyDeviceToDevice, ctx->stream),
                    "native residual copy"));
  MSQ_TRY(quantizeBatch(ctx, format, b, rq));                     // R in the format
  MSQ_TRY(matmulFmaBatch(ctx, b, vectors_t, rq, w1));              // W1 = V^T R
  MSQ_TRY(quantizeBatch(ctx, format, b, w1));
  MSQ_TRY(matmulFmaBatch(ctx, b, w1, vectors, w2));                // W2 = W1 V
  MSQ_TRY(quantizeBatch(ctx, format, b, w2));
  MSQ_TRY(diagonalSylvesterBatch(ctx, b, w2, spectrum, w1));       // C
  MSQ_TRY(quantizeBatch(ctx, format, b, w1));
  MSQ_TRY(matmulFmaBatch(ctx, b, vectors, w1, w2));                // W1' = V C
  MSQ_TRY(quantizeBatch(ctx, format, b, w2));
  MSQ_TRY(matmulFmaBatch(ctx, b, w2, vectors_t, w1));              // E = W1' V^T
  MSQ_TRY(quantizeBatch(ctx, format, b, w1));
  return symmetricAdd(ctx, b, x_hi, x_lo, w1);                       // X += (E + E^T)/2
}

namespace msq {
namespace {

struct Group {
  msq_plan plan;
  std::vector<int> members;  // indices into the caller's batch
};

bool samePlan(const msq_plan &a, const msq_plan &b) {
  return a.format == b.format && a.sweeps == b.sweeps &&
         a.jacobi_tolerance == b.jacobi_tolerance && a.jacobi_max_sweeps == b.jacobi_max_sweeps;
}

// One Jacobi pass: the plan groups of a call run one batched Jacobi over
// their union, gathered group by group into the solver arena, each matrix to
// its own plan's tolerance (the largest budget of the groups); the
// eigenvector mode may use the tensor cores only when every group quantizes
// its basis.  Each group then runs its reconstruction, residuals and
// corrections on its own part of the arena (a sub-batch at the pass's
// offsets), so a call with several plans does not pay one eigensolver
// launch sequence per plan.
struct Pass {
  double jacobi_tolerance;
  int jacobi_max_sweeps;
  bool low_bit;
  std::vector<int> groups;      // indices into the call's groups
  double *tols_host = nullptr;  // per member (pinned), when the tolerances differ
};

struct PassBuffers {
  const DeviceBatch *b = nullptr;          // the pass (members group by group)
  std::vector<const DeviceBatch *> sub;    // per group: its members at pass offsets
  std::vector<int> first;                  // per group: its first member in the pass
  std::vector<int64_t> eig_base;           // per group: its first eigenvalue
  std::vector<int> members;                // caller indices in pass order
  std::vector<int32_t> n;
  std::vector<int64_t> off;
  int64_t total = 0;
  size_t mat = 0;
  float *A, *J, *V, *F, *Xh, *Xl, *R, *W1, *lam, *Bh, *Bl;
  double *norms;
  int32_t *sweeps;
};

// Stream-ordered copies of a group's outcome into pinned host memory:
// ||R0||^2, ||A||^2 per member after the reconstruction, the same after the
// plan's sweeps, and the Jacobi sweeps per member.
struct GroupReport {
  double *initial;
  double *final;
  int32_t *sweeps;
};

// (rounded up to 16 bytes so the next report's doubles stay aligned)
size_t reportBytes(int count) {
  return ((4 * sizeof(double) + sizeof(int32_t)) * count + 64 + 15) & ~static_cast<size_t>(15);
}

GroupReport reportAt(void *base, int count) {
  auto *d = static_cast<double *>(base);
  return {d, d + 2 * count, reinterpret_cast<int32_t *>(d + 4 * count)};
}

// Members [lo, hi) of the pass in runs whose caller offsets are contiguous
// (the arena offsets are contiguous by construction): one copy per run.
template <class Copy>
int forEachRun(const PassBuffers &pb, const int64_t *off_user, int lo, int hi, Copy copy) {
  for (int i = lo; i < hi;) {
    int j = i + 1;
    while (j < hi && pb.members[j] == pb.members[j - 1] + 1 &&
           off_user[pb.members[j]] ==
               off_user[pb.members[j - 1]] +
                   ((static_cast<int64_t>(pb.n[j - 1]) * pb.n[j - 1] + 3) & ~int64_t(3)))
      ++j;
    const int last = j - 1;
    const int64_t bytes =
        (pb.off[last] - pb.off[i] + static_cast<int64_t>(pb.n[last]) * pb.n[last]) * sizeof(float);
    MSQ_TRY(copy(off_user[pb.members[i]], pb.off[i], bytes));
    i = j;
  }
  return MSQ_OK;
}

// Enqueues one pass on ctx->stream with no host synchronisation: gather, the
// pass's Jacobi, then per group factor, reconstruction, residual, the plan's
// sweeps, final residual and the report copies.  `backup`: room for a copy
// of X (the fallback's undo).  `warm`: the pass continues an earlier Jacobi
// of the same matrices instead of starting from A and the identity: its
// rotated matrices at warm[0, total) and their accumulated rotations at
// warm[total, 2 total), in the pass's own layout.
int enqueuePass(msq_ctx *ctx, const float *a_user, const int32_t *n_user,
                const int64_t *off_user, const std::vector<Group> &groups, const Pass &pass,
                const std::vector<GroupReport> &reports, bool backup, PassBuffers *pb,
                const float *warm = nullptr) {
  int64_t total = 0, order_total = 0;
  for (int k : pass.groups) {
    pb->first.push_back(static_cast<int>(pb->members.size()));
    pb->eig_base.push_back(order_total);
    for (int m : groups[k].members) {
      pb->members.push_back(m);
      pb->n.push_back(n_user[m]);
      pb->off.push_back(total);
      total += (static_cast<int64_t>(n_user[m]) * n_user[m] + 3) & ~int64_t(3);
      order_total += n_user[m];
    }
  }
  const int count = static_cast<int>(pb->members.size());
  pb->total = total;
  const DeviceBatch *b = prepareBatch(ctx, pb->n.data(), pb->off.data(), count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  pb->b = b;
  for (size_t q = 0; q < pass.groups.size(); ++q) {
    const int lo = pb->first[q];
    const int c = static_cast<int>(groups[pass.groups[q]].members.size());
    const DeviceBatch *sb =
        pass.groups.size() == 1 ? b : prepareBatch(ctx, pb->n.data() + lo, pb->off.data() + lo, c);
    if (sb == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
    pb->sub.push_back(sb);
  }
  const size_t mat = alignUp(total * sizeof(float));
  pb->mat = mat;
  const size_t vec = alignUp(order_total * sizeof(float));
  const size_t norms_bytes = alignUp(2 * count * sizeof(double));
  const size_t sweeps_bytes = alignUp(count * sizeof(int32_t));
  const size_t backup_bytes = backup ? 2 * mat : 0;
  const size_t tols_bytes = pass.tols_host ? alignUp(count * sizeof(double)) : 0;
  char *w = static_cast<char *>(scratch(
      ctx, 8 * mat + vec + norms_bytes + sweeps_bytes + backup_bytes + tols_bytes, kScratchSolver));
  if (w == nullptr) return MSQ_ERR_CUDA;
  pb->A = reinterpret_cast<float *>(w);
  pb->J = reinterpret_cast<float *>(w + mat);       // Jacobi working copy
  pb->V = reinterpret_cast<float *>(w + 2 * mat);
  pb->F = reinterpret_cast<float *>(w + 3 * mat);
  pb->Xh = reinterpret_cast<float *>(w + 4 * mat);
  pb->Xl = reinterpret_cast<float *>(w + 5 * mat);
  pb->R = reinterpret_cast<float *>(w + 6 * mat);
  pb->W1 = reinterpret_cast<float *>(w + 7 * mat);  // with F: the 2 sweep buffers
  pb->lam = reinterpret_cast<float *>(w + 8 * mat);
  pb->norms = reinterpret_cast<double *>(w + 8 * mat + vec);
  pb->sweeps = reinterpret_cast<int32_t *>(w + 8 * mat + vec + norms_bytes);
  pb->Bh = reinterpret_cast<float *>(w + 8 * mat + vec + norms_bytes + sweeps_bytes);
  pb->Bl = pb->Bh + mat / sizeof(float);
  MSQ_TRY(forEachRun(*pb, off_user, 0, count, [&](int64_t user_off, int64_t arena_off, int64_t bytes) {
    return cudaCheck(ctx, cudaMemcpyAsync(pb->A + arena_off, a_user + user_off, bytes,
                                          cudaMemcpyDeviceToDevice, ctx->stream), "gather A");
  }));
  MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(pb->J, warm != nullptr ? warm : pb->A,
                                         total * sizeof(float), cudaMemcpyDeviceToDevice,
                                         ctx->stream), "jacobi copy"));
  if (warm != nullptr) {
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(pb->V, warm + total, total * sizeof(float),
                                           cudaMemcpyDeviceToDevice, ctx->stream),
                      "vectors copy"));
  }
  const int max_sweeps = pass.jacobi_max_sweeps > 0 ? pass.jacobi_max_sweeps : 15;
  double *tols = nullptr;
  if (pass.tols_host != nullptr) {
    tols = reinterpret_cast<double *>(w + 8 * mat + vec + norms_bytes + sweeps_bytes + backup_bytes);
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(tols, pass.tols_host, count * sizeof(double),
                                           cudaMemcpyHostToDevice, ctx->stream), "tolerances"));
  }
  MSQ_TRY(jacobiEnqueue(ctx, b, pb->J, pb->V, pb->lam, pass.jacobi_tolerance, max_sweeps,
                        pb->sweeps, nullptr, pass.low_bit, tols, pass.tols_host,
                        warm != nullptr));
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(pb->Xl, 0, total * sizeof(float), ctx->stream),
                    "x_lo reset"));
  for (size_t q = 0; q < pass.groups.size(); ++q) {
    const Group &g = groups[pass.groups[q]];
    const DeviceBatch *sb = pb->sub[q];
    const int c = static_cast<int>(g.members.size());
    const GroupReport &rep = reports[q];
    float *lam = pb->lam + pb->eig_base[q];
    double *norms = pb->norms + 2 * pb->first[q];
    MSQ_TRY(makeFactor(ctx, sb, pb->V, lam, pb->F));
    MSQ_TRY(reconstructFromFactor(ctx, sb, g.plan.format, pb->F, pb->Xh));
    // Corrections use the FP32 stable basis V, as the reference's fp32_frozen
    // stage does (src/metal_solver.cpp:304-325).  The plain FP32 plan runs its
    // GEMMs and residuals on the CUDA cores in FP32 / float-float; low-bit
    // plans run the correction GEMMs on the tensor cores (split BF16, FP32
    // accumulation) and the residual of the low-bit X0 too.  A tensor-core
    // residual carries the FP32 accumulation error of an n-long sum (about
    // sqrt(n) 2^-24 of ||A||): negligible against the quantization residual of
    // X0, not against the residual after a correction, which a further
    // correction could not push below it.  So every residual after the first
    // correction, and the one that decides acceptance, are float-float.
    const bool low_bit = g.plan.format != MSQ_PLAN_FP32;
    const int gemm_format = low_bit ? MSQ_FMT_BF16 : MSQ_FMT_FP32;
    auto residual = [&](bool accurate) {
      return low_bit && !accurate ? residualTc(ctx, sb, pb->A, pb->Xh, pb->Xl, pb->R, norms)
                                  : residualFF(ctx, sb, pb->A, pb->Xh, pb->Xl, pb->R, norms);
    };
    MSQ_TRY(residual(g.plan.sweeps == 0));
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(rep.initial, norms, 2 * c * sizeof(double),
                                           cudaMemcpyDeviceToHost, ctx->stream), "norms read"));
    for (int s = 0; s < g.plan.sweeps; ++s) {
      // V's split operands from the previous sweep stay valid: between two
      // sweeps only the float-float residual runs
      MSQ_TRY(sylvesterSweep(ctx, sb, gemm_format, pb->V, lam, pb->R, pb->Xh, pb->Xl, pb->F,
                             pb->W1, s > 0));
      MSQ_TRY(residual(true));
    }
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(rep.final, norms, 2 * c * sizeof(double),
                                           cudaMemcpyDeviceToHost, ctx->stream), "norms read"));
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(rep.sweeps, pb->sweeps + pb->first[q],
                                           c * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                           ctx->stream), "sweeps read"));
  }
  return MSQ_OK;
}

// Scatter X of every member of the pass (hi word; the lo word is below FP32
// resolution of the output).
int scatterPass(msq_ctx *ctx, const int64_t *off_user, const PassBuffers &pb, float *root) {
  return forEachRun(pb, off_user, 0, static_cast<int>(pb.members.size()),
                    [&](int64_t user_off, int64_t arena_off, int64_t bytes) {
    return cudaCheck(ctx, cudaMemcpyAsync(root + user_off, pb.Xh + arena_off, bytes,
                                          cudaMemcpyDeviceToDevice, ctx->stream), "scatter X");
  });
}

double ratio(const double *norms, int i) { return std::sqrt(norms[2 * i] / norms[2 * i + 1]); }

// The FP32 fallback group, run with host decisions: the plan's pipeline,
// then further FP32 sweeps while any member's residual misses `tolerance`
// (at most extra_sweeps), as the reference's plain method corrects until its
// tolerance is met (src/accelerate_backend.cpp:803-1091).  A sweep that does
// not lower a member's residual is undone for that member and the sweeps
// stop (Newton from a basis that no longer contracts diverges).  `warm`:
// the members' rotated matrices and rotations from the plan pass (enqueuePass
// layout), which the fallback's Jacobi continues; their sweeps add to the
// plan pass's in `jsweeps`.
int runFallback(msq_ctx *ctx, const float *a_user, const int32_t *n_user,
                const int64_t *off_user, const Group &g, float *root, double tolerance,
                int extra_sweeps, std::vector<double> &final_res, std::vector<int> &jsweeps,
                int *applied, const float *warm) {
  const int count = static_cast<int>(g.members.size());
  void *host = pinnedScratch(ctx, reportBytes(count));
  if (host == nullptr) return MSQ_ERR_CUDA;
  const std::vector<GroupReport> reports{reportAt(host, count)};
  const GroupReport &rep = reports[0];
  const std::vector<Group> groups{g};
  Pass pass{g.plan.jacobi_tolerance, g.plan.jacobi_max_sweeps, false, {0}};
  PassBuffers gb;
  MSQ_TRY(enqueuePass(ctx, a_user, n_user, off_user, groups, pass, reports, true, &gb, warm));
  MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(ctx->stream), "fallback sync"));
  std::vector<double> norms(rep.final, rep.final + 2 * count);
  int done = g.plan.sweeps;
  for (int extra = 0; extra < extra_sweeps; ++extra) {
    bool all_met = true;
    for (int i = 0; i < count; ++i) all_met = all_met && ratio(norms.data(), i) <= tolerance;
    if (all_met) break;
    const std::vector<double> before = norms;
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(gb.Bh, gb.Xh, gb.total * sizeof(float),
                                           cudaMemcpyDeviceToDevice, ctx->stream), "x backup"));
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(gb.Bl, gb.Xl, gb.total * sizeof(float),
                                           cudaMemcpyDeviceToDevice, ctx->stream), "x backup"));
    MSQ_TRY(sylvesterSweep(ctx, gb.b, MSQ_FMT_FP32, gb.V, gb.lam, gb.R, gb.Xh, gb.Xl, gb.F,
                           gb.W1));
    MSQ_TRY(residualFF(ctx, gb.b, gb.A, gb.Xh, gb.Xl, gb.R, gb.norms));
    ++done;
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(norms.data(), gb.norms, 2 * count * sizeof(double),
                                           cudaMemcpyDeviceToHost, ctx->stream), "norms read"));
    MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(ctx->stream), "norms sync"));
    bool worse = false;
    for (int i = 0; i < count; ++i) {
      if (!(ratio(norms.data(), i) < ratio(before.data(), i))) {
        worse = true;
        const size_t elems = static_cast<size_t>(gb.n[i]) * gb.n[i];
        MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(gb.Xh + gb.off[i], gb.Bh + gb.off[i],
                                               elems * sizeof(float), cudaMemcpyDeviceToDevice,
                                               ctx->stream), "x undo"));
        MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(gb.Xl + gb.off[i], gb.Bl + gb.off[i],
                                               elems * sizeof(float), cudaMemcpyDeviceToDevice,
                                               ctx->stream), "x undo"));
        norms[2 * i] = before[2 * i];
        norms[2 * i + 1] = before[2 * i + 1];
      }
    }
    if (worse) break;
  }
  *applied = done;
  MSQ_TRY(scatterPass(ctx, off_user, gb, root));
  MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(ctx->stream), "group sync"));
  MSQ_TRY(checkDeviceStatus(ctx));
  for (int i = 0; i < count; ++i) {
    final_res[g.members[i]] = ratio(norms.data(), i);
    jsweeps[g.members[i]] = (warm != nullptr ? jsweeps[g.members[i]] : 0) + rep.sweeps[i];
  }
  return MSQ_OK;
}

// Copies the retry members' rotated matrices and rotations out of the plan
// pass's arena (still in place after the pass or its graph replay: every
// group's members in group order, enqueuePass's layout) into the fallback
// arena, in the layout the fallback pass gives them: J of every member, then
// V of every member.  *warm stays null when the plan pass's eigenvectors are
// not FP32 accurate (the tensor-core eigenvector modes, 256 < n <= 512).
int warmStart(msq_ctx *ctx, const int32_t *n, int count, const std::vector<Group> &groups,
              bool low_bit, const std::vector<int> &retry, const float **warm) {
  *warm = nullptr;
  auto elems = [&](int m) { return (static_cast<int64_t>(n[m]) * n[m] + 3) & ~int64_t(3); };
  const int mode = ctx->jacobi_vectors >= 0 ? ctx->jacobi_vectors : (low_bit ? 2 : 0);
  int64_t retry_total = 0;
  for (int m : retry) {
    if (mode >= 2 && n[m] > 256 && n[m] <= 512) return MSQ_OK;
    retry_total += elems(m);
  }
  std::vector<int64_t> member_off(count, -1);  // by caller index
  int64_t total = 0;
  for (const Group &g : groups)
    for (int m : g.members) {
      member_off[m] = total;
      total += elems(m);
    }
  const char *arena = static_cast<const char *>(ctx->scratch[kScratchSolver]);
  if (arena == nullptr) return MSQ_OK;
  const size_t mat = alignUp(total * sizeof(float));
  const float *J = reinterpret_cast<const float *>(arena + mat);
  const float *V = reinterpret_cast<const float *>(arena + 2 * mat);
  auto *out = static_cast<float *>(scratch(ctx, 2 * retry_total * sizeof(float), kScratchFallback));
  if (out == nullptr) return MSQ_ERR_CUDA;
  int64_t at = 0;
  for (size_t i = 0; i < retry.size();) {
    // a run of members adjacent in both layouts: one copy per buffer
    size_t j = i + 1;
    int64_t run = elems(retry[i]);
    while (j < retry.size() && member_off[retry[j]] == member_off[retry[i]] + run) run += elems(retry[j++]);
    const int64_t from = member_off[retry[i]];
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(out + at, J + from, run * sizeof(float),
                                           cudaMemcpyDeviceToDevice, ctx->stream), "warm J"));
    MSQ_TRY(cudaCheck(ctx, cudaMemcpyAsync(out + retry_total + at, V + from, run * sizeof(float),
                                           cudaMemcpyDeviceToDevice, ctx->stream), "warm V"));
    at += run;
    i = j;
  }
  *warm = out;
  return MSQ_OK;
}

uint64_t mix(uint64_t h, uint64_t v) { return (h ^ v) * 1099511628211ull; }

// The whole-solve graph key: layout, plans, buffers, tolerance and the
// context settings the launch sequence depends on.
uint64_t solveKey(msq_ctx *ctx, const float *a, const int32_t *n, const int64_t *offset,
                  int count, const std::vector<Group> &groups, double tolerance,
                  const float *root) {
  uint64_t h = 1469598103934665603ull;
  h = mix(h, static_cast<uint64_t>(count));
  for (int i = 0; i < count; ++i) h = mix(mix(h, static_cast<uint64_t>(n[i])), static_cast<uint64_t>(offset[i]));
  for (const Group &g : groups) {
    uint64_t t;
    std::memcpy(&t, &g.plan.jacobi_tolerance, sizeof(t));
    h = mix(mix(mix(mix(h, g.plan.format), g.plan.sweeps), t), g.plan.jacobi_max_sweeps);
    for (int m : g.members) h = mix(h, static_cast<uint64_t>(m));
  }
  uint64_t tol;
  std::memcpy(&tol, &tolerance, sizeof(tol));
  h = mix(mix(mix(h, tol), reinterpret_cast<uintptr_t>(a)), reinterpret_cast<uintptr_t>(root));
  h = mix(mix(h, ctx->concurrent ? 1 : 0), static_cast<uint64_t>(ctx->jacobi_vectors + 8));
  return mix(h, reinterpret_cast<uintptr_t>(ctx->stream));
}

}  // namespace
}  // namespace msq

extern "C" int msq_solve_batched(msq_ctx *ctx, const float *a, const int32_t *n,
                                 const int64_t *offset, int count, const msq_plan *plans,
                                 double tolerance, float *root, msq_solve_result *results) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  if (a == nullptr || root == nullptr || n == nullptr || offset == nullptr || count <= 0)
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_solve_batched: null or empty input");
  if (!(tolerance > 0.0)) return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "tolerance must be > 0");
  const msq_plan fp32_plan{MSQ_PLAN_FP32, 0, 1e-7, 15, 0};
  std::vector<Group> groups;
  for (int i = 0; i < count; ++i) {
    if (n[i] < 1) return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "order < 1");
    const msq_plan p = plans ? plans[i] : fp32_plan;
    if (p.format < MSQ_PLAN_FP32 || p.format > MSQ_PLAN_MXFP4 || p.sweeps < 0 || p.sweeps > 8)
      return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "invalid plan");
    bool placed = false;
    for (Group &g : groups) {
      if (samePlan(g.plan, p)) {
        g.members.push_back(i);
        placed = true;
        break;
      }
    }
    if (!placed) groups.push_back({p, {i}});
  }
  std::vector<double> final_res(count, NAN), initial_res(count, NAN);
  std::vector<int> jsweeps(count, 0), fallback(count, 0), accepted(count, 0), corrections(count, 0);
  // The plan groups, enqueued back to back with no host synchronisation and
  // their reports copied into pinned host memory; one synchronisation at the
  // end.  From the second call with the same layout, plans, buffers and
  // tolerance (the first sizes every arena and cache), the whole sequence is
  // captured once into a CUDA graph and later calls replay it with one
  // launch, while no freed allocation invalidates it.
  // every group in one Jacobi pass, each matrix to its plan's tolerance
  std::vector<Pass> passes(1);
  {
    Pass &ps = passes[0];
    ps.jacobi_tolerance = groups[0].plan.jacobi_tolerance;
    ps.jacobi_max_sweeps = 0;
    ps.low_bit = true;
    for (size_t k = 0; k < groups.size(); ++k) {
      const msq_plan &p = groups[k].plan;
      ps.groups.push_back(static_cast<int>(k));
      ps.jacobi_max_sweeps =
          std::max(ps.jacobi_max_sweeps, p.jacobi_max_sweeps > 0 ? p.jacobi_max_sweeps : 15);
      ps.low_bit = ps.low_bit && p.format != MSQ_PLAN_FP32;
    }
  }
  bool mixed_tols = false;
  for (const Group &g : groups)
    mixed_tols = mixed_tols || g.plan.jacobi_tolerance != groups[0].plan.jacobi_tolerance;
  size_t report_bytes = 0;
  for (const Group &g : groups) report_bytes += reportBytes(static_cast<int>(g.members.size()));
  const size_t tols_at = report_bytes;
  if (mixed_tols) report_bytes += count * sizeof(double);
  void *host = pinnedScratch(ctx, report_bytes);
  if (host == nullptr) return MSQ_ERR_CUDA;
  if (mixed_tols) {
    double *t = reinterpret_cast<double *>(static_cast<char *>(host) + tols_at);
    size_t i = 0;
    for (const Group &g : groups)
      for (size_t j = 0; j < g.members.size(); ++j) t[i++] = g.plan.jacobi_tolerance;
    passes[0].tols_host = t;
  }
  std::vector<GroupReport> reports;
  {
    char *at = static_cast<char *>(host);
    for (const Group &g : groups) {
      const int c = static_cast<int>(g.members.size());
      reports.push_back(reportAt(at, c));
      at += reportBytes(c);
    }
  }
  const uint64_t key = solveKey(ctx, a, n, offset, count, groups, tolerance, root);
  bool replayed = false;
  for (size_t k = 0; k < ctx->solve_graphs.size(); ++k) {
    auto &e = ctx->solve_graphs[k];
    if (e.key != key) continue;
    if (e.generation != ctx->alloc_generation) {  // captured memory was freed since
      cudaGraphExecDestroy(e.exec);
      ctx->solve_graphs.erase(ctx->solve_graphs.begin() + k);
      break;
    }
    MSQ_TRY(cudaCheck(ctx, cudaGraphLaunch(e.exec, ctx->stream), "solve graph launch"));
    ++ctx->graph_launches;
    ctx->launches += e.launches;
    replayed = true;
    break;
  }
  if (!replayed) {
    const bool seen = std::find(ctx->solve_seen.begin(), ctx->solve_seen.end(), key) !=
                      ctx->solve_seen.end();
    bool capture = seen && ctx->graphs && !ctx->timing && waitTestMode() == kWaitTestOff;
    std::vector<PassBuffers> buffers(passes.size());
    if (capture) {
      // the capture must not allocate or synchronise: every pass's batch,
      // Jacobi plan and tuned launch shapes exist after the direct run
      for (const Pass &ps : passes) {
        std::vector<int32_t> pn;
        std::vector<int64_t> po;
        int64_t total = 0;
        for (int k : ps.groups)
          for (int m : groups[k].members) {
            pn.push_back(n[m]);
            po.push_back(total);
            total += (static_cast<int64_t>(n[m]) * n[m] + 3) & ~int64_t(3);
          }
        const DeviceBatch *b = prepareBatch(ctx, pn.data(), po.data(), static_cast<int>(pn.size()));
        if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
        capture = capture && jacobiCapturable(ctx, b, ps.low_bit);
      }
    }
    const uint64_t generation = ctx->alloc_generation;
    cudaStream_t caller = ctx->stream;
    cudaStream_t capture_stream = capture ? auxStream(ctx, 4) : nullptr;
    if (capture && (capture_stream == nullptr || capture_stream == caller)) capture = false;
    const uint64_t launches0 = ctx->launches;
    if (capture) {
      MSQ_TRY(cudaCheck(ctx, cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal),
                        "solve capture"));
      ctx->stream = capture_stream;
      ctx->capturing = true;
    }
    int status = MSQ_OK;
    for (size_t q = 0; q < passes.size() && status == MSQ_OK; ++q) {
      std::vector<GroupReport> pass_reports;
      for (int k : passes[q].groups) pass_reports.push_back(reports[k]);
      status = enqueuePass(ctx, a, n, offset, groups, passes[q], pass_reports, false, &buffers[q]);
      if (status == MSQ_OK) status = scatterPass(ctx, offset, buffers[q], root);
    }
    if (capture) {
      ctx->stream = caller;
      ctx->capturing = false;
      cudaGraph_t graph = nullptr;
      const cudaError_t end = cudaStreamEndCapture(capture_stream, &graph);
      cudaGraphExec_t exec = nullptr;
      if (status == MSQ_OK && end == cudaSuccess && generation == ctx->alloc_generation &&
          cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
        status = cudaCheck(ctx, cudaGraphLaunch(exec, caller), "solve graph launch");
        ++ctx->graph_launches;
        if (ctx->solve_graphs.size() >= 4) {
          cudaGraphExecDestroy(ctx->solve_graphs.front().exec);
          ctx->solve_graphs.erase(ctx->solve_graphs.begin());
        }
        ctx->solve_graphs.push_back({key, generation, exec, ctx->launches - launches0});
      } else if (status == MSQ_OK) {
        status = setError(ctx, MSQ_ERR_CUDA, "solve graph capture failed");
      }
      if (graph != nullptr) cudaGraphDestroy(graph);
    } else if (status == MSQ_OK && !seen) {
      if (ctx->solve_seen.size() >= 16) ctx->solve_seen.erase(ctx->solve_seen.begin());
      ctx->solve_seen.push_back(key);
    }
    MSQ_TRY(status);
  }
  MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(ctx->stream), "solve sync"));
  MSQ_TRY(checkDeviceStatus(ctx));
  for (size_t k = 0; k < groups.size(); ++k) {
    const Group &g = groups[k];
    for (size_t i = 0; i < g.members.size(); ++i) {
      const int m = g.members[i];
      initial_res[m] = ratio(reports[k].initial, static_cast<int>(i));
      final_res[m] = ratio(reports[k].final, static_cast<int>(i));
      jsweeps[m] = reports[k].sweeps[i];
      corrections[m] = g.plan.sweeps;
    }
  }
  // The fallback is the FP32 path with FP32 correction sweeps until the
  // tolerance is met (at least one, at most kFallbackSweeps): FP32 Jacobi +
  // FP32 reconstruction alone leaves a residual near u * n, which misses
  // tight tolerances at the larger orders, and ill-conditioned large
  // matrices (n = 4096, condition 1e6) need a second sweep.
  constexpr int kFallbackSweeps = 4;
  // (Jacobi budget 20 sweeps: n = 4096 at condition 1e6 needs 16 to 1e-7)
  const msq_plan fallback_plan{MSQ_PLAN_FP32, 1, 1e-7, 20, 0};
  Group retry{fallback_plan, {}};
  for (const Group &g : groups) {
    if (samePlan(g.plan, fallback_plan)) continue;
    for (int m : g.members)
      if (!(final_res[m] <= tolerance)) retry.members.push_back(m);
  }
  for (int i = 0; i < count; ++i) accepted[i] = final_res[i] <= tolerance;
  const std::vector<double> plan_res = final_res;
  if (!retry.members.empty()) {
    int applied = 0;
    // the fallback's Jacobi continues from the plan pass's rotations (a plan
    // stops its Jacobi at 1e-2 or 1e-3, so a few FP32 sweeps reach 1e-7
    // instead of a full solve from A)
    const float *warm = nullptr;
    MSQ_TRY(warmStart(ctx, n, count, groups, passes[0].low_bit, retry.members, &warm));
    MSQ_TRY(runFallback(ctx, a, n, offset, retry, root, tolerance,
                        kFallbackSweeps - fallback_plan.sweeps, final_res, jsweeps, &applied,
                        warm));
    for (int m : retry.members) {
      fallback[m] = 1;
      corrections[m] = applied;
    }
  }
  if (results != nullptr) {
    for (int i = 0; i < count; ++i) {
      results[i].final_residual = final_res[i];
      results[i].initial_residual = initial_res[i];
      results[i].jacobi_sweeps = jsweeps[i];
      results[i].corrections = corrections[i];
      results[i].accepted = accepted[i];
      results[i].fallback = fallback[i];
      results[i].plan_residual = plan_res[i];
    }
  }
  return MSQ_OK;
}
