// Internal declarations shared by the CUDA translation units of libmsq_cuda.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/msq_cuda.h"

namespace msq {

// GB300: 152 SMs on two dies.  Grids of streaming kernels are sized as a
// multiple of this so every SM gets the same number of resident CTAs.
constexpr int kSmCount = 152;

// Device-side status words (one int each) written by kernels that bound a
// wait or check an index or an input; read back by msq_synchronize and the
// solve calls (checkDeviceStatus).
enum DeviceStatus : int {
  kStatusOk = 0,
  kStatusJacobiOrderTooLarge = 1,
  kStatusMbarrierTimeout = 2,
  kStatusTmemAllocFailed = 3,
  kStatusBadOrder = 4,
  kStatusFlagTimeout = 5,
  kStatusBadSpectrum = 6,
};

// Failure injection for the bounded waits (msq_debug_expire_waits): 0 off;
// kWaitTestFlag makes the Jacobi sweep's shared-memory flag waits look for a
// value no warp writes and its tile-load barrier get no copy;
// kWaitTestMbarrier makes the tcgen05 GEMM's producer
// first wait on a barrier nothing arrives at, before it issues any copy.
// Either wait gives up after a short limit and reports its status.
enum WaitTest : int { kWaitTestOff = 0, kWaitTestFlag = 1, kWaitTestMbarrier = 2 };
int waitTestMode();

struct WorkList {
  int tile;
  int4 *work;
  int items;
};

// Batched layout uploaded to the device once per distinct (n, offset) set.
struct DeviceBatch {
  int count = 0;
  int32_t *n = nullptr;         // [count]
  int64_t *offset = nullptr;    // [count] element offset of matrix i
  int64_t *eig_offset = nullptr;// [count] prefix sum of n
  int64_t total_elements = 0;   // sum n^2
  int64_t total_order = 0;      // sum n
  int max_n = 0;
  uint64_t key = 0;
  std::vector<int32_t> host_n;
  std::vector<int64_t> host_offset;
  std::vector<int64_t> host_eig_offset;
  std::vector<WorkList> work_cache;  // tile work lists (msq_dense.cu)
};

// The context's cached Jacobi launch plans (msq_jacobi.cu) and tcgen05 tile
// plans (msq_tc.cu).
struct JacobiPlanCache;
void destroyJacobiPlans(JacobiPlanCache *cache);
struct TcPlanCache;
void destroyTcPlans(TcPlanCache *cache);

// A captured batched-Jacobi launch sequence and what it was captured for.
struct JacobiGraphKey {
  uint64_t plan_serial, batch_key;
  const void *batch, *a, *v, *w, *sweeps, *off, *work, *tols;
  double tol;
  int max_sweeps;
  bool concurrent;
  uint64_t shapes;
  bool operator==(const JacobiGraphKey &o) const {
    return plan_serial == o.plan_serial && batch_key == o.batch_key && batch == o.batch && a == o.a &&
           v == o.v && w == o.w && sweeps == o.sweeps && off == o.off && work == o.work &&
           tols == o.tols &&
           tol == o.tol && max_sweeps == o.max_sweeps && concurrent == o.concurrent &&
           shapes == o.shapes;
  }
};

struct JacobiGraph {
  JacobiGraphKey key;
  cudaGraphExec_t exec;
  uint64_t launches;  // kernel launches the graph holds
};

}  // namespace msq

struct msq_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string error;
  uint64_t launches = 0;
  int *d_status = nullptr;  // device status word
  // Grow-only scratch arenas owned by the context (freed in msq_destroy);
  // one per user so nested stages never share memory.
  void *scratch[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  size_t scratch_bytes[6] = {0, 0, 0, 0, 0, 0};
  // Batch layouts cached by content hash (at most 32, oldest evicted).
  std::vector<msq::DeviceBatch *> batches;
  // Launch timing (msq_timing_begin/end).  Launches on the context stream
  // record one event after each launch (duration = gap to the previous
  // event on that stream); launches on auxiliary streams record a begin and
  // an end event around the kernel.
  struct TimingEntry {
    const char *name;     // nullptr: a marker that only restarts the chain
    cudaEvent_t end;
    cudaEvent_t begin;    // nullptr for context-stream launches
  };
  bool timing = false;
  std::vector<TimingEntry> timing_events;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t pending_begin = nullptr;  // begin recorded for the next aux launch
  // Auxiliary streams (non-blocking, created on first use) that fork from and
  // join back into `stream` through events from sync_pool.
  cudaStream_t aux[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // false: every launch on `stream` (serial order; per-kernel timings are
  // then each kernel's own duration, not shared with concurrent work)
  bool concurrent = true;
  // Eigenvector accumulation of the batched Jacobi for 256 < n <= 512
  // (msq_set_jacobi_vectors): -1 automatic, 0 round-robin + FP32 replay,
  // 1 two-level pairing + FP32 replay, 2 two-level pairing + V on the
  // tensor cores, 3 two-level pairing + A and V on the tensor cores.
  int jacobi_vectors = -1;
  // Per-layout work plans of the Jacobi and of the tensor-core GEMMs.
  msq::JacobiPlanCache *jacobi_plans = nullptr;
  msq::TcPlanCache *tc_plans = nullptr;
  // Batched Jacobi launch sequences captured as CUDA graphs (at most 8).
  bool graphs = true;
  std::vector<msq::JacobiGraph> jacobi_graphs;
  // Grid Jacobi (one large matrix on all SMs): pinned off-norm readback and
  // the captured graph of one sweep, valid for order grid_n and workspace
  // grid_work.
  double *grid_host = nullptr;
  cudaGraphExec_t grid_exec = nullptr;
  int grid_n = 0;
  void *grid_work = nullptr;
  std::vector<cudaEvent_t> sync_pool;
  size_t sync_next = 0;
  // Whole-solve graphs (msq_solve_batched): the plan groups' launch
  // sequence of a call, captured once per (layout, plans, buffers,
  // tolerance) after one direct run of that call (which sizes every
  // scratch arena and cache), replayed while alloc_generation is unchanged.
  // alloc_generation counts every free of memory a captured graph may use
  // (scratch growth, evicted batch layouts and launch plans, pinned
  // staging growth).
  struct SolveGraph {
    uint64_t key;
    uint64_t generation;
    cudaGraphExec_t exec;
    uint64_t launches;
  };
  std::vector<SolveGraph> solve_graphs;
  std::vector<uint64_t> solve_seen;  // keys already run directly once
  uint64_t alloc_generation = 0;
  bool capturing = false;            // a whole-solve capture is open
  uint64_t graph_launches = 0;       // cudaGraphLaunch calls of this context
  void *pinned = nullptr;            // host staging of the solve's reports
  size_t pinned_bytes = 0;
};

namespace msq {

int setError(msq_ctx *ctx, int code, const std::string &message);
int cudaCheck(msq_ctx *ctx, cudaError_t status, const char *what);
// Checks the last launch error and counts one launch (context stream).
int launched(msq_ctx *ctx, const char *what);
// Launches on an auxiliary stream: launchBegin before, launchedOn after.
void launchBegin(msq_ctx *ctx, cudaStream_t stream);
int launchedOn(msq_ctx *ctx, cudaStream_t stream, const char *what);
// Auxiliary stream i (0..4), created non-blocking on first use: 0 replay,
// 1..3 sweep buckets, 4 graph capture.
cudaStream_t auxStream(msq_ctx *ctx, int i);
// A disable-timing event from the context's pool; syncReset() recycles the
// pool at the start of a call (events may be re-recorded once waited on).
cudaEvent_t syncEvent(msq_ctx *ctx);
void syncReset(msq_ctx *ctx);
// `waiter` waits for everything enqueued so far on `source`.
int streamWait(msq_ctx *ctx, cudaStream_t waiter, cudaStream_t source);
// Returns MSQ_ERR_DEVICE_STATUS (and resets the word) if a kernel set it.
int checkDeviceStatus(msq_ctx *ctx);
// Uploads (or finds cached) the batch layout; null on error (ctx->error set).
const DeviceBatch *prepareBatch(msq_ctx *ctx, const int32_t *n,
                                const int64_t *offset, int count);
// Grow-only context scratch arena `slot` (0: Jacobi, 1: solver,
// 2: codec operands, 3: GEMM split operands, 4: grid Jacobi, 5: the rotated
// matrices and eigenvectors a fallback continues from).
enum ScratchSlot : int {
  kScratchJacobi = 0, kScratchSolver = 1, kScratchOperand = 2, kScratchGemm = 3, kScratchGrid = 4,
  kScratchFallback = 5, kScratchSlots = 6
};
void *scratch(msq_ctx *ctx, size_t bytes, int slot);
// Grow-only pinned host staging (for reports copied back inside a graph).
void *pinnedScratch(msq_ctx *ctx, size_t bytes);

// Makes the context's device current for one entry point and restores the
// caller's device on return (a process may drive several GPUs).
struct DeviceGuard {
  int previous = -1;
  explicit DeviceGuard(const msq_ctx *ctx) {
    int current = 0;
    if (cudaGetDevice(&current) == cudaSuccess && current != ctx->device &&
        cudaSetDevice(ctx->device) == cudaSuccess) {
      previous = current;
    }
  }
  ~DeviceGuard() {
    if (previous >= 0) cudaSetDevice(previous);
  }
  DeviceGuard(const DeviceGuard &) = delete;
  DeviceGuard &operator=(const DeviceGuard &) = delete;
};

inline unsigned gridFor(size_t work_items, unsigned threads,
                        unsigned ctas_per_sm = 8) {
  size_t blocks = (work_items + threads - 1) / threads;
  const size_t cap = static_cast<size_t>(kSmCount) * ctas_per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return static_cast<unsigned>(blocks);
}

}  // namespace msq

#define MSQ_TRY(expr)               \
  do {                              \
    const int msq_status_ = (expr); \
    if (msq_status_ != MSQ_OK) {    \
      return msq_status_;           \
    }                               \
  } while (0)
