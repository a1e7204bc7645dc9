// Context, error handling, batch-layout upload and scratch management.
#include "msq_internal.cuh"

#include <atomic>

#include <cstring>
#include <string>

namespace msq {

int setError(msq_ctx *ctx, int code, const std::string &message) {
  if (ctx != nullptr) ctx->error = message;
  return code;
}

int cudaCheck(msq_ctx *ctx, cudaError_t status, const char *what) {
  if (status == cudaSuccess) return MSQ_OK;
  return setError(ctx, MSQ_ERR_CUDA,
                  std::string(what) + ": " + cudaGetErrorString(status));
}

static cudaEvent_t takeEvent(msq_ctx *ctx) {
  if (ctx->event_pool.empty()) {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t e = ctx->event_pool.back();
  ctx->event_pool.pop_back();
  return e;
}

static void recycleTiming(msq_ctx *ctx) {
  for (auto &entry : ctx->timing_events) {
    ctx->event_pool.push_back(entry.end);
    if (entry.begin != nullptr) ctx->event_pool.push_back(entry.begin);
  }
  ctx->timing_events.clear();
  if (ctx->pending_begin != nullptr) {
    ctx->event_pool.push_back(ctx->pending_begin);
    ctx->pending_begin = nullptr;
  }
}

int launched(msq_ctx *ctx, const char *what) {
  ++ctx->launches;
  const int status = cudaCheck(ctx, cudaGetLastError(), what);
  if (status == MSQ_OK && ctx->timing) {
    cudaEvent_t e = takeEvent(ctx);
    cudaEventRecord(e, ctx->stream);
    ctx->timing_events.push_back({what, e, nullptr});
  }
  return status;
}

void launchBegin(msq_ctx *ctx, cudaStream_t stream) {
  // a launch on the context's stream is timed by the event chain instead
  if (!ctx->timing || stream == ctx->stream) return;
  ctx->pending_begin = takeEvent(ctx);
  cudaEventRecord(ctx->pending_begin, stream);
}

int launchedOn(msq_ctx *ctx, cudaStream_t stream, const char *what) {
  if (stream == ctx->stream) return launched(ctx, what);
  ++ctx->launches;
  const int status = cudaCheck(ctx, cudaGetLastError(), what);
  if (ctx->timing && ctx->pending_begin != nullptr) {
    cudaEvent_t e = takeEvent(ctx);
    cudaEventRecord(e, stream);
    ctx->timing_events.push_back({what, e, ctx->pending_begin});
    ctx->pending_begin = nullptr;
  }
  return status;
}

cudaStream_t auxStream(msq_ctx *ctx, int i) {
  if (ctx->aux[i] == nullptr) {
    if (cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking) != cudaSuccess) {
      ctx->aux[i] = nullptr;
      return ctx->stream;  // degrade to the context stream (still correct)
    }
  }
  return ctx->aux[i];
}

void syncReset(msq_ctx *ctx) { ctx->sync_next = 0; }

cudaEvent_t syncEvent(msq_ctx *ctx) {
  if (ctx->sync_next == ctx->sync_pool.size()) {
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    ctx->sync_pool.push_back(e);
  }
  return ctx->sync_pool[ctx->sync_next++];
}

int streamWait(msq_ctx *ctx, cudaStream_t waiter, cudaStream_t source) {
  if (waiter == source) return MSQ_OK;
  cudaEvent_t e = syncEvent(ctx);
  MSQ_TRY(cudaCheck(ctx, cudaEventRecord(e, source), "event record"));
  MSQ_TRY(cudaCheck(ctx, cudaStreamWaitEvent(waiter, e, 0), "stream wait"));
  if (ctx->timing && waiter == ctx->stream) {
    // restart the context-stream chain after a join (the join's wait is not
    // a launch's duration)
    cudaEvent_t m = takeEvent(ctx);
    cudaEventRecord(m, ctx->stream);
    ctx->timing_events.push_back({nullptr, m, nullptr});
  }
  return MSQ_OK;
}

namespace {
std::atomic<int> g_wait_test{0};
}  // namespace

int waitTestMode() { return g_wait_test.load(std::memory_order_relaxed); }

int checkDeviceStatus(msq_ctx *ctx) {
  int status = 0;
  MSQ_TRY(cudaCheck(ctx,
                    cudaMemcpyAsync(&status, ctx->d_status, sizeof(int),
                                    cudaMemcpyDeviceToHost, ctx->stream),
                    "device status read"));
  MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(ctx->stream), "device status sync"));
  if (status != kStatusOk) {
    MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream),
                      "device status reset"));
    const char *why = status == kStatusMbarrierTimeout   ? "bounded mbarrier wait expired"
                      : status == kStatusTmemAllocFailed ? "TMEM allocation failed"
                      : status == kStatusBadOrder        ? "matrix order outside kernel limits"
                      : status == kStatusFlagTimeout     ? "bounded shared-memory flag wait expired"
                      : status == kStatusBadSpectrum     ? "log-spectrum input not finite and positive"
                                                         : "kernel reported an error";
    return setError(ctx, MSQ_ERR_DEVICE_STATUS,
                    std::string("device status ") + std::to_string(status) + ": " + why);
  }
  return MSQ_OK;
}

static uint64_t hashLayout(const int32_t *n, const int64_t *offset, int count) {
  uint64_t h = 1469598103934665603ull ^ static_cast<uint64_t>(count);
  for (int i = 0; i < count; ++i) {
    h = (h ^ static_cast<uint64_t>(n[i])) * 1099511628211ull;
    h = (h ^ static_cast<uint64_t>(offset[i])) * 1099511628211ull;
  }
  return h;
}

const DeviceBatch *prepareBatch(msq_ctx *ctx, const int32_t *n,
                                const int64_t *offset, int count) {
  if (count <= 0 || n == nullptr || offset == nullptr) {
    setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "batch: empty or null layout");
    return nullptr;
  }
  const uint64_t key = hashLayout(n, offset, count);
  for (DeviceBatch *b : ctx->batches) {
    if (b->key == key && b->count == count &&
        std::memcmp(b->host_n.data(), n, count * sizeof(int32_t)) == 0 &&
        std::memcmp(b->host_offset.data(), offset, count * sizeof(int64_t)) == 0) {
      return b;
    }
  }
  auto *b = new DeviceBatch;
  b->count = count;
  b->key = key;
  b->host_n.assign(n, n + count);
  b->host_offset.assign(offset, offset + count);
  b->host_eig_offset.resize(count);
  int64_t eig = 0;
  for (int i = 0; i < count; ++i) {
    if (n[i] < 1 || offset[i] < 0) {
      delete b;
      setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "batch: order < 1 or negative offset");
      return nullptr;
    }
    b->host_eig_offset[i] = eig;
    eig += n[i];
    b->total_elements += static_cast<int64_t>(n[i]) * n[i];
    if (n[i] > b->max_n) b->max_n = n[i];
  }
  b->total_order = eig;
  const size_t bytes = count * (sizeof(int32_t) + 2 * sizeof(int64_t));
  char *device = nullptr;
  if (cudaCheck(ctx, cudaMalloc(&device, bytes + 64), "batch upload alloc") != MSQ_OK) {
    delete b;
    return nullptr;
  }
  b->offset = reinterpret_cast<int64_t *>(device);
  b->eig_offset = b->offset + count;
  b->n = reinterpret_cast<int32_t *>(b->eig_offset + count);
  // Synchronous copies: the layout is uploaded once and then reused.
  if (cudaCheck(ctx, cudaMemcpy(b->offset, offset, count * sizeof(int64_t), cudaMemcpyHostToDevice), "batch upload") != MSQ_OK ||
      cudaCheck(ctx, cudaMemcpy(b->eig_offset, b->host_eig_offset.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice), "batch upload") != MSQ_OK ||
      cudaCheck(ctx, cudaMemcpy(b->n, n, count * sizeof(int32_t), cudaMemcpyHostToDevice), "batch upload") != MSQ_OK) {
    cudaFree(device);
    delete b;
    return nullptr;
  }
  if (ctx->batches.size() >= 32) {
    DeviceBatch *old = ctx->batches.front();
    for (auto &w : old->work_cache) cudaFree(w.work);
    cudaFree(old->offset);
    delete old;
    ctx->batches.erase(ctx->batches.begin());
    ++ctx->alloc_generation;
  }
  ctx->batches.push_back(b);
  return b;
}

void *scratch(msq_ctx *ctx, size_t bytes, int slot) {
  if (bytes <= ctx->scratch_bytes[slot]) return ctx->scratch[slot];
  if (ctx->scratch[slot] != nullptr) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->scratch[slot]);
    ctx->scratch[slot] = nullptr;
    ctx->scratch_bytes[slot] = 0;
    ++ctx->alloc_generation;
  }
  const size_t rounded = (bytes + (1u << 20) - 1) & ~static_cast<size_t>((1u << 20) - 1);
  if (cudaCheck(ctx, cudaMalloc(&ctx->scratch[slot], rounded), "scratch alloc") != MSQ_OK) {
    ctx->scratch[slot] = nullptr;
    return nullptr;
  }
  ctx->scratch_bytes[slot] = rounded;
  return ctx->scratch[slot];
}

void *pinnedScratch(msq_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->pinned_bytes) return ctx->pinned;
  if (ctx->pinned != nullptr) {
    cudaStreamSynchronize(ctx->stream);
    cudaFreeHost(ctx->pinned);
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    ++ctx->alloc_generation;
  }
  const size_t rounded = (bytes + 65535) & ~static_cast<size_t>(65535);
  if (cudaCheck(ctx, cudaMallocHost(&ctx->pinned, rounded), "pinned staging alloc") != MSQ_OK) {
    ctx->pinned = nullptr;
    return nullptr;
  }
  ctx->pinned_bytes = rounded;
  return ctx->pinned;
}

}  // namespace msq

using namespace msq;

extern "C" int msq_create(msq_ctx **out, int device) {
  if (out == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto *ctx = new msq_ctx;
  ctx->device = device;
  if (cudaCheck(ctx, cudaSetDevice(device), "cudaSetDevice") != MSQ_OK ||
      cudaCheck(ctx, cudaMalloc(&ctx->d_status, 256), "status alloc") != MSQ_OK ||
      cudaCheck(ctx, cudaMemset(ctx->d_status, 0, 256), "status reset") != MSQ_OK) {
    static thread_local std::string last;
    last = ctx->error;
    delete ctx;
    return MSQ_ERR_CUDA;
  }
  *out = ctx;
  return MSQ_OK;
}

extern "C" void msq_destroy(msq_ctx *ctx) {
  if (ctx == nullptr) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream != nullptr) cudaStreamSynchronize(ctx->stream);
  else cudaDeviceSynchronize();
  for (DeviceBatch *b : ctx->batches) {
    for (auto &w : b->work_cache) cudaFree(w.work);
    cudaFree(b->offset);
    delete b;
  }
  for (int slot = 0; slot < msq::kScratchSlots; ++slot)
    if (ctx->scratch[slot] != nullptr) cudaFree(ctx->scratch[slot]);
  if (ctx->grid_exec != nullptr) cudaGraphExecDestroy(ctx->grid_exec);
  for (auto &g : ctx->jacobi_graphs) cudaGraphExecDestroy(g.exec);
  for (auto &g : ctx->solve_graphs) cudaGraphExecDestroy(g.exec);
  if (ctx->pinned != nullptr) cudaFreeHost(ctx->pinned);
  destroyJacobiPlans(ctx->jacobi_plans);
  destroyTcPlans(ctx->tc_plans);
  if (ctx->grid_host != nullptr) cudaFreeHost(ctx->grid_host);
  if (ctx->d_status != nullptr) cudaFree(ctx->d_status);
  recycleTiming(ctx);
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->sync_pool) cudaEventDestroy(e);
  for (cudaStream_t s : ctx->aux)
    if (s != nullptr) cudaStreamDestroy(s);
  delete ctx;
}

extern "C" const char *msq_last_error(const msq_ctx *ctx) {
  return ctx == nullptr ? "null context" : ctx->error.c_str();
}

extern "C" int msq_set_stream(msq_ctx *ctx, void *stream) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return MSQ_OK;
}

extern "C" int msq_set_concurrency(msq_ctx *ctx, int enable) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  ctx->concurrent = enable != 0;
  return MSQ_OK;
}

extern "C" int msq_set_graphs(msq_ctx *ctx, int enable) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  ctx->graphs = enable != 0;
  return MSQ_OK;
}

extern "C" int msq_debug_expire_waits(int mode) {
  if (mode < msq::kWaitTestOff || mode > msq::kWaitTestMbarrier) return MSQ_ERR_INVALID_ARGUMENT;
  msq::g_wait_test.store(mode, std::memory_order_relaxed);
  return MSQ_OK;
}

extern "C" int msq_synchronize(msq_ctx *ctx) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  MSQ_TRY(cudaCheck(ctx, cudaStreamSynchronize(ctx->stream), "msq_synchronize"));
  return checkDeviceStatus(ctx);
}

extern "C" uint64_t msq_launch_count(const msq_ctx *ctx) {
  return ctx == nullptr ? 0 : ctx->launches;
}

extern "C" uint64_t msq_graph_launch_count(const msq_ctx *ctx) {
  return ctx == nullptr ? 0 : ctx->graph_launches;
}

namespace msq {
namespace {

// FP32 FMA throughput: eight independent FMA chains per thread, enough
// threads to fill every SM; the result keeps the chains live.
__global__ void __launch_bounds__(256) fmaRateKernel(float *out, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = static_cast<float>(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
  }
  float sum = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) sum += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

}  // namespace
}  // namespace msq

extern "C" int msq_fma_rate(msq_ctx *ctx, double *tflops) {
  if (ctx == nullptr || tflops == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  constexpr int kBlocks = msq::kSmCount * 8, kThreads = 256, kIters = 1 << 15;
  float *out = static_cast<float *>(scratch(ctx, kBlocks * kThreads * sizeof(float), msq::kScratchGemm));
  if (out == nullptr) return MSQ_ERR_CUDA;
  cudaEvent_t start = nullptr, stop = nullptr;
  MSQ_TRY(cudaCheck(ctx, cudaEventCreate(&start), "fma rate event"));
  MSQ_TRY(cudaCheck(ctx, cudaEventCreate(&stop), "fma rate event"));
  float best = 0.0f;
  for (int rep = 0; rep < 4; ++rep) {  // the first launch warms the clocks
    cudaEventRecord(start, ctx->stream);
    msq::fmaRateKernel<<<kBlocks, kThreads, 0, ctx->stream>>>(out, kIters, 0.999999f, 1e-6f);
    cudaEventRecord(stop, ctx->stream);
    MSQ_TRY(launched(ctx, "fma rate"));
    MSQ_TRY(cudaCheck(ctx, cudaEventSynchronize(stop), "fma rate sync"));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, start, stop);
    if (rep > 0 && ms > 0.0f && (best == 0.0f || ms < best)) best = ms;
  }
  cudaEventDestroy(start);
  cudaEventDestroy(stop);
  const double flops = 2.0 * 8.0 * kIters * static_cast<double>(kBlocks) * kThreads;
  *tflops = best > 0.0f ? flops / (best * 1e-3) / 1e12 : 0.0;
  return MSQ_OK;
}

extern "C" int msq_timing_begin(msq_ctx *ctx) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  recycleTiming(ctx);
  cudaEvent_t e = takeEvent(ctx);
  MSQ_TRY(cudaCheck(ctx, cudaEventRecord(e, ctx->stream), "timing begin"));
  ctx->timing_events.push_back({nullptr, e, nullptr});
  ctx->timing = true;
  return MSQ_OK;
}

extern "C" int msq_timing_end(msq_ctx *ctx, char *out, size_t capacity) {
  if (ctx == nullptr || out == nullptr || capacity == 0) return MSQ_ERR_INVALID_ARGUMENT;
  msq::DeviceGuard device_guard(ctx);
  ctx->timing = false;
  MSQ_TRY(cudaCheck(ctx, cudaDeviceSynchronize(), "timing end"));
  struct Acc { double ms = 0.0; long count = 0; };
  std::vector<std::pair<std::string, Acc>> rows;
  cudaEvent_t chain = nullptr;  // last context-stream event
  for (size_t i = 0; i < ctx->timing_events.size(); ++i) {
    const auto &entry = ctx->timing_events[i];
    float ms = 0.0f;
    if (entry.begin != nullptr) {
      cudaEventElapsedTime(&ms, entry.begin, entry.end);
    } else {
      if (chain != nullptr && entry.name != nullptr) cudaEventElapsedTime(&ms, chain, entry.end);
      chain = entry.end;
    }
    if (entry.name == nullptr) continue;  // marker
    const std::string name = entry.name;
    Acc *acc = nullptr;
    for (auto &r : rows)
      if (r.first == name) acc = &r.second;
    if (acc == nullptr) {
      rows.emplace_back(name, Acc{});
      acc = &rows.back().second;
    }
    acc->ms += ms;
    acc->count += 1;
  }
  std::string text;
  for (auto &r : rows) {
    text += r.first + "\t" + std::to_string(r.second.count) + "\t" +
            std::to_string(r.second.ms) + "\n";
  }
  std::strncpy(out, text.c_str(), capacity - 1);
  out[capacity - 1] = '\0';
  recycleTiming(ctx);
  return MSQ_OK;
}
