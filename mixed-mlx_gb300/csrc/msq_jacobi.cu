// Batched parallel-order two-sided Jacobi eigensolver.
//
// Replaces MetalRuntime::symmetricJacobi (src/metal_runtime.cpp:584-646),
// its kernels jacobi_rotations_f32 / jacobi_similarity_vectors_f32 /
// jacobi_root_eigenvalues_f32 (metal_mixed_sqrt.metal:1319-1444) and the
// host-built schedule makeJacobiSchedule (src/metal_solver.cpp:50-79).
//
// Same algorithm, laid out for GB300:
//  * the round-robin pairing is computed arithmetically (no schedule
//    arrays: the reference's needs 3 x n(n-1) u32 per order);
//  * one CTA owns one matrix for a whole sweep; the upper triangle of A is
//    kept packed in shared memory (n <= 336 fits the 227 KB limit) and the
//    disjoint 2x2 blocks of a round are rotated in place, so a round costs
//    one pass over shared memory instead of a global ping-pong;
//  * rotation angles and the off-norm are computed in FP64 (the reference
//    uses FP32 angles and a fixed 8 sweeps; here sweeps stop once
//    off(A) <= tol * ||A||_F);
//  * every round's (c, s) is logged and a second, row-parallel kernel
//    replays the sweep onto V: rows of V evolve independently under
//    right-multiplication by rotations, so V never competes with A for the
//    CTA's shared memory;
//  * launches are size-bucketed (threads per CTA grow with n) and the
//    largest matrices start first.
#include "msq_internal.cuh"

#include <algorithm>
#include <vector>

namespace msq {
namespace {

constexpr int kMaxSmemOrder = 336;  // n(n+1)/2 floats + tables <= 227 KB
constexpr int kVRowsMax = 32;       // rows of V per CTA in the replay kernel
constexpr size_t kSmemLimit = 227 * 1024;

struct JacobiState {
  double norm2;       // ||A||_F^2
  double off_ratio;   // off(A) / ||A||_F at the start of the last sweep
  int sweeps;         // sweeps applied
  int done;           // 1 once converged or out of budget
  int logged;         // 1 if the log holds a sweep not yet applied to V
  int pad;
};

struct JacobiArgs {
  float *a;                 // user matrices (full, column-major)
  float *packed;            // packed upper triangles (global workspace)
  const int64_t *a_offset;  // element offset of matrix i in a
  const int64_t *p_offset;  // element offset of matrix i in packed
  const int64_t *log_offset;// float2 offset of matrix i's rotation log
  const int64_t *eig_offset;
  const int32_t *n;
  float2 *log;
  float *eigenvalues;
  JacobiState *state;
  const int32_t *order;     // matrix ids of this launch, largest first
  int count;
  double tol;
  int max_sweeps;
  int first;                // 1 on the first launch (load from a, set norm)
};

// Slot -> participant of round r (participants 1..m-1 rotate right by one
// per round, slot 0 fixed), the closed form of std::rotate in
// makeJacobiSchedule (src/metal_solver.cpp:75-76).
__device__ __forceinline__ int rrSlot(int slot, int round, int m) {
  if (slot == 0) return 0;
  int k = slot - 1 - round % (m - 1);
  if (k < 0) k += m - 1;
  return 1 + k;
}

__device__ __forceinline__ void rrPair(int pair, int round, int m, int &p, int &q) {
  const int a = rrSlot(pair, round, m);
  const int b = rrSlot(m - 1 - pair, round, m);
  p = a < b ? a : b;
  q = a < b ? b : a;
}

__device__ __forceinline__ int packedIndex(const int *tri, int r, int c) {
  return r <= c ? tri[c] + r : tri[r] + c;
}

// Folded enumeration of the upper triangle {(i, j): i <= j < P} of pair
// blocks: rows i and P-1-i share one folded row of P+1 items.
__device__ __forceinline__ bool foldedBlock(int w, int P, int &i, int &j) {
  const int r = w / (P + 1);
  const int c = w - r * (P + 1);
  if (c < P - r) {
    i = r;
    j = r + c;
    return true;
  }
  if ((P & 1) && r == P / 2) return false;  // middle row of an odd P
  i = P - 1 - r;
  j = c - 1;
  return true;
}

__device__ double blockReduceSum(double v, double *red) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  const int warps = blockDim.x / 32;
  v = threadIdx.x < warps ? red[threadIdx.x] : 0.0;
  if (warp == 0) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  const double total = red[0];
  __syncthreads();
  return total;
}

// One sweep (or the convergence check / write-back) for one matrix per CTA.
// kSmem: packed A staged in shared memory; otherwise it is rotated in place
// in the global packed workspace (L2-resident at these orders).
template <bool kSmem>
__global__ void __launch_bounds__(1024)
jacobiSweepKernel(JacobiArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mi = args.order[blockIdx.x];
  const int n = args.n[mi];
  const int m = n + (n & 1);
  const int P = m / 2;
  JacobiState &st = args.state[mi];
  // Snapshot of the state before any thread writes it (the barriers below
  // keep thread 0's final update after every warp's snapshot).
  const JacobiState s0 = st;
  if (!args.first && s0.done) {
    if (threadIdx.x == 0) st.logged = 0;
    return;
  }

  double *red = reinterpret_cast<double *>(smem_raw);               // 32
  int *tri = reinterpret_cast<int *>(red + 32);                      // m + 1
  int *pair_p = tri + (m + 1);                                       // P
  int *pair_q = pair_p + P;                                          // P
  float *pc = reinterpret_cast<float *>(pair_q + P);                 // P
  float *ps = pc + P;                                                // P
  float *packed_s = ps + P;
  float *A = kSmem ? packed_s : args.packed + args.p_offset[mi];
  const float *full = args.a + args.a_offset[mi];
  float *packed_g = args.packed + args.p_offset[mi];
  const int tri_n = n * (n + 1) / 2;

  for (int k = threadIdx.x; k <= m; k += blockDim.x) tri[k] = k * (k + 1) / 2;
  __syncthreads();

  // Stage the packed upper triangle.
  if (args.first) {
    // Symmetrised load, as working_from_symmetric_f32 and the averaged
    // a_pq of jacobi_rotations_f32 do (metal_mixed_sqrt.metal:1349-1350).
    for (int c = 0; c < n; ++c) {
      for (int r = threadIdx.x; r <= c; r += blockDim.x) {
        A[tri[c] + r] = 0.5f * (full[r + static_cast<int64_t>(c) * n] +
                                full[c + static_cast<int64_t>(r) * n]);
      }
    }
  } else if (kSmem) {
    for (int k = threadIdx.x; k < tri_n; k += blockDim.x) A[k] = packed_g[k];
  }
  __syncthreads();

  // Off-norm and norm in FP64.
  double off2 = 0.0, diag2 = 0.0;
  for (int c = 0; c < n; ++c) {
    for (int r = threadIdx.x; r <= c; r += blockDim.x) {
      const double v = A[tri[c] + r];
      if (r == c) diag2 += v * v; else off2 += 2.0 * v * v;
    }
  }
  off2 = blockReduceSum(off2, red);
  diag2 = blockReduceSum(diag2, red);
  const double norm2 = args.first ? off2 + diag2 : s0.norm2;
  const int sweeps = args.first ? 0 : s0.sweeps;
  const double ratio = norm2 > 0.0 ? sqrt(off2 / norm2) : 0.0;
  const bool stop = ratio <= args.tol || sweeps >= args.max_sweeps;

  if (stop) {
    {
      // Eigenvalues = diagonal (jacobi_root_eigenvalues_f32 takes its sqrt
      // later, :1436-1444); full symmetric write-back of the matrix.
      float *eig = args.eigenvalues + args.eig_offset[mi];
      for (int k = threadIdx.x; k < n; k += blockDim.x) eig[k] = A[tri[k] + k];
      float *out = args.a + args.a_offset[mi];
      for (int c = 0; c < n; ++c) {
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
          out[r + static_cast<int64_t>(c) * n] = A[packedIndex(tri, r, c)];
        }
      }
    }
    if (threadIdx.x == 0) {
      st.norm2 = norm2;
      st.sweeps = sweeps;
      st.off_ratio = ratio;
      st.done = 1;
      st.logged = 0;
    }
    return;
  }

  float2 *log = args.log + args.log_offset[mi];
  for (int round = 0; round < m - 1; ++round) {
    // Angles of the round's disjoint pairs (FP64).
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
      int p, q;
      rrPair(k, round, m, p, q);
      double cs = 1.0, sn = 0.0;
      if (q < n) {
        const double app = A[tri[p] + p];
        const double aqq = A[tri[q] + q];
        const double apq = A[tri[q] + p];
        if (apq != 0.0) {
          const double tau = (aqq - app) / (2.0 * apq);
          const double t = copysign(1.0 / (fabs(tau) + sqrt(1.0 + tau * tau)), tau);
          cs = 1.0 / sqrt(1.0 + t * t);
          sn = t * cs;
        }
      }
      pair_p[k] = p;
      pair_q[k] = q;
      pc[k] = static_cast<float>(cs);
      ps[k] = static_cast<float>(sn);
      log[static_cast<int64_t>(round) * P + k] = make_float2(pc[k], ps[k]);
    }
    __syncthreads();
    // A <- J^T A J on every 2x2 block (i <= j); blocks are disjoint.
    const int items = ((P + 1) / 2) * (P + 1);
    for (int w = threadIdx.x; w < items; w += blockDim.x) {
      int i, j;
      if (!foldedBlock(w, P, i, j)) continue;
      const int pi = pair_p[i], qi = pair_q[i], pj = pair_p[j], qj = pair_q[j];
      const float ci = pc[i], si = ps[i], cj = pc[j], sj = ps[j];
      const bool hi = qi < n, hj = qj < n;
      if (i == j) {
        if (!hi) continue;
        const int kpp = tri[pi] + pi, kqq = tri[qi] + qi, kpq = tri[qi] + pi;
        const float app = A[kpp], aqq = A[kqq], apq = A[kpq];
        // [c -s; s c]^T-free form of J^T M J for the pivot block
        const float t0 = ci * app - si * apq, t1 = ci * apq - si * aqq;
        const float u0 = si * app + ci * apq, u1 = si * apq + ci * aqq;
        A[kpp] = ci * t0 - si * t1;
        A[kqq] = si * u0 + ci * u1;
        A[kpq] = 0.0f;
        continue;
      }
      const int k00 = packedIndex(tri, pi, pj);
      const int k01 = hj ? packedIndex(tri, pi, qj) : 0;
      const int k10 = hi ? packedIndex(tri, qi, pj) : 0;
      const int k11 = hi && hj ? packedIndex(tri, qi, qj) : 0;
      const float m00 = A[k00];
      const float m01 = hj ? A[k01] : 0.0f;
      const float m10 = hi ? A[k10] : 0.0f;
      const float m11 = hi && hj ? A[k11] : 0.0f;
      // T = M J_j, J = [c s; -s c]
      const float t00 = cj * m00 - sj * m01, t01 = sj * m00 + cj * m01;
      const float t10 = cj * m10 - sj * m11, t11 = sj * m10 + cj * m11;
      // M' = J_i^T T
      A[k00] = ci * t00 - si * t10;
      if (hj) A[k01] = ci * t01 - si * t11;
      if (hi) A[k10] = si * t00 + ci * t10;
      if (hi && hj) A[k11] = si * t01 + ci * t11;
    }
    __syncthreads();
  }
  if (kSmem) {
    for (int k = threadIdx.x; k < tri_n; k += blockDim.x) packed_g[k] = A[k];
  }
  if (threadIdx.x == 0) {
    st.norm2 = norm2;
    st.off_ratio = ratio;
    st.sweeps = sweeps + 1;
    st.done = 0;
    st.logged = 1;
  }
}

struct VArgs {
  float *v;
  const int64_t *a_offset;
  const int64_t *log_offset;
  const int32_t *n;
  const float2 *log;
  const JacobiState *state;
  const int32_t *work_matrix;  // per CTA: matrix id
  const int32_t *work_row;     // per CTA: first row
  int rows_per_cta;
};

// Replays one logged sweep onto rows [r0, r0 + 32) of V (V <- V J per round,
// column p: c v_p - s v_q, column q: s v_p + c v_q, the update of
// jacobi_similarity_vectors_f32 z = 1, metal_mixed_sqrt.metal:1380-1390).
__global__ void __launch_bounds__(256)
jacobiReplayKernel(VArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mi = args.work_matrix[blockIdx.x];
  if (!args.state[mi].logged) return;
  const int r0 = args.work_row[blockIdx.x];
  const int n = args.n[mi];
  const int m = n + (n & 1);
  const int P = m / 2;
  const int kVRows = args.rows_per_cta;
  float *vs = reinterpret_cast<float *>(smem_raw);  // [m][kVRows]
  float *v = args.v + args.a_offset[mi];
  const int rows = min(kVRows, n - r0);
  for (int k = threadIdx.x; k < m * kVRows; k += blockDim.x) {
    const int c = k / kVRows, r = k % kVRows;
    vs[k] = (c < n && r < rows) ? v[r0 + r + static_cast<int64_t>(c) * n] : 0.0f;
  }
  __syncthreads();
  const float2 *log = args.log + args.log_offset[mi];
  for (int round = 0; round < m - 1; ++round) {
    for (int k = threadIdx.x; k < P * kVRows; k += blockDim.x) {
      const int pair = k / kVRows, r = k % kVRows;
      int p, q;
      rrPair(pair, round, m, p, q);
      const float2 cs = log[static_cast<int64_t>(round) * P + pair];
      const float vp = vs[p * kVRows + r], vq = vs[q * kVRows + r];
      vs[p * kVRows + r] = cs.x * vp - cs.y * vq;
      vs[q * kVRows + r] = cs.y * vp + cs.x * vq;
    }
    __syncthreads();
  }
  for (int k = threadIdx.x; k < n * kVRows; k += blockDim.x) {
    const int c = k / kVRows, r = k % kVRows;
    if (r < rows) v[r0 + r + static_cast<int64_t>(c) * n] = vs[k];
  }
}

__global__ void identityKernel(float *v, const int64_t *a_offset,
                               const int32_t *n, int count) {
  for (int mi = blockIdx.y; mi < count; mi += gridDim.y) {
    const int64_t nn = static_cast<int64_t>(n[mi]) * n[mi];
    float *out = v + a_offset[mi];
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
      const int64_t r = k % n[mi], c = k / n[mi];
      out[k] = r == c ? 1.0f : 0.0f;
    }
  }
}

__global__ void jacobiReportKernel(const JacobiState *state, int count,
                                   int32_t *sweeps, float *off_ratio) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += gridDim.x * blockDim.x) {
    if (sweeps) sweeps[i] = state[i].sweeps;
    if (off_ratio) off_ratio[i] = static_cast<float>(state[i].off_ratio);
  }
}

size_t sweepSmemBytes(int n, bool smem) {
  const int m = n + (n & 1), P = m / 2;
  size_t bytes = 32 * sizeof(double) + (m + 1 + 2 * P) * sizeof(int) + 2 * P * sizeof(float) + 64;
  if (smem) bytes += static_cast<size_t>(n) * (n + 1) / 2 * sizeof(float);
  return bytes;
}

int threadsFor(int n) {
  if (n <= 32) return 64;
  if (n <= 64) return 128;
  if (n <= 128) return 256;
  if (n <= 256) return 512;
  return 1024;
}

// Per-layout launch plan, kept with the batch layout.
struct JacobiPlan {
  uint64_t key = 0;
  int count = 0;
  int64_t packed_total = 0, log_total = 0;
  int64_t *p_offset = nullptr, *log_offset = nullptr;
  int32_t *order = nullptr;  // all ids grouped by bucket, largest first
  struct Bucket { int threads; bool smem; int first; int count; size_t smem_bytes; };
  std::vector<Bucket> buckets;
  int32_t *work_matrix = nullptr, *work_row = nullptr;
  int work_count = 0;
  size_t v_smem = 0;
  int rows_per_cta = kVRowsMax;
  int device_id = 0;
  void *device = nullptr;
};

std::vector<JacobiPlan *> g_plans;

JacobiPlan *planFor(msq_ctx *ctx, const DeviceBatch *b) {
  for (JacobiPlan *p : g_plans)
    if (p->key == b->key && p->count == b->count && p->device_id == ctx->device) return p;
  auto *plan = new JacobiPlan;
  plan->device_id = ctx->device;
  plan->key = b->key;
  plan->count = b->count;
  const int count = b->count;
  std::vector<int64_t> p_off(count), l_off(count);
  for (int i = 0; i < count; ++i) {
    const int n = b->host_n[i], m = n + (n & 1);
    p_off[i] = plan->packed_total;
    plan->packed_total += static_cast<int64_t>(n) * (n + 1) / 2;
    l_off[i] = plan->log_total;
    plan->log_total += static_cast<int64_t>(m - 1) * (m / 2);
  }
  std::vector<int32_t> ids(count);
  for (int i = 0; i < count; ++i) ids[i] = i;
  std::stable_sort(ids.begin(), ids.end(), [&](int x, int y) {
    const int tx = threadsFor(b->host_n[x]) * (b->host_n[x] <= kMaxSmemOrder ? 1 : 2);
    const int ty = threadsFor(b->host_n[y]) * (b->host_n[y] <= kMaxSmemOrder ? 1 : 2);
    if (tx != ty) return tx > ty;
    return b->host_n[x] > b->host_n[y];
  });
  for (int i = 0; i < count;) {
    const int n0 = b->host_n[ids[i]];
    const int t = threadsFor(n0);
    const bool smem = n0 <= kMaxSmemOrder;
    int j = i;
    size_t bytes = 0;
    while (j < count && threadsFor(b->host_n[ids[j]]) == t &&
           (b->host_n[ids[j]] <= kMaxSmemOrder) == smem) {
      bytes = std::max(bytes, sweepSmemBytes(b->host_n[ids[j]], smem));
      ++j;
    }
    plan->buckets.push_back({t, smem, i, j - i, bytes});
    i = j;
  }
  std::vector<int32_t> wm, wr;
  int max_m = 0;
  for (int i = 0; i < count; ++i) max_m = std::max(max_m, b->host_n[i] + (b->host_n[i] & 1));
  plan->rows_per_cta = static_cast<int>(std::max<size_t>(
      1, std::min<size_t>(kVRowsMax, kSmemLimit / (static_cast<size_t>(max_m) * sizeof(float)))));
  for (int i = 0; i < count; ++i) {
    const int n = b->host_n[ids[i]];
    for (int r = 0; r < n; r += plan->rows_per_cta) {
      wm.push_back(ids[i]);
      wr.push_back(r);
    }
  }
  plan->work_count = static_cast<int>(wm.size());
  plan->v_smem = static_cast<size_t>(max_m) * plan->rows_per_cta * sizeof(float);
  const size_t bytes = 2 * count * sizeof(int64_t) + count * sizeof(int32_t) +
                       2 * wm.size() * sizeof(int32_t) + 64;
  char *dev = nullptr;
  if (cudaCheck(ctx, cudaMalloc(&dev, bytes), "jacobi plan alloc") != MSQ_OK) {
    delete plan;
    return nullptr;
  }
  plan->device = dev;
  plan->p_offset = reinterpret_cast<int64_t *>(dev);
  plan->log_offset = plan->p_offset + count;
  plan->order = reinterpret_cast<int32_t *>(plan->log_offset + count);
  plan->work_matrix = plan->order + count;
  plan->work_row = plan->work_matrix + wm.size();
  cudaMemcpy(plan->p_offset, p_off.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->log_offset, l_off.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->order, ids.data(), count * sizeof(int32_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->work_matrix, wm.data(), wm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  cudaMemcpy(plan->work_row, wr.data(), wr.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (g_plans.size() >= 8) {
    cudaFree(g_plans.front()->device);
    delete g_plans.front();
    g_plans.erase(g_plans.begin());
  }
  g_plans.push_back(plan);
  return plan;
}

}  // namespace

// Enqueues the whole solve; `work` must hold packed + log + state.
int jacobiEnqueue(msq_ctx *ctx, const DeviceBatch *b, float *matrices,
                  float *vectors, float *eigenvalues, double tolerance,
                  int max_sweeps, int32_t *sweeps_done, float *off_ratio) {
  if (b->max_n > 8192) {
    return setError(ctx, MSQ_ERR_UNSUPPORTED, "jacobi: order above 8192");
  }
  JacobiPlan *plan = planFor(ctx, b);
  if (plan == nullptr) return MSQ_ERR_CUDA;
  const size_t state_bytes = (b->count * sizeof(JacobiState) + 255) & ~size_t(255);
  const size_t packed_bytes = (plan->packed_total * sizeof(float) + 255) & ~size_t(255);
  const size_t log_bytes = plan->log_total * sizeof(float2);
  char *work = static_cast<char *>(scratch(ctx, state_bytes + packed_bytes + log_bytes, kScratchJacobi));
  if (work == nullptr) return MSQ_ERR_CUDA;
  JacobiArgs args{};
  args.a = matrices;
  args.state = reinterpret_cast<JacobiState *>(work);
  args.packed = reinterpret_cast<float *>(work + state_bytes);
  args.log = reinterpret_cast<float2 *>(work + state_bytes + packed_bytes);
  args.a_offset = b->offset;
  args.p_offset = plan->p_offset;
  args.log_offset = plan->log_offset;
  args.eig_offset = b->eig_offset;
  args.n = b->n;
  args.eigenvalues = eigenvalues;
  args.count = b->count;
  args.tol = tolerance;
  args.max_sweeps = max_sweeps;

  static bool attributes_set = false;
  if (!attributes_set) {
    MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(jacobiSweepKernel<true>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                227 * 1024), "jacobi smem attr"));
    MSQ_TRY(cudaCheck(ctx, cudaFuncSetAttribute(jacobiReplayKernel,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                227 * 1024), "replay smem attr"));
    attributes_set = true;
  }
  MSQ_TRY(cudaCheck(ctx, cudaMemsetAsync(args.state, 0, state_bytes, ctx->stream), "state reset"));
  {
    dim3 grid(64, std::min(b->count, 65535));
    identityKernel<<<grid, 256, 0, ctx->stream>>>(vectors, b->offset, b->n, b->count);
    MSQ_TRY(launched(ctx, "jacobi identity"));
  }
  VArgs vargs{vectors, b->offset, plan->log_offset, b->n, args.log, args.state,
              plan->work_matrix, plan->work_row, plan->rows_per_cta};
  for (int launch = 0; launch <= max_sweeps; ++launch) {
    args.first = launch == 0;
    for (const auto &bucket : plan->buckets) {
      args.order = plan->order + bucket.first;
      if (bucket.smem) {
        jacobiSweepKernel<true><<<bucket.count, bucket.threads, bucket.smem_bytes, ctx->stream>>>(args);
      } else {
        jacobiSweepKernel<false><<<bucket.count, bucket.threads, bucket.smem_bytes, ctx->stream>>>(args);
      }
      MSQ_TRY(launched(ctx, "jacobi sweep"));
    }
    if (launch < max_sweeps) {
      jacobiReplayKernel<<<plan->work_count, 256, plan->v_smem, ctx->stream>>>(vargs);
      MSQ_TRY(launched(ctx, "jacobi replay"));
    }
  }
  if (sweeps_done != nullptr || off_ratio != nullptr) {
    jacobiReportKernel<<<gridFor(b->count, 256), 256, 0, ctx->stream>>>(
        args.state, b->count, sweeps_done, off_ratio);
    MSQ_TRY(launched(ctx, "jacobi report"));
  }
  return MSQ_OK;
}

}  // namespace msq

using namespace msq;

extern "C" int msq_jacobi_batched(msq_ctx *ctx, float *matrices, float *vectors,
                                  float *eigenvalues, const int32_t *n,
                                  const int64_t *offset, int count,
                                  double tolerance, int max_sweeps,
                                  int32_t *sweeps_done, float *off_ratio) {
  if (ctx == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  if (matrices == nullptr || vectors == nullptr || eigenvalues == nullptr) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT, "msq_jacobi_batched: null buffer");
  }
  if (!(tolerance >= 0.0) || max_sweeps < 0 || max_sweeps > 64) {
    return setError(ctx, MSQ_ERR_INVALID_ARGUMENT,
                    "msq_jacobi_batched: tolerance must be >= 0, max_sweeps in [0, 64]");
  }
  const DeviceBatch *b = prepareBatch(ctx, n, offset, count);
  if (b == nullptr) return MSQ_ERR_INVALID_ARGUMENT;
  return jacobiEnqueue(ctx, b, matrices, vectors, eigenvalues, tolerance,
                       max_sweeps, sweeps_done, off_ratio);
}
