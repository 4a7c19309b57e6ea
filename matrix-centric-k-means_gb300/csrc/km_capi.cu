// C ABI of libkm_sm103 (include/km.h).  Host orchestration only: validation,
// seeded initialisation, CUDA-graph capture of the iteration and the
// device-side stop flag; all arithmetic runs in the kernels.
#include "km_lloyd.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <unordered_set>
#include <vector>

namespace km {
const char* last_error_text();
__global__ void gather_rows_kernel(const float* X, uint32_t d, const int32_t* idx, uint32_t m,
                                   float* out);
__global__ void round_robin_labels_kernel(uint32_t* labels, uint64_t n, uint32_t k);
}  // namespace km

using namespace km;

namespace km {

__global__ void gather_rows_kernel(const float* __restrict__ X, uint32_t d,
                                   const int32_t* __restrict__ idx, uint32_t m,
                                   float* __restrict__ out) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)m * d) return;
  const uint32_t r = (uint32_t)(t / d), j = (uint32_t)(t % d);
  out[t] = X[(uint64_t)idx[r] * d + j];
}

__global__ void round_robin_labels_kernel(uint32_t* labels, uint64_t n, uint32_t k) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) labels[i] = (uint32_t)(i % k);
}

namespace {

uint64_t count_kernel_nodes(cudaGraph_t g) {
  size_t nn = 0;
  if (cudaGraphGetNodes(g, nullptr, &nn) != cudaSuccess) { (void)cudaGetLastError(); return 0; }
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn && cudaGraphGetNodes(g, nodes.data(), &nn) != cudaSuccess) { (void)cudaGetLastError(); return 0; }
  uint64_t c = 0;
  for (cudaGraphNode_t v : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(v, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++c;
  }
  return c;
}

// Seeded sample picks exactly as the reference CPU k-means draws them
// (comparisons/CPU_Kmeans/src/kmeans.cpp:22-29, :49-84): mt19937(seed_seq{seed}),
// uniform_int_distribution<int>(0, n-1), points equal by value to an earlier
// pick are skipped (Point::operator==, src/include/point.hpp:64-70).  Candidate
// rows are fetched from the device in batches; equality is float '=='
// (NaN cannot occur: inputs are checked), hashed on the bit pattern with -0
// folded into +0.
struct RowKey {
  std::string bytes;
  bool operator==(const RowKey& o) const { return bytes == o.bytes; }
};
struct RowKeyHash {
  size_t operator()(const RowKey& r) const { return std::hash<std::string>()(r.bytes); }
};

km_status sample_init(LloydEngine& e, int seed) {
  std::seed_seq ss{seed};
  std::mt19937 gen(ss);
  std::uniform_int_distribution<int> dist(0, (int)(e.n - 1));
  std::unordered_set<RowKey, RowKeyHash> seen;
  std::vector<float> accepted;
  accepted.reserve((size_t)e.k * e.d);
  uint32_t have = 0;
  uint64_t draws = 0;
  const uint64_t max_draws = 1000ull * (e.k + 16) + 100000ull;
  int32_t* d_idx = nullptr;
  float* d_rows = nullptr;
  const uint32_t cap = std::max<uint32_t>(64, 2 * e.k + 16);
  if (cudaMalloc(&d_idx, sizeof(int32_t) * cap) != cudaSuccess ||
      cudaMalloc(&d_rows, sizeof(float) * (size_t)cap * e.d) != cudaSuccess) {
    (void)cudaGetLastError();
    if (d_idx) cudaFree(d_idx);
    return KM_ERR_ALLOC;
  }
  std::vector<int32_t> cand;
  std::vector<float> rows;
  km_status rc = KM_OK;
  while (have < e.k) {
    if (draws > max_draws) { rc = KM_ERR_ARG; break; }  // fewer than k distinct points
    const uint32_t m = std::min<uint32_t>(cap, 2 * (e.k - have) + 16);
    cand.resize(m);
    for (uint32_t i = 0; i < m; ++i) cand[i] = dist(gen);
    draws += m;
    rows.resize((size_t)m * e.d);
    if (cudaMemcpyAsync(d_idx, cand.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, e.stream) != cudaSuccess) { rc = KM_ERR_CUDA; break; }
    gather_rows_kernel<<<(unsigned)(((uint64_t)m * e.d + 255) / 256), 256, 0, e.stream>>>(e.X, e.d, d_idx, m, d_rows);
    if (cudaMemcpyAsync(rows.data(), d_rows, sizeof(float) * m * e.d, cudaMemcpyDeviceToHost, e.stream) != cudaSuccess ||
        cudaStreamSynchronize(e.stream) != cudaSuccess) { rc = KM_ERR_CUDA; break; }
    for (uint32_t i = 0; i < m && have < e.k; ++i) {
      const float* r = rows.data() + (size_t)i * e.d;
      RowKey key;
      key.bytes.resize(sizeof(float) * e.d);
      float* kb = reinterpret_cast<float*>(&key.bytes[0]);
      for (uint32_t j = 0; j < e.d; ++j) kb[j] = (r[j] == 0.0f) ? 0.0f : r[j];
      if (seen.insert(std::move(key)).second) {
        accepted.insert(accepted.end(), r, r + e.d);
        ++have;
      }
    }
  }
  if (rc == KM_OK) {
    if (cudaMemcpyAsync(e.C, accepted.data(), sizeof(float) * e.k * e.d, cudaMemcpyHostToDevice, e.stream) != cudaSuccess ||
        cudaStreamSynchronize(e.stream) != cudaSuccess)
      rc = KM_ERR_CUDA;
  }
  cudaFree(d_idx);
  cudaFree(d_rows);
  return rc;
}

// Initial centroids as exact means of the groups i % k (reference GPU path
// labels, src/kmeans.cu:365-374).
km_status round_robin_init(LloydEngine& e) {
  round_robin_labels_kernel<<<(unsigned)((e.n + 255) / 256), 256, 0, e.stream>>>(e.labels, e.n, e.k);
  KM_TRY(e.enqueue_sort(e.labels));
  return launch_update_sums(e.X, e.perm, e.cstart, e.d, e.k, nullptr, e.C, nullptr, nullptr, e.st,
                            e.stream);
}

}  // namespace
}  // namespace km

struct km_lloyd;
static km_status run_init(km_lloyd* h, const float* C0);

struct km_lloyd {
  km_lloyd_params p;
  LloydEngine eng;
  cudaGraphExec_t graph = nullptr;
  LoopConsts graph_lc{};
  int graph_iters = 0;
  uint64_t graph_kernels = 0;     // kernel nodes in one replay of `graph`
  int32_t* h_done = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

// Resets the loop state and places the initial centroids in e.C.
static km_status run_init(km_lloyd* h, const float* C0) {
  LloydEngine& e = h->eng;
  KM_TRY(e.reset_state());
  switch (h->p.init) {
    case KM_INIT_SAMPLE: KM_TRY(sample_init(e, h->p.seed)); break;
    case KM_INIT_ROUND_ROBIN: KM_TRY(round_robin_init(e)); break;
    case KM_INIT_PLUSPLUS: KM_TRY(plusplus_init(e, h->p.seed)); break;
    case KM_INIT_GIVEN:
      if (!C0) return KM_ERR_ARG;
      KM_CUDA_TRY(cudaMemcpyAsync(e.C, C0, sizeof(float) * e.k * e.d, cudaMemcpyHostToDevice, e.stream));
      break;
    default: return KM_ERR_ARG;
  }
  return e.set_centroids_dev(e.C);
}

extern "C" {

const char* km_status_str(km_status s) {
  switch (s) {
    case KM_OK: return "ok";
    case KM_ERR_ARG: return "invalid argument";
    case KM_ERR_ALLOC: return "allocation failed";
    case KM_ERR_CUDA: return last_error_text()[0] ? last_error_text() : "CUDA error";
    case KM_ERR_TIMEOUT: return "device wait timed out";
    case KM_ERR_UNSUPPORTED: return "unsupported shape/precision";
    case KM_ERR_NO_DEVICE: return "no sm_103 CUDA device";
    case KM_ERR_STATE: return "call out of order";
  }
  return "unknown status";
}

const char* km_version(void) { return "libkm_sm103 0.1 (sm_103a)"; }

int km_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { (void)cudaGetLastError(); return 0; }
  int c = 0;
  for (int i = 0; i < n; ++i) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, i) == cudaSuccess && p.major == 10 && p.minor == 3) ++c;
  }
  return c;
}

km_status km_lloyd_create(const km_lloyd_params* p, km_lloyd** out) {
  if (!p || !out) return KM_ERR_ARG;
  *out = nullptr;
  if (p->init < KM_INIT_SAMPLE || p->init > KM_INIT_PLUSPLUS) return KM_ERR_ARG;
  if (p->conv < KM_CONV_SHIFT || p->conv > KM_CONV_NONE) return KM_ERR_ARG;
  if (p->empty != KM_EMPTY_ZERO && p->empty != KM_EMPTY_EXCLUDE) return KM_ERR_ARG;
  if (!(p->tol >= 0.0f) || p->maxiter == 0) return KM_ERR_ARG;
  km_lloyd* h = new (std::nothrow) km_lloyd();
  if (!h) return KM_ERR_ALLOC;
  h->p = *p;
  km_status s = h->eng.init(p->n, p->d, p->k, p->precision, p->device, p->stream, true);
  if (s == KM_OK && cudaMallocHost(reinterpret_cast<void**>(&h->h_done), sizeof(int32_t)) != cudaSuccess) s = KM_ERR_ALLOC;
  if (s == KM_OK && (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)) s = KM_ERR_CUDA;
  if (s != KM_OK) { km_lloyd_destroy(h); return s; }
  *out = h;
  return KM_OK;
}

km_status km_mem_info(int32_t device, uint64_t* free_bytes, uint64_t* total_bytes) {
  if (!free_bytes || !total_bytes) return KM_ERR_ARG;
  if (km_device_count() == 0) return KM_ERR_NO_DEVICE;
  KM_CUDA_TRY(cudaSetDevice(device));
  size_t f = 0, t = 0;
  KM_CUDA_TRY(cudaMemGetInfo(&f, &t));
  *free_bytes = f;
  *total_bytes = t;
  return KM_OK;
}

km_status km_lloyd_init(km_lloyd* h, const float* C0, float* centroids_out) {
  if (!h || !centroids_out) return KM_ERR_ARG;
  LloydEngine& e = h->eng;
  if (!e.data_ready) return KM_ERR_STATE;
  KM_CUDA_TRY(cudaSetDevice(e.device));
  KM_TRY(run_init(h, C0));
  KM_CUDA_TRY(cudaMemcpyAsync(centroids_out, e.C, sizeof(float) * e.k * e.d, cudaMemcpyDeviceToHost, e.stream));
  KM_CUDA_TRY(cudaStreamSynchronize(e.stream));
  return e.check_device_error();
}

km_status km_lloyd_configure(km_lloyd* h, uint64_t maxiter, float tol, int32_t conv) {
  if (!h || maxiter == 0 || !(tol >= 0.0f) || conv < KM_CONV_SHIFT || conv > KM_CONV_NONE) return KM_ERR_ARG;
  h->p.maxiter = maxiter;
  h->p.tol = tol;
  h->p.conv = conv;
  return KM_OK;
}

km_status km_lloyd_set_data_bf16(km_lloyd* h, const uint16_t* X, int on_device) {
  if (!h || !X) return KM_ERR_ARG;
  return h->eng.set_points_bf16(X, on_device != 0);
}

km_status km_lloyd_set_data(km_lloyd* h, const float* X, int on_device) {
  if (!h || !X) return KM_ERR_ARG;
  return h->eng.set_points(X, on_device != 0, true);
}

km_status km_lloyd_fit(km_lloyd* h, const float* C0, uint32_t* labels_out, float* centroids_out,
                       km_result* res) {
  if (!h) return KM_ERR_ARG;
  LloydEngine& e = h->eng;
  if (!e.data_ready) return KM_ERR_STATE;
  KM_CUDA_TRY(cudaSetDevice(e.device));
  KM_TRY(run_init(h, C0));

  LoopConsts lc{h->p.maxiter, h->p.tol, h->p.conv, h->p.empty};
  // One captured graph = G iterations; relaunched until the device says done.
  const int G = (int)std::min<uint64_t>(h->p.maxiter, h->p.conv == KM_CONV_NONE ? 8 : 2);
  if (!h->graph || h->graph_iters != G || h->graph_lc.maxiter != lc.maxiter ||
      h->graph_lc.tol != lc.tol || h->graph_lc.conv != lc.conv || h->graph_lc.empty != lc.empty) {
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    cudaGraph_t g = nullptr;
    KM_CUDA_TRY(cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal));
    km_status cs = KM_OK;
    for (int i = 0; i < G && cs == KM_OK; ++i) cs = e.enqueue_iteration(lc);
    cudaError_t ce = cudaStreamEndCapture(e.stream, &g);
    if (cs != KM_OK) { if (g) cudaGraphDestroy(g); return cs; }
    KM_CUDA_TRY(ce);
    h->graph_kernels = count_kernel_nodes(g);
    cudaError_t ie = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    KM_CUDA_TRY(ie);
    h->graph_lc = lc;
    h->graph_iters = G;
  }
  KM_CUDA_TRY(cudaEventRecord(h->ev0, e.stream));
  uint64_t launched = 0, replays = 0;
  uint64_t batch = (h->p.conv == KM_CONV_NONE) ? h->p.maxiter : 4;
  while (launched < h->p.maxiter) {
    const uint64_t target = std::min<uint64_t>(h->p.maxiter, launched + batch);
    while (launched < target) {
      KM_CUDA_TRY(cudaGraphLaunch(h->graph, e.stream));
      launched += (uint64_t)G;
      ++replays;
    }
    if (launched >= h->p.maxiter) break;
    KM_CUDA_TRY(cudaMemcpyAsync(h->h_done, &e.st->done, sizeof(int32_t), cudaMemcpyDeviceToHost, e.stream));
    KM_CUDA_TRY(cudaStreamSynchronize(e.stream));
    if (*h->h_done) break;
    batch = std::min<uint64_t>(batch * 2, 64);
  }
  KM_CUDA_TRY(cudaEventRecord(h->ev1, e.stream));
  KM_TRY(e.check_device_error());
  float ms = 0.0f;
  KM_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  const DevState& s = *e.h_st;
  if (labels_out)
    KM_CUDA_TRY(cudaMemcpyAsync(labels_out, e.labels, sizeof(uint32_t) * e.n, cudaMemcpyDeviceToHost, e.stream));
  if (centroids_out)
    KM_CUDA_TRY(cudaMemcpyAsync(centroids_out, e.C, sizeof(float) * e.k * e.d, cudaMemcpyDeviceToHost, e.stream));
  KM_CUDA_TRY(cudaStreamSynchronize(e.stream));
  if (res) {
    std::memset(res, 0, sizeof(*res));
    res->iterations = s.iter;
    res->converged = s.converged_iter != 0;
    res->converged_iter = s.converged_iter ? s.converged_iter : h->p.maxiter;
    res->objective = s.objective;
    res->score = s.score;
    res->max_shift = s.max_shift;
    res->refined_rows = s.refined_total;
    res->full_rescore_rows = s.full_total;
    res->fit_ms = ms;
    res->kernel_launches = replays * h->graph_kernels;
  }
  return KM_OK;
}

km_status km_lloyd_device_results(km_lloyd* h, const uint32_t** labels_dev, const float** centroids_dev,
                                  const uint32_t** counts_dev) {
  if (!h) return KM_ERR_ARG;
  if (labels_dev) *labels_dev = h->eng.labels;
  if (centroids_dev) *centroids_dev = h->eng.C;
  if (counts_dev) *counts_dev = h->eng.counts;
  return KM_OK;
}

km_status km_lloyd_profile(km_lloyd* h, uint64_t iters, double* stage_ms) {
  if (!h || !stage_ms || iters == 0) return KM_ERR_ARG;
  LloydEngine& e = h->eng;
  if (!e.data_ready) return KM_ERR_STATE;
  KM_CUDA_TRY(cudaSetDevice(e.device));
  // Clear the stop flag and the iteration budget so that the stages run.
  KM_TRY(e.read_state());
  e.h_st->done = 0;
  e.h_st->iter = 0;
  e.h_st->fin_ticket = 0;
  e.h_st->scan_ticket = 0;
  KM_CUDA_TRY(cudaMemcpyAsync(e.st, e.h_st, sizeof(DevState), cudaMemcpyHostToDevice, e.stream));
  LoopConsts lc{~0ull, h->p.tol, KM_CONV_NONE, h->p.empty};
  cudaEvent_t ev[6];
  for (auto& x : ev) KM_CUDA_TRY(cudaEventCreate(&x));
  // One iteration captured as a graph (the same kernels as the fit's graph)
  // with event-record nodes between the stages; each replay is one iteration.
  auto enqueue = [&](bool external) -> km_status {
    const unsigned fl = external ? cudaEventRecordExternal : 0u;
    km_status r = KM_OK;
    cudaEventRecordWithFlags(ev[0], e.stream, fl);
    r = e.enqueue_distance(nullptr);
    cudaEventRecordWithFlags(ev[1], e.stream, fl);
    if (r == KM_OK) r = e.enqueue_refine();
    cudaEventRecordWithFlags(ev[2], e.stream, fl);
    if (r == KM_OK) r = e.enqueue_sort(e.labels);
    cudaEventRecordWithFlags(ev[3], e.stream, fl);
    if (r == KM_OK) r = e.enqueue_update_step(h->p.tol);
    cudaEventRecordWithFlags(ev[4], e.stream, fl);
    if (r == KM_OK) r = e.enqueue_finalize(lc);
    cudaEventRecordWithFlags(ev[5], e.stream, fl);
    return r;
  };
  cudaGraphExec_t gx = nullptr;
  {
    cudaGraph_t g = nullptr;
    km_status cs = KM_ERR_CUDA;
    if (cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      cs = enqueue(true);
      if (cudaStreamEndCapture(e.stream, &g) != cudaSuccess) cs = KM_ERR_CUDA;
    }
    if (cs == KM_OK && g && cudaGraphInstantiate(&gx, g, 0) != cudaSuccess) gx = nullptr;
    if (g) cudaGraphDestroy(g);
    (void)cudaGetLastError();   // no graph: the stages are launched directly below
  }
  double acc[5] = {0, 0, 0, 0, 0};
  km_status rc = KM_OK;
  for (uint64_t it = 0; it < iters && rc == KM_OK; ++it) {
    if (gx) {
      if (cudaGraphLaunch(gx, e.stream) != cudaSuccess) { rc = KM_ERR_CUDA; break; }
    } else {
      rc = enqueue(false);
    }
    if (cudaEventSynchronize(ev[5]) != cudaSuccess) { rc = KM_ERR_CUDA; break; }
    for (int s = 0; s < 5; ++s) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[s], ev[s + 1]);
      acc[s] += ms;
    }
  }
  if (gx) cudaGraphExecDestroy(gx);
  for (auto& x : ev) cudaEventDestroy(x);
  KM_TRY(rc);
  KM_TRY(e.check_device_error());
  for (int s = 0; s < 5; ++s) stage_ms[s] = acc[s] / (double)iters;
  return KM_OK;
}

void km_lloyd_destroy(km_lloyd* h) {
  if (!h) return;
  if (h->eng.device >= 0) cudaSetDevice(h->eng.device);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->h_done) cudaFreeHost(h->h_done);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  delete h;
}

static km_status current_device(int* dev) {
  if (cudaGetDevice(dev) != cudaSuccess) { (void)cudaGetLastError(); return KM_ERR_NO_DEVICE; }
  return KM_OK;
}

km_status km_assign(const float* X_dev, const float* C_dev, uint64_t n, uint32_t d, uint32_t k,
                    int32_t precision, uint32_t* labels_dev, float* mindist_dev,
                    uint64_t* refined_rows, void* stream) {
  if (!X_dev || !C_dev || !labels_dev) return KM_ERR_ARG;
  int dev;
  KM_TRY(current_device(&dev));
  LloydEngine e;
  KM_TRY(e.init(n, d, k, precision, dev, stream, false));
  KM_TRY(e.set_points(X_dev, true, false));
  KM_TRY(e.set_centroids_dev(C_dev));
  KM_TRY(e.enqueue_assign(nullptr));
  KM_CUDA_TRY(cudaMemcpyAsync(labels_dev, e.labels, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, e.stream));
  if (mindist_dev)
    KM_CUDA_TRY(cudaMemcpyAsync(mindist_dev, e.mindist, sizeof(float) * n, cudaMemcpyDeviceToDevice, e.stream));
  KM_TRY(e.check_device_error());
  if (refined_rows) *refined_rows = e.h_st->refined_total;
  return KM_OK;
}

km_status km_distances(const float* X_dev, const float* C_dev, uint64_t n, uint32_t d, uint32_t k,
                       int32_t precision, float* D_dev, void* stream) {
  if (!X_dev || !C_dev || !D_dev) return KM_ERR_ARG;
  int dev;
  KM_TRY(current_device(&dev));
  LloydEngine e;
  KM_TRY(e.init(n, d, k, precision, dev, stream, false));
  KM_TRY(e.set_points(X_dev, true, false));
  KM_TRY(e.set_centroids_dev(C_dev));
  KM_TRY(e.enqueue_assign(D_dev));
  return e.check_device_error();
}

km_status km_update(const float* X_dev, const uint32_t* labels_dev, uint64_t n, uint32_t d, uint32_t k,
                    float* C_dev, uint32_t* counts_dev, uint32_t* perm_dev, uint32_t* offsets_dev,
                    void* stream) {
  if (!X_dev || !labels_dev || !C_dev) return KM_ERR_ARG;
  int dev;
  KM_TRY(current_device(&dev));
  LloydEngine e;
  KM_TRY(e.init(n, d, k, KM_PREC_FP32, dev, stream, true));
  e.X = X_dev;
  KM_TRY(e.enqueue_sort(labels_dev));
  KM_TRY(e.check_device_error());   // labels >= k are rejected before the sums run
  KM_TRY(launch_update_sums(X_dev, e.perm, e.cstart, d, k, nullptr, C_dev, nullptr, nullptr, e.st,
                            e.stream));
  if (counts_dev) KM_CUDA_TRY(cudaMemcpyAsync(counts_dev, e.counts, sizeof(uint32_t) * k, cudaMemcpyDeviceToDevice, e.stream));
  if (perm_dev) KM_CUDA_TRY(cudaMemcpyAsync(perm_dev, e.perm, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, e.stream));
  if (offsets_dev) KM_CUDA_TRY(cudaMemcpyAsync(offsets_dev, e.cstart, sizeof(uint32_t) * (k + 1), cudaMemcpyDeviceToDevice, e.stream));
  return e.check_device_error();
}

}  // extern "C"
