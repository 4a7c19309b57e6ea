// Batched Lloyd k-means: many independent problems of uneven n, d, k, each
// with several seeded restarts, in ONE persistent kernel launch.
//
// Every restart of every problem is an "instance".  A CTA takes the next
// instance from a work counter (instances are ordered largest first, so the
// long ones start early) and runs the reference CPU algorithm on it to the
// end, iterations included, without leaving the kernel:
//   assign   each thread owns rows; distances by the CPU formula
//            sum_j fl((x_j - c_j)^2) in column order (exact, no bound or
//            refinement needed), strict '<' over centroids in ascending order
//            (comparisons/CPU_Kmeans/src/kmeans.cpp:86-129);
//   sort     counts in shared memory and a stable counting sort of the rows by
//            label (chunks of blockDim rows, warp match + per-warp counts);
//   update   one thread per (cluster, column): sum of the cluster's rows in row
//            order, then scale by float(1/(double)max(count,1)) (kmeans.cpp:131-155);
//   stop     from the second iteration, every centroid moved <= tol (float
//            sqrt of the column-ordered sum of squares, kmeans.cpp:170-200).
// The centroids live in shared memory (transposed, d x kpad) for the whole
// instance; X, the labels and the per-CTA scratch (permutation, next
// centroids) are in global memory.  Initial centroids are the reference's
// seeded sample picks, drawn on the host (std::mt19937 as the reference does).
//
// Tile shape: each thread computes CG centroids at a time for its row (CG in
// {8, 16, 32}) with NT threads per CTA (128 or 256); the pair is chosen by
// timing the candidates on a sample of the instances (km_batch_fit).
#include "km_lloyd.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace km {

struct BatchInst {
  uint64_t xoff;      // floats: first coordinate of the problem's points
  uint64_t loff;      // uint32: first label of this instance
  uint64_t coff;      // floats: first centroid value of this instance (k*d)
  uint32_t n, d, k, kpad;
  uint32_t prob, restart;
};

struct BatchOut {
  uint64_t converged_iter;
  uint64_t iterations;
  double objective;   // FP64 sum of the final assignment's (FP32 CPU-formula) distances
};

constexpr uint32_t BATCH_MAX_SMEM_C = 160u * 1024u;

namespace {

__device__ __forceinline__ float f_inf_b() { return __int_as_float(0x7f800000); }

template <int NT, int CG>
__global__ void __launch_bounds__(NT)
batch_lloyd_kernel(const float* __restrict__ X, const BatchInst* __restrict__ insts, uint32_t ninst,
                   const float* __restrict__ C0, float* __restrict__ Cout,
                   uint32_t* __restrict__ labels_all, uint32_t* __restrict__ perm_scratch,
                   float* __restrict__ cnew_scratch, uint64_t perm_stride, uint64_t cnew_stride,
                   uint32_t* __restrict__ next, float tol, uint64_t maxiter, BatchOut* __restrict__ out) {
  constexpr int NW = NT / 32;
  extern __shared__ float Cs[];                          // d x kpad, transposed centroids
  __shared__ uint32_t cnt[256], cstart[257], running[256];
  __shared__ uint32_t wcnt[NW][256];
  __shared__ uint32_t s_inst;
  __shared__ int s_moved;
  __shared__ double s_obj[NW];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t* perm = perm_scratch + (uint64_t)blockIdx.x * perm_stride;
  float* Cn = cnew_scratch + (uint64_t)blockIdx.x * cnew_stride;

  for (;;) {
    if (tid == 0) s_inst = atomicAdd(next, 1u);
    __syncthreads();
    const uint32_t ii = s_inst;
    __syncthreads();
    if (ii >= ninst) break;
    const BatchInst I = insts[ii];
    const uint32_t n = I.n, d = I.d, k = I.k, kpad = I.kpad;
    const float* Xp = X + I.xoff;
    uint32_t* lab = labels_all + I.loff;
    // initial centroids, transposed
    for (uint32_t q = tid; q < d * kpad; q += NT) {
      const uint32_t j = q / kpad, c = q % kpad;
      Cs[q] = (c < k) ? C0[I.coff + (uint64_t)c * d + j] : 0.0f;
    }
    for (uint32_t q = tid; q < NW * 256u; q += NT) (&wcnt[0][0])[q] = 0u;
    __syncthreads();
    uint64_t converged = maxiter, iter = 0;
    double obj = 0.0;
    while (iter++ < maxiter) {
      // ---- assign (reference CPU distance and argmin) ----
      double myobj = 0.0;
      for (uint32_t row = tid; row < n; row += NT) {
        const float* x = Xp + (uint64_t)row * d;
        float best = f_inf_b();
        uint32_t bi = 0;
        for (uint32_t g = 0; g < kpad; g += CG) {
          float acc[CG];
#pragma unroll
          for (int c = 0; c < CG; ++c) acc[c] = 0.0f;
          for (uint32_t j = 0; j < d; ++j) {
            const float xj = __ldg(x + j);
            const float4* cs4 = reinterpret_cast<const float4*>(Cs + (uint64_t)j * kpad + g);
#pragma unroll
            for (int c4 = 0; c4 < CG / 4; ++c4) {
              const float4 cc = cs4[c4];
              float t;
              t = __fsub_rn(xj, cc.x); acc[4 * c4 + 0] = __fadd_rn(acc[4 * c4 + 0], __fmul_rn(t, t));
              t = __fsub_rn(xj, cc.y); acc[4 * c4 + 1] = __fadd_rn(acc[4 * c4 + 1], __fmul_rn(t, t));
              t = __fsub_rn(xj, cc.z); acc[4 * c4 + 2] = __fadd_rn(acc[4 * c4 + 2], __fmul_rn(t, t));
              t = __fsub_rn(xj, cc.w); acc[4 * c4 + 3] = __fadd_rn(acc[4 * c4 + 3], __fmul_rn(t, t));
            }
          }
#pragma unroll
          for (int c = 0; c < CG; ++c)
            if (g + c < k && acc[c] < best) { best = acc[c]; bi = g + c; }
        }
        lab[row] = bi;
        myobj += (double)best;
      }
      for (int o = 16; o > 0; o >>= 1) myobj += __shfl_xor_sync(0xffffffffu, myobj, o);
      if (lane == 0) s_obj[warp] = myobj;
      for (uint32_t c = tid; c < k; c += NT) { cnt[c] = 0; running[c] = 0; }
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < NW; ++w) t += s_obj[w];
        obj = t;
      }
      // ---- counts and exclusive scan ----
      for (uint32_t row = tid; row < n; row += NT) atomicAdd(&cnt[lab[row]], 1u);
      __syncthreads();
      if (tid == 0) {
        uint32_t s = 0;
        for (uint32_t c = 0; c < k; ++c) { cstart[c] = s; s += cnt[c]; }
        cstart[k] = s;
      }
      __syncthreads();
      // ---- stable scatter: chunks of NT rows in order ----
      for (uint32_t base = 0; base < n; base += NT) {
        const uint32_t row = base + tid;
        const bool valid = row < n;
        const uint32_t L = valid ? lab[row] : 0xffffffffu;
        const unsigned same = __match_any_sync(0xffffffffu, L);
        const uint32_t rank = (uint32_t)__popc(same & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][L] = (uint32_t)__popc(same);
        __syncthreads();
        if (valid) {
          uint32_t before = 0;
          for (int w = 0; w < warp; ++w) {
            // a warp that had no row with label L left wcnt[w][L] at zero
            before += wcnt[w][L];
          }
          perm[cstart[L] + running[L] + before + rank] = row;
        }
        __syncthreads();
        for (uint32_t c = tid; c < k; c += NT) {
          uint32_t t = 0;
          for (int w = 0; w < NW; ++w) { t += wcnt[w][c]; wcnt[w][c] = 0; }
          running[c] += t;
        }
        __syncthreads();
      }
      // ---- update: ordered sums per (cluster, column) ----
      for (uint32_t q = tid; q < k * d; q += NT) {
        const uint32_t c = q / d, j = q % d;
        const uint32_t p0 = cstart[c], p1 = cstart[c + 1];
        float s = 0.0f;
        uint32_t p = p0;
        for (; p + 4 <= p1; p += 4) {
          const float v0 = __ldg(Xp + (uint64_t)perm[p] * d + j);
          const float v1 = __ldg(Xp + (uint64_t)perm[p + 1] * d + j);
          const float v2 = __ldg(Xp + (uint64_t)perm[p + 2] * d + j);
          const float v3 = __ldg(Xp + (uint64_t)perm[p + 3] * d + j);
          s = __fadd_rn(s, v0); s = __fadd_rn(s, v1); s = __fadd_rn(s, v2); s = __fadd_rn(s, v3);
        }
        for (; p < p1; ++p) s = __fadd_rn(s, __ldg(Xp + (uint64_t)perm[p] * d + j));
        const uint32_t count = (p1 - p0) > 1u ? (p1 - p0) : 1u;
        const float scale = (float)(1.0 / (double)count);
        Cn[q] = __fmul_rn(s, scale);
      }
      if (tid == 0) s_moved = 0;
      __syncthreads();
      // ---- stop rule (from the second iteration) and centroid swap ----
      if (iter > 1) {
        for (uint32_t c = tid; c < k; c += NT) {
          float s = 0.0f;
          for (uint32_t j = 0; j < d; ++j) {
            const float t = __fsub_rn(Cn[(uint64_t)c * d + j], Cs[(uint64_t)j * kpad + c]);
            s = __fadd_rn(s, __fmul_rn(t, t));
          }
          if (sqrtf(s) > tol) s_moved = 1;
        }
      }
      __syncthreads();
      const bool stop = iter > 1 && s_moved == 0;
      for (uint32_t q = tid; q < k * d; q += NT) {
        const uint32_t c = q / d, j = q % d;
        Cs[(uint64_t)j * kpad + c] = Cn[q];
      }
      __syncthreads();
      if (stop) { converged = iter; break; }
    }
    if (iter > maxiter) iter = maxiter;
    // results
    for (uint32_t q = tid; q < k * d; q += NT) {
      const uint32_t c = q / d, j = q % d;
      Cout[I.coff + q] = Cs[(uint64_t)j * kpad + c];
    }
    if (tid == 0) {
      out[ii].converged_iter = converged;
      out[ii].iterations = iter;
      out[ii].objective = obj;
    }
    __syncthreads();
  }
}

// Reference sample picks (kmeans.cpp:22-29, :49-84) on the host copy of X.
bool host_sample_picks(const float* X, uint64_t n, uint32_t d, uint32_t k, int seed, int32_t* picks) {
  std::seed_seq ss{seed};
  std::mt19937 gen(ss);
  std::uniform_int_distribution<int> dist(0, (int)(n - 1));
  uint32_t have = 0;
  uint64_t guard = 0;
  while (have < k) {
    if (++guard > 1000ull * (k + 16) + 100000ull) return false;
    const int p = dist(gen);
    bool found = false;
    for (uint32_t q = 0; q < have && !found; ++q) {
      bool eq = true;
      for (uint32_t j = 0; j < d && eq; ++j) eq = X[(uint64_t)picks[q] * d + j] == X[(uint64_t)p * d + j];
      found = eq;
    }
    if (!found) picks[have++] = p;
  }
  return true;
}

using BatchKernel = void (*)(const float*, const BatchInst*, uint32_t, const float*, float*, uint32_t*,
                             uint32_t*, float*, uint64_t, uint64_t, uint32_t*, float, uint64_t, BatchOut*);

struct BatchVariant {
  BatchKernel fn;
  int nt, cg;
};

const BatchVariant kVariants[] = {
    {batch_lloyd_kernel<128, 8>, 128, 8},   {batch_lloyd_kernel<128, 16>, 128, 16},
    {batch_lloyd_kernel<128, 32>, 128, 32}, {batch_lloyd_kernel<256, 8>, 256, 8},
    {batch_lloyd_kernel<256, 16>, 256, 16}, {batch_lloyd_kernel<256, 32>, 256, 32},
};

}  // namespace
}  // namespace km

using namespace km;

struct km_batch {
  km_batch_params p;
  std::vector<km_batch_problem> probs;
  std::vector<BatchInst> inst;          // LPT order
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uint64_t x_floats = 0, lab_total = 0, c_total = 0, max_n = 0, max_kd = 0;
  size_t smem = 0;
  float* X = nullptr;
  float* C0 = nullptr;
  float* Cout = nullptr;
  uint32_t* labels = nullptr;
  uint32_t* perm = nullptr;
  float* cnew = nullptr;
  BatchInst* dinst = nullptr;
  BatchOut* dout = nullptr;
  uint32_t* next = nullptr;
  int variant = -1;
  double tune_ms[6] = {0, 0, 0, 0, 0, 0};
  bool ready = false;
  ~km_batch() {
    if (device >= 0) cudaSetDevice(device);
    for (void* q : {(void*)X, (void*)C0, (void*)Cout, (void*)labels, (void*)perm, (void*)cnew, (void*)dinst,
                    (void*)dout, (void*)next})
      if (q) cudaFree(q);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};

namespace {

template <typename T>
km_status balloc(T** p, size_t count) {
  if (cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) {
    (void)cudaGetLastError();
    return KM_ERR_ALLOC;
  }
  return KM_OK;
}

// One launch of the persistent kernel over instances [0, ninst) of dinst.
km_status run_batch(km_batch* h, int v, const BatchInst* dinst, uint32_t ninst, uint64_t maxiter,
                    float* ms_out) {
  const BatchVariant& V = kVariants[v];
  const uint64_t perm_stride = (h->max_n + 31) / 32 * 32, cnew_stride = (h->max_kd + 31) / 32 * 32;
  KM_CUDA_TRY(cudaMemsetAsync(h->next, 0, sizeof(uint32_t), h->stream));
  cudaEvent_t e0, e1;
  KM_CUDA_TRY(cudaEventCreate(&e0));
  KM_CUDA_TRY(cudaEventCreate(&e1));
  KM_CUDA_TRY(cudaEventRecord(e0, h->stream));
  V.fn<<<h->num_sms, V.nt, h->smem, h->stream>>>(h->X, dinst, ninst, h->C0, h->Cout, h->labels, h->perm,
                                                  h->cnew, perm_stride, cnew_stride, h->next, h->p.tol,
                                                  maxiter, h->dout);
  cudaError_t le = cudaGetLastError();
  KM_CUDA_TRY(cudaEventRecord(e1, h->stream));
  KM_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  KM_CUDA_TRY(le);
  if (ms_out) *ms_out = ms;
  return KM_OK;
}

}  // namespace

extern "C" {

km_status km_batch_create(const km_batch_params* p, const km_batch_problem* probs, km_batch** out) {
  if (!p || !probs || !out || p->problems == 0 || p->restarts == 0 || p->maxiter == 0 || !(p->tol >= 0.0f))
    return KM_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { (void)cudaGetLastError(); return KM_ERR_NO_DEVICE; }
  km_batch* h = new (std::nothrow) km_batch();
  if (!h) return KM_ERR_ALLOC;
  h->p = *p;
  h->device = p->device;
  h->probs.assign(probs, probs + p->problems);
  uint64_t xoff = 0;
  for (const km_batch_problem& q : h->probs) {
    if (q.n == 0 || q.d == 0 || q.k == 0 || q.k > q.n || q.k > 256 || q.n >= (1ull << 31)) { delete h; return KM_ERR_ARG; }
    const uint32_t kpad = (q.k + 31) / 32 * 32;
    if ((uint64_t)q.d * kpad * 4 > BATCH_MAX_SMEM_C) { delete h; return KM_ERR_UNSUPPORTED; }
    h->max_n = std::max<uint64_t>(h->max_n, q.n);
    h->max_kd = std::max<uint64_t>(h->max_kd, (uint64_t)q.k * q.d);
    h->smem = std::max<size_t>(h->smem, (size_t)q.d * kpad * 4);
    xoff += q.n * q.d;
  }
  h->x_floats = xoff;
  // instances in LPT order (n*k*d descending, then problem, restart)
  uint64_t px = 0;
  std::vector<BatchInst> inst;
  for (uint32_t pi = 0; pi < p->problems; ++pi) {
    const km_batch_problem& q = h->probs[pi];
    for (uint32_t r = 0; r < p->restarts; ++r) {
      BatchInst I{};
      I.xoff = px; I.n = (uint32_t)q.n; I.d = q.d; I.k = q.k; I.kpad = (q.k + 31) / 32 * 32;
      I.prob = pi; I.restart = r;
      inst.push_back(I);
    }
    px += q.n * q.d;
  }
  std::stable_sort(inst.begin(), inst.end(), [](const BatchInst& a, const BatchInst& b) {
    return (uint64_t)a.n * a.k * a.d > (uint64_t)b.n * b.k * b.d;
  });
  uint64_t loff = 0, coff = 0;
  for (BatchInst& I : inst) { I.loff = loff; I.coff = coff; loff += I.n; coff += (uint64_t)I.k * I.d; }
  h->lab_total = loff;
  h->c_total = coff;
  h->inst = inst;
  km_status s = KM_OK;
  if (cudaSetDevice(h->device) != cudaSuccess) { (void)cudaGetLastError(); delete h; return KM_ERR_CUDA; }
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (p->stream) h->stream = static_cast<cudaStream_t>(p->stream);
  else if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess) h->own_stream = true;
  else { (void)cudaGetLastError(); delete h; return KM_ERR_CUDA; }
  if (s == KM_OK) s = balloc(&h->X, h->x_floats);
  if (s == KM_OK) s = balloc(&h->C0, h->c_total);
  if (s == KM_OK) s = balloc(&h->Cout, h->c_total);
  if (s == KM_OK) s = balloc(&h->labels, h->lab_total);
  if (s == KM_OK) s = balloc(&h->perm, (size_t)h->num_sms * ((h->max_n + 31) / 32 * 32));
  if (s == KM_OK) s = balloc(&h->cnew, (size_t)h->num_sms * ((h->max_kd + 31) / 32 * 32));
  if (s == KM_OK) s = balloc(&h->dinst, inst.size());
  if (s == KM_OK) s = balloc(&h->dout, inst.size());
  if (s == KM_OK) s = balloc(&h->next, 1);
  if (s == KM_OK && cudaMemcpyAsync(h->dinst, inst.data(), sizeof(BatchInst) * inst.size(), cudaMemcpyHostToDevice,
                                    h->stream) != cudaSuccess) s = KM_ERR_CUDA;
  if (s == KM_OK) {
    for (const BatchVariant& V : kVariants)
      if (h->smem > 48 * 1024 &&
          cudaFuncSetAttribute(V.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem) != cudaSuccess)
        s = KM_ERR_CUDA;
  }
  if (s != KM_OK) { (void)cudaGetLastError(); delete h; return s; }
  *out = h;
  return KM_OK;
}

km_status km_batch_set_data(km_batch* h, const float* X_host) {
  if (!h || !X_host) return KM_ERR_ARG;
  KM_CUDA_TRY(cudaSetDevice(h->device));
  for (uint64_t q = 0; q < h->x_floats; ++q)
    if (!std::isfinite(X_host[q])) return KM_ERR_ARG;
  // seeded sample picks of every instance: restart r of problem p uses seed + p*restarts + r
  std::vector<float> C0(h->c_total);
  std::vector<uint64_t> pxoff(h->probs.size());
  uint64_t px = 0;
  for (size_t pi = 0; pi < h->probs.size(); ++pi) { pxoff[pi] = px; px += h->probs[pi].n * h->probs[pi].d; }
  for (const BatchInst& I : h->inst) {
    const float* Xp = X_host + pxoff[I.prob];
    std::vector<int32_t> picks(I.k);
    const int seed = h->p.seed + (int)(I.prob * h->p.restarts + I.restart);
    if (!host_sample_picks(Xp, I.n, I.d, I.k, seed, picks.data())) return KM_ERR_ARG;
    for (uint32_t c = 0; c < I.k; ++c)
      std::memcpy(C0.data() + I.coff + (uint64_t)c * I.d, Xp + (uint64_t)picks[c] * I.d, sizeof(float) * I.d);
  }
  KM_CUDA_TRY(cudaMemcpyAsync(h->X, X_host, sizeof(float) * h->x_floats, cudaMemcpyHostToDevice, h->stream));
  KM_CUDA_TRY(cudaMemcpyAsync(h->C0, C0.data(), sizeof(float) * h->c_total, cudaMemcpyHostToDevice, h->stream));
  KM_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->ready = true;
  return KM_OK;
}

km_status km_batch_tune(km_batch* h, int32_t* variant_out, double* ms_per_variant) {
  if (!h) return KM_ERR_ARG;
  if (!h->ready) return KM_ERR_STATE;
  KM_CUDA_TRY(cudaSetDevice(h->device));
  // time every variant on an even sample of the instances, two iterations each
  const uint32_t ninst = (uint32_t)h->inst.size();
  const uint32_t want = std::min<uint32_t>(ninst, (uint32_t)h->num_sms * 2);
  std::vector<BatchInst> sample;
  for (uint32_t s = 0; s < want; ++s) sample.push_back(h->inst[(uint64_t)s * ninst / want]);
  BatchInst* ds = nullptr;
  KM_TRY(balloc(&ds, sample.size()));
  km_status st = KM_OK;
  if (cudaMemcpyAsync(ds, sample.data(), sizeof(BatchInst) * sample.size(), cudaMemcpyHostToDevice, h->stream) !=
      cudaSuccess) st = KM_ERR_CUDA;
  int best = -1;
  double bms = 0;
  const int nv = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
  for (int v = 0; v < nv && st == KM_OK; ++v) {
    float ms = 0.f;
    st = run_batch(h, v, ds, (uint32_t)sample.size(), 2, nullptr);      // warm-up
    if (st == KM_OK) st = run_batch(h, v, ds, (uint32_t)sample.size(), 2, &ms);
    h->tune_ms[v] = ms;
    if (ms_per_variant) ms_per_variant[v] = ms;
    if (st == KM_OK && (best < 0 || ms < bms)) { best = v; bms = ms; }
  }
  cudaFree(ds);
  if (st != KM_OK) return st;
  h->variant = best;
  if (variant_out) *variant_out = best;
  return KM_OK;
}

km_status km_batch_fit(km_batch* h, km_batch_result* results, uint32_t* best_labels, float* best_centroids,
                       double* fit_ms) {
  if (!h) return KM_ERR_ARG;
  if (!h->ready) return KM_ERR_STATE;
  KM_CUDA_TRY(cudaSetDevice(h->device));
  if (h->variant < 0) KM_TRY(km_batch_tune(h, nullptr, nullptr));
  float ms = 0.f;
  KM_TRY(run_batch(h, h->variant, h->dinst, (uint32_t)h->inst.size(), h->p.maxiter, &ms));
  if (fit_ms) *fit_ms = ms;
  std::vector<BatchOut> out(h->inst.size());
  KM_CUDA_TRY(cudaMemcpy(out.data(), h->dout, sizeof(BatchOut) * out.size(), cudaMemcpyDeviceToHost));
  // best restart per problem: lowest objective, then lowest restart
  const uint32_t P = h->p.problems, R = h->p.restarts;
  std::vector<int64_t> best(P, -1);
  for (size_t i = 0; i < h->inst.size(); ++i) {
    const BatchInst& I = h->inst[i];
    if (results) {
      km_batch_result& r = results[(uint64_t)I.prob * R + I.restart];
      r.converged_iter = out[i].converged_iter;
      r.iterations = out[i].iterations;
      r.objective = out[i].objective;
    }
    int64_t& b = best[I.prob];
    if (b < 0 || out[i].objective < out[b].objective ||
        (out[i].objective == out[b].objective && I.restart < h->inst[b].restart))
      b = (int64_t)i;
  }
  uint64_t lo = 0, co = 0;
  for (uint32_t pi = 0; pi < P; ++pi) {
    const BatchInst& I = h->inst[best[pi]];
    if (best_labels)
      KM_CUDA_TRY(cudaMemcpy(best_labels + lo, h->labels + I.loff, sizeof(uint32_t) * I.n, cudaMemcpyDeviceToHost));
    if (best_centroids)
      KM_CUDA_TRY(cudaMemcpy(best_centroids + co, h->Cout + I.coff, sizeof(float) * I.k * I.d,
                             cudaMemcpyDeviceToHost));
    lo += I.n;
    co += (uint64_t)I.k * I.d;
  }
  return KM_OK;
}

km_status km_batch_instance_labels(km_batch* h, uint32_t problem, uint32_t restart, uint32_t* labels_out,
                                   float* centroids_out) {
  if (!h || problem >= h->p.problems || restart >= h->p.restarts) return KM_ERR_ARG;
  KM_CUDA_TRY(cudaSetDevice(h->device));
  for (const BatchInst& I : h->inst) {
    if (I.prob != problem || I.restart != restart) continue;
    if (labels_out)
      KM_CUDA_TRY(cudaMemcpy(labels_out, h->labels + I.loff, sizeof(uint32_t) * I.n, cudaMemcpyDeviceToHost));
    if (centroids_out)
      KM_CUDA_TRY(cudaMemcpy(centroids_out, h->Cout + I.coff, sizeof(float) * I.k * I.d, cudaMemcpyDeviceToHost));
    return KM_OK;
  }
  return KM_ERR_ARG;
}

void km_batch_destroy(km_batch* h) { delete h; }

}  // extern "C"
