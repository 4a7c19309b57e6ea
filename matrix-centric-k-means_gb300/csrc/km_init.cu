// Greedy k-means++ initialisation on the device (the reference's
// init_centroids_plus_plus, src/kmeans.cu:447-769, compiled there behind
// PLUSPLUS): the first centroid is a uniformly drawn point; every further
// round draws s = 2 + ceil(ln k) candidate points with probability
// proportional to their current squared distance to the chosen set
// (raft::random::discrete over min_distances, :585-588), computes for each
// candidate the cost sum_i min(d2_i, ||x_i - x_cand||^2) (:681-693), keeps the
// cheapest (lowest index on equal cost, cub ArgMin :697-715) and updates d2
// with its distances (:721-724).  The reference seeds its generators from
// std::random_device; here the draws come from the caller's seed
// (std::mt19937_64), so the result is reproducible, and every sum has a fixed
// order, so the same seed gives the same centroids on every run.
//
// Rows are processed in chunks of PP_CHUNK; bsum[b] is the FP64 sum of d2
// over chunk b, which the sampler walks to find the chunk holding a draw and
// then scans inside the chunk.  Distances are FP32, ||x - c||^2 with the
// differences squared and summed in column order.
#include "km_lloyd.cuh"

#include <cmath>
#include <random>
#include <vector>

namespace km {

constexpr uint32_t PP_CHUNK = 1024;
constexpr uint32_t PP_MAX_S = 16;

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

// d2_i = ||x_i - x_first||^2; bsum per chunk.
__global__ void __launch_bounds__(256)
pp_first_kernel(const float* __restrict__ X, uint64_t n, uint32_t d, uint64_t first,
                float* __restrict__ d2, double* __restrict__ bsum) {
  __shared__ double red[8];
  const uint64_t r0 = (uint64_t)blockIdx.x * PP_CHUNK;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* c = X + first * d;
  double acc = 0.0;
  for (uint32_t t = warp; t < PP_CHUNK; t += 8) {
    const uint64_t i = r0 + t;
    if (i >= n) break;
    const float* x = X + i * d;
    float s = 0.0f;
    for (uint32_t j = lane; j < d; j += 32) {
      const float u = x[j] - c[j];
      s = fmaf(u, u, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) { d2[i] = s; acc += (double)s; }
  }
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    bsum[blockIdx.x] = t;
  }
}

// One warp per candidate: draw index ~ d2 / sum(d2) for the uniform u[j].
__global__ void pp_sample_kernel(const float* __restrict__ d2, uint64_t n, const double* __restrict__ bsum,
                                 uint32_t nblk, const double* __restrict__ u, uint32_t s,
                                 int32_t* __restrict__ cand) {
  const uint32_t j = blockIdx.x;
  const int lane = threadIdx.x;
  if (j >= s) return;
  double tot = 0.0;
  for (uint32_t b = lane; b < nblk; b += 32) tot += bsum[b];
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (!(tot > 0.0)) {   // every point coincides with a chosen one: uniform draw
    if (lane == 0) cand[j] = (int32_t)umin64(n - 1, (uint64_t)(u[j] * (double)n));
    return;
  }
  double target = u[j] * tot;
  // chunk holding the draw
  uint32_t blk = 0xffffffffu, last_pos = 0;
  double base = 0.0;
  for (uint32_t b0 = 0; b0 < nblk && blk == 0xffffffffu; b0 += 32) {
    const uint32_t b = b0 + lane;
    const double v = (b < nblk) ? bsum[b] : 0.0;
    double inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, b < nblk && v > 0.0 && base + inc > target);
    const unsigned pos = __ballot_sync(0xffffffffu, b < nblk && v > 0.0);
    if (pos) last_pos = b0 + 31 - __clz(pos);
    if (hit) {
      const int l = __ffs(hit) - 1;
      blk = b0 + l;
      const double excl = __shfl_sync(0xffffffffu, base + inc - v, l);
      target -= excl;
    } else {
      base += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
  if (blk == 0xffffffffu) { blk = last_pos; target = -1.0; }   // rounding at the top end
  // row inside the chunk
  const uint64_t r0 = (uint64_t)blk * PP_CHUNK;
  const uint64_t r1 = umin64(n, r0 + PP_CHUNK);
  uint64_t pick = 0xffffffffffffffffull, last_row = r0;
  base = 0.0;
  for (uint64_t i0 = r0; i0 < r1 && pick == 0xffffffffffffffffull; i0 += 32) {
    const uint64_t i = i0 + lane;
    const double v = (i < r1) ? (double)d2[i] : 0.0;
    double inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, i < r1 && v > 0.0 && target >= 0.0 && base + inc > target);
    const unsigned pos = __ballot_sync(0xffffffffu, i < r1 && v > 0.0);
    if (pos) last_row = i0 + 31 - __clz(pos);
    if (hit) pick = i0 + (__ffs(hit) - 1);
    else base += __shfl_sync(0xffffffffu, inc, 31);
  }
  if (pick == 0xffffffffffffffffull) pick = last_row;
  if (lane == 0) cand[j] = (int32_t)pick;
}

// D[i, j] = ||x_i - x_cand_j||^2 and per-chunk FP64 costs sum_i min(d2_i, D[i, j]).
__global__ void __launch_bounds__(256)
pp_cost_kernel(const float* __restrict__ X, uint64_t n, uint32_t d, const int32_t* __restrict__ cand,
               uint32_t s, const float* __restrict__ d2, float* __restrict__ D,
               double* __restrict__ cpart) {
  extern __shared__ float cs[];                    // s x d candidate rows
  __shared__ double red[8][PP_MAX_S];
  for (uint32_t t = threadIdx.x; t < s * d; t += blockDim.x) {
    const uint32_t j = t / d, c = t % d;
    cs[t] = X[(uint64_t)cand[j] * d + c];
  }
  __syncthreads();
  const uint64_t r0 = (uint64_t)blockIdx.x * PP_CHUNK;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[PP_MAX_S];
#pragma unroll
  for (uint32_t j = 0; j < PP_MAX_S; ++j) acc[j] = 0.0;
  for (uint32_t t = warp; t < PP_CHUNK; t += 8) {
    const uint64_t i = r0 + t;
    if (i >= n) break;
    const float* x = X + i * d;
    float p[PP_MAX_S];
#pragma unroll
    for (uint32_t j = 0; j < PP_MAX_S; ++j) p[j] = 0.0f;
    for (uint32_t c = lane; c < d; c += 32) {
      const float xv = x[c];
#pragma unroll
      for (uint32_t j = 0; j < PP_MAX_S; ++j) {
        if (j < s) {
          const float u = xv - cs[j * d + c];
          p[j] = fmaf(u, u, p[j]);
        }
      }
    }
#pragma unroll
    for (uint32_t j = 0; j < PP_MAX_S; ++j) {
      if (j < s) {
        float v = p[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
          D[i * s + j] = v;
          acc[j] += (double)fminf(v, d2[i]);
        }
      }
    }
  }
  if (lane == 0) {
#pragma unroll
    for (uint32_t j = 0; j < PP_MAX_S; ++j) red[warp][j] = acc[j];
  }
  __syncthreads();
  if (threadIdx.x < s) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w][threadIdx.x];
    cpart[(uint64_t)blockIdx.x * s + threadIdx.x] = t;
  }
}

// Single warp: total cost per candidate, the cheapest (lowest index on ties)
// becomes centroid number r.
__global__ void pp_choose_kernel(const double* __restrict__ cpart, uint32_t nblk, uint32_t s,
                                 const int32_t* __restrict__ cand, uint32_t r,
                                 int32_t* __restrict__ chosen, int32_t* __restrict__ best) {
  const int lane = threadIdx.x;
  double bestv = 0.0;
  int bj = -1;
  for (uint32_t j = 0; j < s; ++j) {
    double t = 0.0;
    for (uint32_t b = lane; b < nblk; b += 32) t += cpart[(uint64_t)b * s + j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (bj < 0 || t < bestv) { bestv = t; bj = (int)j; }
  }
  if (lane == 0) {
    chosen[r] = cand[bj];
    *best = bj;
  }
}

// d2_i = min(d2_i, D[i, best]); bsum per chunk.
__global__ void __launch_bounds__(256)
pp_update_kernel(const float* __restrict__ D, uint64_t n, uint32_t s, const int32_t* __restrict__ best,
                 float* __restrict__ d2, double* __restrict__ bsum) {
  __shared__ double red[8];
  const uint64_t r0 = (uint64_t)blockIdx.x * PP_CHUNK;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bj = *best;
  double acc = 0.0;
  for (uint32_t t = threadIdx.x; t < PP_CHUNK; t += blockDim.x) {
    const uint64_t i = r0 + t;
    if (i >= n) break;
    const float v = fminf(d2[i], D[i * s + bj]);
    d2[i] = v;
    acc += (double)v;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    bsum[blockIdx.x] = t;
  }
}

__global__ void pp_gather_kernel(const float* __restrict__ X, uint32_t d, const int32_t* __restrict__ idx,
                                 uint32_t k, float* __restrict__ C) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)k * d) return;
  const uint32_t r = (uint32_t)(t / d), j = (uint32_t)(t % d);
  C[t] = X[(uint64_t)idx[r] * d + j];
}

namespace {
template <typename T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t count) { return cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * count); }
};
}  // namespace

km_status plusplus_init(LloydEngine& e, int seed) {
  const uint64_t n = e.n;
  const uint32_t d = e.d, k = e.k;
  const uint32_t s = 2u + (uint32_t)std::ceil(std::log((double)k));
  if (s > PP_MAX_S) return KM_ERR_UNSUPPORTED;
  const size_t smem = (size_t)s * d * sizeof(float);
  if (smem > 200 * 1024) return KM_ERR_UNSUPPORTED;
  const uint32_t nblk = (uint32_t)((n + PP_CHUNK - 1) / PP_CHUNK);
  std::mt19937_64 gen((uint64_t)(int64_t)seed);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  const uint64_t first = std::uniform_int_distribution<uint64_t>(0, n - 1)(gen);
  std::vector<double> hu((size_t)(k > 1 ? k - 1 : 1) * s);
  for (auto& v : hu) v = uni(gen);
  std::vector<int32_t> hchosen(1, (int32_t)first);

  DevBuf<float> d2, D;
  DevBuf<double> bsum, cpart, u;
  DevBuf<int32_t> cand, chosen, best;
  if (d2.alloc(n) || D.alloc(n * s) || bsum.alloc(nblk) || cpart.alloc((size_t)nblk * s) ||
      u.alloc(hu.size()) || cand.alloc(s) || chosen.alloc(k) || best.alloc(1)) {
    (void)cudaGetLastError();
    return KM_ERR_ALLOC;
  }
  if (smem > 48 * 1024)
    KM_CUDA_TRY(cudaFuncSetAttribute(pp_cost_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaStream_t st = e.stream;
  KM_CUDA_TRY(cudaMemcpyAsync(u.p, hu.data(), sizeof(double) * hu.size(), cudaMemcpyHostToDevice, st));
  KM_CUDA_TRY(cudaMemcpyAsync(chosen.p, hchosen.data(), sizeof(int32_t), cudaMemcpyHostToDevice, st));
  pp_first_kernel<<<nblk, 256, 0, st>>>(e.X, n, d, first, d2.p, bsum.p);
  for (uint32_t r = 1; r < k; ++r) {
    pp_sample_kernel<<<s, 32, 0, st>>>(d2.p, n, bsum.p, nblk, u.p + (size_t)(r - 1) * s, s, cand.p);
    pp_cost_kernel<<<nblk, 256, smem, st>>>(e.X, n, d, cand.p, s, d2.p, D.p, cpart.p);
    pp_choose_kernel<<<1, 32, 0, st>>>(cpart.p, nblk, s, cand.p, r, chosen.p, best.p);
    pp_update_kernel<<<nblk, 256, 0, st>>>(D.p, n, s, best.p, d2.p, bsum.p);
  }
  pp_gather_kernel<<<(unsigned)(((uint64_t)k * d + 255) / 256), 256, 0, st>>>(e.X, d, chosen.p, k, e.C);
  KM_CUDA_TRY(cudaGetLastError());
  // the scratch buffers are freed on return: wait for the kernels using them
  KM_CUDA_TRY(cudaStreamSynchronize(st));
  return KM_OK;
}

}  // namespace km
