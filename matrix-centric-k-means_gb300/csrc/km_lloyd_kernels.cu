// Lloyd k-means kernels for sm_103a: point/centroid preparation, the SIMT FP32
// distance stage with fused top-3 argmin, exact near-tie refinement, the
// stable label sort (one-hot V as a label-sorted permutation), the exact
// centroid update V.X, and the per-iteration finalize / loop-control kernels.
//
// Reference counterparts (HicrestLaboratory/Matrix-Centric-K-Means):
//   distance + argmin     comparisons/CPU_Kmeans/src/kmeans.cpp:86-122;
//                         src/kmeans.cu:847-936 (popcorn SpMM + RAFT argmin)
//   counts                src/kmeans.cu:941-947 (RAFT reduce_cols_by_key)
//   V rebuild             src/kmeans.cu:987-1031, src/kernels/kernels.cuh:296-314
//   centroid update       comparisons/CPU_Kmeans/src/kmeans.cpp:131-148
//   convergence           comparisons/CPU_Kmeans/src/kmeans.cpp:170-200;
//                         src/kmeans.cu:1054-1073 (score rule)
#include "km_lloyd.cuh"

#include <cmath>
#include <cfloat>

namespace km {

static __device__ __forceinline__ float f_inf() { return __int_as_float(0x7f800000); }

// ---------------------------------------------------------------------------
// Preparation
// ---------------------------------------------------------------------------

// One warp per row: ||x||^2 (FP64 sum, stored as float and as a per-row double
// for the deterministic total), non-finite check, and the BF16 hi/lo copies
// padded with zeros to dp columns (only when Xb != nullptr).
__global__ void prep_points_kernel(const float* __restrict__ X, uint64_t n, uint32_t d, uint32_t dp,
                                   float* __restrict__ xn2, double* __restrict__ xn2d,
                                   __nv_bfloat16* __restrict__ Xb, __nv_bfloat16* __restrict__ Xlo,
                                   DevState* st) {
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = warp; r < n; r += nw) {
    const float* x = X + r * d;
    double s = 0.0;
    bool bad = false;
    for (uint32_t j = lane; j < dp; j += 32) {
      float v = (j < d) ? x[j] : 0.0f;
      if (!isfinite(v)) bad = true;
      s += (double)v * (double)v;
      if (Xb) {
        __nv_bfloat16 hi = __float2bfloat16_rn(v);
        Xb[r * dp + j] = hi;
        if (Xlo) Xlo[r * dp + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
      }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&st->err, KM_DEVERR_NONFINITE);
    if (lane == 0) {
      xn2[r] = (float)s;
      if (xn2d) xn2d[r] = s;
    }
  }
}

// Deterministic FP64 sum: fixed-shape tree per block, block partials summed in
// index order by a second single-block pass.
__global__ void reduce_f64_partial_kernel(const double* __restrict__ v, uint64_t n,
                                          double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  const uint64_t per = (n + gridDim.x - 1) / gridDim.x;
  const uint64_t b = per * blockIdx.x, e = min(n, b + per);
  for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) s += v[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void reduce_f64_final_kernel(const double* __restrict__ part, int np, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < np; ++i) s += part[i];
    *out = s;
  }
}

// One warp per centroid: ||c||^2 in FP64 (stored as float), BF16 hi/lo copies
// padded to (kp, dp), +inf norms for the padding centroids, and max ||c||.
__global__ void prep_centroids_kernel(const float* __restrict__ C, uint32_t k, uint32_t kp,
                                      uint32_t d, uint32_t dp, float* __restrict__ cn2,
                                      __nv_bfloat16* __restrict__ Cb,
                                      __nv_bfloat16* __restrict__ Clo, DevState* st) {
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= kp) return;
  const uint32_t c = warp;
  double s = 0.0;
  for (uint32_t j = lane; j < dp; j += 32) {
    float v = (c < k && j < d) ? C[(uint64_t)c * d + j] : 0.0f;
    s += (double)v * (double)v;
    if (Cb) {
      __nv_bfloat16 hi = __float2bfloat16_rn(v);
      Cb[(uint64_t)c * dp + j] = hi;
      if (Clo) Clo[(uint64_t)c * dp + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    float f = (c < k) ? (float)s : f_inf();
    cn2[c] = f;
    if (c < k) atomicMax(reinterpret_cast<unsigned int*>(&st->cmax), __float_as_uint(sqrtf(f)));
  }
}

// ---------------------------------------------------------------------------
// (a)+(b) SIMT FP32 distance GEMM with fused top-3 argmin.
// Tile 128 rows x 128 centroids, 256 threads, 8x8 register micro-tiles,
// K chunks of 16 staged through shared memory with register double buffering.
// Every CTA walks all centroid tiles for its rows, so the row tile is read from
// HBM once and re-read from L2.
// ---------------------------------------------------------------------------
namespace {
constexpr int SM_ = 128, SN_ = 128, SK_ = 16, SPAD = 4;
}

__global__ void __launch_bounds__(256, 1)
assign_f32_kernel(const float* __restrict__ X, const float* __restrict__ C,
                  const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                  uint32_t d, uint32_t k, TieBound tb, DevState* st,
                  uint32_t* __restrict__ labels, float* __restrict__ mindist,
                  RefineEntry* __restrict__ queue, float* __restrict__ Dout) {
  if (st->done) return;
  __shared__ __align__(16) float As[2][SK_][SM_ + SPAD];
  __shared__ __align__(16) float Bs[2][SK_][SN_ + SPAD];
  __shared__ float cns[SN_];
  __shared__ float bv1[SM_], bv2[SM_], bv3[SM_];
  __shared__ uint32_t bi1[SM_], bi2[SM_];

  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const uint64_t m0 = (uint64_t)blockIdx.x * SM_;
  if (tid < SM_) {
    bv1[tid] = bv2[tid] = bv3[tid] = f_inf();
    bi1[tid] = bi2[tid] = 0xffffffffu;
  }
  const uint32_t ntiles = (k + SN_ - 1) / SN_;
  const uint32_t nk = (d + SK_ - 1) / SK_;

  for (uint32_t nt = 0; nt < ntiles; ++nt) {
    const uint32_t c0 = nt * SN_;
    __syncthreads();
    if (tid < SN_) cns[tid] = (c0 + tid < k) ? cn2[c0 + tid] : f_inf();

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    float ra[8], rb[8];
    auto gload = [&](uint32_t kc) {
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int idx = e * 256 + tid;
        const int r = idx >> 4, kk = idx & 15;
        const uint32_t col = kc + kk;
        const uint64_t row = m0 + r;
        ra[e] = (row < n && col < d) ? X[row * d + col] : 0.0f;
        const uint32_t cc = c0 + r;
        rb[e] = (cc < k && col < d) ? C[(uint64_t)cc * d + col] : 0.0f;
      }
    };
    auto sstore = [&](int buf) {
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int idx = e * 256 + tid;
        const int r = idx >> 4, kk = idx & 15;
        As[buf][kk][r] = ra[e];
        Bs[buf][kk][r] = rb[e];
      }
    };
    gload(0);
    sstore(0);
    __syncthreads();
    for (uint32_t kt = 0; kt < nk; ++kt) {
      const int buf = kt & 1;
      if (kt + 1 < nk) gload((kt + 1) * SK_);
#pragma unroll
      for (int kk = 0; kk < SK_; ++kk) {
        const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 8]);
        const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 8 + 4]);
        const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 8]);
        const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 8 + 4]);
        const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
      if (kt + 1 < nk) sstore(buf ^ 1);
      __syncthreads();
    }

    // Epilogue: v = ||c||^2 - 2 x.c, top-3 per row across the 16 lanes of a row.
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty * 8 + i;
      const uint64_t row = m0 + r;
      Top3 t;
      t.init();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint32_t col = c0 + tx * 8 + j;
        const float v = fmaf(-2.0f, acc[i][j], cns[tx * 8 + j]);
        if (Dout && row < n && col < k) Dout[row * k + col] = v + xn2[row];
        if (col < k) t.insert(v, col);
      }
      t.shfl_merge_xor(8);
      t.shfl_merge_xor(4);
      t.shfl_merge_xor(2);
      t.shfl_merge_xor(1);
      if (tx == 0) {
        Top3 b;
        b.v1 = bv1[r]; b.v2 = bv2[r]; b.v3 = bv3[r]; b.i1 = bi1[r]; b.i2 = bi2[r];
        b.merge(t);
        bv1[r] = b.v1; bv2[r] = b.v2; bv3[r] = b.v3; bi1[r] = b.i1; bi2[r] = b.i2;
      }
    }
  }
  __syncthreads();

  // Classify rows (one thread per row) and queue near ties.
  if (tid < SM_) {
    const uint64_t row = m0 + tid;
    const bool valid = row < n;
    int cls = 0;
    uint32_t i1 = bi1[tid] == 0xffffffffu ? 0u : bi1[tid];
    if (valid) {
      const float cn1 = sqrtf(fmaxf(cn2[i1], 0.0f));
      cls = tie_class(xn2[row], bv1[tid], bv2[tid], bv3[tid], cn1, st->cmax, tb);
      labels[row] = i1;
      if (mindist) mindist[row] = bv1[tid] + xn2[row];
    }
    RefineEntry e{(uint32_t)row, (uint32_t)cls, i1, bi2[tid]};
    queue_refine(st, queue, valid && cls != 0, e);
  }
}

// Exact refinement of queued rows: one warp per row; the reference's CPU
// distance (float, j ascending) to the candidates, lowest index on ties.
__global__ void refine_kernel(const float* __restrict__ X, const float* __restrict__ C, uint32_t d,
                              uint32_t k, DevState* st, const RefineEntry* __restrict__ queue,
                              uint32_t* __restrict__ labels, float* __restrict__ mindist) {
  if (st->done) return;
  const uint32_t cnt = st->flag_count;
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t e = warp; e < cnt; e += nw) {
    const RefineEntry en = queue[e];
    const float* x = X + (uint64_t)en.row * d;
    float bv = f_inf();
    uint32_t bi = 0xffffffffu;
    if (en.cls == 1) {
      if (lane < 2) {
        const uint32_t c = lane ? en.c2 : en.c1;
        if (c < k) {
          const float v = cpu_dist(x, C + (uint64_t)c * d, d);
          if (v < bv) { bv = v; bi = c; }
        }
      }
    } else {
      for (uint32_t c = lane; c < k; c += 32) {
        const float v = cpu_dist(x, C + (uint64_t)c * d, d);
        if (v < bv) { bv = v; bi = c; }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (lane == 0) {
      labels[en.row] = (bi == 0xffffffffu) ? 0u : bi;
      if (mindist) mindist[en.row] = bv;
      if (en.cls == 2) atomicAdd(&st->full_total, 1ull);
    }
  }
}

// ---------------------------------------------------------------------------
// (c) One-hot V as a stable label-sorted permutation.
// Segments of `seg` rows, one warp per segment.  seghist is cluster-major
// (k x nseg) so that each cluster's segment counts are contiguous.
// ---------------------------------------------------------------------------
__global__ void seg_hist_kernel(const uint32_t* __restrict__ labels, uint64_t n, uint32_t k,
                                uint32_t seg, uint32_t nseg, uint32_t* __restrict__ seghist,
                                DevState* st) {
  if (st->done) return;
  extern __shared__ uint32_t sh_cnt[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  uint32_t* cnt = sh_cnt + (uint64_t)wib * k;
  const uint32_t s = blockIdx.x * wpb + wib;
  for (uint32_t c = lane; c < k; c += 32) cnt[c] = 0;
  __syncwarp();
  if (s < nseg) {
    const uint64_t r0 = (uint64_t)s * seg, r1 = min(n, r0 + seg);
    bool bad = false;
    for (uint64_t r = r0 + lane; r < r1; r += 32) {
      const uint32_t l = labels[r];
      if (l < k) atomicAdd(&cnt[l], 1u); else bad = true;
    }
    if (bad) atomicOr(&st->err, KM_DEVERR_OVERFLOW);
    __syncwarp();
    for (uint32_t c = lane; c < k; c += 32) seghist[(uint64_t)c * nseg + s] = cnt[c];
  }
}

// One warp per cluster: exclusive scan over its segments, total -> counts.
__global__ void seg_scan_kernel(uint32_t* __restrict__ seghist, uint32_t k, uint32_t nseg,
                                uint32_t* __restrict__ counts, DevState* st) {
  if (st->done) return;
  const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k) return;
  uint32_t* h = seghist + (uint64_t)c * nseg;
  uint32_t carry = 0;
  for (uint32_t b = 0; b < nseg; b += 32) {
    const uint32_t i = b + lane;
    const uint32_t v = (i < nseg) ? h[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (i < nseg) h[i] = carry + x - v;
    carry += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) counts[c] = carry;
}

// Single block: exclusive scan of the k counts -> cstart[0..k] (CSR row
// pointers of V).
__global__ void cluster_scan_kernel(const uint32_t* __restrict__ counts, uint32_t k,
                                    uint32_t* __restrict__ cstart, DevState* st) {
  if (st->done) return;
  __shared__ uint32_t part[1024];
  const uint32_t per = (k + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per, e = min(k, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i) s += counts[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (uint32_t t = 0; t < blockDim.x; ++t) { uint32_t v = part[t]; part[t] = acc; acc += v; }
  }
  __syncthreads();
  uint32_t acc = part[threadIdx.x];
  for (uint32_t i = b; i < e; ++i) { cstart[i] = acc; acc += counts[i]; }
  if (e == k && b < e) cstart[k] = acc;
  if (k == 0 && threadIdx.x == 0) cstart[0] = 0;
}

// One warp per segment: stable scatter of row ids into perm.
__global__ void seg_scatter_kernel(const uint32_t* __restrict__ labels, uint64_t n, uint32_t k,
                                   uint32_t seg, uint32_t nseg, const uint32_t* __restrict__ seghist,
                                   const uint32_t* __restrict__ cstart,
                                   uint32_t* __restrict__ perm, DevState* st) {
  if (st->done) return;
  extern __shared__ uint32_t sh_pos[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  uint32_t* pos = sh_pos + (uint64_t)wib * k;
  const uint32_t s = blockIdx.x * wpb + wib;
  if (s >= nseg) return;
  for (uint32_t c = lane; c < k; c += 32) pos[c] = cstart[c] + seghist[(uint64_t)c * nseg + s];
  __syncwarp();
  const uint64_t r0 = (uint64_t)s * seg, r1 = min(n, r0 + seg);
  for (uint64_t rb = r0; rb < r1; rb += 32) {
    const uint64_t r = rb + lane;
    const bool valid = r < r1;
    const uint32_t l = valid ? labels[r] : 0xffffffffu;
    const bool ok = valid && l < k;
    const unsigned m = __match_any_sync(0xffffffffu, ok ? l : 0xffffffffu);
    const uint32_t rank = __popc(m & ((1u << lane) - 1u));
    uint32_t base = ok ? pos[l] : 0u;
    __syncwarp();
    if (ok) {
      perm[base + rank] = (uint32_t)r;
      if (rank == 0) pos[l] = base + __popc(m);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// (c) Exact centroid update V.X: thread per (cluster, column), rows of the
// cluster in ascending index order (the label-sorted permutation), float sums
// exactly as the reference's CPU loop.  Also: squared move per element for the
// shift test, and the FP64 objective of this iteration's assignment against the
// centroids that produced it (FP32 partials over 64 rows, FP64 above).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
update_sums_kernel(const float* __restrict__ X, const uint32_t* __restrict__ perm,
                   const uint32_t* __restrict__ cstart, uint32_t d, uint32_t k,
                   const float* __restrict__ C, float* __restrict__ Cn,
                   float* __restrict__ dsq, double* __restrict__ objpart, DevState* st) {
  if (st && st->done) return;
  const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (uint64_t)k * d) return;
  const uint32_t c = (uint32_t)(p / d), j = (uint32_t)(p % d);
  const uint32_t s0 = cstart[c], s1 = cstart[c + 1];
  const float cold = C ? C[p] : 0.0f;
  float sum = 0.0f, e32 = 0.0f;
  double e64 = 0.0;
  constexpr int U = 16;
  uint32_t s = s0;
  int chunk = 0;
  for (; s + U <= s1; s += U) {
    uint32_t r[U];
    float v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) r[u] = perm[s + u];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = X[(uint64_t)r[u] * d + j];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      sum = __fadd_rn(sum, v[u]);
      const float t = v[u] - cold;
      e32 = fmaf(t, t, e32);
    }
    if (++chunk == 4) { e64 += e32; e32 = 0.0f; chunk = 0; }
  }
  for (; s < s1; ++s) {
    const float v = X[(uint64_t)perm[s] * d + j];
    sum = __fadd_rn(sum, v);
    const float t = v - cold;
    e32 = fmaf(t, t, e32);
  }
  e64 += e32;
  const uint32_t cnt = s1 - s0;
  const float scale = __double2float_rn(1.0 / (double)(cnt > 1 ? cnt : 1));
  const float cn = __fmul_rn(sum, scale);
  Cn[p] = cn;
  if (dsq) {
    const float t = __fsub_rn(cn, cold);
    dsq[p] = __fmul_rn(t, t);
  }
  if (objpart) objpart[p] = e64;
}

// One warp per cluster: reference shift test (float sum over j ascending, then
// sqrtf(s) > tol, kmeans.cpp:190-200), FP64 move, FP64 objective of the
// cluster, new ||c||^2 and BF16 copies; then C <- Cn.
__global__ void finalize_kernel(const float* __restrict__ Cn, float* __restrict__ C,
                                const float* __restrict__ dsq, const double* __restrict__ objpart,
                                uint32_t d, uint32_t dp, uint32_t k, float tol,
                                float* __restrict__ cn2, __nv_bfloat16* __restrict__ Cb,
                                __nv_bfloat16* __restrict__ Clo, double* __restrict__ shift_c,
                                double* __restrict__ obj_c, DevState* st) {
  if (st->done) return;
  const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k) return;
  const uint64_t base = (uint64_t)c * d;
  double nrm = 0.0, mv = 0.0, ob = 0.0;
  for (uint32_t j = lane; j < dp; j += 32) {
    const float v = (j < d) ? Cn[base + j] : 0.0f;
    if (j < d) {
      nrm += (double)v * v;
      const double t = (double)v - (double)C[base + j];
      mv += t * t;
      ob += objpart[base + j];
    }
    if (Cb) {
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      Cb[(uint64_t)c * dp + j] = hi;
      if (Clo) Clo[(uint64_t)c * dp + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
    mv += __shfl_xor_sync(0xffffffffu, mv, o);
    ob += __shfl_xor_sync(0xffffffffu, ob, o);
  }
  if (lane == 0) {
    float s = 0.0f;
    for (uint32_t j = 0; j < d; ++j) s = __fadd_rn(s, dsq[base + j]);
    if (sqrtf(s) > tol) st->moved = 1u;
    cn2[c] = (float)nrm;
    shift_c[c] = sqrt(mv);
    obj_c[c] = ob;
  }
  __syncwarp();
  for (uint32_t j = lane; j < d; j += 32) C[base + j] = Cn[base + j];
}

// Single block: end of iteration.  Deterministic reductions over clusters,
// stop decision, counters for the next iteration.
__global__ void control_kernel(const float* __restrict__ cn2, const double* __restrict__ shift_c,
                               const double* __restrict__ obj_c, uint32_t k, LoopConsts lc,
                               DevState* st) {
  if (st->done) return;
  __shared__ double s_obj[256];
  __shared__ double s_sh[256];
  __shared__ float s_cm[256];
  double ob = 0.0, sh = 0.0;
  float cm = 0.0f;
  const uint32_t per = (k + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per, e = min(k, b + per);
  for (uint32_t c = b; c < e; ++c) {
    ob += obj_c[c];
    sh = fmax(sh, shift_c[c]);
    cm = fmaxf(cm, sqrtf(cn2[c]));
  }
  s_obj[threadIdx.x] = ob; s_sh[threadIdx.x] = sh; s_cm[threadIdx.x] = cm;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s_obj[threadIdx.x] += s_obj[threadIdx.x + o];
      s_sh[threadIdx.x] = fmax(s_sh[threadIdx.x], s_sh[threadIdx.x + o]);
      s_cm[threadIdx.x] = fmaxf(s_cm[threadIdx.x], s_cm[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const uint32_t it = st->iter + 1;
    st->iter = it;
    st->objective = s_obj[0];
    st->max_shift = s_sh[0];
    st->cmax = s_cm[0] * 1.000001f;
    const double score = s_obj[0] - st->sum_x2;
    st->score = score;
    st->refined_total += st->flag_count;
    st->flag_count = 0;
    bool stop = false;
    if (lc.conv == KM_CONV_SHIFT) {
      if (it > 1 && st->moved == 0u) { st->converged_iter = it; stop = true; }
    } else if (lc.conv == KM_CONV_SCORE) {
      if (it < lc.maxiter && it > 1 && fabs(score - st->last_score) < (double)lc.tol) {
        st->converged_iter = it; stop = true;
      }
      st->last_score = score;
    }
    st->moved = 0u;
    if (it >= lc.maxiter) stop = true;
    if (stop) st->done = 1u;
  }
}

}  // namespace km
