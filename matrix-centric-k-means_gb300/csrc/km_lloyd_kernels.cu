// Lloyd k-means kernels for sm_103a: point/centroid preparation, the SIMT FP32
// distance stage with fused top-3 argmin, exact near-tie refinement, the
// stable label sort (one-hot V as a label-sorted permutation), the exact
// centroid update V.X, and the per-iteration finalize kernel (whose last block
// takes the loop decision).
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

// One warp per row: ||x||^2 (an FP32 pair, stored as float and as a per-row
// double for the deterministic total), non-finite check, and the BF16 hi/lo
// copies padded with zeros to dp columns (only when Xb != nullptr).
__global__ void prep_points_kernel(const float* __restrict__ X, uint64_t n, uint32_t d, uint32_t dp,
                                   float* __restrict__ xn2, double* __restrict__ xn2d,
                                   __nv_bfloat16* __restrict__ Xb, __nv_bfloat16* __restrict__ Xlo,
                                   DevState* st) {
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  // ||x||^2 as an unevaluated FP32 pair (hi + lo): each square split exactly
  // by an FMA, each addition by TwoSum (the FP64 units of this GPU are a
  // small fraction of its FP32 rate); the pair is within a few units of 2^-48
  // of the exact value, and float(hi + lo) is the correctly rounded norm.
  auto two_sum = [](float& h, float& l, float a, float al) {
    const float t = __fadd_rn(h, a), bp = __fsub_rn(t, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bp)), __fsub_rn(a, bp));
    h = t;
    l = __fadd_rn(l, __fadd_rn(al, err));
  };
  // NaN/Inf and non-BF16 coordinates are flagged once per warp (after its
  // rows), not once per row: an atomic per row on one word serialises.
  bool bad = false, inexact = false;
  for (uint64_t r = warp; r < n; r += nw) {
    const float* x = X + r * d;
    float sh = 0.0f, sl = 0.0f;
    for (uint32_t j = lane; j < dp; j += 32) {
      float v = (j < d) ? x[j] : 0.0f;
      if (!isfinite(v)) bad = true;
      if ((__float_as_uint(v) & 0xffffu) != 0u) inexact = true;    // not a BF16 value
      const float p = __fmul_rn(v, v);
      two_sum(sh, sl, p, fmaf(v, v, -p));
      if (Xb) {
        __nv_bfloat16 hi = __float2bfloat16_rn(v);
        Xb[r * dp + j] = hi;
        if (Xlo) Xlo[r * dp + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, sh, o), ol = __shfl_xor_sync(0xffffffffu, sl, o);
      two_sum(sh, sl, oh, ol);
    }
    const double s = (double)sh + (double)sl;
    if (lane == 0) {
      xn2[r] = (float)s;
      if (xn2d) xn2d[r] = s;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&st->err, KM_DEVERR_NONFINITE);
  if (__any_sync(0xffffffffu, inexact) && lane == 0) atomicOr(&st->x_not_bf16, 1u);
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
                                      __nv_bfloat16* __restrict__ Clo, float* __restrict__ Ct,
                                      DevState* st, uint32_t kp64) {
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= kp) {
    // +inf norms up to whole 64-column groups (read by the distance epilogue)
    if (warp < kp64 && lane == 0) cn2[warp] = f_inf();
    return;
  }
  const uint32_t c = warp;
  double s = 0.0;
  for (uint32_t j = lane; j < dp; j += 32) {
    float v = (c < k && j < d) ? C[(uint64_t)c * d + j] : 0.0f;
    if (c < k && j < d) Ct[(uint64_t)j * k + c] = v;
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
// K chunks of 16 staged through shared memory with register double buffering
// (16-byte global loads when d % 4 == 0 and the rows are 16-byte aligned).
// Every CTA walks all centroid tiles for its rows, so the row tile is read from
// HBM once and re-read from L2.
// ---------------------------------------------------------------------------
namespace {
constexpr int SM_ = 128, SN_ = 128, SK_ = 16, SPAD = 4;
// Dynamic shared memory of assign_f32_kernel: each thread's running top-3 of
// its eight rows, five arrays (v1, v2, v3, i1, i2) of [128 rows][F32_TOP_LD]
// words, lane tx of a row at column tx.  The stride 18 keeps the epilogue's
// accesses (two rows 8 apart per warp) conflict-free and the final per-row
// merge two-way at most.
constexpr int F32_TOP_LD = 18;
constexpr size_t F32_TOP_SMEM = 5 * 128 * F32_TOP_LD * sizeof(float);
}

// Thread (tx, ty) of the 16 x 16 grid owns rows ty*8 .. ty*8+7 and the two
// column quads tx*4 .. tx*4+3 and 64 + tx*4 .. +3 of the 128 x 128 tile: the
// quarter-warps' 16-byte centroid loads from shared memory then cover 128
// contiguous bytes (no bank conflicts), and two CTAs fit an SM.
// DOUT (distance-matrix output): one CTA per SM, so that its stores do not spill.
template <bool V4, bool DOUT>
__global__ void __launch_bounds__(256, DOUT ? 1 : 2)
assign_f32_kernel(const float* __restrict__ X, const float* __restrict__ C,
                  const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                  uint32_t d, uint32_t k, TieBound tb, DevState* st,
                  uint32_t* __restrict__ labels, float* __restrict__ mindist,
                  RefineQueues rq, float* __restrict__ Dout, const uint32_t* __restrict__ ridx,
                  const uint32_t* __restrict__ nidx) {
  griddep_wait();
  if (st->done) return;
  // Gather mode (ridx != null): logical row li of the tiles is row ridx[li] of X,
  // for li < *nidx; queue segments are taken over the logical rows.
  const uint64_t n_log = ridx ? (uint64_t)*nidx : n;
  if ((uint64_t)blockIdx.x * SM_ >= n_log) return;
  __shared__ uint32_t rmap[SM_];
  __shared__ __align__(16) float As[2][SK_][SM_ + SPAD];
  __shared__ __align__(16) float Bs[2][SK_][SN_ + SPAD];
  __shared__ float cns[SN_];
  // Each thread's running top-3 of its eight rows over the column tiles so far.
  // A thread visits its columns in ascending order (tx*4 + j, then 64 + tx*4 +
  // j, tile by tile), so strict-order insertion keeps the lowest index on
  // ties; after the last tile one thread per row merges the row's 16 lists
  // under the (v, i) order.
  extern __shared__ float f32_top[];
  constexpr int TA = SM_ * F32_TOP_LD;
  float* const tv1 = f32_top;
  float* const tv2 = f32_top + TA;
  float* const tv3 = f32_top + 2 * TA;
  uint32_t* const ti1 = reinterpret_cast<uint32_t*>(f32_top + 3 * TA);
  uint32_t* const ti2 = reinterpret_cast<uint32_t*>(f32_top + 4 * TA);

  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int o = (ty * 8 + i) * F32_TOP_LD + tx;
    tv1[o] = tv2[o] = tv3[o] = f_inf();
    ti1[o] = ti2[o] = 0xffffffffu;
  }
  const uint64_t m0 = (uint64_t)blockIdx.x * SM_;
  if (tid < SM_) {
    const uint64_t li = m0 + tid;
    rmap[tid] = ridx ? (li < n_log ? ridx[li] : 0u) : (uint32_t)li;
  }
  __syncthreads();
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
      if constexpr (V4) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int idx = e * 256 + tid;
          const int r = idx >> 2, c4 = idx & 3;
          const uint32_t col = kc + 4u * (uint32_t)c4;
          const bool rv = m0 + r < n_log;
          const uint64_t row = rmap[r];
          const uint32_t cc = c0 + r;
          float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
          if (rv && col < d) a = __ldg(reinterpret_cast<const float4*>(X + row * d + col));
          if (cc < k && col < d) b = __ldg(reinterpret_cast<const float4*>(C + (uint64_t)cc * d + col));
          ra[4 * e + 0] = a.x; ra[4 * e + 1] = a.y; ra[4 * e + 2] = a.z; ra[4 * e + 3] = a.w;
          rb[4 * e + 0] = b.x; rb[4 * e + 1] = b.y; rb[4 * e + 2] = b.z; rb[4 * e + 3] = b.w;
        }
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int idx = e * 256 + tid;
          const int r = idx >> 4, kk = idx & 15;
          const uint32_t col = kc + kk;
          const uint64_t row = rmap[r];
          ra[e] = (m0 + r < n_log && col < d) ? X[row * d + col] : 0.0f;
          const uint32_t cc = c0 + r;
          rb[e] = (cc < k && col < d) ? C[(uint64_t)cc * d + col] : 0.0f;
        }
      }
    };
    auto sstore = [&](int buf) {
      if constexpr (V4) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int idx = e * 256 + tid;
          const int r = idx >> 2, c4 = idx & 3;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            As[buf][4 * c4 + q][r] = ra[4 * e + q];
            Bs[buf][4 * c4 + q][r] = rb[4 * e + q];
          }
        }
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int idx = e * 256 + tid;
          const int r = idx >> 4, kk = idx & 15;
          As[buf][kk][r] = ra[e];
          Bs[buf][kk][r] = rb[e];
        }
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
        const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
        const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
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

    // Epilogue: v = ||c||^2 - 2 x.c into the thread's running top-3 per row.
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty * 8 + i;
      const uint64_t row = m0 + r;                      // Dout is written in direct mode only
      const int o = r * F32_TOP_LD + tx;
      Top3 t;
      t.v1 = tv1[o]; t.v2 = tv2[o]; t.v3 = tv3[o]; t.i1 = ti1[o]; t.i2 = ti2[o];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint32_t cl = (j < 4) ? (uint32_t)(tx * 4 + j) : (uint32_t)(64 + tx * 4 + j - 4);
        const uint32_t col = c0 + cl;
        const float v = fmaf(-2.0f, acc[i][j], cns[cl]);
        if (DOUT && row < n && col < k) Dout[row * k + col] = v + xn2[row];
        // columns at or past k hold ||c||^2 = +inf, so v is +inf (or NaN)
        // there and the strict insertion never takes them
        t.insert_asc(v, col);
      }
      tv1[o] = t.v1; tv2[o] = t.v2; tv3[o] = t.v3; ti1[o] = t.i1; ti2[o] = t.i2;
    }
  }
  __syncthreads();

  // One thread per row: merge the row's 16 lists, classify, queue near ties.
  if (tid < SM_) {
    Top3 b;
    b.init();
#pragma unroll 4
    for (int l = 0; l < 16; ++l) {
      const int o = tid * F32_TOP_LD + l;
      Top3 u;
      u.v1 = tv1[o]; u.v2 = tv2[o]; u.v3 = tv3[o]; u.i1 = ti1[o]; u.i2 = ti2[o];
      b.merge(u);
    }
    const uint64_t li = m0 + tid;
    const bool valid = li < n_log;
    const uint64_t row = rmap[tid];
    int cls = 0;
    uint32_t i1 = b.i1 == 0xffffffffu ? 0u : b.i1;
    if (valid) {
      const float cn1 = sqrtf(fmaxf(cn2[i1], 0.0f));
      cls = tie_class(xn2[row], b.v1, b.v2, b.v3, cn1, st->cmax, tb);
      labels[row] = i1;
      if (mindist) mindist[row] = b.v1 + xn2[row];
    }
    RefineEntry e{(uint32_t)row, 2u, {i1, b.i2, 0u, 0u}};
    const uint64_t seg = li >> 5;
    seg_push(rq.cand, rq.ccnt, seg, valid && cls == 1, e);
    seg_push(rq.full, rq.fcnt, seg, valid && cls == 2, (uint32_t)row);
  }
}

km_status launch_assign_f32(const float* X, const float* C, const float* cn2, const float* xn2,
                            uint64_t n, uint32_t d, uint32_t k, TieBound tb, DevState* st,
                            uint32_t* labels, float* mindist, const RefineQueues& rq,
                            float* Dout, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n + SM_ - 1) / SM_);
  const bool v4 = (d % 4 == 0) && (reinterpret_cast<uintptr_t>(X) % 16 == 0) &&
                  (reinterpret_cast<uintptr_t>(C) % 16 == 0);
  auto kern = v4 ? (Dout ? assign_f32_kernel<true, true> : assign_f32_kernel<true, false>)
                 : (Dout ? assign_f32_kernel<false, true> : assign_f32_kernel<false, false>);
  kern<<<blocks, 256, F32_TOP_SMEM, s>>>(X, C, cn2, xn2, n, d, k, tb, st, labels, mindist, rq, Dout, nullptr,
                                         nullptr);
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

// Exact re-score of rows with 2..4 candidates, for rows that are not 16-byte
// aligned or d % 4 != 0 (refine_staged_kernel below is the vector path): four
// lanes per row, one candidate per lane, the reference's CPU distance (float,
// j ascending); smallest distance wins, lowest index on ties.  The candidate
// set provably holds the reference argmin over all k (tie_tau / tie_class).
// One warp per RC_SEGS consecutive queue segments, their entries flattened so
// that every pass keeps eight rows in flight; the grid covers all segments at
// once (no loop over segments, so a warp pays one count load and its rows).
constexpr int RC_SEGS = 2;
constexpr int RC_WARPS = 8;

__global__ void __launch_bounds__(32 * RC_WARPS)
refine_cands_kernel(const float* __restrict__ X, const float* __restrict__ C, uint32_t d,
                    DevState* st, RefineQueues rq, uint32_t* __restrict__ labels,
                    float* __restrict__ mindist, bool count) {
  griddep_wait();
  if (st->done) return;
  __shared__ uint32_t block_rows;
  if (threadIdx.x == 0) block_rows = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t seg0 = warp * RC_SEGS;
  // inclusive prefix of the RC_SEGS segment counts, kept in every lane
  const uint32_t c = (lane < RC_SEGS && seg0 + (uint64_t)lane < rq.nseg) ? rq.ccnt[seg0 + lane] : 0u;
  uint32_t pre[RC_SEGS];
  uint32_t run = 0;
#pragma unroll
  for (int q = 0; q < RC_SEGS; ++q) {
    run += __shfl_sync(0xffffffffu, c, q);
    pre[q] = run;
  }
  const uint32_t total = run;
  const uint32_t slot = (uint32_t)lane & 3u;
  for (uint32_t base = 0; base < total; base += 8) {
    const uint32_t qi = base + (uint32_t)(lane >> 2);
    float bv = f_inf();
    uint32_t bi = 0xffffffffu;
    uint32_t row = 0;
    if (qi < total) {
      uint32_t sg = 0, before = 0;
#pragma unroll
      for (int q = 0; q < RC_SEGS - 1; ++q)
        if (qi >= pre[q]) { sg = (uint32_t)q + 1u; before = pre[q]; }
      const RefineEntry en = rq.cand[(seg0 + sg) * 32 + (qi - before)];
      row = en.row;
      if (slot < en.cnt) {
        const uint32_t cc = en.c[slot];
        const float* x = X + (uint64_t)row * d;
        const float* cr = C + (uint64_t)cc * d;
        const float v = cpu_dist(x, cr, d);
        if (v < bv) { bv = v; bi = cc; }
      }
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (qi < total && slot == 0) {
      labels[row] = (bi == 0xffffffffu) ? 0u : bi;
      if (mindist) mindist[row] = bv;
    }
  }
  if (count && lane == 0 && total) atomicAdd(&block_rows, total);
  __syncthreads();
  if (count && threadIdx.x == 0 && block_rows)
    atomicAdd(&st->refined_total, (unsigned long long)block_rows);
}

// Reference CPU distance with 16-byte loads (d % 4 == 0 and 16-byte aligned
// rows): the operation order of cpu_dist, the loads arranged for memory-level
// parallelism (below).
__device__ __forceinline__ float4 ldg_nc_v4(const float4* p) {
  float4 v;
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}
__device__ __forceinline__ float cpu_dist_v4(const float* __restrict__ x, const float* __restrict__ c,
                                                 uint32_t d) {
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const float4* c4 = reinterpret_cast<const float4*>(c);
  const uint32_t d4 = d / 4;
  float s = 0.0f;
  auto step = [&](const float4 a, const float4 b) {
    float t = __fsub_rn(a.x, b.x); s = __fadd_rn(s, __fmul_rn(t, t));
    t = __fsub_rn(a.y, b.y); s = __fadd_rn(s, __fmul_rn(t, t));
    t = __fsub_rn(a.z, b.z); s = __fadd_rn(s, __fmul_rn(t, t));
    t = __fsub_rn(a.w, b.w); s = __fadd_rn(s, __fmul_rn(t, t));
  };
  // Groups of four 128-byte lines of each row: the first 16 bytes of all eight
  // lines are loaded together (eight misses in flight), so the rest of each
  // line is already in L1 when the ordered chain reaches it.
  uint32_t q = 0;
  for (; q + 32 <= d4; q += 32) {
    float4 a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) { a[i] = ldg_nc_v4(x4 + q + 8 * i); b[i] = ldg_nc_v4(c4 + q + 8 * i); }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      step(a[i], b[i]);
      float4 ra[7], rb[7];
#pragma unroll
      for (int r = 0; r < 7; ++r) { ra[r] = __ldg(x4 + q + 8 * i + 1 + r); rb[r] = __ldg(c4 + q + 8 * i + 1 + r); }
#pragma unroll
      for (int r = 0; r < 7; ++r) step(ra[r], rb[r]);
    }
  }
  for (; q < d4; ++q) step(x4[q], c4[q]);
  return s;
}

// Exact re-score of a group of up to FULL_ROWS rows (row ids rows[0..nr))
// against all k centroids by one warp: lanes over centroids (eight chains per
// lane and row), centroids read from the transposed copy Ct (d x k) so that
// every load of the warp is one coalesced 128-byte line and serves all rows of
// the group.  Per lane the centroids are visited in ascending order with a
// strict '<' and the warp reduction keeps the lowest index on ties: the
// reference's argmin (kmeans.cpp:106-122).
constexpr int FULL_ROWS = 4;

__device__ __forceinline__ void full_rescore_group(const float* __restrict__ X, const float* __restrict__ Ct,
                                                   uint32_t d, uint32_t k, const uint32_t* rows, uint32_t nr,
                                                   uint32_t* __restrict__ labels, float* __restrict__ mindist) {
  const int lane = threadIdx.x & 31;
  uint32_t row[FULL_ROWS];
  const float* x[FULL_ROWS];
#pragma unroll
  for (int r = 0; r < FULL_ROWS; ++r) {
    row[r] = rows[min((uint32_t)r, nr - 1)];   // pad with the last row
    x[r] = X + (uint64_t)row[r] * d;
  }
  float bv[FULL_ROWS];
  uint32_t bi[FULL_ROWS];
#pragma unroll
  for (int r = 0; r < FULL_ROWS; ++r) { bv[r] = f_inf(); bi[r] = 0xffffffffu; }
  for (uint32_t cb = 0; cb < k; cb += 256) {
    float s[FULL_ROWS][8];
#pragma unroll
    for (int r = 0; r < FULL_ROWS; ++r)
#pragma unroll
      for (int t = 0; t < 8; ++t) s[r][t] = 0.0f;
    // Four j steps per group: all their loads (the rows' x_j, the lanes'
    // centroid columns from Ct) are issued before the group's arithmetic,
    // which keeps 48 loads in flight per lane instead of one step's.
    for (uint32_t j0 = 0; j0 < d; j0 += 4) {
      float xj[4][FULL_ROWS], cv[4][8];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t j = j0 + (uint32_t)q;
        const bool jin = j < d;
#pragma unroll
        for (int r = 0; r < FULL_ROWS; ++r) xj[q][r] = jin ? x[r][j] : 0.0f;
        const float* ct = Ct + (uint64_t)(jin ? j : 0u) * k + cb + lane;
#pragma unroll
        for (int t = 0; t < 8; ++t) cv[q][t] = (jin && cb + lane + 32 * t < k) ? ct[32 * t] : 0.0f;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (j0 + (uint32_t)q >= d) break;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
#pragma unroll
          for (int r = 0; r < FULL_ROWS; ++r) {
            const float tt = __fsub_rn(xj[q][r], cv[q][t]);
            s[r][t] = __fadd_rn(s[r][t], __fmul_rn(tt, tt));
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const uint32_t c = cb + lane + 32 * t;
#pragma unroll
      for (int r = 0; r < FULL_ROWS; ++r)
        if (c < k && s[r][t] < bv[r]) { bv[r] = s[r][t]; bi[r] = c; }
    }
  }
#pragma unroll
  for (int r = 0; r < FULL_ROWS; ++r) {
    float v = bv[r];
    uint32_t i = bi[r];
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, v, o);
      const uint32_t oi = __shfl_xor_sync(0xffffffffu, i, o);
      if (ov < v || (ov == v && oi < i)) { v = ov; i = oi; }
    }
    if (lane == 0 && (uint32_t)r < nr) {
      labels[row[r]] = (i == 0xffffffffu) ? 0u : i;
      if (mindist) mindist[row[r]] = v;
    }
  }
}

// Rows of the full queue, warp by warp: segments warp, warp + nw, warp + 2 nw,
// ... (a dense queue spreads over all warps); 32 of their counts per load,
// only the non-empty ones visited.
__global__ void __launch_bounds__(256, 2)
refine_full_kernel(const float* __restrict__ X, const float* __restrict__ Ct, uint32_t d, uint32_t k,
                   DevState* st, RefineQueues rq, uint32_t* __restrict__ labels,
                   float* __restrict__ mindist, bool count) {
  griddep_wait();
  if (st->done) return;
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint32_t done_rows = 0;
  for (uint64_t g0 = warp; g0 < rq.nseg; g0 += nw * 32) {
    const uint64_t sgl = g0 + (uint64_t)lane * nw;
    const uint32_t cl = (sgl < rq.nseg) ? rq.fcnt[sgl] : 0u;
    uint32_t nz = __ballot_sync(0xffffffffu, cl != 0u);
    while (nz) {
      const int sl = __ffs(nz) - 1;
      nz &= nz - 1u;
      const uint64_t seg = g0 + (uint64_t)sl * nw;
      const uint32_t cnt = __shfl_sync(0xffffffffu, cl, sl);
      done_rows += cnt;
      for (uint32_t e0 = 0; e0 < cnt; e0 += FULL_ROWS)
        full_rescore_group(X, Ct, d, k, rq.full + seg * 32 + e0, min(cnt - e0, (uint32_t)FULL_ROWS), labels,
                           mindist);
    }
  }
  if (count && lane == 0 && done_rows) {
    atomicAdd(&st->refined_total, (unsigned long long)done_rows);
    atomicAdd(&st->full_total, (unsigned long long)done_rows);
  }
}

// Exact re-score of the candidate queue with its operands staged in shared
// memory (d % 4 == 0, 16-byte aligned rows).  Each warp owns ranges of `span`
// (<= 32) consecutive queue segments, one segment count per lane, and walks a
// range's entries in passes.  A pass takes the leading entries whose point
// rows and candidate centroid rows fit RS_ROWS staged rows: the entries' point
// rows at [0, ne), the pairs' centroid rows at [ne, ne + np), pair p on lane p.
// The rows are copied by the TMA engine, one bulk copy per row issued by the
// lane that owns the row, RS_CH columns per round trip (all of d when d <=
// RS_CH), completing on the warp's mbarrier; the loads of the next pass's
// entries are issued before the copies are waited on.  (16-byte cp.async per
// lane, one row per instruction, spent most of the pass issuing the copies.)  Every lane then runs the reference's ordered
// chain (float, j ascending, no contraction) from shared memory.  A lane that
// loads its own rows straight from global memory touches up to 32 lines per
// instruction, and the L1 wavefronts, not DRAM, then set the time.  The
// entry's lane picks the smallest distance over its candidates in ascending
// index order with a strict '<' (lowest index on ties).  The candidate set
// provably holds the reference argmin over all k (tie_tau / tie_class).
// FULL: the grid's warps then re-score the full queue against all k
// (full_rescore_group), so that one launch covers the whole refinement.
constexpr int RS_WARPS = 5;
constexpr int RS_ROWS = 40;              // staged rows per pass (at most 32 pairs)
constexpr uint32_t RS_CH = 128;          // staged columns per round trip
constexpr int RS_BLOCKS_PER_SM = 2;
constexpr uint64_t RS_WAIT_NS = 2000000000ull;   // bound of a wait for the warp's copies
// Shared row stride in floats for chunks of ch columns, with (stride / 4) odd
// so that float4 reads of eight consecutive rows cover the 32 banks.
__host__ __device__ constexpr uint32_t rs_ld(uint32_t ch) { return ((ch + 4u) / 4u) % 2u ? ch + 4u : ch + 8u; }
constexpr size_t RS_SMEM_MAX = (size_t)RS_WARPS * RS_ROWS * rs_ld(RS_CH) * sizeof(float);

template <bool FULL>
__global__ void __launch_bounds__(32 * RS_WARPS, RS_BLOCKS_PER_SM)
refine_staged_kernel(const float* __restrict__ X, const float* __restrict__ C, const float* __restrict__ Ct,
                     uint32_t d, uint32_t k, uint32_t span, DevState* st, RefineQueues rq,
                     uint32_t* __restrict__ labels, float* __restrict__ mindist, bool count) {
  griddep_wait();
  if (st->done) return;
  extern __shared__ __align__(16) float rs_smem[];
  __shared__ __align__(8) uint64_t rs_bar[RS_WARPS];
  __shared__ int rs_no_abort[RS_WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t ch = min(d, RS_CH), ld = rs_ld(ch);
  float* const stg = rs_smem + (size_t)wib * RS_ROWS * ld;
  uint64_t* const bar = &rs_bar[wib];   // this warp's copies
  if (lane == 0) {
    mbar_init(bar, 1);
    rs_no_abort[wib] = 0;
    mbar_fence_init();
  }
  __syncwarp();
  uint32_t ph = 0;   // parity of the barrier phase the next wait completes
  const uint64_t nranges = (rq.nseg + span - 1) / span;
  const uint64_t nw = (uint64_t)gridDim.x * RS_WARPS;
  uint32_t cand_rows = 0, full_rows = 0;
  for (uint64_t rg = (uint64_t)blockIdx.x * RS_WARPS + wib; rg < nranges; rg += nw) {
    const uint64_t seg0 = rg * span;
    const bool segok = (uint32_t)lane < span && seg0 + (uint64_t)lane < rq.nseg;
    const uint32_t c = segok ? rq.ccnt[seg0 + lane] : 0u;
    uint32_t pre = c;   // inclusive prefix of the segment counts over the lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
    cand_rows += total;
    // Entry t of the range (all lanes call; loads only for t < total): its
    // segment is the number of lanes whose prefix is <= t.
    auto load_entry = [&](uint32_t t) {
      uint32_t sg = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint32_t pv = __shfl_sync(0xffffffffu, pre, (int)(sg + (uint32_t)step - 1u));
        if (pv <= t) sg += (uint32_t)step;
      }
      const uint32_t before = __shfl_sync(0xffffffffu, pre, (int)((sg + 31u) & 31u));
      RefineEntry r{0u, 0u, {0u, 0u, 0u, 0u}};
      if (t < total) r = rq.cand[(seg0 + sg) * 32 + (t - (sg ? before : 0u))];
      return r;
    };
    RefineEntry en = load_entry((uint32_t)lane);
    for (uint32_t e0 = 0; e0 < total;) {
      const bool has = e0 + (uint32_t)lane < total;
      const uint32_t cl = has ? max(1u, min(en.cnt, 4u)) : 0u;
      uint32_t incl = cl;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      // entries of this pass: the leading lanes whose rows (one point row per
      // entry, one centroid row per pair) fit RS_ROWS and whose pairs fit the
      // 32 lanes (at least eight entries, cl <= 4)
      const uint32_t ne = (uint32_t)__popc(
          __ballot_sync(0xffffffffu, has && incl <= 32u && (uint32_t)lane + 1u + incl <= (uint32_t)RS_ROWS));
      const uint32_t np = __shfl_sync(0xffffffffu, incl, (int)ne - 1);
      const uint32_t off = incl - cl;
      // pair p = lane: its entry e (the last entry lane with off <= p)
      const uint32_t p = (uint32_t)lane;
      uint32_t e = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint32_t t = e + (uint32_t)step;
        const uint32_t ot = __shfl_sync(0xffffffffu, off, (int)(t & 31u));
        if (t < ne && ot <= p) e = t;
      }
      const uint32_t m = p - __shfl_sync(0xffffffffu, off, (int)e);
      const uint32_t q0 = __shfl_sync(0xffffffffu, en.c[0], (int)e);
      const uint32_t q1 = __shfl_sync(0xffffffffu, en.c[1], (int)e);
      const uint32_t q2 = __shfl_sync(0xffffffffu, en.c[2], (int)e);
      const uint32_t q3 = __shfl_sync(0xffffffffu, en.c[3], (int)e);
      const uint32_t cand = m == 0 ? q0 : m == 1 ? q1 : m == 2 ? q2 : q3;   // meaningful for p < np
      const uint32_t nrows = ne + np;
      // Source rows of the staged rows: lane r holds staged row r (r < 32) and
      // lane r - 32 holds staged row r >= 32 (16-byte aligned: d % 4 == 0).
      const uint32_t crl = __shfl_sync(0xffffffffu, cand, (int)(((uint32_t)lane - ne) & 31u));
      const uint32_t crh = __shfl_sync(0xffffffffu, cand, (int)(((uint32_t)lane + 32u - ne) & 31u));
      const uint64_t srcl = (uint32_t)lane < ne ? reinterpret_cast<uint64_t>(X + (uint64_t)en.row * d)
                                                : reinterpret_cast<uint64_t>(C + (uint64_t)crl * d);
      const uint64_t srch = reinterpret_cast<uint64_t>(C + (uint64_t)crh * d);
      // columns [j0, j0 + nc) of the pass's rows: one bulk copy per row (a
      // multiple of 16 bytes between 16-byte aligned addresses)
      auto stage = [&](uint32_t j0) {
        const uint32_t bytes = min(ch, d - j0) * 4u;
        // Every earlier read of the rows has returned its value (the chain's
        // sums went through the lane reduction) before any lane gets here.
        if (lane == 0) mbar_arrive_expect_tx(bar, nrows * bytes);
        __syncwarp();
        if ((uint32_t)lane < nrows)
          bulk_copy_g2s(stg + lane * ld, reinterpret_cast<const float*>(srcl) + j0, bytes, bar);
        if ((uint32_t)lane + 32u < nrows)
          bulk_copy_g2s(stg + (32u + lane) * ld, reinterpret_cast<const float*>(srch) + j0, bytes, bar);
      };
      stage(0);
      const uint32_t e0n = e0 + ne;
      const RefineEntry enn = load_entry(e0n + (uint32_t)lane);   // in flight during this pass
      float s = 0.0f;
      auto step4 = [&](const float4 a, const float4 b) {
        float t = __fsub_rn(a.x, b.x); s = __fadd_rn(s, __fmul_rn(t, t));
        t = __fsub_rn(a.y, b.y); s = __fadd_rn(s, __fmul_rn(t, t));
        t = __fsub_rn(a.z, b.z); s = __fadd_rn(s, __fmul_rn(t, t));
        t = __fsub_rn(a.w, b.w); s = __fadd_rn(s, __fmul_rn(t, t));
      };
      for (uint32_t j0 = 0; j0 < d; j0 += ch) {
        if (j0) stage(j0);
        const bool okw = mbar_wait_bounded(bar, ph, &rs_no_abort[wib], RS_WAIT_NS);
        ph ^= 1u;
        if (!__all_sync(0xffffffffu, okw)) {
          // copies that never landed: flag, give the ones in flight a bounded
          // second wait, and end this warp (no block barrier follows)
          if (lane == 0) atomicOr(&st->err, KM_DEVERR_TIMEOUT);
          mbar_wait_bounded(bar, ph ^ 1u, &rs_no_abort[wib], RS_WAIT_NS);
          return;
        }
        if (p < np) {
          const float4* xs = reinterpret_cast<const float4*>(stg + e * ld);
          const float4* cs = reinterpret_cast<const float4*>(stg + (ne + p) * ld);
          const uint32_t nc4 = min(ch, d - j0) / 4u;
          if (nc4 == RS_CH / 4u) {
#pragma unroll 8
            for (uint32_t q = 0; q < RS_CH / 4u; ++q) step4(xs[q], cs[q]);
          } else {
            for (uint32_t q = 0; q < nc4; ++q) step4(xs[q], cs[q]);
          }
        }
        __syncwarp();   // the rows are restaged only after every lane's chain
      }
      // entry lane: the smallest of its cl candidates (pairs off .. off+cl-1)
      float bv = 0.0f;
      uint32_t bi = 0u;
#pragma unroll
      for (uint32_t mm = 0; mm < 4; ++mm) {
        const int src = (int)((off + mm) & 31u);
        const float v = __shfl_sync(0xffffffffu, s, src);
        const uint32_t ci = __shfl_sync(0xffffffffu, cand, src);
        if (mm == 0 || (mm < cl && v < bv)) { bv = v; bi = ci; }
      }
      if ((uint32_t)lane < ne) {
        labels[en.row] = bi;
        if (mindist) mindist[en.row] = bv;
      }
      en = enn;
      e0 = e0n;
    }
  }
  if (FULL) {
    // The full queue, interleaved over every warp of the grid as in
    // refine_full_kernel (its rows can be many and bunched: e.g. the FP32 pass
    // at very large k); 32 segment counts per load, only non-empty ones visited.
    for (uint64_t g0 = (uint64_t)blockIdx.x * RS_WARPS + wib; g0 < rq.nseg; g0 += nw * 32) {
      const uint64_t sgl = g0 + (uint64_t)lane * nw;
      const uint32_t fl = (sgl < rq.nseg) ? rq.fcnt[sgl] : 0u;
      uint32_t nz = __ballot_sync(0xffffffffu, fl != 0u);
      while (nz) {
        const int sl = __ffs(nz) - 1;
        nz &= nz - 1u;
        const uint64_t seg = g0 + (uint64_t)sl * nw;
        const uint32_t cnt = __shfl_sync(0xffffffffu, fl, sl);
        full_rows += cnt;
        for (uint32_t f0 = 0; f0 < cnt; f0 += FULL_ROWS)
          full_rescore_group(X, Ct, d, k, rq.full + seg * 32 + f0, min(cnt - f0, (uint32_t)FULL_ROWS), labels,
                             mindist);
      }
    }
  }
  if (count && lane == 0 && cand_rows + full_rows)
    atomicAdd(&st->refined_total, (unsigned long long)(cand_rows + full_rows));
  if (count && lane == 0 && full_rows) atomicAdd(&st->full_total, (unsigned long long)full_rows);
}

// Launch shape of refine_staged_kernel: a persistent grid, each warp a range
// of `span` consecutive segments.
struct StagedShape {
  unsigned blocks;
  uint32_t span;
  size_t smem;
};
static StagedShape staged_shape(int num_sms, uint64_t nseg, uint32_t d) {
  const uint64_t max_warps = (uint64_t)num_sms * RS_BLOCKS_PER_SM * RS_WARPS;
  const uint32_t span = (uint32_t)std::min<uint64_t>(32, std::max<uint64_t>(1, (nseg + max_warps - 1) / max_warps));
  const uint64_t ranges = (nseg + span - 1) / span;
  StagedShape sh;
  sh.blocks = (unsigned)std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t)num_sms * RS_BLOCKS_PER_SM, (ranges + RS_WARPS - 1) / RS_WARPS));
  sh.span = span;
  sh.smem = (size_t)RS_WARPS * RS_ROWS * rs_ld(std::min<uint32_t>(d, RS_CH)) * sizeof(float);
  return sh;
}

static void launch_refine_cands(bool v4, int num_sms, const float* X, const float* C, uint32_t d,
                                DevState* st, const RefineQueues& rq, uint32_t* labels, float* mindist,
                                bool count, cudaStream_t s) {
  if (v4) {
    const StagedShape sh = staged_shape(num_sms, rq.nseg, d);
    (void)launch_pdl(refine_staged_kernel<false>, sh.blocks, 32 * RS_WARPS, sh.smem, s, X, C,
                     (const float*)nullptr, d, 0u, sh.span, st, rq, labels, mindist, count);
  } else {
    const uint64_t warps = (rq.nseg + RC_SEGS - 1) / RC_SEGS;
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, (warps + RC_WARPS - 1) / RC_WARPS);
    (void)launch_pdl(refine_cands_kernel, blocks, 32 * RC_WARPS, 0, s, X, C, d, st, rq, labels, mindist, count);
  }
}

// Rows of the full queue gathered into one list (order irrelevant: every row
// is re-scored on its own), counted as fully re-scored rows.
__global__ void full_compact_kernel(DevState* st, RefineQueues rq, uint32_t* __restrict__ out,
                                    uint32_t* __restrict__ nout) {
  griddep_wait();
  if (st->done) return;
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint32_t done_rows = 0;
  for (uint64_t seg = warp; seg < rq.nseg; seg += nw) {
    const uint32_t cnt = rq.fcnt[seg];
    if (cnt == 0u) continue;
    done_rows += cnt;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(nout, cnt);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((uint32_t)lane < cnt) out[base + lane] = rq.full[seg * 32 + lane];
  }
  if (lane == 0 && done_rows) {
    atomicAdd(&st->refined_total, (unsigned long long)done_rows);
    atomicAdd(&st->full_total, (unsigned long long)done_rows);
  }
}

// Exact re-score of rows with 5..L candidates (chunked distance kernel): one
// warp per row, lanes stride over the row's candidates, the reference's CPU
// distance; smallest distance wins, lowest index on ties.
template <bool V4>
__global__ void __launch_bounds__(256, 2)
refine_wide_kernel(const float* __restrict__ X, const float* __restrict__ C, uint32_t d,
                   DevState* st, RefineQueues rq, uint32_t* __restrict__ labels,
                   float* __restrict__ mindist) {
  griddep_wait();
  if (st->done) return;
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint32_t done_rows = 0;
  for (uint64_t seg = warp; seg < rq.nseg; seg += nw) {
    const uint32_t cnt = rq.wcnt[seg];
    done_rows += cnt;
    for (uint32_t e = 0; e < cnt; ++e) {
      const uint32_t row = rq.wide[seg * 32 + e];
      const uint32_t nc = min(rq.wlc[row], rq.L);
      float bv = f_inf();
      uint32_t bi = 0xffffffffu;
      const float* x = X + (uint64_t)row * d;
      for (uint32_t e = (uint32_t)lane; e < nc; e += 32u) {
        const uint32_t c = rq.wl[(uint64_t)row * rq.L + e].x;
        const float* cc = C + (uint64_t)c * d;
        const float v = V4 ? cpu_dist_v4(x, cc, d) : cpu_dist(x, cc, d);
        if (v < bv || (v == bv && c < bi)) { bv = v; bi = c; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov < bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
      }
      if (lane == 0) {
        labels[row] = (bi == 0xffffffffu) ? 0u : bi;
        if (mindist) mindist[row] = bv;
      }
    }
  }
  if (lane == 0 && done_rows) atomicAdd(&st->refined_total, (unsigned long long)done_rows);
}

km_status refine_prepare() {
  // assign_f32_kernel: 37 KB static + F32_TOP_SMEM dynamic is above the default 48 KB
  for (auto kern : {assign_f32_kernel<true, true>, assign_f32_kernel<true, false>, assign_f32_kernel<false, true>,
                    assign_f32_kernel<false, false>})
    KM_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F32_TOP_SMEM));
  KM_CUDA_TRY(cudaFuncSetAttribute(refine_staged_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)RS_SMEM_MAX));
  KM_CUDA_TRY(cudaFuncSetAttribute(refine_staged_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)RS_SMEM_MAX));
  return KM_OK;
}

km_status launch_refine(bool v4, int num_sms, const float* X, const float* C, const float* Ct,
                        uint32_t d, uint32_t k, DevState* st, const RefineQueues& rq,
                        uint32_t* labels, float* mindist, cudaStream_t s) {
  // Every row sits in one queue at most, so the queues are re-scored in any order.
  if (v4) {
    // candidate and full queues in one launch
    const StagedShape sh = staged_shape(num_sms, rq.nseg, d);
    KM_CUDA_TRY(launch_pdl(refine_staged_kernel<true>, sh.blocks, 32 * RS_WARPS, sh.smem, s, X, C, Ct, d, k,
                           sh.span, st, rq, labels, mindist, true));
    if (rq.wide)
      KM_CUDA_TRY(launch_pdl(refine_wide_kernel<true>, num_sms * 8, 256, 0, s, X, C, d, st, rq, labels, mindist));
  } else {
    launch_refine_cands(false, num_sms, X, C, d, st, rq, labels, mindist, true, s);
    if (rq.wide)
      KM_CUDA_TRY(launch_pdl(refine_wide_kernel<false>, num_sms * 8, 256, 0, s, X, C, d, st, rq, labels, mindist));
    KM_CUDA_TRY(launch_pdl(refine_full_kernel, num_sms * 4, 256, 0, s, X, Ct, d, k, st, rq, labels, mindist, true));
  }
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

km_status launch_refine_gemm(bool v4, int num_sms, const float* X, const float* C, const float* Ct,
                             const float* cn2, const float* xn2, uint64_t n, uint32_t d, uint32_t k,
                             TieBound tb32, DevState* st, const RefineQueues& rq,
                             const RefineQueues& rq2, uint32_t* fidx, uint32_t* nfull,
                             uint32_t* labels, float* mindist, cudaStream_t s) {
  launch_refine_cands(v4, num_sms, X, C, d, st, rq, labels, mindist, true, s);
  if (rq.wide) {
    if (v4)
      refine_wide_kernel<true><<<num_sms * 8, 256, 0, s>>>(X, C, d, st, rq, labels, mindist);
    else
      refine_wide_kernel<false><<<num_sms * 8, 256, 0, s>>>(X, C, d, st, rq, labels, mindist);
  }
  // rows of the full queue: FP32 distance pass over all k on those rows alone,
  // then the exact re-score of its own near ties
  KM_CUDA_TRY(cudaMemsetAsync(nfull, 0, sizeof(uint32_t), s));
  // the gather pass writes the counts of the segments its rows reach only:
  // every other segment of rq2 must read as empty
  KM_CUDA_TRY(cudaMemsetAsync(rq2.ccnt, 0, sizeof(uint32_t) * rq2.nseg, s));
  KM_CUDA_TRY(cudaMemsetAsync(rq2.fcnt, 0, sizeof(uint32_t) * rq2.nseg, s));
  full_compact_kernel<<<num_sms * 4, 256, 0, s>>>(st, rq, fidx, nfull);
  const unsigned blocks = (unsigned)((n + SM_ - 1) / SM_);
  const bool gv4 = v4 && (reinterpret_cast<uintptr_t>(C) % 16 == 0);
  if (gv4)
    assign_f32_kernel<true, false><<<blocks, 256, F32_TOP_SMEM, s>>>(X, C, cn2, xn2, n, d, k, tb32, st, labels, mindist,
                                                   rq2, nullptr, fidx, nfull);
  else
    assign_f32_kernel<false, false><<<blocks, 256, F32_TOP_SMEM, s>>>(X, C, cn2, xn2, n, d, k, tb32, st, labels, mindist,
                                                    rq2, nullptr, fidx, nfull);
  launch_refine_cands(v4, num_sms, X, C, d, st, rq2, labels, mindist, false, s);
  refine_full_kernel<<<num_sms * 4, 256, 0, s>>>(X, Ct, d, k, st, rq2, labels, mindist, false);
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

// ---------------------------------------------------------------------------
// (c) One-hot V as a stable label-sorted permutation.
// Segments of `seg` rows, one warp per segment.  seghist is cluster-major
// (k x nseg) so that each cluster's segment counts are contiguous.
// ---------------------------------------------------------------------------
__global__ void seg_hist_kernel(const uint32_t* __restrict__ labels, uint64_t n, uint32_t k,
                                uint32_t seg, uint32_t nseg, uint32_t* __restrict__ seghist,
                                DevState* st) {
  griddep_wait();
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
    for (uint64_t g = r0; g < r1; g += 32u * 32u) {
      uint32_t lv[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const uint64_t r = g + (uint64_t)q * 32u + (uint64_t)lane;
        lv[q] = (r < r1) ? labels[r] : 0u;
      }
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        if (g + (uint64_t)q * 32u + (uint64_t)lane >= r1) break;
        const uint32_t l = lv[q];
        if (l < k) atomicAdd(&cnt[l], 1u); else bad = true;
      }
    }
    if (bad) atomicOr(&st->err, KM_DEVERR_OVERFLOW);
    __syncwarp();
    for (uint32_t c = lane; c < k; c += 32) seghist[(uint64_t)c * nseg + s] = cnt[c];
  }
}

// Exclusive scan of the k counts -> cstart[0..k] (CSR row pointers of V) by one
// block (any size up to 1024 threads); order (nullable, k <= 1024): clusters by
// descending count, ties by index.  Counts are read from L2 (other blocks may
// have written them in the same launch).
__device__ void cluster_scan_block(const uint32_t* counts, uint32_t k, uint32_t* __restrict__ cstart,
                                   uint32_t* __restrict__ order, uint32_t* part, uint32_t* scnt) {
  if (order && k <= 1024u) {
    // largest cluster first, so that the longest ordered sums start first
    for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) scnt[c] = __ldcg(counts + c);
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) {
      const uint32_t v = scnt[c];
      uint32_t rank = 0;
      for (uint32_t o = 0; o < k; ++o) {
        const uint32_t w = scnt[o];
        rank += (w > v || (w == v && o < c)) ? 1u : 0u;
      }
      order[rank] = c;
    }
    __syncthreads();
  }
  const uint32_t per = (k + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per, e = min(k, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i) s += __ldcg(counts + i);
  // exclusive block scan of s: warp shuffles, then the warp totals
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) part[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const uint32_t nw = blockDim.x >> 5;
    uint32_t t = (uint32_t)lane < nw ? part[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if ((uint32_t)lane < nw) part[lane] = t;       // inclusive warp totals
  }
  __syncthreads();
  uint32_t acc = x - s + (wid > 0 ? part[wid - 1] : 0u);
  for (uint32_t i = b; i < e; ++i) { cstart[i] = acc; acc += __ldcg(counts + i); }
  if (e == k && b < e) cstart[k] = acc;
  if (k == 0 && threadIdx.x == 0) cstart[0] = 0;
}

// One warp per cluster: exclusive scan over its segments, total -> counts.
// With cstart, the block that finishes last (a ticket in DevState) then runs
// the cluster scan, which saves a dependent launch.  At most 512 threads per
// block (80 registers a thread).
__global__ void __launch_bounds__(512) seg_scan_kernel(uint32_t* __restrict__ seghist, uint32_t k, uint32_t nseg,
                                uint32_t* __restrict__ counts, DevState* st, uint32_t* __restrict__ cstart,
                                uint32_t* __restrict__ order) {
  griddep_wait();
  if (st->done) return;
  const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c < k) {
    uint32_t* h = seghist + (uint64_t)c * nseg;
    uint32_t carry = 0;
    // groups of 32 coalesced chunks: every load of a group is issued before the
    // scans that use them
    for (uint32_t g = 0; g < nseg; g += 32u * 32u) {
      uint32_t v[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const uint32_t i = g + (uint32_t)q * 32u + (uint32_t)lane;
        v[q] = (i < nseg) ? h[i] : 0u;
      }
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const uint32_t i = g + (uint32_t)q * 32u + (uint32_t)lane;
        uint32_t x = v[q];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        if (i < nseg) h[i] = carry + x - v[q];
        carry += __shfl_sync(0xffffffffu, x, 31);
      }
    }
    if (lane == 0) counts[c] = carry;
  }
  if (!cstart) return;
  __shared__ uint32_t part[32];
  __shared__ uint32_t scnt[1024];
  __shared__ int is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = (atomicAdd(&st->scan_ticket, 1u) == gridDim.x - 1u) ? 1 : 0;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  cluster_scan_block(counts, k, cstart, order, part, scnt);
  if (threadIdx.x == 0) reinterpret_cast<volatile DevState*>(st)->scan_ticket = 0u;
}

// Single block: cluster_scan_block as a kernel of its own.
__global__ void cluster_scan_kernel(const uint32_t* __restrict__ counts, uint32_t k,
                                    uint32_t* __restrict__ cstart, DevState* st,
                                    uint32_t* __restrict__ order) {
  griddep_wait();
  if (st->done) return;
  __shared__ uint32_t part[32];
  __shared__ uint32_t scnt[1024];
  cluster_scan_block(counts, k, cstart, order, part, scnt);
}

// One warp per segment: stable scatter of row ids into perm.
__global__ void seg_scatter_kernel(const uint32_t* __restrict__ labels, uint64_t n, uint32_t k,
                                   uint32_t seg, uint32_t nseg, const uint32_t* __restrict__ seghist,
                                   const uint32_t* __restrict__ cstart,
                                   uint32_t* __restrict__ perm, DevState* st) {
  griddep_wait();
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
  // labels of up to 32 chunks into registers first (one load latency per group)
  for (uint64_t g = r0; g < r1; g += 32u * 32u) {
   uint32_t lv[32];
#pragma unroll
   for (int q = 0; q < 32; ++q) {
     const uint64_t r = g + (uint64_t)q * 32u + (uint64_t)lane;
     lv[q] = (r < r1) ? labels[r] : 0xffffffffu;
   }
#pragma unroll
   for (int q = 0; q < 32; ++q) {
    const uint64_t rb = g + (uint64_t)q * 32u;
    if (rb >= r1) break;
    const uint64_t r = rb + lane;
    const bool valid = r < r1;
    const uint32_t l = lv[q];
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
}

// ---------------------------------------------------------------------------
// (c) Exact centroid update V.X.  One warp per (cluster, 32*VEC-column chunk),
// each lane on VEC adjacent columns: the cluster's rows are visited in
// ascending index order (the label-sorted permutation) and summed in float
// exactly as the reference's CPU loop (kmeans.cpp:133-137).  Row segments are
// gathered with cp.async (16 bytes per lane for VEC = 4, 4 bytes for VEC = 1,
// zero-filled past d) into a per-warp ring of UPD_STAGES batches of UPD_ROWS
// rows, so that three batches are in flight while the ordered additions consume
// the fourth; the permutation indices of a batch come in with one coalesced
// load and are broadcast by shuffles.  Also: squared move per element for the
// shift test and the FP64 objective of this iteration's assignment against the
// centroids that produced it (FP32 partials per batch, FP64 above).
// ---------------------------------------------------------------------------
namespace {
constexpr int UPD_ROWS = 32, UPD_STAGES = 8;

__device__ __forceinline__ void cp_async_16(void* smem, const void* gmem, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_4(void* smem, const void* gmem, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(smem)), "l"(gmem),
               "r"(src_bytes)
               : "memory");
}
}  // namespace

template <int VEC>
__global__ void __launch_bounds__(32)
update_sums_kernel(const float* __restrict__ X, const uint32_t* __restrict__ perm,
                   const uint32_t* __restrict__ cstart, uint32_t d, uint32_t k,
                   const float* __restrict__ C, float* __restrict__ Cn,
                   float* __restrict__ dsq, double* __restrict__ objpart, DevState* st) {
  griddep_wait();
  if (st && st->done) return;
  extern __shared__ __align__(128) float ring[];   // [UPD_STAGES][UPD_ROWS][32 * VEC]
  constexpr uint32_t W = 32u * VEC;
  const uint32_t nchunk = (d + W - 1) / W;
  const uint64_t gw = blockIdx.x;
  if (gw >= (uint64_t)k * nchunk) return;
  const int lane = threadIdx.x & 31;
  const uint32_t c = (uint32_t)(gw / nchunk);
  const uint32_t j0 = (uint32_t)(gw % nchunk) * W + (uint32_t)lane * VEC;
  const uint32_t s0 = cstart[c], s1 = cstart[c + 1];
  const uint32_t nb = (s1 - s0 + UPD_ROWS - 1) / UPD_ROWS;
  float cold[VEC], sum[VEC];
  double e64[VEC];
#pragma unroll
  for (int q = 0; q < VEC; ++q) {
    cold[q] = (C && j0 + q < d) ? C[(uint64_t)c * d + j0 + q] : 0.0f;
    sum[q] = 0.0f;
    e64[q] = 0.0;
  }
  // Permutation index of this lane's row in batch b (loaded one batch ahead of
  // its use so that the gather issue never waits on it).
  auto load_perm = [&](uint32_t b) -> uint32_t {
    const uint32_t i = s0 + b * UPD_ROWS + (uint32_t)lane;
    return (b < nb && i < s1) ? perm[i] : 0u;
  };
  auto issue = [&](uint32_t b, uint32_t rl) {
    if (b < nb) {
      const uint32_t base = s0 + b * UPD_ROWS;
      const uint32_t m = min((uint32_t)UPD_ROWS, s1 - base);
      float* dst = ring + (size_t)(b % UPD_STAGES) * UPD_ROWS * W + (uint32_t)lane * VEC;
#pragma unroll 8
      for (int u = 0; u < UPD_ROWS; ++u) {
        const uint32_t r = __shfl_sync(0xffffffffu, rl, u);
        const bool ok = (uint32_t)u < m && j0 < d;
        const float* src = ok ? X + (uint64_t)r * d + j0 : X;
        if constexpr (VEC == 4) cp_async_16(dst + (size_t)u * W, src, ok ? 16u : 0u);
        else cp_async_4(dst + (size_t)u * W, src, ok ? 4u : 0u);
      }
    }
    cp_async_commit();
  };
  {
    uint32_t p0[UPD_STAGES - 1];
#pragma unroll
    for (int b = 0; b < UPD_STAGES - 1; ++b) p0[b] = load_perm((uint32_t)b);
#pragma unroll
    for (int b = 0; b < UPD_STAGES - 1; ++b) issue((uint32_t)b, p0[b]);
  }
  // pq[i] holds the permutation indices of batch b + UPD_STAGES - 1 + i: the
  // load of a batch's indices is issued UPD_PREFETCH iterations before use.
  // The loop is unrolled by UPD_PREFETCH so that pq[i] is consumed in place,
  // UPD_PREFETCH batches after its load was issued.
  constexpr int UPD_PREFETCH = 8;
  uint32_t pq[UPD_PREFETCH];
#pragma unroll
  for (int i = 0; i < UPD_PREFETCH; ++i) pq[i] = load_perm((uint32_t)(UPD_STAGES - 1 + i));
  for (uint32_t b0 = 0; b0 < nb; b0 += UPD_PREFETCH)
#pragma unroll
  for (int i = 0; i < UPD_PREFETCH; ++i) {
    const uint32_t b = b0 + (uint32_t)i;
    if (b >= nb) break;
    issue(b + UPD_STAGES - 1, pq[i]);
    pq[i] = load_perm(b + UPD_STAGES - 1 + UPD_PREFETCH);
    cp_async_wait<UPD_STAGES - 1>();
    __syncwarp();
    const uint32_t m = min((uint32_t)UPD_ROWS, s1 - (s0 + b * UPD_ROWS));
    const float* src = ring + (size_t)(b % UPD_STAGES) * UPD_ROWS * W + (uint32_t)lane * VEC;
    float e32[VEC];
#pragma unroll
    for (int q = 0; q < VEC; ++q) e32[q] = 0.0f;
#pragma unroll 8
    for (int u = 0; u < UPD_ROWS; ++u) {
      if ((uint32_t)u < m) {
        float v[VEC];
        if constexpr (VEC == 4) {
          const float4 f = *reinterpret_cast<const float4*>(src + (size_t)u * W);
          v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
        } else {
          v[0] = src[(size_t)u * W];
        }
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          sum[q] = __fadd_rn(sum[q], v[q]);
          const float t = v[q] - cold[q];
          e32[q] = fmaf(t, t, e32[q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < VEC; ++q) e64[q] += e32[q];
    __syncwarp();
  }
  cp_async_wait<0>();
  const uint32_t cnt = s1 - s0;
  const float scale = __double2float_rn(1.0 / (double)(cnt > 1 ? cnt : 1));
#pragma unroll
  for (int q = 0; q < VEC; ++q) {
    if (j0 + q >= d) break;
    const uint64_t p = (uint64_t)c * d + j0 + q;
    const float cn = __fmul_rn(sum[q], scale);
    Cn[p] = cn;
    if (dsq) {
      const float t = __fsub_rn(cn, cold[q]);
      dsq[p] = __fmul_rn(t, t);
    }
    if (objpart) objpart[p] = e64[q];
  }
}

// Pipelined variant (d % 4 == 0, 16-byte aligned X): one CTA per (cluster,
// 32-column block), so a cluster's d/32 column chains run on as many SMs.
// Warps 0..BLK_PROD-1 produce: producer p fills batches p, p + BLK_PROD, ...
// with 16-byte cp.async per lane (one instruction copies BLK_RPI row segments)
// into a BLK_STAGES-deep ring; arrival on the stage's mbarrier fires when its
// copies land (cp.async.mbarrier.arrive.noinc).  A single producer warp caps a
// CTA at about half the row rate of three.  Warp BLK_PROD consumes, lane =
// column: a full batch is loaded into registers first, then summed in row
// order exactly as the reference (kmeans.cpp:133-137).  The objective term is
// summed per batch in FP32 and across batches as an unevaluated FP32 pair
// (TwoSum), which keeps FP64-level accuracy without a loop-carried FP64 add
// (a long-latency operation on this GPU).  Every wait is bounded; on timeout
// the CTA flags KM_DEVERR_TIMEOUT and drains its copies before exiting.
// Permutation indices are prefetched P batches ahead in registers consumed in
// place.  A batch is BLK_ROWS = 128 rows (four groups of 32): every batch costs
// the consumer one wait and one release of fixed latency, which at 32 rows per
// batch capped a CTA at about 140 rows/us (measured); at 128 rows the largest
// clusters' chains run at about 280 rows/us.  BLK_STAGES is a multiple of
// BLK_PROD, so a stage is always refilled by the same producer, which waits on
// its phases in order (a parity wait can never alias a later phase).
namespace {
constexpr int BLK_ROWS = 128, BLK_GRP = 32, BLK_STAGES = 6, BLK_COLS = 32, BLK_PROD = 3;
static_assert(BLK_STAGES % BLK_PROD == 0, "a stage must always belong to the same producer");
static_assert(BLK_ROWS % BLK_GRP == 0, "batches are whole groups of 32 rows");
constexpr uint64_t BLK_WAIT_NS = 2000000000ull;
constexpr uint32_t BLK_SUSPEND_NS = 2000;       // try_wait suspend hint
constexpr size_t BLK_SMEM = (size_t)BLK_STAGES * BLK_ROWS * BLK_COLS * sizeof(float);
constexpr int BLK_LPR = BLK_COLS / 4;           // lanes per row (16 bytes each)
constexpr int BLK_RPI = 32 / BLK_LPR;           // rows per copy instruction
constexpr int BLK_THREADS = 32 * (BLK_PROD + (BLK_COLS + 31) / 32);
}  // namespace

__global__ void __launch_bounds__(BLK_THREADS)
update_sums_bulk_kernel(const float* __restrict__ X, const uint32_t* __restrict__ perm,
                        const uint32_t* __restrict__ cstart, uint32_t d, uint32_t k,
                        const float* __restrict__ C, float* __restrict__ Cn,
                        float* __restrict__ dsq, double* __restrict__ objpart, DevState* st,
                        const uint32_t* __restrict__ order) {
  griddep_wait();
  if (st && st->done) return;
  extern __shared__ __align__(128) float ring[];        // [BLK_STAGES][BLK_ROWS][BLK_COLS]
  __shared__ __align__(8) uint64_t full[BLK_STAGES], empty[BLK_STAGES];
  __shared__ int abort_flag;
  const uint32_t nblk = (d + BLK_COLS - 1) / BLK_COLS;
  // with an order, CTAs take the largest clusters first (they are scheduled in
  // index order), so that the longest ordered sums start first
  const uint32_t c = order ? order[blockIdx.x / nblk] : blockIdx.x / nblk;
  const uint32_t j0 = (blockIdx.x % nblk) * BLK_COLS;
  const uint32_t w = min((uint32_t)BLK_COLS, d - j0);   // columns of this block (multiple of 4)
  const uint32_t nc = (w + 31) / 32;                    // consumer warps doing work
  const uint32_t s0 = cstart[c], s1 = cstart[c + 1];
  const uint32_t nb = (s1 - s0 + BLK_ROWS - 1) / BLK_ROWS;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < BLK_STAGES; ++s) { mbar_init(&full[s], 32); mbar_init(&empty[s], nc); }
    abort_flag = 0;
    mbar_fence_init();
  }
  __syncthreads();
  volatile int* ab = &abort_flag;
  auto fail = [&]() {
    abort_flag = 1;
    if (st) atomicOr(&st->err, KM_DEVERR_TIMEOUT);
  };

  if (warp < BLK_PROD) {
    constexpr int P = 2;                       // batches of indices prefetched per producer
    constexpr int G = BLK_ROWS / BLK_GRP;
    const uint32_t p0 = (uint32_t)warp;
    uint32_t pq[P][G];
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const uint32_t b = p0 + (uint32_t)i * BLK_PROD;
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const uint32_t idx = s0 + b * BLK_ROWS + (uint32_t)(g * BLK_GRP) + (uint32_t)lane;
        pq[i][g] = (b < nb && idx < s1) ? perm[idx] : 0u;
      }
    }
    // Unrolled by P so that pq[i] is consumed in place, P batches after its
    // load was issued (moving a register whose load is in flight would wait).
    bool ok = true;
    for (uint32_t lb0 = 0; p0 + lb0 * BLK_PROD < nb && ok; lb0 += P) {
#pragma unroll
      for (int i = 0; i < P; ++i) {
        const uint32_t b = p0 + (lb0 + (uint32_t)i) * BLK_PROD;
        if (b >= nb || !ok) break;
        const uint32_t s = b % BLK_STAGES, ph = (b / BLK_STAGES) & 1u;
        const bool okw = mbar_wait_bounded(&empty[s], ph ^ 1u, ab, BLK_WAIT_NS, BLK_SUSPEND_NS);
        if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(); ok = false; break; }
        const uint32_t m = min((uint32_t)BLK_ROWS, s1 - (s0 + b * BLK_ROWS));
        // One instruction copies BLK_RPI rows: BLK_LPR lanes of 16 bytes per
        // row; columns past w and rows past m zero-fill.
        const uint32_t sub = (uint32_t)lane / BLK_LPR, c4 = ((uint32_t)lane % BLK_LPR) * 4u;
        const bool lane_has_cols = c4 < w;
        const float* xl = X + j0 + c4;
#pragma unroll
        for (int g = 0; g < G; ++g) {
          float* dst = ring + ((size_t)s * BLK_ROWS + (size_t)(g * BLK_GRP) + sub) * BLK_COLS + c4;
          // All row indices of the group first: each cp.async is an ordered asm
          // statement, so a shuffle placed between two of them would put its
          // latency on every row.
          uint32_t rr[BLK_GRP / BLK_RPI];
#pragma unroll
          for (int ii = 0; ii < BLK_GRP / BLK_RPI; ++ii)
            rr[ii] = __shfl_sync(0xffffffffu, pq[i][g], ii * BLK_RPI + (int)sub);
#pragma unroll
          for (int ii = 0; ii < BLK_GRP / BLK_RPI; ++ii) {
            const uint32_t u = (uint32_t)(g * BLK_GRP + ii * BLK_RPI) + sub;
            const bool okr = u < m && lane_has_cols;
            const float* src = okr ? xl + (uint64_t)rr[ii] * d : X;
            cp_async16_zfill(dst + (size_t)ii * BLK_RPI * BLK_COLS, src, okr ? 16u : 0u);
          }
        }
        cp_async_mbar_arrive_noinc(&full[s]);
        const uint32_t nbb = b + (uint32_t)P * BLK_PROD;
#pragma unroll
        for (int g = 0; g < G; ++g) {
          const uint32_t idx = s0 + nbb * BLK_ROWS + (uint32_t)(g * BLK_GRP) + (uint32_t)lane;
          pq[i][g] = (nbb < nb && idx < s1) ? perm[idx] : 0u;
        }
      }
    }
    // Drain: this warp's copies must land before the CTA exits.
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else if ((uint32_t)(warp - BLK_PROD) < nc) {
    const uint32_t col = (uint32_t)(warp - BLK_PROD) * 32u + (uint32_t)lane;   // column within the block
    const bool vj = col < w;
    const uint64_t p = (uint64_t)c * d + j0 + col;
    const float cold = (C && vj) ? C[p] : 0.0f;
    float sum = 0.0f;
    float eh = 0.0f, el = 0.0f;          // objective: FP32 pair hi + lo
    for (uint32_t b = 0; b < nb; ++b) {
      const uint32_t s = b % BLK_STAGES, ph = (b / BLK_STAGES) & 1u;
      const bool ok = mbar_wait_bounded(&full[s], ph, ab, BLK_WAIT_NS, BLK_SUSPEND_NS);
      if (!__all_sync(0xffffffffu, ok)) { if (lane == 0) fail(); break; }
      const uint32_t m = min((uint32_t)BLK_ROWS, s1 - (s0 + b * BLK_ROWS));
      // Groups of 32 rows in order; the group's objective partial joins the
      // FP32 pair, as one batch of 32 rows did.
      for (uint32_t g0 = 0; g0 < m; g0 += BLK_GRP) {
        const uint32_t mg = min((uint32_t)BLK_GRP, m - g0);
        const float* src = ring + ((size_t)s * BLK_ROWS + g0) * BLK_COLS + col;
        float e32 = 0.0f, e32b = 0.0f;
        if (mg == (uint32_t)BLK_GRP) {
          // Full group: all loads first, then the ordered chain (no branch or
          // load latency on the dependent additions).
          float v[BLK_GRP];
#pragma unroll
          for (int u = 0; u < BLK_GRP; ++u) v[u] = vj ? src[(size_t)u * BLK_COLS] : 0.0f;
#pragma unroll
          for (int u = 0; u < BLK_GRP; ++u) {
            sum = __fadd_rn(sum, v[u]);
            const float t = v[u] - cold;
            if (u & 1) e32b = fmaf(t, t, e32b); else e32 = fmaf(t, t, e32);
          }
        } else {
          for (uint32_t u = 0; u < mg; ++u) {
            const float v = vj ? src[(size_t)u * BLK_COLS] : 0.0f;
            sum = __fadd_rn(sum, v);
            const float t = v - cold;
            e32 = fmaf(t, t, e32);
          }
        }
        e32 = __fadd_rn(e32, e32b);
        // TwoSum: eh + e32 = s_ + err exactly; err accumulates into el
        const float s_ = __fadd_rn(eh, e32), bb = __fsub_rn(s_, eh);
        el = __fadd_rn(el, __fadd_rn(__fsub_rn(eh, __fsub_rn(s_, bb)), __fsub_rn(e32, bb)));
        eh = s_;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
    if (vj) {
      const uint32_t cnt = s1 - s0;
      const float scale = __double2float_rn(1.0 / (double)(cnt > 1 ? cnt : 1));
      const float cn = __fmul_rn(sum, scale);
      Cn[p] = cn;
      if (dsq) {
        const float t = __fsub_rn(cn, cold);
        dsq[p] = __fmul_rn(t, t);
      }
      if (objpart) objpart[p] = (double)eh + (double)el;
    }
  }
}

// Opt-in shared memory for the VEC = 4 ring; called before any capture.
km_status update_sums_prepare() {
  KM_CUDA_TRY(cudaFuncSetAttribute(update_sums_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   UPD_STAGES * UPD_ROWS * 128 * (int)sizeof(float)));
  KM_CUDA_TRY(cudaFuncSetAttribute(update_sums_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)BLK_SMEM));
  return KM_OK;
}

// One lane per column (32 columns per warp) exposes the most independent
// (cluster, column) chains: the largest cluster is spread over d/32 warps, each
// with UPD_STAGES*UPD_ROWS rows in flight.  The 4-column variant is used only
// when the chains already outnumber the GPU many times over.
km_status launch_update_sums(const float* X, const uint32_t* perm, const uint32_t* cstart, uint32_t d,
                             uint32_t k, const float* C, float* Cn, float* dsq, double* objpart,
                             DevState* st, cudaStream_t s, const uint32_t* order) {
  if (d % 4 == 0 && reinterpret_cast<uintptr_t>(X) % 16 == 0) {
    const uint64_t ctas = (uint64_t)k * ((d + BLK_COLS - 1) / BLK_COLS);
    KM_CUDA_TRY(launch_pdl(update_sums_bulk_kernel, (unsigned)ctas, BLK_THREADS, BLK_SMEM, s, X, perm, cstart, d,
                           k, C, Cn, dsq, objpart, st, order));
    KM_CUDA_TRY(cudaGetLastError());
    return KM_OK;
  }
  const bool v4 = false;
  const uint32_t W = v4 ? 128u : 32u;
  const uint64_t warps = (uint64_t)k * ((d + W - 1) / W);
  const size_t smem = (size_t)UPD_STAGES * UPD_ROWS * W * sizeof(float);
  if (v4) {
    update_sums_kernel<4><<<(unsigned)warps, 32, smem, s>>>(X, perm, cstart, d, k, C, Cn, dsq, objpart, st);
  } else {
    update_sums_kernel<1><<<(unsigned)warps, 32, smem, s>>>(X, perm, cstart, d, k, C, Cn, dsq, objpart, st);
  }
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

// One warp per cluster: reference shift test (float sum over j ascending, then
// sqrtf(s) > tol, kmeans.cpp:190-200), FP64 move, FP64 objective of the
// cluster, new ||c||^2 and BF16 copies; then C <- Cn.  The block that finishes
// last (a ticket in DevState) then ends the iteration: deterministic
// reductions over the clusters, the stop decision, counters for the next
// iteration.
__global__ void __launch_bounds__(256)
finalize_kernel(const float* __restrict__ Cn, float* __restrict__ C,
                const float* __restrict__ dsq, const double* __restrict__ objpart,
                const uint32_t* __restrict__ counts, int32_t empty_excl,
                uint32_t d, uint32_t dp, uint32_t k, float tol,
                float* __restrict__ cn2, __nv_bfloat16* __restrict__ Cb,
                __nv_bfloat16* __restrict__ Clo, float* __restrict__ Ct,
                double* __restrict__ shift_c, double* __restrict__ obj_c,
                DevState* st, LoopConsts lc) {
  griddep_wait();
  if (st->done) return;
  __shared__ double s_obj[256];
  __shared__ double s_sh[256];
  __shared__ float s_cm[256];
  __shared__ int is_last;
  const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c < k) {
    const uint64_t base = (uint64_t)c * d;
    // Reference GPU rule (src/kernels/distances.cu:588-599): an empty cluster's
    // distance is +inf from then on, so it is never chosen again.  Its norm and
    // its column of Ct become +inf; its (zero) centroid row stays finite.
    const bool excl = empty_excl && counts[c] == 0u;
    double nrm = 0.0, mv = 0.0, ob = 0.0;
    float s = 0.0f;   // reference shift test: float sum of dsq over j ascending
    // 128 columns per pass, j = j0 + lane + 32 q: all of the pass's loads are
    // issued before its arithmetic; the ordered float sum takes the terms from
    // the lanes by shuffle (j ascending), the FP64 sums keep each lane's order.
    for (uint32_t j0 = 0; j0 < dp; j0 += 128) {
      float v[4], co[4], dq[4];
      double op[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t j = j0 + (uint32_t)lane + 32u * q;
        const bool in = j < d;
        v[q] = in ? Cn[base + j] : 0.0f;
        co[q] = in ? C[base + j] : 0.0f;
        dq[q] = in ? dsq[base + j] : 0.0f;
        op[q] = in ? objpart[base + j] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t j = j0 + (uint32_t)lane + 32u * q;
        if (j < d) {
          nrm += (double)v[q] * v[q];
          const double t = (double)v[q] - (double)co[q];
          mv += t * t;
          ob += op[q];
          Ct[(uint64_t)j * k + c] = excl ? f_inf() : v[q];
          C[base + j] = v[q];
        }
        if (Cb && j < dp) {
          const __nv_bfloat16 hi = __float2bfloat16_rn(v[q]);
          Cb[(uint64_t)c * dp + j] = hi;
          if (Clo) Clo[(uint64_t)c * dp + j] = __float2bfloat16_rn(v[q] - __bfloat162float(hi));
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t jq = j0 + 32u * q;
#pragma unroll
        for (int l = 0; l < 32; ++l) {
          const float tq = __shfl_sync(0xffffffffu, dq[q], l);
          if (jq + (uint32_t)l < d) s = __fadd_rn(s, tq);
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
      mv += __shfl_xor_sync(0xffffffffu, mv, o);
      ob += __shfl_xor_sync(0xffffffffu, ob, o);
    }
    if (lane == 0) {
      if (sqrtf(s) > tol) st->moved = 1u;
      cn2[c] = excl ? f_inf() : (float)nrm;
      shift_c[c] = sqrt(mv);
      obj_c[c] = ob;
    }
  }
  // ---- last block: end of iteration ----
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = (atomicAdd(&st->fin_ticket, 1u) == gridDim.x - 1u) ? 1 : 0;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // other blocks' results: read past L1 (this SM may hold stale lines)
  volatile DevState* vs = st;
  double ob = 0.0, sh = 0.0;
  float cm = 0.0f;
  const uint32_t per = (k + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per, e = min(k, b + per);
  for (uint32_t cc = b; cc < e; ++cc) {
    ob += __ldcg(obj_c + cc);
    sh = fmax(sh, __ldcg(shift_c + cc));
    const float v = __ldcg(cn2 + cc);
    if (v < f_inf()) cm = fmaxf(cm, sqrtf(v));   // excluded (empty) clusters hold +inf
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
    const uint32_t it = vs->iter + 1;
    vs->iter = it;
    vs->objective = s_obj[0];
    vs->max_shift = s_sh[0];
    vs->cmax = s_cm[0] * 1.000001f;
    const double score = s_obj[0] - vs->sum_x2;
    vs->score = score;
    bool stop = false;
    if (lc.conv == KM_CONV_SHIFT) {
      if (it > 1 && vs->moved == 0u) { vs->converged_iter = it; stop = true; }
    } else if (lc.conv == KM_CONV_SCORE) {
      if (it < lc.maxiter && it > 1 && fabs(score - vs->last_score) < (double)lc.tol) {
        vs->converged_iter = it; stop = true;
      }
      vs->last_score = score;
    }
    vs->moved = 0u;
    if (it >= lc.maxiter) stop = true;
    if (stop) vs->done = 1u;
    vs->fin_ticket = 0u;
  }
}

}  // namespace km
