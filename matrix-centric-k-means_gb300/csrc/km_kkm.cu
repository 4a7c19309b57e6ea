// Kernel k-means for sm_103a (the reference's current "popcorn" GPU path).
//
//  (a) kernel matrix  K = f(X X^T)  (src/kernels/kernels.cuh:43-118, :568-718):
//      tcgen05 GEMM (BF16 or split-BF16x3 operands, FP32 accumulators in TMEM,
//      TMA-fed) or SIMT FP32 GEMM, with the kernel function applied in the
//      epilogue and K (and diag K) stored once.  The reference stores
//      B = -2 f(.) and runs an n^2 Thrust pass; here f is fused and the -2 is
//      folded into the distance.
//  (c) one iteration (src/kmeans.cu:772-1073, src/kernels/distances.cu:895-1002):
//      E = K V^T streamed over the rows of K once (E[i,c] = sum_{j in c} K_ij,
//      per-lane shared-memory bins, deterministic order), ctilde_c =
//      (1/|c|^2) sum_{i in c} E[i,c] = diag(V K V^T) in FP64 over the
//      label-sorted permutation, then D[i,c] = -2 E[i,c]/|c| + ctilde_c
//      (ctilde_c == 0 -> +inf, distances.cu:588-599), argmin keeping the lowest
//      index from (0, FLT_MAX) (kmeans.cu:923-936), score = sum_i min_c D
//      (kmeans.cu:1054-1061; it leaves out K_ii), stop on |score - last| < tol
//      from iteration 2 when checking (kmeans.cu:1064-1073).
#include "km_lloyd.cuh"

#include <cudaTypedefs.h>
#include <cmath>
#include <cstring>
#include <cfloat>
#include <new>

namespace km {

__global__ void round_robin_labels_kernel(uint32_t* labels, uint64_t n, uint32_t k);  // km_capi.cu

struct KFn {
  int kind;        // km_kernel_fn
  float gamma, coef, inv2s2;
  int degree;
};

__device__ __forceinline__ float kfn_apply(const KFn& f, float dot, float ni, float nj) {
  switch (f.kind) {
    case KM_KERNEL_LINEAR: return dot;
    case KM_KERNEL_POLY: {
      const float b = fmaf(f.gamma, dot, f.coef);
      float r = 1.0f;
      for (int e = 0; e < f.degree; ++e) r *= b;
      return r;
    }
    case KM_KERNEL_SIGMOID: return tanhf(fmaf(f.gamma, dot, f.coef));
    default: {
      const float d2 = fmaxf(ni + nj - 2.0f * dot, 0.0f);
      return expf(-d2 * f.inv2s2);
    }
  }
}

// The same functions with the kind fixed at compile time (one small body per
// kernel-matrix instantiation; the tensor-core epilogue unrolls it per column).
template <int KIND>
__device__ __forceinline__ float kfn_apply_k(const KFn& f, float dot, float ni, float nj) {
  if constexpr (KIND == KM_KERNEL_LINEAR) {
    return dot;
  } else if constexpr (KIND == KM_KERNEL_POLY) {
    const float b = fmaf(f.gamma, dot, f.coef);
    if (f.degree == 2) return b * b;          // the loop's 1 * b * b, without the loop
    float r = 1.0f;
#pragma unroll 1
    for (int e = 0; e < f.degree; ++e) r *= b;
    return r;
  } else if constexpr (KIND == KM_KERNEL_SIGMOID) {
    return tanhf(fmaf(f.gamma, dot, f.coef));
  } else {
    const float d2 = fmaxf(ni + nj - 2.0f * dot, 0.0f);
    return expf(-d2 * f.inv2s2);
  }
}

// ||x_i||^2 of the operands the tensor cores see (hi, or hi + lo): the
// Gaussian epilogue's ||x_i||^2 + ||x_j||^2 - 2 x_i.x_j is then the squared
// distance of those operands (K_ii = 1 exactly), instead of mixing FP32 norms
// with a BF16 dot product.
__global__ void kmat_operand_norms_kernel(const __nv_bfloat16* __restrict__ Xb,
                                          const __nv_bfloat16* __restrict__ Xlo, uint64_t n,
                                          uint32_t dp, float* __restrict__ out) {
  const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  double s = 0.0;
  for (uint32_t j = lane; j < dp; j += 32) {
    float v = __bfloat162float(Xb[r * dp + j]);
    if (Xlo) v += __bfloat162float(Xlo[r * dp + j]);
    s += (double)v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[r] = (float)s;
}

template <bool OUT_BF16>
__device__ __forceinline__ void kstore(void* K, uint64_t idx, float v) {
  if (OUT_BF16) reinterpret_cast<__nv_bfloat16*>(K)[idx] = __float2bfloat16_rn(v);
  else reinterpret_cast<float*>(K)[idx] = v;
}

// ---------------------------------------------------------------------------
// (a) SIMT FP32 kernel-matrix GEMM: 128 x 128 tiles, 256 threads, 8 x 8
// micro-tiles, K chunks of 16 through shared memory.  Builds rows
// [row0, row_end) of K into K (row stride n, first row = row0); with `stop`
// set it does nothing once the fit has stopped (panels rebuilt per iteration).
// ---------------------------------------------------------------------------
template <bool OUT_BF16>
__global__ void __launch_bounds__(256)
kmat_f32_kernel(const float* __restrict__ X, const float* __restrict__ xn2, uint64_t n, uint32_t d,
                uint64_t row0, uint64_t row_end, KFn f, void* __restrict__ K, float* __restrict__ diag,
                const DevState* stop) {
  if (stop && stop->done) return;
  __shared__ __align__(16) float As[16][128 + 4];
  __shared__ __align__(16) float Bs[16][128 + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const uint64_t m0 = row0 + (uint64_t)blockIdx.y * 128, c0 = (uint64_t)blockIdx.x * 128;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  for (uint32_t kc = 0; kc < d; kc += 16) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int idx = e * 256 + tid;
      const int r = idx >> 4, kk = idx & 15;
      const uint32_t col = kc + kk;
      As[kk][r] = (m0 + r < row_end && col < d) ? X[(m0 + r) * d + col] : 0.0f;
      Bs[kk][r] = (c0 + r < n && col < d) ? X[(c0 + r) * d + col] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[8], b[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) { a[i] = As[kk][ty * 8 + i]; b[i] = Bs[kk][tx * 8 + i]; }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint64_t row = m0 + ty * 8 + i;
    if (row >= row_end) continue;
    const float ni = xn2[row];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint64_t col = c0 + tx * 8 + j;
      if (col >= n) continue;
      const float v = kfn_apply(f, acc[i][j], ni, xn2[col]);
      kstore<OUT_BF16>(K, (row - row0) * n + col, v);
      if (diag && row == col) diag[row] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// (a) tcgen05 kernel-matrix GEMM.  Persistent CTAs walk 128 x 256 output
// tiles; per K-block the A tile (128 rows) and B tile (256 rows) of the BF16
// copy of X (hi, and lo for X3) come in by TMA into a ring of stages; one
// thread issues the MMAs into a TMEM accumulator (two buffers of 256
// columns); eight epilogue warps (two sets, one per buffer; warp w on TMEM
// lanes 32*(w%4)) read the accumulator 64 columns at a time, apply f and store
// K.  Every wait is bounded (2 s) and a timeout raises KM_DEVERR_TIMEOUT after
// draining this CTA's copies and MMAs.  The kernel builds rows
// [prow0, prow_end) of K into K (row stride n, first row = prow0): all of K,
// or one panel of it; with skip_done it does nothing once the fit has stopped.
//
// Symmetry: K is symmetric, so only tiles (row tile mi, column block nj) with
// mi/2 <= nj are computed (the 256-row blocks on or above the diagonal), as
// the reference's SYRK path builds one triangle and mirrors it
// (src/kernels/kernels.cuh:596-649).  A tile strictly above the diagonal
// (mi/2 < nj) also stores its transpose: each warp holds 32 consecutive rows
// in its lanes, so column c of the tile leaves as one contiguous run of row
// c of K.  The tiles come from a list built on the host (kmat_tile_list):
// (mi, nj | direct << 30 | mirror << 31), `direct` when the tile's own rows
// lie in [prow0, prow_end) and `mirror` when its transposed rows do, so a
// panel receives exactly the values the whole matrix holds.  This halves the
// MMA work of a resident build.
// ---------------------------------------------------------------------------
namespace {
constexpr int KM_M = 128, KM_N = 256;
constexpr uint32_t KA_BYTES = KM_M * 128;   // 64-column BF16 K-block of A
constexpr uint32_t KB_BYTES = KM_N * 128;   // 64-column BF16 K-block of B
constexpr uint64_t KWAIT_NS = 2000000000ull;

constexpr uint64_t KM_GROUP = 16;   // row tiles per raster group of the kernel-matrix build


constexpr uint32_t KM_STG_BYTES = 8u * 32u * 32u * 4u;   // epilogue staging tiles, one per epilogue warp

struct KmSmem {
  uint64_t full[8];
  uint64_t empty[8];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t tdone;
  uint32_t tmem_base;
  int abort;
};
}  // namespace

template <bool X3, bool OUT_BF16, int KIND>
__global__ void __launch_bounds__(384, 1)
kmat_tc_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tAlo,
               const __grid_constant__ CUtensorMap tB, const __grid_constant__ CUtensorMap tBlo,
               const float* __restrict__ xn2, uint64_t n, uint64_t prow0, uint64_t prow_end, uint32_t KB,
               uint32_t S, KFn f, void* __restrict__ K, float* __restrict__ diag, int vec, int skip_done,
               DevState* st, const uint32_t* __restrict__ tlist, uint64_t ntiles) {
  if (skip_done && st->done) return;   // uniform over the grid: written by an earlier launch
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const uint32_t stage_bytes = (KA_BYTES + KB_BYTES) * (X3 ? 2u : 1u);
  float* stg_all = reinterpret_cast<float*>(smem + (size_t)S * stage_bytes);    // [8 warps][32][32]
  KmSmem* ts = reinterpret_cast<KmSmem*>(smem + (size_t)S * stage_bytes + KM_STG_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < S; ++s) { mbar_init(&ts->full[s], 1); mbar_init(&ts->empty[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&ts->tfull[b], 1); mbar_init(&ts->tempty[b], 4); }
    mbar_init(&ts->tdone, 1);
    ts->abort = 0;
    mbar_fence_init();
  }
  if (warp == 2) tmem_alloc(&ts->tmem_base, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = ts->tmem_base;
  volatile int* abort_flag = &ts->abort;
  auto fail = [&](uint32_t where) {
    ts->abort = 1;
    if (atomicOr(&st->err, KM_DEVERR_TIMEOUT) == 0u) st->err_where = 100u + where;
  };
  // tile t -> (mi, nj) from the list (groups of KM_GROUP row tiles, column
  // blocks in the inner loop, so that a group's A tiles stay in L2)
  if (warp == 0) {
    if (lane == 0) {
      uint64_t u = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const uint64_t mi = tlist[2 * tile], nj = tlist[2 * tile + 1] & 0x3fffffffu;
        for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
          const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
          if (!mbar_wait_bounded(&ts->empty[s], ph ^ 1u, abort_flag, KWAIT_NS)) { fail(1); ok = false; break; }
          mbar_arrive_expect_tx(&ts->full[s], stage_bytes);
          uint8_t* dst = smem + (size_t)s * stage_bytes;
          tma_load_2d(dst, &tA, (int)(kb * 64), (int)(mi * KM_M), &ts->full[s]);
          tma_load_2d(dst + KA_BYTES, &tB, (int)(kb * 64), (int)(nj * KM_N), &ts->full[s]);
          if (X3) {
            tma_load_2d(dst + KA_BYTES + KB_BYTES, &tAlo, (int)(kb * 64), (int)(mi * KM_M), &ts->full[s]);
            tma_load_2d(dst + 2 * KA_BYTES + KB_BYTES, &tBlo, (int)(kb * 64), (int)(nj * KM_N), &ts->full[s]);
          }
        }
      }
      volatile int no_abort = 0;
      const uint64_t first = u > S ? u - S : 0;
      for (uint64_t v = first; v < u; ++v)
        mbar_wait_bounded(&ts->full[v % S], (uint32_t)((v / S) & 1u), &no_abort, KWAIT_NS);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(KM_M, KM_N);
      const uint32_t s0 = smem_u32(smem);
      uint64_t u = 0, t = 0;
      bool ok = true, issued = false;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++t) {
        const uint32_t buf = (uint32_t)(t & 1u), use = (uint32_t)(t >> 1);
        if (!mbar_wait_bounded(&ts->tempty[buf], (use & 1u) ^ 1u, abort_flag, KWAIT_NS)) { fail(2); ok = false; break; }
        tc_fence_after();
        const uint32_t dt = tmem_base + buf * 256u;
        for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
          const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
          if (!mbar_wait_bounded(&ts->full[s], ph, abort_flag, KWAIT_NS)) { fail(3); ok = false; break; }
          tc_fence_after();
          const uint32_t a0 = s0 + s * stage_bytes, b0 = a0 + KA_BYTES;
#pragma unroll
          for (uint32_t kk = 0; kk < 4; ++kk) {
            const uint64_t ad = smem_desc_sw128(a0 + kk * 32u);
            const uint64_t bd = smem_desc_sw128(b0 + kk * 32u);
            tc_mma_bf16(dt, ad, bd, idesc, (kb | kk) != 0u ? 1u : 0u);
            if (X3) {
              const uint64_t adl = smem_desc_sw128(a0 + KA_BYTES + KB_BYTES + kk * 32u);
              const uint64_t bdl = smem_desc_sw128(a0 + 2 * KA_BYTES + KB_BYTES + kk * 32u);
              tc_mma_bf16(dt, ad, bdl, idesc, 1u);
              tc_mma_bf16(dt, adl, bd, idesc, 1u);
            }
          }
          tc_commit(&ts->empty[s]);
          issued = true;
        }
        if (!ok) break;
        tc_commit(&ts->tfull[buf]);
      }
      if (issued) {
        tc_commit(&ts->tdone);
        volatile int no_abort = 0;
        mbar_wait_bounded(&ts->tdone, 0, &no_abort, KWAIT_NS);
      }
    }
  } else if (warp >= 4) {
    const int q = warp & 3, set = (warp - 4) >> 2;
    const uint32_t r = (uint32_t)q * 32u + (uint32_t)lane;
    const uint32_t tbase = tmem_base + (((uint32_t)q * 32u) << 16) + (uint32_t)set * 256u;
    uint64_t t = (uint64_t)set;
    for (uint64_t tile = blockIdx.x + (uint64_t)set * gridDim.x; tile < ntiles;
         tile += 2ull * gridDim.x, t += 2) {
      const uint64_t mi = tlist[2 * tile];
      const uint32_t njf = tlist[2 * tile + 1];
      const uint64_t nj = njf & 0x3fffffffu;
      const bool direct = (njf >> 30) & 1u, mirror = (njf >> 31) & 1u;
      const uint64_t row = mi * KM_M + r, c0 = nj * KM_N;
      const bool row_in = row < n;
      const float ni = row_in ? xn2[row] : 0.0f;
      // column norms only matter for the Gaussian kernel (broadcast loads)
      auto colnorm = [&](uint64_t c) -> float {
        return (KIND == KM_KERNEL_GAUSSIAN && c < n) ? __ldg(xn2 + c) : 0.0f;
      };
      const bool okw = mbar_wait_bounded(&ts->tfull[set], (uint32_t)(t >> 1) & 1u, abort_flag, KWAIT_NS);
      if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(4); break; }
      tc_fence_after();
      // Values of this lane's row go to the warp's staging tile (32 rows x 32
      // columns, 16-byte chunks XOR-swizzled by row) and leave as whole
      // 128-byte row segments: eight lanes per row, four rows per store.
      float* stg = stg_all + (size_t)(warp - 4) * 32 * 32;
      const uint64_t row0 = mi * KM_M + (uint64_t)q * 32u;  // first row of this warp
#pragma unroll 1
      for (uint32_t pr = 0; pr < KM_N / 64; ++pr) {       // not unrolled: the body is large
        uint32_t acc[64];
        tmem_ld_32x32b_x64(tbase + pr * 64u, acc);
        tmem_ld_wait();
        if (pr + 1 == KM_N / 64) {
          // the accumulator's last columns are in registers: the MMAs of the
          // next tile on this buffer may start while this one is stored
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ts->tempty[set]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint64_t cb = c0 + pr * 64u + (uint32_t)h * 32u;
          __syncwarp();                                  // the previous half has been read back
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            float4 o;
            o.x = kfn_apply_k<KIND>(f, __uint_as_float(acc[h * 32 + 4 * c + 0]), ni, colnorm(cb + 4 * c + 0));
            o.y = kfn_apply_k<KIND>(f, __uint_as_float(acc[h * 32 + 4 * c + 1]), ni, colnorm(cb + 4 * c + 1));
            o.z = kfn_apply_k<KIND>(f, __uint_as_float(acc[h * 32 + 4 * c + 2]), ni, colnorm(cb + 4 * c + 2));
            o.w = kfn_apply_k<KIND>(f, __uint_as_float(acc[h * 32 + 4 * c + 3]), ni, colnorm(cb + 4 * c + 3));
            if (diag && direct && row >= prow0 && row < prow_end) {
              if (cb + 4 * c + 0 == row) diag[row] = o.x;
              if (cb + 4 * c + 1 == row) diag[row] = o.y;
              if (cb + 4 * c + 2 == row) diag[row] = o.z;
              if (cb + 4 * c + 3 == row) diag[row] = o.w;
            }
            *reinterpret_cast<float4*>(stg + lane * 32 + ((c ^ (lane & 7)) * 4)) = o;
            if (mirror && row_in) {
              // transposed: K[gcol][row]; the warp's lanes write one contiguous run
              const float ov[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
              for (int qq = 0; qq < 4; ++qq) {
                const uint64_t gcol = cb + 4 * c + qq;
                if (gcol >= prow0 && gcol < prow_end) {
                  if (OUT_BF16)
                    reinterpret_cast<__nv_bfloat16*>(K)[(gcol - prow0) * n + row] = __float2bfloat16_rn(ov[qq]);
                  else
                    reinterpret_cast<float*>(K)[(gcol - prow0) * n + row] = ov[qq];
                }
              }
            }
          }
          __syncwarp();
          if (!direct) continue;                         // the staged copy is stored only for own rows
#pragma unroll
          for (int step = 0; step < 8; ++step) {
            const uint32_t rr = (uint32_t)step * 4u + ((uint32_t)lane >> 3);   // row within the warp's 32
            const uint32_t ch = (uint32_t)lane & 7u;                           // 16-byte chunk of the row
            const float4 o = *reinterpret_cast<const float4*>(stg + rr * 32 + ((ch ^ (rr & 7u)) * 4u));
            const uint64_t grow = row0 + rr, gcol = cb + ch * 4u;
            if (grow < prow0 || grow >= prow_end) continue;
            if (OUT_BF16) {
              __nv_bfloat16* Kp = reinterpret_cast<__nv_bfloat16*>(K) + (grow - prow0) * n + gcol;
              if (vec && gcol + 3 < n) {
                const __nv_bfloat162 a = __floats2bfloat162_rn(o.x, o.y), b = __floats2bfloat162_rn(o.z, o.w);
                uint2 u;
                u.x = *reinterpret_cast<const uint32_t*>(&a);
                u.y = *reinterpret_cast<const uint32_t*>(&b);
                *reinterpret_cast<uint2*>(Kp) = u;
              } else {
                if (gcol + 0 < n) Kp[0] = __float2bfloat16_rn(o.x);
                if (gcol + 1 < n) Kp[1] = __float2bfloat16_rn(o.y);
                if (gcol + 2 < n) Kp[2] = __float2bfloat16_rn(o.z);
                if (gcol + 3 < n) Kp[3] = __float2bfloat16_rn(o.w);
              }
            } else {
              float* Kp = reinterpret_cast<float*>(K) + (grow - prow0) * n + gcol;
              if (vec && gcol + 3 < n) {
                *reinterpret_cast<float4*>(Kp) = o;
              } else {
                if (gcol + 0 < n) Kp[0] = o.x;
                if (gcol + 1 < n) Kp[1] = o.y;
                if (gcol + 2 < n) Kp[2] = o.z;
                if (gcol + 3 < n) Kp[3] = o.w;
              }
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(tmem_base, 512);
}

// ---------------------------------------------------------------------------
// (c') E = K V^T without K in memory.  The columns of K are taken in
// label-sorted order: the B operand is a copy of the points permuted by the
// stable label sort (perm), so cluster c owns the contiguous columns
// [cstart[c], cstart[c+1]) and E[i,c] is a running sum along row i of
// f(x_i . x_perm(j)), j ascending.  Persistent CTAs take whole 128-row blocks
// of K and sweep its 256-column tiles in order: warp 0 the TMA producer,
// warp 1 the MMA issuer into two TMEM accumulators, warp 2 the TMEM
// allocation, warps 4-7 the epilogue with one row per thread (TMEM lane
// quadrant warp % 4).  Per 64-column chunk the epilogue applies f and, when no
// cluster ends inside the chunk, adds the chunk's pairwise-tree sum to the
// row's running sum; a chunk holding a boundary goes column by column through
// a shared staging tile.  Each E[i,c] is written once, by its row's thread.
// The order of the sum is fixed by the data (deterministic); it is not the
// resident V.K kernel's lane-interleaved order.  Waits are bounded as in
// kmat_tc_kernel.
// ---------------------------------------------------------------------------
namespace {
constexpr uint32_t KF_STG_BYTES = 4u * 64u * 32u * 4u;   // per epilogue warp: 64 columns x 32 rows

struct KfSmem {
  uint64_t full[8];
  uint64_t empty[8];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t tdone;
  uint32_t tmem_base;
  int abort;
};
}  // namespace

template <bool X3, int KIND>
__global__ void __launch_bounds__(256, 1)
kkm_fused_tc_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tAlo,
                    const __grid_constant__ CUtensorMap tB, const __grid_constant__ CUtensorMap tBlo,
                    const float* __restrict__ xn2, const float* __restrict__ xn2p, uint64_t n, uint32_t KB,
                    uint32_t S, KFn f, const uint32_t* __restrict__ cstart, uint32_t k, float* __restrict__ E,
                    DevState* st) {
  if (st->done) return;   // uniform over the grid: written by an earlier launch
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const uint32_t stage_bytes = (KA_BYTES + KB_BYTES) * (X3 ? 2u : 1u);
  float* stg_all = reinterpret_cast<float*>(smem + (size_t)S * stage_bytes);   // [4 warps][64][32]
  KfSmem* ts = reinterpret_cast<KfSmem*>(smem + (size_t)S * stage_bytes + KF_STG_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t mt = (n + KM_M - 1) / KM_M, nt = (n + KM_N - 1) / KM_N;
  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < S; ++s) { mbar_init(&ts->full[s], 1); mbar_init(&ts->empty[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&ts->tfull[b], 1); mbar_init(&ts->tempty[b], 4); }
    mbar_init(&ts->tdone, 1);
    ts->abort = 0;
    mbar_fence_init();
  }
  if (warp == 2) tmem_alloc(&ts->tmem_base, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = ts->tmem_base;
  volatile int* abort_flag = &ts->abort;
  auto fail = [&](uint32_t where) {
    ts->abort = 1;
    if (atomicOr(&st->err, KM_DEVERR_TIMEOUT) == 0u) st->err_where = 110u + where;
  };
  if (warp == 0) {
    if (lane == 0) {
      uint64_t u = 0;
      bool ok = true;
      for (uint64_t mi = blockIdx.x; mi < mt && ok; mi += gridDim.x) {
        for (uint64_t nj = 0; nj < nt && ok; ++nj) {
          for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
            const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
            if (!mbar_wait_bounded(&ts->empty[s], ph ^ 1u, abort_flag, KWAIT_NS)) { fail(1); ok = false; break; }
            mbar_arrive_expect_tx(&ts->full[s], stage_bytes);
            uint8_t* dst = smem + (size_t)s * stage_bytes;
            tma_load_2d(dst, &tA, (int)(kb * 64), (int)(mi * KM_M), &ts->full[s]);
            tma_load_2d(dst + KA_BYTES, &tB, (int)(kb * 64), (int)(nj * KM_N), &ts->full[s]);
            if (X3) {
              tma_load_2d(dst + KA_BYTES + KB_BYTES, &tAlo, (int)(kb * 64), (int)(mi * KM_M), &ts->full[s]);
              tma_load_2d(dst + 2 * KA_BYTES + KB_BYTES, &tBlo, (int)(kb * 64), (int)(nj * KM_N), &ts->full[s]);
            }
          }
        }
      }
      volatile int no_abort = 0;
      const uint64_t first = u > S ? u - S : 0;
      for (uint64_t v = first; v < u; ++v)
        mbar_wait_bounded(&ts->full[v % S], (uint32_t)((v / S) & 1u), &no_abort, KWAIT_NS);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(KM_M, KM_N);
      const uint32_t s0 = smem_u32(smem);
      uint64_t u = 0, t = 0;
      bool ok = true, issued = false;
      for (uint64_t mi = blockIdx.x; mi < mt && ok; mi += gridDim.x) {
        for (uint64_t nj = 0; nj < nt && ok; ++nj, ++t) {
          const uint32_t buf = (uint32_t)(t & 1u), use = (uint32_t)(t >> 1);
          if (!mbar_wait_bounded(&ts->tempty[buf], (use & 1u) ^ 1u, abort_flag, KWAIT_NS)) { fail(2); ok = false; break; }
          tc_fence_after();
          const uint32_t dt = tmem_base + buf * 256u;
          for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
            const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
            if (!mbar_wait_bounded(&ts->full[s], ph, abort_flag, KWAIT_NS)) { fail(3); ok = false; break; }
            tc_fence_after();
            const uint32_t a0 = s0 + s * stage_bytes, b0 = a0 + KA_BYTES;
#pragma unroll
            for (uint32_t kk = 0; kk < 4; ++kk) {
              const uint64_t ad = smem_desc_sw128(a0 + kk * 32u);
              const uint64_t bd = smem_desc_sw128(b0 + kk * 32u);
              tc_mma_bf16(dt, ad, bd, idesc, (kb | kk) != 0u ? 1u : 0u);
              if (X3) {
                const uint64_t adl = smem_desc_sw128(a0 + KA_BYTES + KB_BYTES + kk * 32u);
                const uint64_t bdl = smem_desc_sw128(a0 + 2 * KA_BYTES + KB_BYTES + kk * 32u);
                tc_mma_bf16(dt, ad, bdl, idesc, 1u);
                tc_mma_bf16(dt, adl, bd, idesc, 1u);
              }
            }
            tc_commit(&ts->empty[s]);
            issued = true;
          }
          if (!ok) break;
          tc_commit(&ts->tfull[buf]);
        }
      }
      if (issued) {
        tc_commit(&ts->tdone);
        volatile int no_abort = 0;
        mbar_wait_bounded(&ts->tdone, 0, &no_abort, KWAIT_NS);
      }
    }
  } else if (warp >= 4) {
    const int q = warp & 3;
    const uint32_t tq = tmem_base + (((uint32_t)q * 32u) << 16);
    float* stg = stg_all + (size_t)q * 64 * 32;
    auto colnorm = [&](uint64_t j) -> float {
      return (KIND == KM_KERNEL_GAUSSIAN) ? __ldg(xn2p + j) : 0.0f;
    };
    uint64_t t = 0;
    bool ok = true;
    for (uint64_t mi = blockIdx.x; mi < mt && ok; mi += gridDim.x) {
      const uint64_t row = mi * KM_M + (uint64_t)q * 32u + (uint64_t)lane;
      const bool valid = row < n;
      const float ni = (KIND == KM_KERNEL_GAUSSIAN && valid) ? xn2[row] : 0.0f;
      float* Er = E + row * k;
      uint32_t cur = 0;                 // cluster of the running sum
      uint64_t nb = cstart[1];          // first column after cluster cur
      float run = 0.0f;
      for (uint64_t nj = 0; nj < nt; ++nj, ++t) {
        const uint32_t buf = (uint32_t)(t & 1u);
        const bool okw = mbar_wait_bounded(&ts->tfull[buf], (uint32_t)(t >> 1) & 1u, abort_flag, KWAIT_NS);
        if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(4); ok = false; break; }
        tc_fence_after();
        for (uint32_t pr = 0; pr < KM_N / 64; ++pr) {
          const uint64_t j0 = nj * KM_N + pr * 64u;
          if (j0 >= n) break;                                   // warp-uniform
          uint32_t acc[64];
          tmem_ld_32x32b_x64(tq + buf * 256u + pr * 64u, acc);
          tmem_ld_wait();
          if (nb >= j0 + 64 && j0 + 64 <= n) {
            float v[64];
#pragma unroll
            for (int c = 0; c < 64; ++c) v[c] = kfn_apply_k<KIND>(f, __uint_as_float(acc[c]), ni, colnorm(j0 + c));
#pragma unroll
            for (int w = 32; w >= 1; w >>= 1)
#pragma unroll
              for (int c = 0; c < w; ++c) v[c] += v[c + w];
            run += v[0];
          } else {
            // a cluster ends inside this chunk (or the points do): column by column
#pragma unroll
            for (int c = 0; c < 64; ++c)
              stg[c * 32 + lane] = (j0 + c < n) ? kfn_apply_k<KIND>(f, __uint_as_float(acc[c]), ni, colnorm(j0 + c))
                                                : 0.0f;
            __syncwarp();
            const uint32_t cols = (uint32_t)((n - j0) < 64 ? (n - j0) : 64);
#pragma unroll 1
            for (uint32_t c = 0; c < cols; ++c) {
              const uint64_t j = j0 + c;
              while (j == nb) {                                 // cluster cur ended before column j
                if (valid) Er[cur] = run;
                run = 0.0f;
                ++cur;
                nb = cstart[cur + 1];
              }
              run += stg[c * 32 + lane];
            }
            __syncwarp();
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ts->tempty[buf]);
      }
      if (!ok) break;
      // the last non-empty cluster, then the empty ones after it
      for (; cur < k; ++cur) {
        if (valid) Er[cur] = run;
        run = 0.0f;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(tmem_base, 512);
}

// Label-sorted copies of the tensor-core operands and of their norms: row j of
// a copy is row perm[j] of the original.  One warp per row, 16-byte copies
// (dp is a multiple of 64).
__global__ void kkm_permute_points_kernel(const __nv_bfloat16* __restrict__ Xb,
                                          const __nv_bfloat16* __restrict__ Xlo, const float* __restrict__ xn2,
                                          const uint32_t* __restrict__ perm, uint64_t n, uint32_t dp,
                                          __nv_bfloat16* __restrict__ Xbp, __nv_bfloat16* __restrict__ Xlop,
                                          float* __restrict__ xn2p, const DevState* st) {
  if (st->done) return;
  const uint64_t j = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  const uint64_t src = perm[j];
  const uint32_t w16 = dp / 8;
  const uint4* a = reinterpret_cast<const uint4*>(Xb + src * dp);
  uint4* b = reinterpret_cast<uint4*>(Xbp + j * dp);
  for (uint32_t w = lane; w < w16; w += 32) b[w] = __ldg(a + w);
  if (Xlo) {
    const uint4* al = reinterpret_cast<const uint4*>(Xlo + src * dp);
    uint4* bl = reinterpret_cast<uint4*>(Xlop + j * dp);
    for (uint32_t w = lane; w < w16; w += 32) bl[w] = __ldg(al + w);
  }
  if (lane == 0) xn2p[j] = xn2[src];
}

// ---------------------------------------------------------------------------
// (c) E = K V^T.  One warp per row of K at a time; the labels of all n points
// are bytes (k <= 256), in shared memory when they fit next to the bins
// (GLAB false) or else read from a global byte copy (GLAB true, L2-resident);
// every lane accumulates its columns into private bins bins[c][lane] (no
// atomics, fixed order), then each lane reduces two bins over the 32 lanes in
// lane order.  K rows are read once with 16-byte (FP32) or 8-byte (BF16)
// loads.  Rows [row0, row_end) are done; K holds them from row row0 on (the
// whole matrix with row0 = 0, or one panel).  Both label sources give the
// same sums in the same order.
// ---------------------------------------------------------------------------
template <bool KBF16, bool GLAB>
__global__ void __launch_bounds__(512)
kkm_vk_kernel(const void* __restrict__ K, uint64_t n, uint32_t k, const uint32_t* __restrict__ labels,
              const uint8_t* __restrict__ lab8, uint64_t row0, uint64_t row_end, float* __restrict__ E,
              DevState* st) {
  if (st->done) return;
  extern __shared__ __align__(16) uint8_t kk_smem[];
  const uint8_t* lab = GLAB ? lab8 : kk_smem;                        // n bytes
  float* bins = reinterpret_cast<float*>(kk_smem + (GLAB ? 0ull : ((n + 15) & ~15ull)));  // [warps][k][32]
  if (!GLAB) {
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) kk_smem[i] = (uint8_t)labels[i];
    __syncthreads();
  }
  auto lab4 = [&](uint64_t j) -> uint32_t {     // labels j..j+3 (j % 4 == 0)
    return GLAB ? __ldg(reinterpret_cast<const uint32_t*>(lab + j)) : *reinterpret_cast<const uint32_t*>(lab + j);
  };
  auto lab1 = [&](uint64_t j) -> uint32_t { return GLAB ? (uint32_t)__ldg(lab + j) : (uint32_t)lab[j]; };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* B = bins + (size_t)warp * k * 32;
  for (uint32_t c = 0; c < k; ++c) B[c * 32 + lane] = 0.0f;
  __syncwarp();
  const uint32_t wpb = blockDim.x >> 5;
  const uint64_t nw = (uint64_t)gridDim.x * wpb;
  for (uint64_t row = row0 + (uint64_t)blockIdx.x * wpb + warp; row < row_end; row += nw) {
    // With n % 4 == 0 every row starts 16-byte (FP32) / 8-byte (BF16)
    // aligned: lane l takes columns 4l..4l+3 of each 128-column stride.
    // Otherwise one column per lane with plain loads.
    const bool v4 = (n & 3) == 0;
    if (KBF16) {
      const __nv_bfloat16* Kr = reinterpret_cast<const __nv_bfloat16*>(K) + (row - row0) * n;
      if (v4) {
        // U loads in flight per lane before the (ordered) bin updates
        constexpr int U = 16;
        for (uint64_t j0 = (uint64_t)lane * 4; j0 < n; j0 += 128 * U) {
          uint2 raw[U];
          uint32_t l4[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const uint64_t j = j0 + 128ull * u;
            raw[u] = j < n ? __ldg(reinterpret_cast<const uint2*>(Kr + j)) : make_uint2(0u, 0u);
            l4[u] = j < n ? lab4(j) : 0u;
          }
#pragma unroll
          for (int u = 0; u < U; ++u) {
            if (j0 + 128ull * u >= n) break;
            const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw[u].x));
            const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw[u].y));
            B[((l4[u] >> 0) & 255u) * 32 + lane] += a.x;
            B[((l4[u] >> 8) & 255u) * 32 + lane] += a.y;
            B[((l4[u] >> 16) & 255u) * 32 + lane] += b.x;
            B[((l4[u] >> 24) & 255u) * 32 + lane] += b.y;
          }
        }
      } else {
        for (uint64_t j = lane; j < n; j += 32) B[lab1(j) * 32 + lane] += __bfloat162float(Kr[j]);
      }
    } else {
      const float* Kr = reinterpret_cast<const float*>(K) + (row - row0) * n;
      if (v4) {
        // U loads in flight per lane before the (ordered) bin updates
        constexpr int U = 8;
        for (uint64_t j0 = (uint64_t)lane * 4; j0 < n; j0 += 128 * U) {
          float4 v[U];
          uint32_t l4[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const uint64_t j = j0 + 128ull * u;
            v[u] = j < n ? __ldg(reinterpret_cast<const float4*>(Kr + j)) : make_float4(0.f, 0.f, 0.f, 0.f);
            l4[u] = j < n ? lab4(j) : 0u;
          }
#pragma unroll
          for (int u = 0; u < U; ++u) {
            if (j0 + 128ull * u >= n) break;
            B[((l4[u] >> 0) & 255u) * 32 + lane] += v[u].x;
            B[((l4[u] >> 8) & 255u) * 32 + lane] += v[u].y;
            B[((l4[u] >> 16) & 255u) * 32 + lane] += v[u].z;
            B[((l4[u] >> 24) & 255u) * 32 + lane] += v[u].w;
          }
        }
      } else {
        for (uint64_t j = lane; j < n; j += 32) B[lab1(j) * 32 + lane] += Kr[j];
      }
    }
    __syncwarp();
    for (uint32_t c = lane; c < k; c += 32) {
      float s = 0.0f;
      for (int l = 0; l < 32; ++l) s += B[c * 32 + l];
      E[row * k + c] = s;
    }
    __syncwarp();
    for (uint32_t c = 0; c < k; ++c) B[c * 32 + lane] = 0.0f;
    __syncwarp();
  }
}

// ctilde_c = (1/|c|^2) sum_{i in c} E[i, c] in FP64, one warp per cluster over
// its rows (label-sorted permutation), fixed reduction order.
__global__ void kkm_ctilde_kernel(const float* __restrict__ E, uint32_t k, const uint32_t* __restrict__ perm,
                                  const uint32_t* __restrict__ cstart, double* __restrict__ ct,
                                  DevState* st) {
  if (st->done) return;
  const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k) return;
  const uint32_t s0 = cstart[c], s1 = cstart[c + 1];
  double s = 0.0;
  for (uint32_t p = s0 + lane; p < s1; p += 32) s += (double)E[(uint64_t)perm[p] * k + c];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const double cnt = (double)(s1 - s0);
    ct[c] = (s1 > s0) ? s / (cnt * cnt) : 0.0;
  }
}

// D[i,c] = -2 E[i,c]/|c| + ctilde_c (ctilde == 0 -> +inf), argmin from
// (0, FLT_MAX) with strict '<', new label and min; per-block FP64 score partials.
__global__ void __launch_bounds__(256)
kkm_dist_kernel(const float* __restrict__ E, uint64_t n, uint32_t k, const uint32_t* __restrict__ counts,
                const double* __restrict__ ct, uint32_t* __restrict__ newlab,
                double* __restrict__ part, DevState* st) {
  if (st->done) return;
  extern __shared__ float kd_smem[];
  float* inv = kd_smem;            // -2/|c| (0 for empty clusters)
  float* add = kd_smem + k;        // ctilde (+inf where 0)
  for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) {
    const uint32_t cnt = counts[c];
    inv[c] = cnt ? -2.0f / (float)cnt : 0.0f;
    const float cf = (float)ct[c];
    add[c] = (cf == 0.0f) ? __int_as_float(0x7f800000) : cf;
  }
  __syncthreads();
  double acc = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float* e = E + i * k;
    float val = FLT_MAX;
    uint32_t key = 0;
    for (uint32_t c = 0; c < k; ++c) {
      const float v = fmaf(inv[c], e[c], add[c]);
      if (v < val) { val = v; key = c; }
    }
    newlab[i] = key;
    acc += (double)val;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// End of iteration: score (fixed-order sum of the block partials), the stop
// rule, label hand-over.
__global__ void kkm_control_kernel(const double* __restrict__ part, int np, LoopConsts lc,
                                   int check, DevState* st) {
  if (st->done) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < np; ++i) s += part[i];
    const uint32_t it = st->iter + 1;
    st->iter = it;
    st->score = s;
    st->objective = s;
    bool stop = false;
    if (it >= lc.maxiter) stop = true;
    else if (check && it > 1 && fabs(s - st->last_score) < (double)lc.tol) { st->converged_iter = it; stop = true; }
    st->last_score = s;
    if (stop) st->done = 1u;
  }
}

// dst8 (optional): the byte copy of the labels that the V.K kernel reads when
// they do not fit shared memory.
__global__ void kkm_copy_labels_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                       uint8_t* __restrict__ dst8, uint64_t n, DevState* st) {
  // runs after the control kernel: the labels of the final iteration are
  // copied too (the done flag is set by then), so only stop after copying.
  if (st->iter == 0) return;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    dst[i] = src[i];
    if (dst8) dst8[i] = (uint8_t)src[i];
  }
}

__global__ void kkm_label_bytes_kernel(const uint32_t* __restrict__ src, uint8_t* __restrict__ dst8, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    dst8[i] = (uint8_t)src[i];
}

}  // namespace km

using namespace km;

struct km_kkm {
  km_kkm_params p;
  LloydEngine eng;          // sort machinery, stream, state (no Lloyd buffers used)
  void* K = nullptr;        // n x n (resident) or panel x n (panels), float or bf16
  float* diag = nullptr;
  uint64_t panel = 0;       // rows of K per panel, 0 when K is resident
  uint8_t* lab8 = nullptr;  // byte labels for the V.K kernel when they do not fit shared memory
  bool glab = false;
  uint64_t kpi = 0;         // kernels launched per iteration
  // fused mode (no K): label-sorted operand copies and the fused kernel's plan
  bool fused = false;
  __nv_bfloat16* Xbp = nullptr;
  __nv_bfloat16* Xlop = nullptr;
  float* xn2p = nullptr;
  CUtensorMap fA{}, fAlo{}, fB{}, fBlo{};
  uint32_t fS = 0;
  size_t fsmem = 0;
  int fgrid = 0;
  float* E = nullptr;       // n x k
  double* ct = nullptr;
  uint32_t* lab = nullptr;  // current labels
  uint32_t* nlab = nullptr; // next labels
  double* part = nullptr;
  int dist_blocks = 0;
  size_t vk_smem = 0;
  uint32_t vk_warps = 8;          // warps per V.K block: as many as the bins leave room for (<= 16)
  bool ready = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int32_t* h_done = nullptr;
  double kbuild_ms = 0.0;   // device time of the last kernel-matrix build
};

namespace km {
namespace {

KFn make_kfn(const km_kkm_params& p) {
  KFn f;
  f.kind = p.kernel_fn;
  f.gamma = p.gamma;
  f.coef = p.coef;
  f.degree = p.degree;
  f.inv2s2 = (p.sigma > 0) ? (float)(1.0 / (2.0 * (double)p.sigma * p.sigma)) : 0.0f;
  return f;
}

km_status kfn_valid(int kind, int degree, float sigma) {
  if (kind < KM_KERNEL_LINEAR || kind > KM_KERNEL_GAUSSIAN) return KM_ERR_ARG;
  if (kind == KM_KERNEL_POLY && (degree < 1 || degree > 16)) return KM_ERR_ARG;
  if (kind == KM_KERNEL_GAUSSIAN && !(sigma > 0)) return KM_ERR_ARG;
  return KM_OK;
}

// Gaussian kernel on the tensor cores: norms of the BF16 operands (see
// kmat_operand_norms_kernel); they overwrite xn2, which the kernel-matrix path
// does not otherwise use.  Once per set of points.
km_status prepare_kmat_norms(LloydEngine& e, uint64_t n, const KFn& f, int precision) {
  if (precision == KM_PREC_FP32 || f.kind != KM_KERNEL_GAUSSIAN) return KM_OK;
  kmat_operand_norms_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, e.stream>>>(
      e.Xb, precision == KM_PREC_BF16X3 ? e.Xlo : nullptr, n, e.dp, e.xn2);
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

// Builds rows [row0, row_end) of K (and of diag) from points X (device,
// n x d) on the engine's stream into K (row stride n, first row = row0).  For
// the tensor-core precisions it uses the BF16 copies prepared by the engine
// and the operand norms of prepare_kmat_norms.  skip_done: the launch does
// nothing once the fit has stopped (panels rebuilt inside the iteration).
// Tiles of the symmetric tensor-core build of rows [row0, row_end): row tile
// mi (128 rows) against column block nj (256 columns) for mi / 2 <= nj, in
// groups of KM_GROUP row tiles with the column blocks inside; `direct` when
// the tile's rows meet [row0, row_end), `mirror` (strictly above the
// diagonal blocks) when its transposed rows do.
std::vector<uint32_t> kmat_tile_list(uint64_t n, uint64_t row0, uint64_t row_end) {
  const uint64_t mt = (n + KM_M - 1) / KM_M, nt = (n + KM_N - 1) / KM_N;
  std::vector<uint32_t> t;
  for (uint64_t g = 0; g < mt; g += KM_GROUP)
    for (uint64_t nj = 0; nj < nt; ++nj)
      for (uint64_t mi = g; mi < std::min<uint64_t>(mt, g + KM_GROUP); ++mi) {
        if (mi / 2 > nj) continue;
        const bool direct = mi * KM_M < row_end && mi * KM_M + KM_M > row0;
        const bool mirror = mi / 2 < nj && nj * KM_N < row_end && nj * KM_N + KM_N > row0;
        if (!direct && !mirror) continue;
        t.push_back((uint32_t)mi);
        t.push_back((uint32_t)nj | (direct ? 1u << 30 : 0u) | (mirror ? 1u << 31 : 0u));
      }
  return t;
}

// The device tile list of rows [row0, row_end), built and copied on first use
// (which must not be inside a stream capture: prepare_kmat_lists covers the
// panels of a fit before its graph is captured).
km_status kmat_tiles_dev(LloydEngine& e, uint64_t n, uint64_t row0, uint64_t row_end, const uint32_t** dev,
                         uint64_t* count) {
  for (const auto& l : e.kmat_lists)
    if (l.row0 == row0 && l.row_end == row_end) { *dev = l.dev; *count = l.count; return KM_OK; }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  KM_CUDA_TRY(cudaStreamIsCapturing(e.stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return KM_ERR_STATE;
  const std::vector<uint32_t> t = kmat_tile_list(n, row0, row_end);
  KmatTileList l;
  l.row0 = row0;
  l.row_end = row_end;
  l.count = t.size() / 2;
  if (cudaMalloc(&l.dev, sizeof(uint32_t) * std::max<size_t>(2, t.size())) != cudaSuccess) {
    (void)cudaGetLastError();
    return KM_ERR_ALLOC;
  }
  e.kmat_lists.push_back(l);
  KM_CUDA_TRY(cudaMemcpy(l.dev, t.data(), sizeof(uint32_t) * t.size(), cudaMemcpyHostToDevice));
  *dev = l.dev;
  *count = l.count;
  return KM_OK;
}

km_status build_kernel_matrix(LloydEngine& e, const float* X, uint64_t n, uint32_t d, const KFn& f,
                              int precision, bool out_bf16, void* K, float* diag, uint64_t row0,
                              uint64_t row_end, bool skip_done) {
  cudaStream_t s = e.stream;
  if (row0 >= row_end || row_end > n) return KM_ERR_ARG;
  const uint64_t rows = row_end - row0;
  if (precision == KM_PREC_FP32) {
    if ((rows + 127) / 128 > 65535) return KM_ERR_UNSUPPORTED;
    dim3 grid((unsigned)((n + 127) / 128), (unsigned)((rows + 127) / 128));
    const DevState* stop = skip_done ? e.st : nullptr;
    if (out_bf16) kmat_f32_kernel<true><<<grid, 256, 0, s>>>(X, e.xn2, n, d, row0, row_end, f, K, diag, stop);
    else kmat_f32_kernel<false><<<grid, 256, 0, s>>>(X, e.xn2, n, d, row0, row_end, f, K, diag, stop);
    KM_CUDA_TRY(cudaGetLastError());
    return KM_OK;
  }
  const bool x3 = precision == KM_PREC_BF16X3;
  CUtensorMap tA{}, tAlo{}, tB{}, tBlo{};
  KM_TRY(encode_tmap_bf16(&tA, e.Xb, e.dp, n, 64, KM_M));
  KM_TRY(encode_tmap_bf16(&tB, e.Xb, e.dp, n, 64, KM_N));
  if (x3) {
    KM_TRY(encode_tmap_bf16(&tAlo, e.Xlo, e.dp, n, 64, KM_M));
    KM_TRY(encode_tmap_bf16(&tBlo, e.Xlo, e.dp, n, 64, KM_N));
  } else {
    tAlo = tA;
    tBlo = tB;
  }
  const uint32_t KBn = e.dp / 64;
  const size_t stage = (size_t)(KA_BYTES + KB_BYTES) * (x3 ? 2 : 1);
  const size_t fixed = 1024 + KM_STG_BYTES + sizeof(KmSmem) + 64;
  size_t S = (227 * 1024 - fixed) / stage;
  if (S > 8) S = 8;
  if (S < 2) return KM_ERR_UNSUPPORTED;
  const size_t smem = fixed + S * stage;
  const uint32_t* tl = nullptr;
  uint64_t tiles = 0;
  KM_TRY(kmat_tiles_dev(e, n, row0, row_end, &tl, &tiles));
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)e.num_sms));
  const int vec = (n % 4 == 0) && (reinterpret_cast<uintptr_t>(K) % 16 == 0);
#define KM_LAUNCH_KMAT(X3_, BF_, KIND_)                                                            \
  do {                                                                                             \
    KM_CUDA_TRY(cudaFuncSetAttribute(kmat_tc_kernel<X3_, BF_, KIND_>,                              \
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));     \
    kmat_tc_kernel<X3_, BF_, KIND_><<<grid, 384, smem, s>>>(tA, tAlo, tB, tBlo, e.xn2, n, row0,    \
                                                            row_end, KBn, (uint32_t)S, f, K, diag, \
                                                            vec, skip_done ? 1 : 0, e.st, tl, tiles); \
  } while (0)
#define KM_LAUNCH_KIND(X3_, BF_)                                                                   \
  do {                                                                                             \
    switch (f.kind) {                                                                              \
      case KM_KERNEL_LINEAR: KM_LAUNCH_KMAT(X3_, BF_, KM_KERNEL_LINEAR); break;                    \
      case KM_KERNEL_POLY: KM_LAUNCH_KMAT(X3_, BF_, KM_KERNEL_POLY); break;                        \
      case KM_KERNEL_SIGMOID: KM_LAUNCH_KMAT(X3_, BF_, KM_KERNEL_SIGMOID); break;                  \
      default: KM_LAUNCH_KMAT(X3_, BF_, KM_KERNEL_GAUSSIAN); break;                                \
    }                                                                                              \
  } while (0)
  if (x3) { if (out_bf16) KM_LAUNCH_KIND(true, true); else KM_LAUNCH_KIND(true, false); }
  else { if (out_bf16) KM_LAUNCH_KIND(false, true); else KM_LAUNCH_KIND(false, false); }
#undef KM_LAUNCH_KIND
#undef KM_LAUNCH_KMAT
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

// Per iteration: V.K (with the K panel builds before each panel's V.K when
// K is not resident), 4 sort kernels, c~, distances/argmin, control, label
// copy; fused: the sort, the operand permutation and the fused kernel
// instead of V.K.
uint64_t kkm_kernels_per_iter(uint64_t n, uint64_t panel, bool fused) {
  if (fused) return 10;
  return panel ? 8 + 2 * ((n + panel - 1) / panel) : 9;
}

template <bool X3, int KIND>
km_status kkm_fused_attr(size_t smem) {
  KM_CUDA_TRY(cudaFuncSetAttribute(kkm_fused_tc_kernel<X3, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  return KM_OK;
}

template <bool X3>
km_status kkm_fused_attr_kind(int kind, size_t smem) {
  switch (kind) {
    case KM_KERNEL_LINEAR: return kkm_fused_attr<X3, KM_KERNEL_LINEAR>(smem);
    case KM_KERNEL_POLY: return kkm_fused_attr<X3, KM_KERNEL_POLY>(smem);
    case KM_KERNEL_SIGMOID: return kkm_fused_attr<X3, KM_KERNEL_SIGMOID>(smem);
    default: return kkm_fused_attr<X3, KM_KERNEL_GAUSSIAN>(smem);
  }
}

// Operand copies, tensor maps and launch shape of the fused kernel.
km_status kkm_fused_plan(km_kkm* h) {
  LloydEngine& e = h->eng;
  const uint64_t n = h->p.n;
  const bool x3 = h->p.precision == KM_PREC_BF16X3;
  if (cudaMalloc(&h->Xbp, sizeof(__nv_bfloat16) * n * e.dp) != cudaSuccess ||
      (x3 && cudaMalloc(&h->Xlop, sizeof(__nv_bfloat16) * n * e.dp) != cudaSuccess) ||
      cudaMalloc(&h->xn2p, sizeof(float) * n) != cudaSuccess) {
    (void)cudaGetLastError();
    return KM_ERR_ALLOC;
  }
  KM_TRY(encode_tmap_bf16(&h->fA, e.Xb, e.dp, n, 64, KM_M));
  KM_TRY(encode_tmap_bf16(&h->fB, h->Xbp, e.dp, n, 64, KM_N));
  if (x3) {
    KM_TRY(encode_tmap_bf16(&h->fAlo, e.Xlo, e.dp, n, 64, KM_M));
    KM_TRY(encode_tmap_bf16(&h->fBlo, h->Xlop, e.dp, n, 64, KM_N));
  } else {
    h->fAlo = h->fA;
    h->fBlo = h->fB;
  }
  const size_t stage = (size_t)(KA_BYTES + KB_BYTES) * (x3 ? 2 : 1);
  const size_t fixed = 1024 + KF_STG_BYTES + sizeof(KfSmem) + 64;
  size_t S = (227 * 1024 - fixed) / stage;
  if (S > 8) S = 8;
  if (S < 2) return KM_ERR_UNSUPPORTED;
  h->fS = (uint32_t)S;
  h->fsmem = fixed + S * stage;
  h->fgrid = (int)std::min<uint64_t>((n + KM_M - 1) / KM_M, (uint64_t)e.num_sms);
  if (x3) KM_TRY(kkm_fused_attr_kind<true>(h->p.kernel_fn, h->fsmem));
  else KM_TRY(kkm_fused_attr_kind<false>(h->p.kernel_fn, h->fsmem));
  return KM_OK;
}

km_status kkm_launch_fused(km_kkm* h) {
  LloydEngine& e = h->eng;
  const uint64_t n = h->p.n;
  const bool x3 = h->p.precision == KM_PREC_BF16X3;
  cudaStream_t s = e.stream;
  kkm_permute_points_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(
      e.Xb, x3 ? e.Xlo : nullptr, e.xn2, e.perm, n, e.dp, h->Xbp, h->Xlop, h->xn2p, e.st);
  KM_CUDA_TRY(cudaGetLastError());
  const KFn f = make_kfn(h->p);
  const uint32_t KBn = e.dp / 64;
#define KM_LAUNCH_FUSED(X3_, KIND_)                                                                \
  kkm_fused_tc_kernel<X3_, KIND_><<<h->fgrid, 256, h->fsmem, s>>>(h->fA, h->fAlo, h->fB, h->fBlo,  \
                                                                  e.xn2, h->xn2p, n, KBn, h->fS,   \
                                                                  f, e.cstart, h->p.k, h->E, e.st)
#define KM_LAUNCH_FUSED_KIND(X3_)                                                                  \
  do {                                                                                             \
    switch (f.kind) {                                                                              \
      case KM_KERNEL_LINEAR: KM_LAUNCH_FUSED(X3_, KM_KERNEL_LINEAR); break;                        \
      case KM_KERNEL_POLY: KM_LAUNCH_FUSED(X3_, KM_KERNEL_POLY); break;                            \
      case KM_KERNEL_SIGMOID: KM_LAUNCH_FUSED(X3_, KM_KERNEL_SIGMOID); break;                      \
      default: KM_LAUNCH_FUSED(X3_, KM_KERNEL_GAUSSIAN); break;                                    \
    }                                                                                              \
  } while (0)
  if (x3) KM_LAUNCH_FUSED_KIND(true);
  else KM_LAUNCH_FUSED_KIND(false);
#undef KM_LAUNCH_FUSED_KIND
#undef KM_LAUNCH_FUSED
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

km_status kkm_launch_vk(km_kkm* h, uint64_t r0, uint64_t r1) {
  LloydEngine& e = h->eng;
  const dim3 grid(e.num_sms), block(h->vk_warps * 32);
  const uint64_t n = h->p.n;
  const uint32_t k = h->p.k;
  cudaStream_t s = e.stream;
  if (h->p.k_bf16) {
    if (h->glab) kkm_vk_kernel<true, true><<<grid, block, h->vk_smem, s>>>(h->K, n, k, h->lab, h->lab8, r0, r1, h->E, e.st);
    else kkm_vk_kernel<true, false><<<grid, block, h->vk_smem, s>>>(h->K, n, k, h->lab, h->lab8, r0, r1, h->E, e.st);
  } else {
    if (h->glab) kkm_vk_kernel<false, true><<<grid, block, h->vk_smem, s>>>(h->K, n, k, h->lab, h->lab8, r0, r1, h->E, e.st);
    else kkm_vk_kernel<false, false><<<grid, block, h->vk_smem, s>>>(h->K, n, k, h->lab, h->lab8, r0, r1, h->E, e.st);
  }
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

km_status kkm_enqueue_iteration(km_kkm* h, const LoopConsts& lc) {
  LloydEngine& e = h->eng;
  const uint64_t n = h->p.n;
  const uint32_t k = h->p.k;
  cudaStream_t s = e.stream;
  if (h->fused) {
    // no K: the label sort first (its permutation orders the columns), then
    // the fused K.V^T
    KM_TRY(e.enqueue_sort(h->lab));
    KM_TRY(kkm_launch_fused(h));
  } else if (h->panel) {
    // K is not resident: rebuild it panel by panel, each panel streamed into
    // its rows of E before the next one overwrites it (stream order)
    const KFn f = make_kfn(h->p);
    for (uint64_t r0 = 0; r0 < n; r0 += h->panel) {
      const uint64_t r1 = std::min<uint64_t>(n, r0 + h->panel);
      KM_TRY(build_kernel_matrix(e, e.X, n, h->p.d, f, h->p.precision, h->p.k_bf16 != 0, h->K, nullptr, r0, r1,
                                 true));
      KM_TRY(kkm_launch_vk(h, r0, r1));
    }
  } else {
    KM_TRY(kkm_launch_vk(h, 0, n));
  }
  if (!h->fused) KM_TRY(e.enqueue_sort(h->lab));
  kkm_ctilde_kernel<<<(k * 32 + 255) / 256, 256, 0, s>>>(h->E, k, e.perm, e.cstart, h->ct, e.st);
  kkm_dist_kernel<<<h->dist_blocks, 256, 2 * k * sizeof(float), s>>>(h->E, n, k, e.counts, h->ct, h->nlab,
                                                                      h->part, e.st);
  kkm_control_kernel<<<1, 32, 0, s>>>(h->part, h->dist_blocks, lc, h->p.check_converged, e.st);
  kkm_copy_labels_kernel<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      h->nlab, h->lab, h->glab ? h->lab8 : nullptr, n, e.st);
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

}  // namespace
}  // namespace km

extern "C" {

km_status km_kernel_matrix(const float* X_dev, uint64_t n, uint32_t d, int32_t kernel_fn, float gamma,
                           float coef, int32_t degree, float sigma, int32_t precision, int32_t out_bf16,
                           void* K_dev, float* diag_dev, void* stream) {
  if (!X_dev || !K_dev || n == 0 || d == 0) return KM_ERR_ARG;
  KM_TRY(kfn_valid(kernel_fn, degree, sigma));
  int dev;
  if (cudaGetDevice(&dev) != cudaSuccess) { (void)cudaGetLastError(); return KM_ERR_NO_DEVICE; }
  LloydEngine e;
  KM_TRY(e.init(n, d, 1, precision, dev, stream, false));
  KM_TRY(e.set_points(X_dev, true, false));
  km_kkm_params p{};
  p.kernel_fn = kernel_fn; p.gamma = gamma; p.coef = coef; p.degree = degree; p.sigma = sigma;
  const KFn f = make_kfn(p);
  KM_TRY(prepare_kmat_norms(e, n, f, precision));
  KM_TRY(build_kernel_matrix(e, X_dev, n, d, f, precision, out_bf16 != 0, K_dev, diag_dev, 0, n, false));
  return e.check_device_error();
}

km_status km_kkm_create(const km_kkm_params* p, km_kkm** out) {
  if (!p || !out) return KM_ERR_ARG;
  *out = nullptr;
  if (p->n == 0 || p->d == 0 || p->k == 0 || p->k > p->n || p->maxiter == 0) return KM_ERR_ARG;
  if (p->k > 256) return KM_ERR_UNSUPPORTED;   // byte labels
  if (!(p->tol >= 0.0f)) return KM_ERR_ARG;
  KM_TRY(kfn_valid(p->kernel_fn, p->degree, p->sigma));
  const uint64_t nn = p->n * p->n;
  if (nn / p->n != p->n) return KM_ERR_ARG;
  // V.K: per-warp bins (k x 32 floats), next to the byte labels when those
  // fit beside eight warps' bins, else the labels come from a global byte
  // copy; more warps keep more K rows in flight
  constexpr size_t SMEM = 227 * 1024;
  const size_t lab_bytes = (p->n + 15) & ~15ull, bin_bytes = (size_t)p->k * 32 * sizeof(float);
  const bool glab = lab_bytes + 8 * bin_bytes > SMEM;
  const size_t lb = glab ? 0 : lab_bytes;
  uint32_t vk_warps = glab ? 1 : 8;
  while (vk_warps < 16 && lb + (size_t)(vk_warps + 1) * bin_bytes <= SMEM) ++vk_warps;
  const size_t vk_smem = lb + (size_t)vk_warps * bin_bytes;
  if (vk_smem > SMEM) return KM_ERR_UNSUPPORTED;
  km_kkm* h = new (std::nothrow) km_kkm();
  if (!h) return KM_ERR_ALLOC;
  h->p = *p;
  h->vk_smem = vk_smem;
  h->vk_warps = vk_warps;
  h->glab = glab;
  km_status s = h->eng.init(p->n, p->d, p->k, p->precision, p->device, p->stream, true);
  auto fail = [&](km_status st) { km_kkm_destroy(h); return st; };
  if (s != KM_OK) return fail(s);
  if (cudaMalloc(&h->diag, sizeof(float) * p->n) != cudaSuccess ||
      cudaMalloc(&h->E, sizeof(float) * p->n * p->k) != cudaSuccess ||
      cudaMalloc(&h->ct, sizeof(double) * p->k) != cudaSuccess ||
      cudaMalloc(&h->lab, sizeof(uint32_t) * p->n) != cudaSuccess ||
      cudaMalloc(&h->nlab, sizeof(uint32_t) * p->n) != cudaSuccess ||
      cudaMalloc(&h->part, sizeof(double) * 1024) != cudaSuccess ||
      (glab && cudaMalloc(&h->lab8, lab_bytes) != cudaSuccess)) {
    (void)cudaGetLastError();
    return fail(KM_ERR_ALLOC);
  }
  // K last: resident (n x n), one panel of rows, or none (fused)
  const size_t bpe = p->k_bf16 ? 2 : 4;
  const bool tensor = p->precision != KM_PREC_FP32;
  uint64_t panel = 0;
  bool fused = false;
  if (p->panel_rows == KM_KKM_FUSED) {
    if (!tensor) return fail(KM_ERR_UNSUPPORTED);
    fused = true;
  } else if (p->panel_rows == KM_KKM_PANEL_AUTO) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { (void)cudaGetLastError(); return fail(KM_ERR_CUDA); }
    if ((double)nn * bpe > 0.9 * (double)fr) {
      if (tensor) {
        fused = true;
      } else {
        const uint64_t r = (uint64_t)(0.5 * (double)fr / ((double)p->n * bpe)) / 128 * 128;
        panel = std::min<uint64_t>(std::max<uint64_t>(r, 128), p->n);
      }
    }
  } else if (p->panel_rows > 0) {
    panel = std::min<uint64_t>(p->panel_rows, p->n);
  }
  h->panel = panel;
  h->fused = fused;
  h->kpi = kkm_kernels_per_iter(p->n, panel, fused);
  if (fused) {
    s = kkm_fused_plan(h);
    if (s != KM_OK) return fail(s);
  } else {
    const size_t kbytes = (panel ? panel * p->n : nn) * bpe;
    if (cudaMalloc(&h->K, kbytes) != cudaSuccess) { (void)cudaGetLastError(); return fail(KM_ERR_ALLOC); }
  }
  h->dist_blocks = (int)std::min<uint64_t>((p->n + 255) / 256, 1024);
  bool attr_ok = true;
  if (glab) {
    attr_ok = cudaFuncSetAttribute(kkm_vk_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)vk_smem) == cudaSuccess &&
              cudaFuncSetAttribute(kkm_vk_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)vk_smem) == cudaSuccess;
  } else {
    attr_ok = cudaFuncSetAttribute(kkm_vk_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)vk_smem) == cudaSuccess &&
              cudaFuncSetAttribute(kkm_vk_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)vk_smem) == cudaSuccess;
  }
  if (!attr_ok || cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void**>(&h->h_done), sizeof(int32_t)) != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(KM_ERR_CUDA);
  }
  *out = h;
  return KM_OK;
}

km_status km_kkm_set_data(km_kkm* h, const float* X, int on_device) {
  if (!h || !X) return KM_ERR_ARG;
  LloydEngine& e = h->eng;
  KM_TRY(e.set_points(X, on_device != 0, true));
  const KFn f = make_kfn(h->p);
  KM_CUDA_TRY(cudaEventRecord(h->ev0, e.stream));
  KM_TRY(prepare_kmat_norms(e, h->p.n, f, h->p.precision));
  // with panels (or fused), K is built inside every iteration instead; the
  // panels' tile lists are made here, before any iteration is captured
  if (h->panel && h->p.precision != KM_PREC_FP32) {
    for (uint64_t r0 = 0; r0 < h->p.n; r0 += h->panel) {
      const uint32_t* tl = nullptr;
      uint64_t cnt = 0;
      KM_TRY(kmat_tiles_dev(e, h->p.n, r0, std::min<uint64_t>(h->p.n, r0 + h->panel), &tl, &cnt));
    }
  }
  if (!h->panel && !h->fused)
    KM_TRY(build_kernel_matrix(e, e.X, h->p.n, h->p.d, f, h->p.precision, h->p.k_bf16 != 0, h->K, h->diag, 0,
                               h->p.n, false));
  KM_CUDA_TRY(cudaEventRecord(h->ev1, e.stream));
  KM_CUDA_TRY(cudaEventSynchronize(h->ev1));
  float ms = 0.f;
  KM_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->kbuild_ms = ms;
  KM_TRY(e.check_device_error());
  h->ready = true;
  return KM_OK;
}

km_status km_kkm_panel_rows(km_kkm* h, uint64_t* rows) {
  if (!h || !rows) return KM_ERR_ARG;
  *rows = h->fused ? KM_KKM_FUSED : h->panel;
  return KM_OK;
}

km_status km_kkm_build_ms(km_kkm* h, double* ms) {
  if (!h || !ms) return KM_ERR_ARG;
  if (!h->ready) return KM_ERR_STATE;
  *ms = h->kbuild_ms;
  return KM_OK;
}

km_status km_kkm_configure(km_kkm* h, uint64_t maxiter, float tol, int32_t check_converged) {
  if (!h || maxiter == 0 || !(tol >= 0.0f)) return KM_ERR_ARG;
  h->p.maxiter = maxiter;
  h->p.tol = tol;
  h->p.check_converged = check_converged != 0;
  return KM_OK;
}

km_status km_kkm_fit(km_kkm* h, const uint32_t* init_labels, uint32_t* labels_out, km_result* res) {
  if (!h) return KM_ERR_ARG;
  if (!h->ready) return KM_ERR_STATE;
  LloydEngine& e = h->eng;
  KM_CUDA_TRY(cudaSetDevice(e.device));
  KM_TRY(e.reset_state());
  const uint64_t n = h->p.n;
  if (init_labels) {
    for (uint64_t i = 0; i < n; ++i)
      if (init_labels[i] >= h->p.k) return KM_ERR_ARG;
    KM_CUDA_TRY(cudaMemcpyAsync(h->lab, init_labels, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, e.stream));
  } else {
    round_robin_labels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, e.stream>>>(h->lab, n, h->p.k);
    KM_CUDA_TRY(cudaGetLastError());
  }
  if (h->glab) {
    kkm_label_bytes_kernel<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, e.stream>>>(h->lab,
                                                                                                   h->lab8, n);
    KM_CUDA_TRY(cudaGetLastError());
  }
  LoopConsts lc{h->p.maxiter, h->p.tol, h->p.check_converged ? KM_CONV_SCORE : KM_CONV_NONE, 0};
  KM_CUDA_TRY(cudaEventRecord(h->ev0, e.stream));
  uint64_t launched = 0, batch = h->p.check_converged ? 4 : h->p.maxiter;
  while (launched < h->p.maxiter) {
    const uint64_t target = std::min<uint64_t>(h->p.maxiter, launched + batch);
    for (; launched < target; ++launched) KM_TRY(kkm_enqueue_iteration(h, lc));
    if (launched >= h->p.maxiter) break;
    KM_CUDA_TRY(cudaMemcpyAsync(h->h_done, &e.st->done, sizeof(int32_t), cudaMemcpyDeviceToHost, e.stream));
    KM_CUDA_TRY(cudaStreamSynchronize(e.stream));
    if (*h->h_done) break;
    batch = std::min<uint64_t>(batch * 2, 64);
  }
  KM_CUDA_TRY(cudaEventRecord(h->ev1, e.stream));
  KM_TRY(e.check_device_error());
  float ms = 0;
  KM_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  if (labels_out)
    KM_CUDA_TRY(cudaMemcpyAsync(labels_out, h->lab, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, e.stream));
  KM_CUDA_TRY(cudaStreamSynchronize(e.stream));
  const DevState& s = *e.h_st;
  if (res) {
    std::memset(res, 0, sizeof(*res));
    res->iterations = s.iter;
    res->converged = s.converged_iter != 0;
    res->converged_iter = s.converged_iter ? s.converged_iter : h->p.maxiter;
    res->objective = s.objective;
    res->score = s.score;
    res->fit_ms = ms;
    res->kernel_launches = launched * h->kpi;
  }
  return KM_OK;
}

void km_kkm_destroy(km_kkm* h) {
  if (!h) return;
  if (h->eng.device >= 0) cudaSetDevice(h->eng.device);
  if (h->K) cudaFree(h->K);
  if (h->diag) cudaFree(h->diag);
  if (h->E) cudaFree(h->E);
  if (h->ct) cudaFree(h->ct);
  if (h->lab) cudaFree(h->lab);
  if (h->nlab) cudaFree(h->nlab);
  if (h->lab8) cudaFree(h->lab8);
  if (h->Xbp) cudaFree(h->Xbp);
  if (h->Xlop) cudaFree(h->Xlop);
  if (h->xn2p) cudaFree(h->xn2p);
  if (h->part) cudaFree(h->part);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->h_done) cudaFreeHost(h->h_done);
  delete h;
}

}  // extern "C"
