// (a)+(b) Tensor-core distance stage for sm_103a: tcgen05.mma (kind::f16, BF16
// operands, FP32 accumulators in TMEM), TMA tile loads with 128-byte swizzle,
// and the argmin epilogue fused on the TMEM read-back.
//
// One persistent CTA per SM.  The centroid operand (k padded to kp <= 256,
// d padded to dp) is loaded once per CTA and stays in shared memory; point
// tiles of 128 rows stream through a ring of K-block stages.  Two TMEM
// accumulator buffers (kp columns each) let the epilogue of tile t overlap the
// MMAs of tile t+1.
//
//   warp 0       TMA producer (one elected lane)
//   warp 1       MMA issuer (one elected lane)
//   warp 2       TMEM allocator
//   warps 4-19   epilogue, four warps per TMEM lane quadrant (warp w reads
//                lanes 32*(w%4)..+31), each on a quarter of the column chunks:
//                pass 1  v = ||c||^2 - 2 acc kept in registers, row minimum v1;
//                        the TMEM buffer is released right after the loads;
//                pass 2  candidates {c : v(c) <= tau(v1)} (tie_tau); one
//                        candidate: the label is proven; 2..4: queued for the
//                        exact re-score of those; more: full re-score.
//                The four warps of a quadrant combine through shared memory
//                with bounded mbarrier hand-offs.
//
// Every mbarrier wait is bounded (2 s); on timeout the CTA raises an abort
// flag, records KM_DEVERR_TIMEOUT, waits (bounded) for its own copies and MMAs
// in flight, frees TMEM and returns.
//
// Split-BF16x3 (x3): x = hi + lo with hi = bf16(x), lo = bf16(x - hi); the
// accumulator receives hi*hi + hi*lo + lo*hi.
//
// Reference counterpart: the distance stage of Kmeans::run (src/kmeans.cu:847-936)
// and the Lloyd distance of comparisons/CPU_Kmeans/src/kmeans.cpp:86-104; the
// reference has no tensor-core kernel (it calls cuBLAS/cuSPARSE).
#include "km_lloyd.cuh"

#include <cudaTypedefs.h>

namespace km {

namespace {

constexpr int TC_EPI_WARPS = 16;
constexpr int TC_THREADS = 32 * (4 + TC_EPI_WARPS);
constexpr int TC_M = 128;
constexpr uint64_t WAIT_NS = 2000000000ull;
constexpr uint32_t A_UNIT = TC_M * 128;  // bytes of one 128-row x 64-col BF16 K-block

struct TcSmem {
  uint64_t full[16];
  uint64_t empty[16];
  uint64_t bfull;
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t tdone;
  uint64_t x1[4];     // per quadrant: partial minima written
  uint64_t x2[4];     // per quadrant: partial candidate lists written
  uint32_t tmem_base;
  int abort;
  float xmin[4][TC_M];
  uint32_t xcnt[4][TC_M];
  uint32_t xcand[4][TC_M][4];
};

template <bool X3>
__global__ void __launch_bounds__(TC_THREADS, 1)
assign_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                 const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
                 const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                 uint32_t k, uint32_t kp, uint32_t KB, uint32_t S, uint32_t nalloc, TieBound tb,
                 DevState* st, uint32_t* __restrict__ labels, float* __restrict__ mindist,
                 RefineQueues rq, float* __restrict__ Dout) {
  if (st->done) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const uint32_t b_bytes = KB * kp * 128u;              // one of hi / lo
  uint8_t* sB = smem;
  uint8_t* sA = smem + b_bytes * (X3 ? 2u : 1u);
  const uint32_t unit_bytes = A_UNIT * (X3 ? 2u : 1u);
  float* cns = reinterpret_cast<float*>(sA + (size_t)S * unit_bytes);
  TcSmem* ts = reinterpret_cast<TcSmem*>(cns + ((kp + 31) & ~31u));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t ntiles = (n + TC_M - 1) / TC_M;
  const float cmax = st->cmax;

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < S; ++s) { mbar_init(&ts->full[s], 1); mbar_init(&ts->empty[s], 1); }
    mbar_init(&ts->bfull, 1);
    for (int b = 0; b < 2; ++b) { mbar_init(&ts->tfull[b], 1); mbar_init(&ts->tempty[b], TC_EPI_WARPS); }
    mbar_init(&ts->tdone, 1);
    for (int q = 0; q < 4; ++q) { mbar_init(&ts->x1[q], 128); mbar_init(&ts->x2[q], 128); }
    ts->abort = 0;
    mbar_fence_init();
  }
  const uint32_t kp32 = (kp + 31) & ~31u;
  for (uint32_t c = threadIdx.x; c < kp32; c += blockDim.x)
    cns[c] = (c < k) ? cn2[c] : __int_as_float(0x7f800000);
  if (warp == 2) tmem_alloc(&ts->tmem_base, 2u * nalloc);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = ts->tmem_base;
  volatile int* abort_flag = &ts->abort;

  auto fail = [&](uint32_t where) {
    ts->abort = 1;
    if (atomicOr(&st->err, KM_DEVERR_TIMEOUT) == 0u) st->err_where = where;
  };

  if (warp == 0) {
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      if (X3) { tma_prefetch_desc(&tmAlo); tma_prefetch_desc(&tmBlo); }
      mbar_arrive_expect_tx(&ts->bfull, b_bytes * (X3 ? 2u : 1u));
      for (uint32_t kb = 0; kb < KB; ++kb) {
        tma_load_2d(sB + (size_t)kb * kp * 128u, &tmB, (int)(kb * 64), 0, &ts->bfull);
        if (X3) tma_load_2d(sB + b_bytes + (size_t)kb * kp * 128u, &tmBlo, (int)(kb * 64), 0, &ts->bfull);
      }
      uint64_t u = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
          const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
          if (!mbar_wait_bounded(&ts->empty[s], ph ^ 1u, abort_flag, WAIT_NS)) { fail(1); ok = false; break; }
          mbar_arrive_expect_tx(&ts->full[s], unit_bytes);
          uint8_t* dst = sA + (size_t)s * unit_bytes;
          tma_load_2d(dst, &tmA, (int)(kb * 64), (int)(tile * TC_M), &ts->full[s]);
          if (X3) tma_load_2d(dst + A_UNIT, &tmAlo, (int)(kb * 64), (int)(tile * TC_M), &ts->full[s]);
        }
      }
      // Drain: every issued copy must land before the CTA exits (these waits
      // ignore the abort flag but stay bounded).
      volatile int no_abort = 0;
      mbar_wait_bounded(&ts->bfull, 0, &no_abort, WAIT_NS);
      const uint64_t first = u > S ? u - S : 0;
      for (uint64_t v = first; v < u; ++v) {
        const uint32_t s = (uint32_t)(v % S), ph = (uint32_t)((v / S) & 1u);
        mbar_wait_bounded(&ts->full[s], ph, &no_abort, WAIT_NS);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(TC_M, kp);
      bool ok = mbar_wait_bounded(&ts->bfull, 0, abort_flag, WAIT_NS);
      if (!ok) fail(2);
      tc_fence_after();
      const uint32_t sA0 = smem_u32(sA), sB0 = smem_u32(sB);
      uint64_t u = 0, t = 0;
      bool issued = false;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++t) {
        const uint32_t buf = (uint32_t)(t & 1u), use = (uint32_t)(t >> 1);
        if (!mbar_wait_bounded(&ts->tempty[buf], (use & 1u) ^ 1u, abort_flag, WAIT_NS)) { fail(3); ok = false; break; }
        tc_fence_after();
        const uint32_t dt = tmem_base + buf * nalloc;
        for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
          const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
          if (!mbar_wait_bounded(&ts->full[s], ph, abort_flag, WAIT_NS)) { fail(4); ok = false; break; }
          tc_fence_after();
          const uint32_t a0 = sA0 + s * unit_bytes;
          const uint32_t b0 = sB0 + kb * kp * 128u;
#pragma unroll
          for (uint32_t kk = 0; kk < 4; ++kk) {
            const uint64_t ad = smem_desc_sw128(a0 + kk * 32u);
            const uint64_t bd = smem_desc_sw128(b0 + kk * 32u);
            tc_mma_bf16(dt, ad, bd, idesc, (kb | kk) != 0u ? 1u : 0u);
            if (X3) {
              const uint64_t adl = smem_desc_sw128(a0 + A_UNIT + kk * 32u);
              const uint64_t bdl = smem_desc_sw128(b0 + b_bytes + kk * 32u);
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
      // All MMAs of this thread complete before teardown.
      if (issued) {
        tc_commit(&ts->tdone);
        volatile int no_abort = 0;
        mbar_wait_bounded(&ts->tdone, 0, &no_abort, WAIT_NS);
      }
    }
  } else if (warp >= 4) {
    const int q = warp & 3, sub = (warp - 4) >> 2;
    const uint32_t nch = (kp + 31) / 32;            // <= 8, so <= 2 chunks per warp
    const uint32_t r = (uint32_t)q * 32u + (uint32_t)lane;
    uint64_t t = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++t) {
      const uint32_t buf = (uint32_t)(t & 1u), use = (uint32_t)(t >> 1), xp = (uint32_t)(t & 1u);
      const bool okw = mbar_wait_bounded(&ts->tfull[buf], use & 1u, abort_flag, WAIT_NS);
      if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(5); break; }
      tc_fence_after();
      const uint64_t row = tile * TC_M + r;
      const float x2 = (row < n) ? xn2[row] : 0.0f;
      // ---- pass 1: values into registers, row minimum ----
      float v[64];
      float m0 = __int_as_float(0x7f800000), m1 = m0, m2 = m0, m3 = m0;
#pragma unroll
      for (int c2 = 0; c2 < 2; ++c2) {
        const uint32_t ch = (uint32_t)sub + 4u * (uint32_t)c2;
        if (ch < nch) {
          uint32_t acc[32];
          tmem_ld_32x32b_x32(tmem_base + (((uint32_t)q * 32u) << 16) + buf * nalloc + ch * 32u, acc);
          tmem_ld_wait();
          const float4* cn4 = reinterpret_cast<const float4*>(cns + ch * 32u);
#pragma unroll
          for (int j4 = 0; j4 < 8; ++j4) {
            const float4 cc = cn4[j4];
            const float a = fmaf(-2.0f, __uint_as_float(acc[4 * j4 + 0]), cc.x);
            const float b = fmaf(-2.0f, __uint_as_float(acc[4 * j4 + 1]), cc.y);
            const float c = fmaf(-2.0f, __uint_as_float(acc[4 * j4 + 2]), cc.z);
            const float e = fmaf(-2.0f, __uint_as_float(acc[4 * j4 + 3]), cc.w);
            v[c2 * 32 + 4 * j4 + 0] = a; v[c2 * 32 + 4 * j4 + 1] = b;
            v[c2 * 32 + 4 * j4 + 2] = c; v[c2 * 32 + 4 * j4 + 3] = e;
            m0 = fminf(m0, a); m1 = fminf(m1, b); m2 = fminf(m2, c); m3 = fminf(m3, e);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[c2 * 32 + j] = __int_as_float(0x7f800000);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&ts->tempty[buf]);     // accumulator buffer free
      if (Dout && row < n) {
#pragma unroll
        for (int c2 = 0; c2 < 2; ++c2) {
          const uint32_t ch = (uint32_t)sub + 4u * (uint32_t)c2;
          if (ch < nch)
            for (int j = 0; j < 32; ++j)
              if (ch * 32u + j < k) Dout[row * k + ch * 32u + j] = v[c2 * 32 + j] + x2;
        }
      }
      ts->xmin[sub][r] = fminf(fminf(m0, m1), fminf(m2, m3));
      mbar_arrive(&ts->x1[q]);
      const bool ok1 = mbar_wait_bounded(&ts->x1[q], xp, abort_flag, WAIT_NS);
      if (!__all_sync(0xffffffffu, ok1)) { if (lane == 0) fail(6); break; }
      const float v1 = fminf(fminf(ts->xmin[0][r], ts->xmin[1][r]), fminf(ts->xmin[2][r], ts->xmin[3][r]));
      // ---- pass 2: candidates v <= tau ----
      const float tau = tie_tau(x2, v1, cmax, tb);
      uint32_t cnt = 0, k0 = 0, k1 = 0, k2 = 0, k3 = 0;
#pragma unroll
      for (int c2 = 0; c2 < 2; ++c2) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const uint32_t col = ((uint32_t)sub + 4u * (uint32_t)c2) * 32u + (uint32_t)j;
          if (v[c2 * 32 + j] <= tau && col < k) {
            k0 = (cnt == 0) ? col : k0; k1 = (cnt == 1) ? col : k1;
            k2 = (cnt == 2) ? col : k2; k3 = (cnt == 3) ? col : k3;
            ++cnt;
          }
        }
      }
      // NaN anywhere (tau or v1) leaves cnt == 0: such a row takes the full path.
      ts->xcnt[sub][r] = cnt;
      ts->xcand[sub][r][0] = k0; ts->xcand[sub][r][1] = k1;
      ts->xcand[sub][r][2] = k2; ts->xcand[sub][r][3] = k3;
      mbar_arrive(&ts->x2[q]);
      const bool ok2 = mbar_wait_bounded(&ts->x2[q], xp, abort_flag, WAIT_NS);
      if (!__all_sync(0xffffffffu, ok2)) { if (lane == 0) fail(7); break; }
      if (sub == 0) {
        uint32_t total = 0, l0 = 0, l1 = 0, l2 = 0, l3 = 0, best = 0xffffffffu;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const uint32_t cw = ts->xcnt[w][r];
#pragma unroll
          for (uint32_t i = 0; i < 4; ++i) {
            if (i < cw) {
              const uint32_t c = ts->xcand[w][r][i];
              const uint32_t pos = total + i;
              l0 = (pos == 0) ? c : l0; l1 = (pos == 1) ? c : l1;
              l2 = (pos == 2) ? c : l2; l3 = (pos == 3) ? c : l3;
              best = min(best, c);
            }
          }
          total += cw;
        }
        const bool valid = row < n;
        if (valid) {
          labels[row] = (total == 1) ? l0 : (best == 0xffffffffu ? 0u : best);
          if (mindist) mindist[row] = v1 + x2;
        }
        RefineEntry e{(uint32_t)row, total, {l0, l1, l2, l3}};
        const uint64_t seg = row >> 5;
        seg_push(rq.cand, rq.ccnt, seg, valid && total >= 2 && total <= 4, e);
        seg_push(rq.full, rq.fcnt, seg, valid && (total == 0 || total > 4), (uint32_t)row);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(tmem_base, 2u * nalloc);
}

}  // namespace

TcPlan plan_tc(uint32_t dp, uint32_t kp, bool x3, uint64_t n, int num_sms) {
  TcPlan p;
  if (dp == 0 || dp % 64 != 0 || kp < 16 || kp > 256 || kp % 16 != 0) return p;
  p.KB = dp / 64;
  const size_t mult = x3 ? 2 : 1;
  const size_t b_bytes = (size_t)p.KB * kp * 128 * mult;
  const size_t unit = (size_t)A_UNIT * mult;
  const size_t fixed = 1024 /*align*/ + ((kp + 31) & ~31u) * 4 + sizeof(TcSmem) + 64;
  const size_t budget = 227 * 1024;
  if (b_bytes + fixed + 2 * unit > budget) return p;
  size_t s = (budget - b_bytes - fixed) / unit;
  if (s > 8) s = 8;
  p.stages = (uint32_t)s;
  p.nalloc = 32;
  while (p.nalloc < kp) p.nalloc <<= 1;
  p.smem = b_bytes + fixed + s * unit;
  const uint64_t ntiles = (n + TC_M - 1) / TC_M;
  p.grid = (int)std::min<uint64_t>(ntiles, (uint64_t)num_sms);
  if (p.grid < 1) p.grid = 1;
  p.ok = true;
  return p;
}

km_status encode_tmap_bf16(CUtensorMap* tm, const void* base, uint64_t inner, uint64_t outer,
                           uint32_t box_inner, uint32_t box_outer) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return KM_ERR_CUDA;
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {inner * 2};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? KM_OK : KM_ERR_CUDA;
}

km_status tc_set_attributes(const TcPlan& pl, bool x3) {
  if (!pl.ok) return KM_ERR_UNSUPPORTED;
  if (x3)
    KM_CUDA_TRY(cudaFuncSetAttribute(assign_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
  else
    KM_CUDA_TRY(cudaFuncSetAttribute(assign_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
  return KM_OK;
}

km_status launch_assign_tc(const TcPlan& pl, bool x3, const CUtensorMap& tmA,
                           const CUtensorMap& tmAlo, const CUtensorMap& tmB,
                           const CUtensorMap& tmBlo, const float* cn2, const float* xn2,
                           uint64_t n, uint32_t k, uint32_t kp, TieBound tb, DevState* st,
                           uint32_t* labels, float* mindist, const RefineQueues& rq,
                           float* Dout, cudaStream_t s) {
  if (!pl.ok) return KM_ERR_UNSUPPORTED;
  if (x3) {
    assign_tc_kernel<true><<<pl.grid, TC_THREADS, pl.smem, s>>>(
        tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, pl.KB, pl.stages, pl.nalloc, tb, st, labels,
        mindist, rq, Dout);
  } else {
    assign_tc_kernel<false><<<pl.grid, TC_THREADS, pl.smem, s>>>(
        tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, pl.KB, pl.stages, pl.nalloc, tb, st, labels,
        mindist, rq, Dout);
  }
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

}  // namespace km
