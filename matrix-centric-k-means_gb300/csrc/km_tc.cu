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
//   warps 4-11   epilogue, all eight on the same tile: warp w reads TMEM
//                lanes 32*(w%4)..+31 (its rows) and one half of the kp
//                columns, so the accumulator buffer is released after half a
//                row's column work and the MMAs of the next tile on that
//                buffer start early:
//                pass 1  partial row minimum of v = ||c||^2 - 2 acc, exchanged
//                        with the other half: v1;
//                pass 2  candidates {c : v(c) <= tau(v1)} (tie_tau) as
//                        per-chunk bit masks (TMEM is read a second time); the
//                        upper half hands its count and first candidates over;
//                one candidate: the label is proven; 2..4: queued for the
//                exact re-score of those; more: full re-score.
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

#include <algorithm>

namespace km {

namespace {

constexpr int TC_EPI_WARPS = 8;
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
  uint64_t pairbar[4];      // epilogue: the two warps of TMEM lane quadrant q
  uint32_t tmem_base;
  int abort;
};

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1)
assign_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                 const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
                 const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                 uint32_t k, uint32_t kp, uint32_t KB, uint32_t S, uint32_t nalloc, TieBound tb,
                 DevState* st, uint32_t* __restrict__ labels, float* __restrict__ mindist,
                 RefineQueues rq, float* __restrict__ Dout) {
  constexpr bool ALO = MODE == TC_SPLIT3;      // point operand has a lo part
  constexpr bool BLO = MODE != TC_PLAIN;       // centroid operand has a lo part
  if (st->done) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const uint32_t b_bytes = KB * kp * 128u;              // one of hi / lo
  uint8_t* sB = smem;
  uint8_t* sA = smem + b_bytes * (BLO ? 2u : 1u);
  const uint32_t unit_bytes = A_UNIT * (ALO ? 2u : 1u);
  float* xch = reinterpret_cast<float*>(sA + (size_t)S * unit_bytes);   // [2][TC_M] row exchange
  TcSmem* ts = reinterpret_cast<TcSmem*>(xch + 2 * TC_M);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t ntiles = (n + TC_M - 1) / TC_M;
  const float cmax = st->cmax;

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < S; ++s) { mbar_init(&ts->full[s], 1); mbar_init(&ts->empty[s], 1); }
    mbar_init(&ts->bfull, 1);
    for (int b = 0; b < 2; ++b) { mbar_init(&ts->tfull[b], 1); mbar_init(&ts->tempty[b], TC_EPI_WARPS); }
    mbar_init(&ts->tdone, 1);
    for (int qq = 0; qq < 4; ++qq) mbar_init(&ts->pairbar[qq], 2);
    ts->abort = 0;
    mbar_fence_init();
  }
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
      if (ALO) tma_prefetch_desc(&tmAlo);
      if (BLO) tma_prefetch_desc(&tmBlo);
      mbar_arrive_expect_tx(&ts->bfull, b_bytes * (BLO ? 2u : 1u));
      for (uint32_t kb = 0; kb < KB; ++kb) {
        tma_load_2d(sB + (size_t)kb * kp * 128u, &tmB, (int)(kb * 64), 0, &ts->bfull);
        if (BLO) tma_load_2d(sB + b_bytes + (size_t)kb * kp * 128u, &tmBlo, (int)(kb * 64), 0, &ts->bfull);
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
          if (ALO) tma_load_2d(dst + A_UNIT, &tmAlo, (int)(kb * 64), (int)(tile * TC_M), &ts->full[s]);
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
            if (BLO) tc_mma_bf16(dt, ad, smem_desc_sw128(b0 + b_bytes + kk * 32u), idesc, 1u);
            if (ALO) tc_mma_bf16(dt, smem_desc_sw128(a0 + A_UNIT + kk * 32u), bd, idesc, 1u);
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
    // Epilogue: the eight warps take every tile of this CTA together.  Warp w
    // owns TMEM lanes (rows) 32*(w%4)..+31 and half h = (w-4)/4 of the 64-column
    // loads (h = 0 the lower columns), so a tile's accumulator is released after
    // half the column work of one warp.  The two warps of a quadrant exchange the
    // row's partial minimum, then the upper half's candidate summary, through
    // xch and their pair mbarrier (two phases per tile, bounded waits).
    const int q = warp & 3, h = (warp - 4) >> 2;
    const uint32_t npair = (kp + 63) / 64;          // 64-column loads in all
    const uint32_t nlo = (npair + 1) / 2;           // of which half 0 takes the first nlo
    const uint32_t pr0 = h ? nlo : 0u, pr1 = h ? npair : nlo;
    const uint32_t r = (uint32_t)q * 32u + (uint32_t)lane;
    uint64_t* pb = &ts->pairbar[q];
    uint32_t pbuse = 0;                             // completed phases of pb
    auto pair_sync = [&]() -> bool {
      __syncwarp();
      if (lane == 0) mbar_arrive(pb);
      const bool ok = mbar_wait_bounded(pb, pbuse & 1u, abort_flag, WAIT_NS);
      ++pbuse;
      return __all_sync(0xffffffffu, ok);
    };
    uint64_t t = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++t) {
      const uint32_t buf = (uint32_t)(t & 1u), use = (uint32_t)(t >> 1);
      const uint64_t row = tile * TC_M + r;
      const float x2 = (row < n) ? xn2[row] : 0.0f;
      const bool okw = mbar_wait_bounded(&ts->tfull[buf], use & 1u, abort_flag, WAIT_NS);
      if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(5); break; }
      tc_fence_after();
      const uint32_t tbase = tmem_base + (((uint32_t)q * 32u) << 16) + buf * nalloc;
      // ---- pass 1: partial row minimum of v = ||c||^2 - 2 acc over this half ----
      // eight independent min chains (four steps per 64 columns each)
      float mv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) mv[i] = __int_as_float(0x7f800000);
      for (uint32_t pr = pr0; pr < pr1; ++pr) {
        uint32_t acc[64];
        tmem_ld_32x32b_x64(tbase + pr * 64u, acc);
        tmem_ld_wait();
        const float4* cn4 = reinterpret_cast<const float4*>(cn2 + pr * 64u);
#pragma unroll
        for (int j4 = 0; j4 < 16; ++j4) {
          const float4 cc = __ldg(cn4 + j4);
          const float2 va = dist_pair(acc[4 * j4 + 0], acc[4 * j4 + 1], cc.x, cc.y);
          const float2 vb = dist_pair(acc[4 * j4 + 2], acc[4 * j4 + 3], cc.z, cc.w);
          mv[(2 * j4) & 7] = fmin3(mv[(2 * j4) & 7], va.x, va.y);
          mv[(2 * j4 + 1) & 7] = fmin3(mv[(2 * j4 + 1) & 7], vb.x, vb.y);
        }
      }
      const float mh = fminf(fmin3(mv[0], mv[1], mv[2]), fmin3(mv[3], mv[4], fmin3(mv[5], mv[6], mv[7])));
      xch[h * TC_M + r] = mh;
      if (!pair_sync()) { if (lane == 0) fail(6); break; }
      const float v1 = fminf(mh, xch[(1 - h) * TC_M + r]);
      const float tau = tie_tau(x2, v1, cmax, tb);
      // ---- pass 2: this half's candidates {c < k : v(c) <= tau} in ascending order ----
      uint32_t cnt = 0, got = 0, k0 = 0, k1 = 0, k2 = 0, k3 = 0;
      bool released = false;
      for (uint32_t pr = pr0; pr < pr1; ++pr) {
        uint32_t acc[64];
        tmem_ld_32x32b_x64(tbase + pr * 64u, acc);
        tmem_ld_wait();
        if (pr + 1 == pr1) {
          // the last load of this tile has landed: the accumulator is free
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ts->tempty[buf]);
          released = true;
        }
        const float4* cn4 = reinterpret_cast<const float4*>(cn2 + pr * 64u);
        uint32_t mm[2];
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          // four independent partial masks, one per column residue mod 4
          uint32_t q0 = 0u, q1 = 0u, q2 = 0u, q3 = 0u;
#pragma unroll
          for (int j4 = 0; j4 < 8; ++j4) {
            const float4 cc = __ldg(cn4 + 8 * hh + j4);
            const int a = 32 * hh + 4 * j4;
            const float2 va = dist_pair(acc[a + 0], acc[a + 1], cc.x, cc.y);
            const float2 vb = dist_pair(acc[a + 2], acc[a + 3], cc.z, cc.w);
            q0 |= (va.x <= tau ? 1u : 0u) << (4 * j4 + 0);
            q1 |= (va.y <= tau ? 1u : 0u) << (4 * j4 + 1);
            q2 |= (vb.x <= tau ? 1u : 0u) << (4 * j4 + 2);
            q3 |= (vb.y <= tau ? 1u : 0u) << (4 * j4 + 3);
          }
          mm[hh] = (q0 | q1) | (q2 | q3);
        }
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const uint32_t c0 = pr * 64u + (uint32_t)hh * 32u;
          uint32_t m = mm[hh] & ((c0 >= k) ? 0u : (k - c0 >= 32u ? 0xffffffffu : ((1u << (k - c0)) - 1u)));
          cnt += (uint32_t)__popc(m);
          while (m != 0u && got < 4u) {
            const uint32_t col = c0 + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            k0 = (got == 0) ? col : k0; k1 = (got == 1) ? col : k1;
            k2 = (got == 2) ? col : k2; k3 = (got == 3) ? col : k3;
            ++got;
          }
        }
        if (Dout && row < n) {
          for (int j = 0; j < 64; ++j)
            if (pr * 64u + j < k)
              Dout[row * k + pr * 64u + j] = fmaf(-2.0f, __uint_as_float(acc[j]), __ldg(cn2 + pr * 64u + j)) + x2;
        }
      }
      if (!released) {                                   // this half had no columns
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ts->tempty[buf]);
      }
      // The upper half hands its summary to the lower half: min(cnt, 7) and up
      // to four column offsets (7 bits each, relative to the half's first
      // column), written to the lower half's exchange slot, which only the
      // upper half reads and has already read.
      const uint32_t hbase = nlo * 64u;
      if (h == 1) {
        const uint32_t info = min(cnt, 7u) | (((k0 - hbase) & 127u) << 3) | (((k1 - hbase) & 127u) << 10) |
                              (((k2 - hbase) & 127u) << 17) | (((k3 - hbase) & 127u) << 24);
        xch[r] = __uint_as_float(info);
      }
      if (!pair_sync()) { if (lane == 0) fail(7); break; }
      if (h == 1) continue;
      {
        const uint32_t info = __float_as_uint(xch[r]);
        const uint32_t cb = info & 7u;
        // merge: the lower half's candidates come first (lower columns)
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
          if (i < cb && got < 4u) {
            const uint32_t col = hbase + ((info >> (3 + 7 * i)) & 127u);
            k0 = (got == 0) ? col : k0; k1 = (got == 1) ? col : k1;
            k2 = (got == 2) ? col : k2; k3 = (got == 3) ? col : k3;
            ++got;
          }
        }
        cnt += cb;
      }
      // Candidates in ascending column order: k0 is the lowest index.  NaN
      // anywhere (tau or v1) leaves cnt == 0: such a row takes the full path.
      const bool valid = row < n;
      if (valid) {
        labels[row] = k0;
        if (mindist) mindist[row] = v1 + x2;
      }
      RefineEntry e{(uint32_t)row, cnt, {k0, k1, k2, k3}};
      const uint64_t seg = row >> 5;
      seg_push(rq.cand, rq.ccnt, seg, valid && cnt >= 2 && cnt <= 4, e);
      seg_push(rq.full, rq.fcnt, seg, valid && (cnt == 0 || cnt > 4), (uint32_t)row);
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(tmem_base, 2u * nalloc);
}


// ---------------------------------------------------------------------------
// k > 256: the centroid operand no longer fits one MMA (N <= 256) nor shared
// memory, so it is walked in chunks of NC (256 or 128) centroids.
//
// Rows are processed in bands of gridDim.x * T tiles (T even, a band of X
// stays in L2): for each band every CTA takes its T tiles and, for each
// chunk j, loads chunk j of the centroids (one B slot per 64-column K block,
// each slot reloaded as soon as the MMAs of the previous chunk have read it)
// and runs its T tiles against it.  Each row keeps its running minimum m in
// shared memory and appends every centroid with v(c) <= tau(m) to its own
// list of up to L (index, value) pairs in global memory.  tau grows with m and
// m only falls, so after the last chunk the entries with v(c) <= tau(m_final)
// are exactly the candidate set of all k centroids; a full list is first
// compacted with the current tau, and a list that still overflows sends the
// row to the full re-score.  Final classification: one candidate = proven
// label, 2..4 = the short re-score queue, 5..L = the wide queue (one warp per
// row re-scores its list), otherwise the full re-score.
//
// Tile i of a band always goes to epilogue set i % 2 and TMEM buffer i % 2,
// so a row's state is only touched by one thread.
// ---------------------------------------------------------------------------
constexpr uint32_t TCC_OVF = 0xffffffffu;     // candidate list overflowed

struct TcSmemC {
  uint64_t full[16];
  uint64_t empty[16];
  uint64_t bfull[8];
  uint64_t bempty[8];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t tdone;
  uint32_t tmem_base;
  int abort;
};

__host__ __device__ constexpr uint32_t tcc_state_bytes(uint32_t T) { return T * TC_M * 8u; }

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1)
assign_tc_chunked_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                         const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
                         const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                         uint32_t k, uint32_t kp, uint32_t NC, uint32_t KB, uint32_t S, uint32_t T,
                         TieBound tb, DevState* st, uint32_t* __restrict__ labels,
                         float* __restrict__ mindist, RefineQueues rq, float* __restrict__ Dout) {
  constexpr bool ALO = MODE == TC_SPLIT3;
  constexpr bool BLO = MODE != TC_PLAIN;
  if (st->done) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const uint32_t slot_bytes = NC * 128u;                // one 64-column K block of NC centroids
  const uint32_t b_bytes = KB * slot_bytes;             // one of hi / lo
  uint8_t* sB = smem;
  uint8_t* sA = smem + b_bytes * (BLO ? 2u : 1u);
  const uint32_t unit_bytes = A_UNIT * (ALO ? 2u : 1u);
  uint8_t* sState = sA + (size_t)S * unit_bytes;
  const uint32_t rows_T = T * TC_M;
  float* st_m = reinterpret_cast<float*>(sState);       // running minimum per row
  uint32_t* st_cnt = reinterpret_cast<uint32_t*>(st_m + rows_T);   // entries in the row's list
  TcSmemC* ts = reinterpret_cast<TcSmemC*>(sState + tcc_state_bytes(T));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t ntiles = (n + TC_M - 1) / TC_M;
  const uint32_t nchunks = kp / NC;
  const uint64_t band_tiles = (uint64_t)gridDim.x * T;
  const float cmax = st->cmax;
  // valid tiles of this CTA in band b: i = 0..Tc-1 (tile = b*band_tiles + i*gridDim.x + blockIdx.x)
  auto tiles_in_band = [&](uint64_t b) -> uint32_t {
    const uint64_t first = b * band_tiles + blockIdx.x;
    if (first >= ntiles) return 0u;
    const uint64_t c = (ntiles - first + gridDim.x - 1) / gridDim.x;
    return (uint32_t)(c < T ? c : T);
  };
  auto tile_of = [&](uint64_t b, uint32_t i) -> uint64_t {
    return b * band_tiles + (uint64_t)i * gridDim.x + blockIdx.x;
  };

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < S; ++s) { mbar_init(&ts->full[s], 1); mbar_init(&ts->empty[s], 1); }
    for (uint32_t kb = 0; kb < KB; ++kb) { mbar_init(&ts->bfull[kb], 1); mbar_init(&ts->bempty[kb], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&ts->tfull[b], 1); mbar_init(&ts->tempty[b], 4); }
    mbar_init(&ts->tdone, 1);
    ts->abort = 0;
    mbar_fence_init();
  }
  if (warp == 2) tmem_alloc(&ts->tmem_base, 2u * NC);
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
      if (ALO) tma_prefetch_desc(&tmAlo);
      if (BLO) tma_prefetch_desc(&tmBlo);
      uint64_t u = 0, p = 0;
      bool ok = true;
      for (uint64_t b = 0; ok; ++b) {
        const uint32_t Tc = tiles_in_band(b);
        if (Tc == 0u) break;
        for (uint32_t j = 0; j < nchunks && ok; ++j, ++p) {
          for (uint32_t kb = 0; kb < KB; ++kb) {
            if (p > 0 && !mbar_wait_bounded(&ts->bempty[kb], (uint32_t)((p - 1) & 1u), abort_flag, WAIT_NS)) {
              fail(11); ok = false; break;
            }
            mbar_arrive_expect_tx(&ts->bfull[kb], slot_bytes * (BLO ? 2u : 1u));
            tma_load_2d(sB + (size_t)kb * slot_bytes, &tmB, (int)(kb * 64), (int)(j * NC), &ts->bfull[kb]);
            if (BLO) tma_load_2d(sB + b_bytes + (size_t)kb * slot_bytes, &tmBlo, (int)(kb * 64), (int)(j * NC),
                                &ts->bfull[kb]);
          }
          for (uint32_t i = 0; i < Tc && ok; ++i) {
            const uint64_t tile = tile_of(b, i);
            for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
              const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
              if (!mbar_wait_bounded(&ts->empty[s], ph ^ 1u, abort_flag, WAIT_NS)) { fail(12); ok = false; break; }
              mbar_arrive_expect_tx(&ts->full[s], unit_bytes);
              uint8_t* dst = sA + (size_t)s * unit_bytes;
              tma_load_2d(dst, &tmA, (int)(kb * 64), (int)(tile * TC_M), &ts->full[s]);
              if (ALO) tma_load_2d(dst + A_UNIT, &tmAlo, (int)(kb * 64), (int)(tile * TC_M), &ts->full[s]);
            }
          }
        }
      }
      // Drain every issued copy before the CTA exits (bounded, abort ignored).
      volatile int no_abort = 0;
      if (p > 0)
        for (uint32_t kb = 0; kb < KB; ++kb) mbar_wait_bounded(&ts->bfull[kb], (uint32_t)((p - 1) & 1u), &no_abort, WAIT_NS);
      const uint64_t first = u > S ? u - S : 0;
      for (uint64_t v = first; v < u; ++v) {
        const uint32_t s = (uint32_t)(v % S), ph = (uint32_t)((v / S) & 1u);
        mbar_wait_bounded(&ts->full[s], ph, &no_abort, WAIT_NS);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(TC_M, NC);
      const uint32_t sA0 = smem_u32(sA), sB0 = smem_u32(sB);
      uint64_t u = 0, p = 0;
      uint32_t use0 = 0u, use1 = 0u;                 // items issued on TMEM buffer 0 / 1
      bool ok = true, issued = false;
      for (uint64_t b = 0; ok; ++b) {
        const uint32_t Tc = tiles_in_band(b);
        if (Tc == 0u) break;
        for (uint32_t j = 0; j < nchunks && ok; ++j, ++p) {
          for (uint32_t i = 0; i < Tc && ok; ++i) {
            const uint32_t buf = i & 1u;
            const uint32_t ub = buf ? use1 : use0;
            if (!mbar_wait_bounded(&ts->tempty[buf], (ub & 1u) ^ 1u, abort_flag, WAIT_NS)) {
              fail(13); ok = false; break;
            }
            if (buf) ++use1; else ++use0;
            tc_fence_after();
            const uint32_t dt = tmem_base + buf * NC;
            for (uint32_t kb = 0; kb < KB; ++kb, ++u) {
              if (i == 0u) {
                if (!mbar_wait_bounded(&ts->bfull[kb], (uint32_t)(p & 1u), abort_flag, WAIT_NS)) {
                  fail(14); ok = false; break;
                }
              }
              const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
              if (!mbar_wait_bounded(&ts->full[s], ph, abort_flag, WAIT_NS)) { fail(15); ok = false; break; }
              tc_fence_after();
              const uint32_t a0 = sA0 + s * unit_bytes;
              const uint32_t b0 = sB0 + kb * slot_bytes;
#pragma unroll
              for (uint32_t kk = 0; kk < 4; ++kk) {
                const uint64_t ad = smem_desc_sw128(a0 + kk * 32u);
                const uint64_t bd = smem_desc_sw128(b0 + kk * 32u);
                tc_mma_bf16(dt, ad, bd, idesc, (kb | kk) != 0u ? 1u : 0u);
                if (BLO) tc_mma_bf16(dt, ad, smem_desc_sw128(b0 + b_bytes + kk * 32u), idesc, 1u);
                if (ALO) tc_mma_bf16(dt, smem_desc_sw128(a0 + A_UNIT + kk * 32u), bd, idesc, 1u);
              }
              tc_commit(&ts->empty[s]);
              if (i + 1u == Tc) tc_commit(&ts->bempty[kb]);   // B slot kb free once these complete
              issued = true;
            }
            if (!ok) break;
            tc_commit(&ts->tfull[buf]);
          }
        }
      }
      if (issued) {
        tc_commit(&ts->tdone);
        volatile int no_abort = 0;
        mbar_wait_bounded(&ts->tdone, 0, &no_abort, WAIT_NS);
      }
    }
  } else if (warp >= 4) {
    const int q = warp & 3;
    const uint32_t set = (uint32_t)(warp - 4) >> 2;
    const uint32_t npair = NC / 64u;
    const uint32_t r = (uint32_t)q * 32u + (uint32_t)lane;
    const uint32_t tbase = tmem_base + (((uint32_t)q * 32u) << 16) + set * NC;
    const float finf = __int_as_float(0x7f800000);
    uint32_t use = 0;
    bool ok = true;
    for (uint64_t b = 0; ok; ++b) {
      const uint32_t Tc = tiles_in_band(b);
      if (Tc == 0u) break;
      for (uint32_t j = 0; j < nchunks && ok; ++j) {
        const bool last = (j + 1u == nchunks);
        for (uint32_t i = set; i < Tc; i += 2u) {
          const uint64_t row = tile_of(b, i) * TC_M + r;
          const bool valid = row < n;
          const float x2 = valid ? xn2[row] : 0.0f;
          const uint32_t si = i * TC_M + r;
          // running minimum and candidate count of this row (list in global memory)
          float m = finf;
          uint32_t cnt = 0;
          if (j > 0) { m = st_m[si]; cnt = st_cnt[si]; }
          uint2* lst = rq.wl + (valid ? row : 0) * (uint64_t)rq.L;
          const bool okw = mbar_wait_bounded(&ts->tfull[set], use & 1u, abort_flag, WAIT_NS);
          ++use;
          if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(16); ok = false; break; }
          tc_fence_after();
          const float* cnj = cn2 + (size_t)j * NC;
          // ---- pass 1: chunk minimum ----
          float m0 = finf, m1 = finf, m2 = finf, m3 = finf;
          for (uint32_t pr = 0; pr < npair; ++pr) {
            uint32_t acc[64];
            tmem_ld_32x32b_x64(tbase + pr * 64u, acc);
            tmem_ld_wait();
            const float4* cn4 = reinterpret_cast<const float4*>(cnj + pr * 64u);
#pragma unroll
            for (int j4 = 0; j4 < 16; j4 += 2) {
              const float4 ca = __ldg(cn4 + j4), cb = __ldg(cn4 + j4 + 1);
              const float2 va = dist_pair(acc[4 * j4 + 0], acc[4 * j4 + 1], ca.x, ca.y);
              const float2 vb = dist_pair(acc[4 * j4 + 2], acc[4 * j4 + 3], ca.z, ca.w);
              const float2 vc = dist_pair(acc[4 * j4 + 4], acc[4 * j4 + 5], cb.x, cb.y);
              const float2 vd = dist_pair(acc[4 * j4 + 6], acc[4 * j4 + 7], cb.z, cb.w);
              m0 = fmin3(m0, va.x, va.y);
              m1 = fmin3(m1, vb.x, vb.y);
              m2 = fmin3(m2, vc.x, vc.y);
              m3 = fmin3(m3, vd.x, vd.y);
            }
          }
          const float mc = fmin3(m0, m1, fminf(m2, m3));
          const float mn = fminf(m, mc);
          const float tau = tie_tau(x2, mn, cmax, tb);
          // ---- pass 2: append this chunk's {c < k : v(c) <= tau} to the row's list ----
          // Entries of earlier chunks above the final tau are dropped after the
          // last chunk; tau only falls, so the list is a superset until then.
          const bool collect = tau < finf && valid;       // tau = +inf only while every value is +inf
          for (uint32_t pr = 0; pr < npair; ++pr) {
            uint32_t acc[64];
            tmem_ld_32x32b_x64(tbase + pr * 64u, acc);
            tmem_ld_wait();
            const float4* cn4 = reinterpret_cast<const float4*>(cnj + pr * 64u);
            uint32_t mm[2] = {0u, 0u};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
#pragma unroll
              for (int j4 = 0; j4 < 8; ++j4) {
                const float4 cc = __ldg(cn4 + 8 * h + j4);
                const int a = 32 * h + 4 * j4;
                const float2 va = dist_pair(acc[a + 0], acc[a + 1], cc.x, cc.y);
                const float2 vb = dist_pair(acc[a + 2], acc[a + 3], cc.z, cc.w);
                mm[h] |= (va.x <= tau ? 1u : 0u) << (4 * j4 + 0);
                mm[h] |= (va.y <= tau ? 1u : 0u) << (4 * j4 + 1);
                mm[h] |= (vb.x <= tau ? 1u : 0u) << (4 * j4 + 2);
                mm[h] |= (vb.y <= tau ? 1u : 0u) << (4 * j4 + 3);
              }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint32_t col0 = j * NC + pr * 64u + (uint32_t)h * 32u;     // global centroid index
              uint32_t mk = collect ? mm[h] : 0u;
              mk &= (col0 >= k) ? 0u : (k - col0 >= 32u ? 0xffffffffu : ((1u << (k - col0)) - 1u));
              while (mk != 0u && cnt != TCC_OVF) {
                const uint32_t bit = (uint32_t)(__ffs(mk) - 1);
                mk &= mk - 1u;
                if (cnt == rq.L) {
                  // full: drop entries of earlier chunks that the current tau excludes
                  uint32_t kept = 0;
                  for (uint32_t e = 0; e < cnt; ++e) {
                    const uint2 en = lst[e];
                    if (__uint_as_float(en.y) <= tau) { if (kept != e) lst[kept] = en; ++kept; }
                  }
                  cnt = kept;
                  if (cnt == rq.L) { cnt = TCC_OVF; break; }
                }
                // the candidate's accumulator by selection (static register indices)
                uint32_t a = 0u;
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) a = ((uint32_t)jj == bit) ? acc[h * 32 + jj] : a;
                const float vv = fmaf(-2.0f, __uint_as_float(a), __ldg(cnj + pr * 64u + h * 32u + bit));
                lst[cnt] = make_uint2(col0 + bit, __float_as_uint(vv));
                ++cnt;
              }
            }
            if (Dout && valid) {
#pragma unroll
              for (int jj = 0; jj < 64; ++jj) {
                const uint32_t col = j * NC + pr * 64u + (uint32_t)jj;
                if (col < k) Dout[row * k + col] = fmaf(-2.0f, __uint_as_float(acc[jj]), cnj[pr * 64u + jj]) + x2;
              }
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ts->tempty[set]);     // accumulator buffer free
          if (!last) {
            st_m[si] = mn;
            st_cnt[si] = cnt;
          } else {
            // Final filter with tau(m): keep {c : v(c) <= tau}, compacted in
            // list order; note the first four for the short queue.
            uint32_t kept = 0, c0 = 0, c1 = 0, c2 = 0, c3 = 0;
            if (cnt != TCC_OVF) {
              for (uint32_t e = 0; e < cnt; ++e) {
                const uint2 en = lst[e];
                if (__uint_as_float(en.y) <= tau) {
                  if (kept != e) lst[kept] = en;
                  c0 = (kept == 0) ? en.x : c0; c1 = (kept == 1) ? en.x : c1;
                  c2 = (kept == 2) ? en.x : c2; c3 = (kept == 3) ? en.x : c3;
                  ++kept;
                }
              }
            }
            // NaN leaves kept == 0: full re-score, as does an overflowed list.
            const uint32_t cf = (cnt == TCC_OVF) ? TCC_OVF : kept;
            if (valid) {
              labels[row] = c0;
              if (mindist) mindist[row] = mn + x2;
              if (cf > 4u && cf != 0xffffffffu) rq.wlc[row] = cf;
            }
            RefineEntry e{(uint32_t)row, cf, {c0, c1, c2, c3}};
            const uint64_t seg = row >> 5;
            seg_push(rq.cand, rq.ccnt, seg, valid && cf >= 2u && cf <= 4u, e);
            seg_push(rq.wide, rq.wcnt, seg, valid && cf > 4u && cf <= rq.L, (uint32_t)row);
            seg_push(rq.full, rq.fcnt, seg, valid && (cf == 0u || cf > rq.L), (uint32_t)row);
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(tmem_base, 2u * NC);
}

}  // namespace

TcPlan plan_tc(uint32_t dp, uint32_t kp, int mode, uint64_t n, int num_sms) {
  TcPlan p;
  if (dp == 0 || dp % 64 != 0 || kp < 16 || kp > 256 || kp % 16 != 0) return p;
  p.KB = dp / 64;
  const size_t b_bytes = (size_t)p.KB * kp * 128 * (mode != TC_PLAIN ? 2 : 1);
  const size_t unit = (size_t)A_UNIT * (mode == TC_SPLIT3 ? 2 : 1);
  const size_t fixed = 1024 /*align*/ + 2 * TC_M * sizeof(float) /*xch*/ + sizeof(TcSmem) + 64;
  const size_t budget = 227 * 1024;
  if (b_bytes + fixed + 2 * unit > budget) return p;
  size_t s = (budget - b_bytes - fixed) / unit;
  if (s > 8) s = 8;
  p.stages = (uint32_t)s;
  p.nalloc = 64;                 // >= 64: a 64-column TMEM load never leaves the buffer
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

TcPlan plan_tc_chunked(uint32_t dp, uint32_t k, int mode, uint64_t n, int num_sms) {
  TcPlan p;
  if (dp == 0 || dp % 64 != 0 || k == 0) return p;
  const uint32_t KB = dp / 64;
  if (KB > 8) return p;
  const size_t bmult = mode != TC_PLAIN ? 2 : 1, amult = mode == TC_SPLIT3 ? 2 : 1;
  const size_t unit = (size_t)A_UNIT * amult;
  const size_t budget = 227 * 1024;
  const size_t band_max = 48ull << 20;             // rows of one band stay in L2
  for (uint32_t NC : {256u, 128u}) {
    if (NC == 256u && k <= 128u) continue;         // one 128-wide chunk wastes less
    const size_t b_bytes = (size_t)KB * NC * 128 * bmult;
    for (uint32_t T : {8u, 6u, 4u, 2u}) {
      const size_t band = (size_t)num_sms * T * TC_M * dp * 2 * amult;
      if (band > band_max && T > 2) continue;
      const size_t fixed = 1024 + b_bytes + tcc_state_bytes(T) + sizeof(TcSmemC) + 64;
      if (fixed + 2 * unit > budget) continue;
      size_t s = (budget - fixed) / unit;
      if (s > 8) s = 8;
      p.chunked = true;
      p.KB = KB;
      p.NC = NC;
      p.T = T;
      p.kp = (k + NC - 1) / NC * NC;
      p.stages = (uint32_t)s;
      p.nalloc = NC;
      p.smem = fixed + s * unit;
      const uint64_t ntiles = (n + TC_M - 1) / TC_M;
      p.grid = (int)std::min<uint64_t>(ntiles, (uint64_t)num_sms);
      if (p.grid < 1) p.grid = 1;
      p.ok = true;
      return p;
    }
  }
  return p;
}

namespace {
template <int MODE>
km_status set_attr_mode(const TcPlan& pl) {
  if (pl.chunked)
    KM_CUDA_TRY(cudaFuncSetAttribute(assign_tc_chunked_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
  else
    KM_CUDA_TRY(cudaFuncSetAttribute(assign_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
  return KM_OK;
}

template <int MODE>
void launch_mode(const TcPlan& pl, const CUtensorMap& tmA, const CUtensorMap& tmAlo, const CUtensorMap& tmB,
                 const CUtensorMap& tmBlo, const float* cn2, const float* xn2, uint64_t n, uint32_t k,
                 uint32_t kp, TieBound tb, DevState* st, uint32_t* labels, float* mindist,
                 const RefineQueues& rq, float* Dout, cudaStream_t s) {
  if (pl.chunked)
    assign_tc_chunked_kernel<MODE><<<pl.grid, TC_THREADS, pl.smem, s>>>(
        tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, pl.NC, pl.KB, pl.stages, pl.T, tb, st, labels,
        mindist, rq, Dout);
  else
    assign_tc_kernel<MODE><<<pl.grid, TC_THREADS, pl.smem, s>>>(
        tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, pl.KB, pl.stages, pl.nalloc, tb, st, labels,
        mindist, rq, Dout);
}
}  // namespace

km_status tc_set_attributes(const TcPlan& pl, int mode) {
  if (!pl.ok) return KM_ERR_UNSUPPORTED;
  switch (mode) {
    case TC_PLAIN: return set_attr_mode<TC_PLAIN>(pl);
    case TC_SPLIT3: return set_attr_mode<TC_SPLIT3>(pl);
    case TC_SPLIT2: return set_attr_mode<TC_SPLIT2>(pl);
  }
  return KM_ERR_ARG;
}

km_status launch_assign_tc(const TcPlan& pl, int mode, const CUtensorMap& tmA,
                           const CUtensorMap& tmAlo, const CUtensorMap& tmB,
                           const CUtensorMap& tmBlo, const float* cn2, const float* xn2,
                           uint64_t n, uint32_t k, uint32_t kp, TieBound tb, DevState* st,
                           uint32_t* labels, float* mindist, const RefineQueues& rq,
                           float* Dout, cudaStream_t s) {
  if (!pl.ok) return KM_ERR_UNSUPPORTED;
  switch (mode) {
    case TC_PLAIN: launch_mode<TC_PLAIN>(pl, tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, tb, st, labels, mindist, rq, Dout, s); break;
    case TC_SPLIT3: launch_mode<TC_SPLIT3>(pl, tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, tb, st, labels, mindist, rq, Dout, s); break;
    case TC_SPLIT2: launch_mode<TC_SPLIT2>(pl, tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, tb, st, labels, mindist, rq, Dout, s); break;
    default: return KM_ERR_ARG;
  }
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

}  // namespace km
