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

// Epilogue sets of four warps in the k <= 256 kernel, by form: the split
// forms (two or three MMAs per K step) keep pace with two sets, whose warps then
// get 168 registers (no spill); the single-BF16 form, with a third of the MMA
// work per tile, is faster with three (128 registers).  Measured at n = 1M,
// d = 128, k = 256: split-BF16x3 distance 0.150 ms with two sets, 0.153 with
// three; single-BF16 iterations 3322 it/s with two sets, 3476 with three.
__host__ __device__ constexpr int tc_sets(int mode) { return mode == TC_PLAIN ? 3 : 2; }
__host__ __device__ constexpr int tc_threads(int mode) { return 32 * (4 + 4 * tc_sets(mode)); }
constexpr int TCC_THREADS = 32 * (4 + 8);               // chunked kernel: two sets of four
constexpr int TC_M = 128;
constexpr uint64_t WAIT_NS = 2000000000ull;
constexpr uint32_t A_UNIT = TC_M * 128;  // bytes of one 128-row x 64-col BF16 K-block
constexpr uint32_t TC_MAX_UNITS = 16;
// Suspend-time hint of the k <= 256 kernel's waits: a waiting warp sleeps
// (until the phase completes) instead of spinning on issue slots the epilogue needs.
constexpr uint32_t TC_HINT_NS = 1000;
// Accumulator-full barriers: tile t (this CTA's t-th) completes tfull[t % NTF],
// NTF = 2 x sets.  Each of them is waited on by one epilogue set only (set
// t % sets), tile after tile, so a parity wait never aliases another set's phase.
constexpr int TC_NTF_MAX = 6;

struct TcSmem {
  uint64_t full[TC_MAX_UNITS];
  uint64_t empty[TC_MAX_UNITS];
  uint64_t bfull;
  uint64_t tfull[TC_NTF_MAX];
  uint64_t tempty[2];
  uint64_t tdone;
  uint32_t tmem_base;
  int abort;
};

// Centroid norms as the epilogue reads them: padded with +inf to 256.
struct TcXch {
  float cn2[256];
};

__device__ __forceinline__ void tmem_ld_32x32b_x16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

// DOUT: the distance-matrix output (km_distances); a template parameter so that
// the assignment-only instance carries none of its code or registers.
template <int MODE, bool DOUT>
__global__ void __launch_bounds__(tc_threads(MODE), 1)
assign_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                 const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
                 const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                 uint32_t k, uint32_t kp, uint32_t KB, uint32_t S, uint32_t nalloc, TieBound tb,
                 DevState* st, uint32_t* __restrict__ labels, float* __restrict__ mindist,
                 RefineQueues rq, float* __restrict__ Dout) {
  constexpr bool ALO = MODE == TC_SPLIT3;      // point operand has a lo part
  constexpr bool BLO = MODE != TC_PLAIN;       // centroid operand has a lo part
  constexpr uint32_t UPK = ALO ? 2u : 1u;      // ring units per K block (hi, then lo)
  constexpr int SETS = tc_sets(MODE), NTF = 2 * SETS, EPI_WARPS = 4 * SETS;
  static_assert(NTF <= TC_NTF_MAX, "accumulator-full barriers");
  griddep_wait();
  if (st->done) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const uint32_t b_bytes = KB * kp * 128u;              // one of hi / lo
  uint8_t* sB = smem;
  uint8_t* sA = smem + b_bytes * (BLO ? 2u : 1u);
  TcXch* xch = reinterpret_cast<TcXch*>(sA + (size_t)S * A_UNIT);
  TcSmem* ts = reinterpret_cast<TcSmem*>(xch + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t ntiles = (n + TC_M - 1) / TC_M;
  const float cmax = st->cmax;
  const float finf = __int_as_float(0x7f800000);

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < S; ++s) { mbar_init(&ts->full[s], 1); mbar_init(&ts->empty[s], 1); }
    mbar_init(&ts->bfull, 1);
    for (int b = 0; b < NTF; ++b) mbar_init(&ts->tfull[b], 1);
    for (int b = 0; b < 2; ++b) mbar_init(&ts->tempty[b], 4);
    mbar_init(&ts->tdone, 1);
    ts->abort = 0;
    mbar_fence_init();
  }
  if (warp >= 4) {
    // centroid norms (padded with +inf by the host to a multiple of 64) into
    // shared memory, +inf up to 256
    const uint32_t kp64 = (kp + 63u) & ~63u;
    for (uint32_t i = threadIdx.x - 128u; i < 256u; i += 32u * EPI_WARPS)
      xch->cn2[i] = i < kp64 ? cn2[i] : finf;
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
      // Ring of S units of one 128 x 64 BF16 block each: per K block the hi
      // part, then (split form) the lo part.
      uint64_t u = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        for (uint32_t kb = 0; kb < KB && ok; ++kb) {
#pragma unroll
          for (uint32_t part = 0; part < UPK; ++part, ++u) {
            const uint32_t s = (uint32_t)(u % S), ph = (uint32_t)((u / S) & 1u);
            if (!mbar_wait_bounded(&ts->empty[s], ph ^ 1u, abort_flag, WAIT_NS, TC_HINT_NS)) {
              fail(1); ok = false; break;
            }
            mbar_arrive_expect_tx(&ts->full[s], A_UNIT);
            tma_load_2d(sA + (size_t)s * A_UNIT, part ? &tmAlo : &tmA, (int)(kb * 64), (int)(tile * TC_M),
                        &ts->full[s]);
          }
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
        if (!mbar_wait_bounded(&ts->tempty[buf], (use & 1u) ^ 1u, abort_flag, WAIT_NS, TC_HINT_NS)) {
          fail(3); ok = false; break;
        }
        tc_fence_after();
        const uint32_t dt = tmem_base + buf * nalloc;
        for (uint32_t kb = 0; kb < KB; ++kb, u += UPK) {
          const uint32_t sh = (uint32_t)(u % S), phh = (uint32_t)((u / S) & 1u);
          const uint32_t sl = (uint32_t)((u + 1) % S), phl = (uint32_t)(((u + 1) / S) & 1u);
          if (!mbar_wait_bounded(&ts->full[sh], phh, abort_flag, WAIT_NS, TC_HINT_NS) ||
              (ALO && !mbar_wait_bounded(&ts->full[sl], phl, abort_flag, WAIT_NS, TC_HINT_NS))) {
            fail(4); ok = false; break;
          }
          tc_fence_after();
          const uint32_t a0 = sA0 + sh * A_UNIT, al = sA0 + sl * A_UNIT;
          const uint32_t b0 = sB0 + kb * kp * 128u;
#pragma unroll
          for (uint32_t kk = 0; kk < 4; ++kk) {
            const uint64_t ad = smem_desc_sw128(a0 + kk * 32u);
            const uint64_t bd = smem_desc_sw128(b0 + kk * 32u);
            tc_mma_bf16(dt, ad, bd, idesc, (kb | kk) != 0u ? 1u : 0u);
            if (BLO) tc_mma_bf16(dt, ad, smem_desc_sw128(b0 + b_bytes + kk * 32u), idesc, 1u);
            if (ALO) tc_mma_bf16(dt, smem_desc_sw128(al + kk * 32u), bd, idesc, 1u);
          }
          tc_commit(&ts->empty[sh]);
          if (ALO) tc_commit(&ts->empty[sl]);
          issued = true;
        }
        if (!ok) break;
        tc_commit(&ts->tfull[t % NTF]);
      }
      // All MMAs of this thread complete before teardown.
      if (issued) {
        tc_commit(&ts->tdone);
        volatile int no_abort = 0;
        mbar_wait_bounded(&ts->tdone, 0, &no_abort, WAIT_NS);
      }
    }
  } else if (warp >= 4) {
    // Epilogue: SETS sets of four warps; set s takes this CTA's tiles
    // t = s, s + SETS, ... (TMEM buffer t % 2), so several tiles are in the
    // epilogue at once and no warp waits for another.  Warp w of a set owns
    // TMEM lanes (rows) 32*(w%4)..+31 and each thread sweeps its whole row in
    // groups of 64 columns: v = ||c||^2 - 2 acc, the group minimum, the running
    // minimum m, and the group's candidate mask {c < k : v(c) <= tau(m)}
    // (tie_tau).  tau only grows with m, so each mask is a superset of the
    // group's part of the final set {c : v(c) <= tau(v1)}, and a group whose
    // minimum is above tau(v1) holds none of it.  The buffer is released after
    // the last group's load.  Final candidates: the masks of the groups whose
    // minimum is <= tau(v1); extra entries can only be centroids with
    // v(c) > tau(v1), which the exact re-score never picks.
    const int q = warp & 3, set = (warp - 4) >> 2;
    const uint32_t r = (uint32_t)q * 32u + (uint32_t)lane;
    const uint32_t ng = (kp + 63u) / 64u;                // 64-column groups (1..4)
    const float* cns = xch->cn2;
    for (uint64_t t = (uint64_t)set;; t += SETS) {
      const uint64_t tile = blockIdx.x + t * gridDim.x;
      if (tile >= ntiles) break;
      const uint32_t buf = (uint32_t)(t & 1u);
      const uint64_t row = tile * TC_M + r;
      const bool valid = row < n;
      const float x2 = valid ? xn2[row] : 0.0f;
      const TauRow tr = tie_tau_row(x2, cmax, tb);
      const bool okw = mbar_wait_bounded(&ts->tfull[t % NTF], (uint32_t)((t / NTF) & 1u), abort_flag,
                                         WAIT_NS, TC_HINT_NS);
      if (!__all_sync(0xffffffffu, okw)) { if (lane == 0) fail(5); break; }
      tc_fence_after();
      const uint32_t tb0 = tmem_base + (((uint32_t)q * 32u) << 16) + buf * nalloc;
      float m = finf;
      float gmin[4];
      uint32_t glo[4], ghi[4];
#pragma unroll
      for (uint32_t g = 0; g < 4; ++g) {
        gmin[g] = finf; glo[g] = 0u; ghi[g] = 0u;
        if (g >= ng) continue;
        const uint32_t cg = g * 64u;
        const uint32_t nld = min(4u, (kp - cg) / 16u);   // 16-column loads in this group
        // acc holds the accumulator, then (in place) v = ||c||^2 - 2 acc
        uint32_t acc[64];
        if (nld == 4u) {
          tmem_ld_32x32b_x64(tb0 + cg, acc);
        } else {
#pragma unroll
          for (uint32_t u = 0; u < 4; ++u) {
            if (u < nld) {
              tmem_ld_32x32b_x16(tb0 + cg + u * 16u, acc + 16u * u);
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j) acc[16u * u + j] = 0u;  // v = +inf from the padded norms
            }
          }
        }
        tmem_ld_wait();
        if (g + 1u == ng) {
          // last load of this tile: the accumulator buffer is free
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ts->tempty[buf]);
        }
        {
          float m0 = finf, m1 = finf, m2 = finf, m3 = finf;
#pragma unroll
          for (int j4 = 0; j4 < 16; ++j4) {
            const float4 cc = *reinterpret_cast<const float4*>(cns + cg + 4 * j4);
            const float2 va = dist_pair(acc[4 * j4 + 0], acc[4 * j4 + 1], cc.x, cc.y);
            const float2 vb = dist_pair(acc[4 * j4 + 2], acc[4 * j4 + 3], cc.z, cc.w);
            acc[4 * j4 + 0] = __float_as_uint(va.x); acc[4 * j4 + 1] = __float_as_uint(va.y);
            acc[4 * j4 + 2] = __float_as_uint(vb.x); acc[4 * j4 + 3] = __float_as_uint(vb.y);
            if (j4 & 1) { m2 = fmin3(m2, va.x, va.y); m3 = fmin3(m3, vb.x, vb.y); }
            else        { m0 = fmin3(m0, va.x, va.y); m1 = fmin3(m1, vb.x, vb.y); }
          }
          gmin[g] = fminf(fminf(m0, m1), fminf(m2, m3));
        }
        m = fminf(m, gmin[g]);
        const float tau = tie_tau_at(tr, m, tb);
        const uint32_t nval = cg < k ? min(64u, k - cg) : 0u;   // columns < k of this group
        uint32_t p0 = 0u, p1 = 0u, p2 = 0u, p3 = 0u;
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          p0 |= (__uint_as_float(acc[j + 0]) <= tau ? 1u : 0u) << (j + 0);
          p1 |= (__uint_as_float(acc[j + 1]) <= tau ? 1u : 0u) << (j + 1);
          p2 |= (__uint_as_float(acc[j + 2]) <= tau ? 1u : 0u) << (j + 2);
          p3 |= (__uint_as_float(acc[j + 3]) <= tau ? 1u : 0u) << (j + 3);
        }
        glo[g] = ((p0 | p1) | (p2 | p3)) & (nval >= 32u ? 0xffffffffu : ((1u << nval) - 1u));
        p0 = p1 = p2 = p3 = 0u;
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          p0 |= (__uint_as_float(acc[32 + j + 0]) <= tau ? 1u : 0u) << (j + 0);
          p1 |= (__uint_as_float(acc[32 + j + 1]) <= tau ? 1u : 0u) << (j + 1);
          p2 |= (__uint_as_float(acc[32 + j + 2]) <= tau ? 1u : 0u) << (j + 2);
          p3 |= (__uint_as_float(acc[32 + j + 3]) <= tau ? 1u : 0u) << (j + 3);
        }
        ghi[g] = ((p0 | p1) | (p2 | p3)) &
                 (nval >= 64u ? 0xffffffffu : (nval > 32u ? ((1u << (nval - 32u)) - 1u) : 0u));
        if (DOUT && valid) {
#pragma unroll
          for (int j = 0; j < 64; ++j)
            if ((uint32_t)j < nval) Dout[row * k + cg + j] = __uint_as_float(acc[j]) + x2;
        }
      }
      // Final set: the masks of the groups whose minimum is within tau(v1),
      // in column order; k0 is the lowest candidate index.  NaN anywhere
      // (tau or v1) leaves cnt == 0: such a row takes the full path.
      const float v1 = m;
      const float tau = tie_tau_at(tr, v1, tb);
      uint32_t cnt = 0, got = 0, k0 = 0, k1 = 0, k2 = 0, k3 = 0;
#pragma unroll
      for (uint32_t g = 0; g < 4; ++g) {
        if (!(gmin[g] <= tau)) continue;
        cnt += (uint32_t)(__popc(glo[g]) + __popc(ghi[g]));
#pragma unroll
        for (uint32_t hh = 0; hh < 2; ++hh) {
          uint32_t mk = hh ? ghi[g] : glo[g];
          while (mk != 0u && got < 4u) {
            const uint32_t col = g * 64u + hh * 32u + (uint32_t)(__ffs(mk) - 1);
            mk &= mk - 1u;
            k0 = (got == 0) ? col : k0; k1 = (got == 1) ? col : k1;
            k2 = (got == 2) ? col : k2; k3 = (got == 3) ? col : k3;
            ++got;
          }
        }
      }
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
__global__ void __launch_bounds__(TCC_THREADS, 1)
assign_tc_chunked_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                         const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
                         const float* __restrict__ cn2, const float* __restrict__ xn2, uint64_t n,
                         uint32_t k, uint32_t kp, uint32_t NC, uint32_t KB, uint32_t S, uint32_t T,
                         TieBound tb, DevState* st, uint32_t* __restrict__ labels,
                         float* __restrict__ mindist, RefineQueues rq, float* __restrict__ Dout) {
  constexpr bool ALO = MODE == TC_SPLIT3;
  constexpr bool BLO = MODE != TC_PLAIN;
  griddep_wait();
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
  const size_t upk = mode == TC_SPLIT3 ? 2 : 1;             // ring units per K block
  const size_t fixed = 1024 /*align*/ + sizeof(TcXch) + sizeof(TcSmem) + 64;
  const size_t budget = 227 * 1024;
  if (b_bytes + fixed + 2 * upk * A_UNIT > budget) return p;
  size_t s = (budget - b_bytes - fixed) / A_UNIT;
  if (s > TC_MAX_UNITS) s = TC_MAX_UNITS;
  p.stages = (uint32_t)s;
  p.nalloc = 64;                 // >= 64: a 64-column TMEM load never leaves the buffer
  while (p.nalloc < kp) p.nalloc <<= 1;
  p.smem = b_bytes + fixed + s * A_UNIT;
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
  else {
    KM_CUDA_TRY(cudaFuncSetAttribute(assign_tc_kernel<MODE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pl.smem));
    KM_CUDA_TRY(cudaFuncSetAttribute(assign_tc_kernel<MODE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pl.smem));
  }
  return KM_OK;
}

template <int MODE>
void launch_mode(const TcPlan& pl, const CUtensorMap& tmA, const CUtensorMap& tmAlo, const CUtensorMap& tmB,
                 const CUtensorMap& tmBlo, const float* cn2, const float* xn2, uint64_t n, uint32_t k,
                 uint32_t kp, TieBound tb, DevState* st, uint32_t* labels, float* mindist,
                 const RefineQueues& rq, float* Dout, cudaStream_t s) {
  if (pl.chunked)
    (void)launch_pdl(assign_tc_chunked_kernel<MODE>, pl.grid, TCC_THREADS, pl.smem, s, tmA, tmAlo, tmB, tmBlo, cn2,
                     xn2, n, k, kp, pl.NC, pl.KB, pl.stages, pl.T, tb, st, labels, mindist, rq, Dout);
  else
    (void)launch_pdl(Dout ? assign_tc_kernel<MODE, true> : assign_tc_kernel<MODE, false>, pl.grid, tc_threads(MODE),
                     pl.smem, s, tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k, kp, pl.KB, pl.stages, pl.nalloc, tb, st,
                     labels, mindist, rq, Dout);
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
