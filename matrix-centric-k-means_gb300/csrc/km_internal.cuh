// Internal definitions shared by the libkm_sm103 translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>

#include "../../include/km.h"

namespace km {

// ---------------------------------------------------------------------------
// Host-side error plumbing: every CUDA call maps to a km_status; nothing exits.
// ---------------------------------------------------------------------------
#define KM_CUDA_TRY(expr)                                                        \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess) {                                                     \
      km::set_last_error(_e, #expr, __FILE__, __LINE__);                         \
      return (_e == cudaErrorMemoryAllocation) ? KM_ERR_ALLOC : KM_ERR_CUDA;     \
    }                                                                            \
  } while (0)

#define KM_TRY(expr)                          \
  do {                                        \
    km_status _s = (expr);                    \
    if (_s != KM_OK) return _s;               \
  } while (0)

void set_last_error(cudaError_t e, const char* what, const char* file, int line);

// ---------------------------------------------------------------------------
// Device-resident loop state of one fit.  Every per-iteration kernel reads
// `done` first and returns when it is set, so iterations enqueued past the stop
// cost one empty launch each and no host synchronisation is needed per
// iteration.
// ---------------------------------------------------------------------------
struct DevState {
  uint32_t done;            // fit finished (stop rule fired or maxiter reached)
  uint32_t iter;            // iterations executed
  uint32_t converged_iter;  // iteration at which the stop rule fired (0: not yet)
  uint32_t moved;           // some centroid moved more than tol in this iteration
  uint32_t x_not_bf16;      // set_data: some coordinate is not exactly a BF16 value
  uint32_t err;             // device error bits (KM_DEVERR_*)
  uint32_t err_where;       // first wait that ran out (diagnostics)
  uint32_t fin_ticket;       // finalize blocks done in this iteration (the last one resets it)
  unsigned long long refined_total;  // rows re-scored (all iterations)
  unsigned long long full_total;     // of those, against all k centroids
  float cmax;               // max_c ||c|| of the centroids the next assignment uses
  uint32_t scan_ticket;      // seg_scan blocks done in this iteration (the last one resets it)
  double objective;         // FP64 objective of the last assignment
  double last_score;
  double score;
  double max_shift;
  double sum_x2;            // FP64 sum_i ||x_i||^2
};

enum : uint32_t {
  KM_DEVERR_TIMEOUT = 1u,   // a bounded wait ran out
  KM_DEVERR_NONFINITE = 2u, // input held NaN/Inf
  KM_DEVERR_OVERFLOW = 4u   // refinement list overflow (cannot happen: list holds n)
};

// Programmatic dependent launch.  A kernel launched with launch_pdl may be
// scheduled while its predecessor in the stream is still draining; it calls
// griddep_wait() before it reads anything the predecessor wrote (the wait
// returns once the predecessor grid has completed and its writes are
// visible).  In a kernel launched without the attribute the wait is a no-op.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// Host mapping of the device error bits to a status (timeouts first).
inline km_status status_of_device_error(uint32_t err) {
  if (err & KM_DEVERR_TIMEOUT) return KM_ERR_TIMEOUT;
  if (err & (KM_DEVERR_NONFINITE | KM_DEVERR_OVERFLOW)) return KM_ERR_ARG;
  return KM_OK;
}

// Per-fit constants passed by value to the kernels that end an iteration
// (finalize_kernel, kkm_control_kernel).
struct LoopConsts {
  uint64_t maxiter;
  float tol;
  int32_t conv;       // km_conv
  int32_t empty;      // km_empty
};

// ---------------------------------------------------------------------------
// Near-tie bound.  A fast-path distance is v(c) = fl(||c||^2 - 2 * dot(x, c)),
// with |v(c) - (||c||^2 - 2 x.c)| <= E(c) = A*||x||*||c|| + B*||c||^2, where
// A = 2*eps_dot + 2u covers the dot-product error and the final rounding and
// B = 2u covers the rounding of ||c||^2 and of the subtraction.  The
// reference's CPU distance sum_j fl(fl(x_j - c_j)^2), summed in float, has
// relative error at most g = gamma_{d+2}.  If, with T an upper bound of
// ||x||^2, v1 <= v2 <= v3 the three smallest fast values and c1 the argmin,
//   (v2 - v1) > Emax + E1 + g * (2T + v1 + v2 + E1 - Emax)
// then the reference's argmin is c1 (class 0).  The same test with v3 in place
// of v2 proves it is one of the two best fast candidates (class 1); otherwise
// the row is re-scored against all k centroids (class 2).  Both refinements use
// the reference's exact formula, so the final labels equal the reference's.
// ---------------------------------------------------------------------------
struct TieBound {
  float A;      // coefficient of ||x||*||c||
  float B;      // coefficient of ||c||^2
  float g;      // relative error of the reference CPU distance
  float safety; // multiplier on the right-hand side (covers this test's own rounding)
};

// a_exact: every point coordinate is exactly a BF16 value, so only the
// centroid operand carries a rounding error.
TieBound make_tie_bound(int precision, uint32_t d, bool a_exact);

__device__ __forceinline__ int tie_class(float X2, float v1, float v2, float v3, float cn1,
                                         float cmax, const TieBound& tb) {
  const float nx = sqrtf(X2) * 1.0000005f;
  const float T = X2 * 1.0000003f;
  const float E1 = tb.A * nx * cn1 + tb.B * cn1 * cn1;
  const float Em = tb.A * nx * cmax + tb.B * cmax * cmax;
  const float base = Em + E1;
  const float s = fmaxf(0.0f, 2.0f * T + v1 + E1 - Em);
  const float rhs2 = tb.safety * (base + tb.g * (s + v2)) + 1e-30f;
  const float rhs3 = tb.safety * (base + tb.g * (s + v3)) + 1e-30f;
  // NaN or Inf anywhere makes the comparisons false: such rows take the full path.
  const bool fin = isfinite(T + v1 + E1 + Em);
  if (fin && (v2 - v1) > rhs2) return 0;
  if (fin && (v3 - v1) > rhs3) return 1;
  return 2;
}

// Top-3 of (value, index) under the order (v, i) < (w, j) iff v < w or
// (v == w and i < j).  Only the two best keep their index; the third value can
// never move into the top two when two such lists are merged.
struct Top3 {
  float v1, v2, v3;
  uint32_t i1, i2;
  __device__ __forceinline__ void init() {
    v1 = v2 = v3 = __int_as_float(0x7f800000);
    i1 = i2 = 0xffffffffu;
  }
  __device__ __forceinline__ void insert(float v, uint32_t i) {
    if (v < v1 || (v == v1 && i < i1)) {
      v3 = v2; v2 = v1; i2 = i1; v1 = v; i1 = i;
    } else if (v < v2 || (v == v2 && i < i2)) {
      v3 = v2; v2 = v; i2 = i;
    } else if (v < v3) {
      v3 = v;
    }
  }
  // Branch-free insertion under the (v, i) order (selects only, so that lanes
  // of a warp never diverge).
  __device__ __forceinline__ void insert_nb(float v, uint32_t i) {
    const bool c1 = v < v1 || (v == v1 && i < i1);
    const bool c2 = v < v2 || (v == v2 && i < i2);
    const bool c3 = v < v3;
    v3 = c2 ? v2 : (c3 ? v : v3);
    v2 = c1 ? v1 : (c2 ? v : v2);
    i2 = c1 ? i1 : (c2 ? i : i2);
    v1 = c1 ? v : v1;
    i1 = c1 ? i : i1;
  }
  // Insertion when every index already held is below i (columns visited in
  // ascending order): a tie keeps the earlier entry, so strict '<' gives the
  // (v, i) order for finite values.
  __device__ __forceinline__ void insert_asc(float v, uint32_t i) {
    const bool c1 = v < v1, c2 = v < v2, c3 = v < v3;
    v3 = c2 ? v2 : (c3 ? v : v3);
    v2 = c1 ? v1 : (c2 ? v : v2);
    i2 = c1 ? i1 : (c2 ? i : i2);
    v1 = c1 ? v : v1;
    i1 = c1 ? i : i1;
  }
  __device__ __forceinline__ void merge(const Top3& o) {
    insert_nb(o.v1, o.i1);
    insert_nb(o.v2, o.i2);
    v3 = fminf(v3, o.v3);
  }
  __device__ __forceinline__ void shfl_merge_xor(int mask, unsigned members = 0xffffffffu) {
    Top3 o;
    o.v1 = __shfl_xor_sync(members, v1, mask);
    o.v2 = __shfl_xor_sync(members, v2, mask);
    o.v3 = __shfl_xor_sync(members, v3, mask);
    o.i1 = __shfl_xor_sync(members, i1, mask);
    o.i2 = __shfl_xor_sync(members, i2, mask);
    merge(o);
  }
};

// Refinement queue entry: a row whose reference argmin is proven to be one of
// `cnt` (2..4) candidate centroids.  Rows with more candidates go to the
// full-rescore queue (row index only).
struct RefineEntry {
  uint32_t row;
  uint32_t cnt;
  uint32_t c[4];
};

// The two refinement queues and their per-segment counts.
struct RefineQueues {
  RefineEntry* cand;   // rows with 2..4 candidates
  uint32_t* full;      // rows re-scored against all k
  uint32_t* ccnt;      // per 32-row segment: entries in cand
  uint32_t* fcnt;      // per 32-row segment: entries in full
  uint64_t nseg;       // segments (rows rounded up to whole 128-row tiles, / 32)
  // chunked distance kernel only (null otherwise): rows with 5..L candidates
  uint32_t* wide;      // row ids, segmented like full
  uint32_t* wcnt;      // per segment: entries in wide
  uint2* wl;           // per row: L (centroid, value bits) pairs, candidates first (L <= 256)
  uint32_t* wlc;       // per row: candidates in wl (valid for rows in wide)
  uint32_t L;
};

// Refinement queues are segmented by rows: the 32 rows r with r >> 5 == seg own
// slots [32*seg, 32*seg + 32) and a count cnt[seg].  The full warp that
// classified those rows writes both, so no global counter (and no atomic
// round-trip on the distance kernels' critical path) is involved, and the
// queue order is deterministic.  Must be called by all 32 lanes.
template <class T>
__device__ __forceinline__ void seg_push(T* q, uint32_t* cnt, uint64_t seg, bool want, const T& e) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  const int lane = threadIdx.x & 31;
  if (want) q[seg * 32 + __popc(m & ((1u << lane) - 1u))] = e;
  if (lane == 0) cnt[seg] = (uint32_t)__popc(m);
}

// Candidate threshold for one row: every centroid with fast value v(c) > tau
// has a reference CPU distance strictly above the row's best (the TieBound
// argument with E1 <= Emax), so the reference argmin lies in {c : v(c) <= tau}.
// The row-dependent part of tie_tau (T = bound of ||x||^2, Em = the largest
// fast-path error), so that tau can be evaluated for several v1 of one row.
struct TauRow {
  float T, Em;
};
__device__ __forceinline__ TauRow tie_tau_row(float X2, float cmax, const TieBound& tb) {
  const float nx = sqrtf(X2) * 1.0000005f;
  return TauRow{X2 * 1.0000003f, tb.A * nx * cmax + tb.B * cmax * cmax};
}
// Non-decreasing in v1 (every operation is monotone), so a threshold taken at
// a running minimum is never below the one of the final minimum.
__device__ __forceinline__ float tie_tau_at(const TauRow& r, float v1, const TieBound& tb) {
  const float s = fmaxf(0.0f, 2.0f * r.T + v1 + 2.0f * r.Em);
  const float sg = tb.safety * tb.g;
  float tau = (v1 + tb.safety * (2.0f * r.Em + tb.g * s) + 1e-30f) / (1.0f - sg);
  return fmaxf(tau, v1);
}
__device__ __forceinline__ float tie_tau(float X2, float v1, float cmax, const TieBound& tb) {
  return tie_tau_at(tie_tau_row(X2, cmax, tb), v1, tb);
}

// Reference CPU distance, bit-exact: float, j ascending, no contraction.
__device__ __forceinline__ float cpu_dist(const float* __restrict__ x, const float* __restrict__ c,
                                          uint32_t d) {
  float s = 0.0f;
  for (uint32_t j = 0; j < d; ++j) {
    const float t = __fsub_rn(x[j], c[j]);
    s = __fadd_rn(s, __fmul_rn(t, t));
  }
  return s;
}

// ---------------------------------------------------------------------------
// Bounded waits (mbarrier) and tcgen05 / TMA wrappers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait with a suspend-time hint: the thread may sleep up to hint_ns (or
// until the phase completes) instead of returning at once.
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Waits for the phase with the given parity to complete, at most `limit_ns`
// nanoseconds.  Returns false on timeout (or when *abort is raised by a peer).
// hint_ns > 0 lets a waiting warp sleep between checks, leaving issue slots to
// the other warps of its scheduler.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  volatile int* abort, uint64_t limit_ns,
                                                  uint32_t hint_ns = 0) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  uint32_t spins = 0;
  while (true) {
    if (hint_ns ? mbar_try_wait_hint(bar, parity, hint_ns) : mbar_try_wait(bar, parity)) return true;
    if (hint_ns || (++spins & 63u) == 0) {
      if (*abort) return false;
      if (globaltimer_ns() - t0 > limit_ns) return false;
    }
  }
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 2-D tiled TMA load into shared memory, completing on an mbarrier.
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const void* tmap, int32_t x, int32_t y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Non-tensor bulk copy global -> shared (16-byte aligned addresses, size a
// multiple of 16), completing on an mbarrier.
__device__ __forceinline__ void bulk_copy_g2s(void* smem_dst, const void* gsrc, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// 16-byte cp.async (zero-filled beyond src_bytes) and an mbarrier arrival that
// fires when all of this thread's prior cp.async copies have landed (the
// barrier's expected count must include this arrival: .noinc).
__device__ __forceinline__ void cp_async16_zfill(void* smem, const void* gmem, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem),
               "r"(src_bytes)
               : "memory");
}
// cp.async groups: close the thread's open group; wait until at most N of its
// groups are still in flight (the landed copies are visible to this thread;
// __syncwarp / __syncthreads then orders them for the others).
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_mbar_arrive_noinc(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const void* tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}

// tcgen05: TMEM allocation (one warp), MMA (one thread), commit, loads.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D(tmem) (+)= A(smem desc) * B(smem desc)^T, kind::f16 (BF16 inputs, FP32 accumulate).
__device__ __forceinline__ void tc_mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on an mbarrier when all previously issued MMAs of this thread complete.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 32 lanes x 32 bit, 32 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

// 32 lanes x 32 bit, 64 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld_32x32b_x64(uint32_t taddr, uint32_t (&r)[64]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
      "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
      "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]),
        "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]),
        "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]),
        "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]),
        "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]),
        "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr)
      : "memory");
}

// Three-input minimum (one instruction on sm_100 and later); a NaN input is
// ignored as by fminf.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// v = c - 2 a for two adjacent accumulator columns in one packed FMA; each
// half is rounded exactly as fmaf(-2, a, c).
__device__ __forceinline__ float2 dist_pair(uint32_t a0, uint32_t a1, float c0, float c1) {
  return __ffma2_rn(make_float2(-2.0f, -2.0f), make_float2(__uint_as_float(a0), __uint_as_float(a1)),
                    make_float2(c0, c1));
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor for a K-major operand in the 128-byte swizzle
// layout: 8-row groups of 128-byte rows, groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t desc = 0;
  desc |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
  desc |= (uint64_t)(16u >> 4) << 16;                    // leading byte offset (unused for SW128 K-major)
  desc |= (uint64_t)(1024u >> 4) << 32;                  // stride byte offset: 8 rows x 128 B
  desc |= (uint64_t)1 << 46;                             // descriptor version (tcgen05)
  desc |= (uint64_t)2 << 61;                             // layout: 128-byte swizzle
  return desc;
}

// Instruction descriptor, kind::f16: BF16 A/B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// ---------------------------------------------------------------------------
// Launch helpers implemented in the .cu files.
// ---------------------------------------------------------------------------
struct Scratch;  // per-call scratch owned by a handle or a stateless call

}  // namespace km
