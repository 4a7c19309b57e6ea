// Lloyd engine: device buffers of one (n, d, k) problem and the launchers of
// the per-iteration kernel sequence.
#pragma once

#include <cuda.h>

#include <vector>
#include "km_internal.cuh"

namespace km {

// ---- kernels (km_lloyd_kernels.cu) ----
__global__ void prep_points_kernel(const float* X, uint64_t n, uint32_t d, uint32_t dp, float* xn2,
                                   double* xn2d, __nv_bfloat16* Xb, __nv_bfloat16* Xlo,
                                   DevState* st);
__global__ void reduce_f64_partial_kernel(const double* v, uint64_t n, double* part);
__global__ void reduce_f64_final_kernel(const double* part, int np, double* out);
__global__ void prep_centroids_kernel(const float* C, uint32_t k, uint32_t kp, uint32_t d,
                                      uint32_t dp, float* cn2, __nv_bfloat16* Cb,
                                      __nv_bfloat16* Clo, float* Ct, DevState* st, uint32_t kp64);
km_status launch_assign_f32(const float* X, const float* C, const float* cn2, const float* xn2,
                            uint64_t n, uint32_t d, uint32_t k, TieBound tb, DevState* st,
                            uint32_t* labels, float* mindist, const RefineQueues& rq,
                            float* Dout, cudaStream_t s);
km_status launch_refine(bool v4, int num_sms, const float* X, const float* C, const float* Ct,
                        uint32_t d, uint32_t k, DevState* st, const RefineQueues& rq,
                        uint32_t* labels, float* mindist, cudaStream_t s);
// Chunked-kernel refinement: candidate and wide queues as launch_refine; rows
// of the full queue go through the FP32 distance kernel on those rows alone
// (gathered by index into fidx) and then the exact re-score of its near ties.
km_status launch_refine_gemm(bool v4, int num_sms, const float* X, const float* C, const float* Ct,
                             const float* cn2, const float* xn2, uint64_t n, uint32_t d, uint32_t k,
                             TieBound tb32, DevState* st, const RefineQueues& rq,
                             const RefineQueues& rq2, uint32_t* fidx, uint32_t* nfull,
                             uint32_t* labels, float* mindist, cudaStream_t s);
__global__ void seg_hist_kernel(const uint32_t* labels, uint64_t n, uint32_t k, uint32_t seg,
                                uint32_t nseg, uint32_t* seghist, DevState* st);
// cstart non-null: the block that finishes last also runs cluster_scan_kernel's
// work (at most 512 threads per block).
__global__ void seg_scan_kernel(uint32_t* seghist, uint32_t k, uint32_t nseg, uint32_t* counts,
                                DevState* st, uint32_t* cstart, uint32_t* order);
// order (nullable, k <= 1024): clusters by descending count, ties by index.
__global__ void cluster_scan_kernel(const uint32_t* counts, uint32_t k, uint32_t* cstart,
                                    DevState* st, uint32_t* order);
__global__ void seg_scatter_kernel(const uint32_t* labels, uint64_t n, uint32_t k, uint32_t seg,
                                   uint32_t nseg, const uint32_t* seghist, const uint32_t* cstart,
                                   uint32_t* perm, DevState* st);
__global__ void finalize_kernel(const float* Cn, float* C, const float* dsq, const double* objpart,
                                const uint32_t* counts, int32_t empty_excl,
                                uint32_t d, uint32_t dp, uint32_t k, float tol, float* cn2,
                                __nv_bfloat16* Cb, __nv_bfloat16* Clo, float* Ct,
                                double* shift_c, double* obj_c, DevState* st, LoopConsts lc);

// ---- tensor-core distance stage (km_tc.cu) ----
struct TcPlan {
  bool ok = false;
  bool chunked = false;  // k > 256: centroids walked in chunks of NC (assign_tc_chunked_kernel)
  uint32_t KB = 0;       // K blocks of 64 columns
  uint32_t stages = 0;   // A pipeline depth (K-block units)
  uint32_t nalloc = 0;   // TMEM columns per accumulator buffer
  uint32_t NC = 0;       // chunked: centroids per chunk (128 or 256)
  uint32_t T = 0;        // chunked: tiles per CTA per band (even)
  uint32_t kp = 0;       // chunked: k padded to a multiple of NC
  size_t smem = 0;       // dynamic shared memory bytes
  int grid = 0;
};
// Operand modes of the tensor-core distance kernels.  PLAIN: BF16 x BF16.
// SPLIT3: x = hi + lo and c = hi + lo, hi*hi + hi*lo + lo*hi.  SPLIT2: the
// points are exact in BF16 (lo = 0), so hi*hi + hi*lo_c alone.
enum : int { TC_PLAIN = 0, TC_SPLIT3 = 1, TC_SPLIT2 = 2 };
TcPlan plan_tc(uint32_t dp, uint32_t kp, int mode, uint64_t n, int num_sms);
TcPlan plan_tc_chunked(uint32_t dp, uint32_t k, int mode, uint64_t n, int num_sms);
km_status encode_tmap_bf16(CUtensorMap* tm, const void* base, uint64_t inner, uint64_t outer,
                           uint32_t box_inner, uint32_t box_outer);
km_status tc_set_attributes(const TcPlan& pl, int mode);
km_status launch_assign_tc(const TcPlan& pl, int mode, const CUtensorMap& tmA,
                           const CUtensorMap& tmAlo, const CUtensorMap& tmB,
                           const CUtensorMap& tmBlo, const float* cn2, const float* xn2,
                           uint64_t n, uint32_t k, uint32_t kp, TieBound tb, DevState* st,
                           uint32_t* labels, float* mindist, const RefineQueues& rq,
                           float* Dout, cudaStream_t s);

km_status update_sums_prepare();
// Shared-memory limits of the staged re-score and FP32 distance kernels (once
// per process and device, before their first launch).
km_status refine_prepare();
// order (nullable): the clusters' processing order (largest first).
km_status launch_update_sums(const float* X, const uint32_t* perm, const uint32_t* cstart, uint32_t d,
                             uint32_t k, const float* C, float* Cn, float* dsq, double* objpart,
                             DevState* st, cudaStream_t s, const uint32_t* order = nullptr);

// ---- engine ----
// Tile list of one symmetric kernel-matrix build of rows [row0, row_end)
// (device array of `count` (row tile, column block | flags) pairs).
struct KmatTileList {
  uint64_t row0 = 0, row_end = 0, count = 0;
  uint32_t* dev = nullptr;
};

struct LloydEngine {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t aux = nullptr;           // second stream of the chunked host-to-device copy
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int num_sms = 0;
  uint64_t n = 0;
  uint32_t d = 0, k = 0, dp = 0, kp = 0;
  int precision = KM_PREC_FP32;

  const float* X = nullptr;   // points (owned copy or borrowed)
  float* X_owned = nullptr;
  float* xn2 = nullptr;
  double* xn2d = nullptr;
  __nv_bfloat16* Xb = nullptr;
  __nv_bfloat16* Xlo = nullptr;
  float* C = nullptr;
  float* Cn = nullptr;
  float* cn2 = nullptr;
  float* dsq = nullptr;
  double* objpart = nullptr;
  double* shift_c = nullptr;
  double* obj_c = nullptr;
  __nv_bfloat16* Cb = nullptr;
  __nv_bfloat16* Clo = nullptr;
  uint32_t* labels = nullptr;
  float* mindist = nullptr;
  RefineEntry* queue = nullptr;
  uint32_t* qfull = nullptr;
  uint32_t* qcnt = nullptr;   // per 32-row segment counts of queue / qfull
  uint32_t* qfcnt = nullptr;
  RefineQueues rq{};
  float* Ct = nullptr;        // centroids transposed (d x k) for the full re-score
  bool refine_v4 = false;
  uint32_t* seghist = nullptr;
  uint32_t* counts = nullptr;
  uint32_t* cstart = nullptr;
  uint32_t* perm = nullptr;
  double* red_part = nullptr;
  DevState* st = nullptr;
  DevState* h_st = nullptr;   // pinned mirror
  uint32_t seg = 1024, nseg = 0;
  int sort_wpb = 8;
  size_t sort_smem = 0;
  RefineQueues rq2{};           // chunked kernel: queues of the FP32 pass over full rows
  RefineEntry* q2 = nullptr;
  uint32_t *q2full = nullptr, *q2cnt = nullptr, *q2fcnt = nullptr, *fidx = nullptr, *nfull = nullptr;
  TieBound tb32{};
  uint32_t* order = nullptr;   // clusters by descending size (centroid sums, k <= 1024)
  uint32_t* qwide = nullptr;   // chunked kernel: rows with 5..32 candidates
  uint32_t* qwcnt = nullptr;
  uint32_t* wlc = nullptr;
  uint2* wl = nullptr;
  TieBound tb{};
  TcPlan tc{};
  int tc_mode = 0;          // TC_PLAIN / TC_SPLIT3 / TC_SPLIT2
  bool a_exact = false;     // every point coordinate is a BF16 value
  CUtensorMap tmA{}, tmAlo{}, tmB{}, tmBlo{};
  bool data_ready = false;
  std::vector<KmatTileList> kmat_lists;   // symmetric kernel-matrix builds (km_kkm.cu)

  ~LloydEngine();
  km_status init(uint64_t n, uint32_t d, uint32_t k, int precision, int device, void* stream,
                 bool need_update);
  km_status set_points(const float* Xsrc, bool on_device, bool copy);
  // Points stored as BF16 (raw bit patterns, n*d): decoded once to the FP32
  // copy, which is then exactly representable in BF16 (Xb = the input).
  km_status set_points_bf16(const uint16_t* Xsrc, bool on_device);
  km_status set_centroids_dev(const float* Csrc_dev);   // C <- src, prep norms/bf16, cmax
  km_status reset_state();
  km_status enqueue_distance(float* Dout);   // distance + argmin kernel only
  km_status enqueue_refine();                // exact re-score of the queued rows
  km_status enqueue_assign(float* Dout);     // both
  km_status enqueue_finalize(const LoopConsts& lc);
  km_status enqueue_sort(const uint32_t* lab);
  km_status enqueue_update_step(float tol);
  km_status enqueue_iteration(const LoopConsts& lc);
  km_status read_state();
  km_status check_device_error();
};

// Greedy k-means++ centroids into e.C (km_init.cu).
km_status plusplus_init(LloydEngine& e, int seed);

}  // namespace km
