/*
 * km.h — C ABI of libkm_sm103, the GB300 (sm_103a) k-means iteration library.
 *
 * Plain C: pointers, sizes and status codes only.  Host arrays are ordinary
 * pointers; "dev" arguments are CUDA device pointers on the handle's device.
 * Streams are passed as void* (a cudaStream_t), NULL meaning the library's own
 * stream.  Every function returns a km_status; nothing calls exit().
 *
 * Reference interfaces replaced (HicrestLaboratory/Matrix-Centric-K-Means):
 *   Kmeans::Kmeans(n,d,k,tol,seed,points,...)  src/kmeans.cuh:117-121, src/kmeans.cu:71-305
 *   Kmeans::run(maxiter, check_converged)       src/kmeans.cuh:130, src/kmeans.cu:772-1105
 *   Kmeans::get_score()                         src/kmeans.cuh:139
 *   CPU Kmeans::Kmeans / run                    comparisons/CPU_Kmeans/include/kmeans.h:31-33
 *   init_kernel_mtx<Kernel>(...)                src/kernels/kernels.cuh:653-718 (+ :43-118)
 *   compute_distances_popcorn_spmv(...)         src/kernels/distances.cu:895-1002
 *   RAFT coalescedReduction argmin + counts     src/kmeans.cu:923-947
 *   compute_v_sparse_csr + exclusive_scan       src/kernels/kernels.cuh:296-314, src/kmeans.cu:987-1031
 *   CPU compute_centroids / cmp_centroids       comparisons/CPU_Kmeans/src/kmeans.cpp:131-155, :190-200
 *   CHECK_* exit-on-error macros                src/cuda_utils.cu:10-41 (replaced by km_status)
 */
#ifndef KM_H
#define KM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The gpukmeans CLI maps them to the reference's exit codes
 * (src/include/utils.hpp:34-37). */
typedef enum km_status {
  KM_OK = 0,
  KM_ERR_ARG = 1,          /* invalid argument (k > n, k == 0, d == 0, size overflow, NaN input, ...) */
  KM_ERR_ALLOC = 2,        /* device or host allocation failed */
  KM_ERR_CUDA = 3,         /* a CUDA runtime/driver call failed */
  KM_ERR_TIMEOUT = 4,      /* a bounded device-side wait ran out; the kernel stopped and reported it */
  KM_ERR_UNSUPPORTED = 5,  /* shape/precision combination this build does not run */
  KM_ERR_NO_DEVICE = 6,    /* no sm_103 device (the library has no CPU path) */
  KM_ERR_STATE = 7         /* call out of order (e.g. fit before set_data) */
} km_status;

/* Initialisation.  KM_INIT_SAMPLE: k distinct seeded sample picks exactly as the
 * reference CPU k-means draws them (mt19937(seed_seq{seed}) +
 * uniform_int_distribution<int>(0,n-1), comparisons/CPU_Kmeans/src/kmeans.cpp:22-29,49-84).
 * KM_INIT_ROUND_ROBIN: labels i % k, as the reference GPU path
 * (src/kmeans.cu:365-374).  KM_INIT_GIVEN: caller-supplied centroids.
 * KM_INIT_PLUSPLUS: greedy k-means++ on the device with s = 2 + ceil(ln k)
 * D^2-sampled candidates per round (src/kmeans.cu:447-769), drawn from `seed`
 * (the reference draws from std::random_device); k <= e^14. */
typedef enum km_init {
  KM_INIT_SAMPLE = 0,
  KM_INIT_ROUND_ROBIN = 1,
  KM_INIT_GIVEN = 2,
  KM_INIT_PLUSPLUS = 3
} km_init;

/* Arithmetic of the distance stage.  FP32: SIMT FP32 GEMM.  BF16: tcgen05
 * tensor cores on BF16 operands, FP32 accumulate.  BF16X3: split-BF16
 * (hi*hi + hi*lo + lo*hi) on tcgen05.  In every precision, rows whose top-2
 * distance margin is inside the proven error bound are re-scored with the
 * reference CPU formula, so labels equal the reference's. */
typedef enum km_precision {
  KM_PREC_FP32 = 0,
  KM_PREC_BF16 = 1,
  KM_PREC_BF16X3 = 2
} km_precision;

/* Stop rule.  SHIFT: every centroid moved <= tol (float, reference CPU rule,
 * kmeans.cpp:190-200), tested from iteration 2.  SCORE: |score - last| < tol
 * (reference GPU rule with -c 1, src/kmeans.cu:1068-1073).  NONE: run maxiter. */
typedef enum km_conv {
  KM_CONV_SHIFT = 0,
  KM_CONV_SCORE = 1,
  KM_CONV_NONE = 2
} km_conv;

/* Kernel functions for kernel k-means (src/kernels/kernels.cuh:43-118 plus
 * Gaussian).  K_ij = f(x_i, x_j):
 *   LINEAR   x.y
 *   POLY     (gamma x.y + coef)^degree   (reference: gamma=1, coef=1, degree=2)
 *   SIGMOID  tanh(gamma x.y + coef)      (reference: gamma=1, coef=1)
 *   GAUSSIAN exp(-||x-y||^2 / (2 sigma^2)) */
typedef enum km_kernel_fn {
  KM_KERNEL_LINEAR = 0,
  KM_KERNEL_POLY = 1,
  KM_KERNEL_SIGMOID = 2,
  KM_KERNEL_GAUSSIAN = 3
} km_kernel_fn;

/* Empty clusters.  ZERO: the centroid of an empty cluster is the zero vector
 * and stays selectable (reference CPU rule, comparisons/CPU_Kmeans/src/kmeans.cpp:131-155).
 * EXCLUDE: an empty cluster's distance is +inf from then on, so it is never
 * chosen again (reference GPU rule: c~ = 0 -> +inf, src/kernels/distances.cu:588-599). */
typedef enum km_empty {
  KM_EMPTY_ZERO = 0,
  KM_EMPTY_EXCLUDE = 1
} km_empty;

typedef struct km_lloyd_params {
  uint64_t n;          /* points */
  uint32_t d;          /* dimensions */
  uint32_t k;          /* clusters, 1 <= k <= n */
  float tol;           /* -t */
  int32_t seed;        /* -s */
  uint64_t maxiter;    /* -m */
  int32_t init;        /* km_init */
  int32_t precision;   /* km_precision */
  int32_t conv;        /* km_conv */
  int32_t device;      /* CUDA device ordinal */
  void* stream;        /* cudaStream_t, or NULL */
  int32_t empty;       /* km_empty */
} km_lloyd_params;

typedef struct km_result {
  uint64_t converged_iter;  /* what the reference's run() returns: converged iteration or maxiter */
  uint64_t iterations;      /* iterations executed */
  int32_t converged;        /* 1 if the stop rule fired */
  int32_t reserved0;
  double objective;         /* FP64 sum_i ||x_i - c_{label_i}||^2 of the last assignment step */
  double score;             /* reference GPU score: objective - sum_i ||x_i||^2 (src/kmeans.cu:1054-1061) */
  double max_shift;         /* FP64 largest centroid move in the last iteration */
  uint64_t refined_rows;    /* rows re-scored with the CPU formula, all iterations */
  uint64_t full_rescore_rows; /* of those, rows re-scored against all k centroids */
  double fit_ms;            /* device time of the iteration loop */
  uint64_t kernel_launches; /* kernels this library launched inside the timed iteration loop */
} km_result;

typedef struct km_lloyd km_lloyd;
typedef struct km_kkm km_kkm;

const char* km_status_str(km_status s);
const char* km_version(void);

/* Number of sm_103 devices visible; 0 when none. */
int km_device_count(void);

/* Free and total device memory of `device` (the reference prints the footprint
 * from cudaMemGetInfo, src/kmeans.cu:1090-1096). */
km_status km_mem_info(int32_t device, uint64_t* free_bytes, uint64_t* total_bytes);

/* ---- Lloyd k-means handle: replaces Kmeans(...) + run() + get_score() ---- */

/* Validates the parameters and allocates the device buffers for (n, d, k). */
km_status km_lloyd_create(const km_lloyd_params* p, km_lloyd** out);

/* Copies the n*d row-major float32 points in (host pointer if on_device == 0,
 * device pointer on the handle's device otherwise), rejects NaN/Inf, and
 * prepares the per-point data (norms, BF16 copies) once. */
km_status km_lloyd_set_data(km_lloyd* h, const float* X, int on_device);

/* Points stored as BF16 (n*d raw bit patterns, row-major; host pointer if
 * on_device == 0).  The points ARE these BF16 values: they are widened once
 * to FP32 (exact) for the re-score and the centroid update, and used as they
 * are as the tensor-core operand. */
km_status km_lloyd_set_data_bf16(km_lloyd* h, const uint16_t* X, int on_device);

/* Runs the iteration.  C0: k*d host centroids for KM_INIT_GIVEN, else NULL.
 * labels_out: n host uint32 (may be NULL); centroids_out: k*d host floats
 * (may be NULL); res may be NULL. */
km_status km_lloyd_fit(km_lloyd* h, const float* C0, uint32_t* labels_out,
                       float* centroids_out, km_result* res);

/* Runs only the configured initialisation and returns the k*d initial
 * centroids (host array); C0 as in km_lloyd_fit. */
km_status km_lloyd_init(km_lloyd* h, const float* C0, float* centroids_out);

/* Changes the iteration budget and stop rule of a handle before its next fit
 * (Kmeans::run(maxiter, check_converged) sets both at run time,
 * src/kmeans.cuh:130). */
km_status km_lloyd_configure(km_lloyd* h, uint64_t maxiter, float tol, int32_t conv);

/* Device-resident results of the last fit (valid until the next fit/destroy). */
km_status km_lloyd_device_results(km_lloyd* h, const uint32_t** labels_dev,
                                  const float** centroids_dev, const uint32_t** counts_dev);

/* Stage timing (the reference's [PERFORMANCE] lines, src/kmeans.cu:837-1048):
 * continues from the state of the last fit for `iters` more iterations, without
 * the stop rule.  One iteration (the fit's kernels) is captured as a CUDA graph
 * with event-record nodes between the stages and replayed `iters` times on the
 * handle's stream (launched directly, stage by stage, if the capture fails);
 * writes the mean milliseconds per iteration of each stage to stage_ms[0..4]:
 * 0 distance+argmin, 1 near-tie refinement, 2 label sort (V), 3 centroid sums
 * (V.X), 4 finalize + loop control.  Labels and centroids advance as in a fit. */
km_status km_lloyd_profile(km_lloyd* h, uint64_t iters, double* stage_ms);

void km_lloyd_destroy(km_lloyd* h);

/* ---- Kernel groups on device pointers (stream-ordered, no host sync) ---- */

/* (a)+(b) Distance stage fused with argmin, plus exact near-tie refinement:
 * labels[i] = argmin_c sum_j (x_ij - c_cj)^2 evaluated as the reference CPU
 * does (kmeans.cpp:86-122: float, j ascending, lowest index on ties).
 * Replaces the reference's distance + RAFT argmin steps (src/kmeans.cu:847-936).
 * mindist (optional, may be NULL): the row's fast-path distance estimate. */
km_status km_assign(const float* X_dev, const float* C_dev, uint64_t n, uint32_t d,
                    uint32_t k, int32_t precision, uint32_t* labels_dev,
                    float* mindist_dev, uint64_t* refined_rows, void* stream);

/* Numerics probe of the distance stage alone: D[i,c] = ||x_i||^2 + ||c||^2 - 2 x_i.c
 * as the fast path computes it (n*k row-major float32, device). */
km_status km_distances(const float* X_dev, const float* C_dev, uint64_t n, uint32_t d,
                       uint32_t k, int32_t precision, float* D_dev, void* stream);

/* (c) Centroid update as the one-hot SpMM V.X over a stable label-sorted
 * permutation: C[c] = (sum_{i in c, i ascending} x_i) * float(1/(double)max(|c|,1)),
 * float sums in point order (kmeans.cpp:131-148); counts exact.
 * perm_dev (optional) receives the label-sorted permutation, offsets_dev
 * (optional, k+1) the cluster start offsets (CSR row pointers of V). */
km_status km_update(const float* X_dev, const uint32_t* labels_dev, uint64_t n, uint32_t d,
                    uint32_t k, float* C_dev, uint32_t* counts_dev, uint32_t* perm_dev,
                    uint32_t* offsets_dev, void* stream);

/* km_update without any device allocation.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory, such as hosts that
 * own all device memory through their own pool and forbid cudaMalloc/cudaFree
 * after start-up (those calls synchronise the device and fragment the pool),
 * or latency-critical loops where an allocation is an unbounded stall.
 *
 * Same arithmetic and results as km_update (C and counts), but its scratch
 * (label-sort counters and the label-sorted permutation) is one file-scope
 * device array of KM_NOALLOC_SCRATCH_BYTES that every GPU loading the library
 * holds until the process exits; it calls no cudaMalloc, cudaFree or other
 * allocating routine.  Limits: n <= KM_NOALLOC_MAX_N and k <= KM_NOALLOC_MAX_K;
 * larger sizes return KM_ERR_UNSUPPORTED before any work.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress, with that
 * device current); with CUDA's lazy module loading that is also when the array
 * is placed on the device, so make the first call before a pool claims the
 * device's memory (or set CUDA_MODULE_LOADING=EAGER).  Every call shares the
 * array and the call clears what must start at zero: calls that overlap on the
 * GPU (other streams or host threads) race and must not be issued.
 * The call enqueues all of its work on `stream`, then synchronises that stream
 * once, at the end, to read the error bits back; so it blocks the host until
 * the update is done, and it cannot be used while the stream is being captured.
 * Labels >= k return KM_ERR_ARG (C_dev is then undefined), a device wait that
 * ran out KM_ERR_TIMEOUT.  counts_dev may be NULL. */
#define KM_NOALLOC_MAX_N 1048576u
#define KM_NOALLOC_MAX_K 1024u
#define KM_NOALLOC_SCRATCH_BYTES 5505024u
km_status km_update_noalloc(const float* X_dev, const uint32_t* labels_dev, uint64_t n, uint32_t d,
                            uint32_t k, float* C_dev, uint32_t* counts_dev, void* stream);

/* ---- Kernel k-means (popcorn formulation, src/kmeans.cu + distances.cu:895-1002) ---- */

/* K = f(X X^T) (n*n row-major).  out_bf16 == 0 stores float32, 1 stores bf16.
 * precision: KM_PREC_FP32 (SIMT FP32), KM_PREC_BF16 or KM_PREC_BF16X3 (tcgen05).
 * diag_dev (optional, n floats) receives K_ii. */
km_status km_kernel_matrix(const float* X_dev, uint64_t n, uint32_t d, int32_t kernel_fn,
                           float gamma, float coef, int32_t degree, float sigma,
                           int32_t precision, int32_t out_bf16, void* K_dev,
                           float* diag_dev, void* stream);

typedef struct km_kkm_params {
  uint64_t n;
  uint32_t d;
  uint32_t k;
  float tol;
  uint64_t maxiter;
  int32_t kernel_fn;   /* km_kernel_fn */
  float gamma, coef, sigma;
  int32_t degree;
  int32_t precision;   /* K build arithmetic (km_precision) */
  int32_t k_bf16;      /* store K as bf16 (1) or float32 (0) */
  int32_t check_converged; /* reference -c: stop on |score - last| < tol */
  int32_t device;
  void* stream;
  /* Where K lives.  0: the whole n*n matrix stays resident (the reference's
   * B, src/kmeans.cu:143), built once by km_kkm_set_data.  r > 0: only a
   * panel of min(r, n) rows is held; every iteration rebuilds K panel by
   * panel and streams each panel into E = K V^T, so memory is r*n instead
   * of n*n and n is no longer capped by n^2 bytes.  The panels hold the same
   * values as the resident matrix, so labels and score are identical.
   * KM_KKM_FUSED (tensor-core precisions): no K at all; every iteration
   * multiplies X by a label-sorted copy of X on the tensor cores and sums
   * each row's kernel values per cluster in the epilogue (memory n*d; labels
   * within tolerance of the resident path, not bitwise: another summation
   * order; k_bf16 does not apply).  KM_KKM_PANEL_AUTO: resident when n*n fits
   * in 90% of the free device memory, else fused (tensor-core precisions) or
   * panels sized to half of it (FP32). */
  uint64_t panel_rows;
} km_kkm_params;

#define KM_KKM_PANEL_AUTO UINT64_MAX
#define KM_KKM_FUSED (UINT64_MAX - 1)

km_status km_kkm_create(const km_kkm_params* p, km_kkm** out);
/* Builds K from n*d points (host or device). */
km_status km_kkm_set_data(km_kkm* h, const float* X, int on_device);
/* Device time of the kernel-matrix build done by the last km_kkm_set_data
 * (with panels: only the operand preparation, K is built per iteration). */
km_status km_kkm_build_ms(km_kkm* h, double* ms);
/* Rows of K per panel chosen at create (0: K resident, KM_KKM_FUSED: no K). */
km_status km_kkm_panel_rows(km_kkm* h, uint64_t* rows);
/* Changes maxiter, tol and the -c stop rule before the next fit. */
km_status km_kkm_configure(km_kkm* h, uint64_t maxiter, float tol, int32_t check_converged);
/* init_labels: n host labels, or NULL for the reference's i % k. */
km_status km_kkm_fit(km_kkm* h, const uint32_t* init_labels, uint32_t* labels_out, km_result* res);
void km_kkm_destroy(km_kkm* h);

/* ---- Batched Lloyd: many independent problems, several restarts each ---- */

/* One problem: n points of d coordinates, k clusters (k <= n, k <= 256,
 * d * round_up(k, 32) * 4 bytes <= 160 KiB).  Points of all problems are
 * packed one after the other (problem order, row-major). */
typedef struct km_batch_problem {
  uint64_t n;
  uint32_t d;
  uint32_t k;
} km_batch_problem;

typedef struct km_batch_params {
  uint32_t problems;
  uint32_t restarts;   /* instances per problem (the reference's -r repeats, here seeded restarts) */
  int32_t seed;        /* restart r of problem p draws its sample picks with seed + p*restarts + r */
  float tol;
  uint64_t maxiter;
  int32_t device;
  void* stream;
} km_batch_params;

typedef struct km_batch_result {
  uint64_t converged_iter;  /* as the reference's run(): converged iteration or maxiter */
  uint64_t iterations;
  double objective;         /* FP64 sum of the final assignment's distances */
} km_batch_result;

typedef struct km_batch km_batch;

/* No counterpart in the reference (its -r repeats one problem sequentially,
 * src/main.cu:95-120): every restart of every problem runs the reference CPU
 * algorithm (seeded sample picks, kmeans.cpp:49-200) with labels and
 * centroids identical to a single run, all in one persistent kernel launch. */
km_status km_batch_create(const km_batch_params* p, const km_batch_problem* problems, km_batch** out);
/* X: all problems' points, packed, host memory. */
km_status km_batch_set_data(km_batch* h, const float* X);
/* Times the kernel's tile variants on a sample of the instances and keeps the
 * fastest (km_batch_fit does this on first use). variant_out / ms (6 doubles)
 * may be NULL. */
km_status km_batch_tune(km_batch* h, int32_t* variant_out, double* ms_per_variant);
/* results: problems*restarts entries (problem-major).  best_labels: the labels
 * of each problem's lowest-objective restart, packed (n per problem);
 * best_centroids: k*d per problem, packed.  Any output may be NULL. */
km_status km_batch_fit(km_batch* h, km_batch_result* results, uint32_t* best_labels,
                       float* best_centroids, double* fit_ms);
/* Labels (n) and centroids (k*d) of one instance of the last fit. */
km_status km_batch_instance_labels(km_batch* h, uint32_t problem, uint32_t restart,
                                   uint32_t* labels_out, float* centroids_out);
void km_batch_destroy(km_batch* h);

/* ---- Synthetic data (deterministic on every platform) ---- */

/* Gaussian-blob points: centers uniform in [lo,hi]^d, one blob per point drawn
 * uniformly (zipf_s > 0: blob b with weight (b+1)^-zipf_s), noise N(0, sigma_b^2)
 * with sigma_b = sigma, or uniform in [sigma_lo, sigma_hi] when sigma_hi > 0.
 * round_clip != 0 rounds to integers and clips to [lo, hi].  Counter-based
 * splitmix64 stream; normals are (u1+u2+u3+u4-2)*sqrt(3).  blob_out optional. */
km_status km_synth_blobs(uint64_t n, uint32_t d, uint32_t blobs, double lo, double hi,
                         double sigma, double sigma_lo, double sigma_hi, double zipf_s,
                         int32_t round_clip, uint64_t seed, int32_t nthreads,
                         float* X_out, uint32_t* blob_out);

#ifdef __cplusplus
}
#endif

#endif /* KM_H */
