// kmeans.hpp — the reference's Kmeans class (src/kmeans.cuh:51-140) as a
// host C++ class over the C ABI of libkm_sm103 (km.h).  Link with
// -lkmeans_host -lkm_sm103.
//
// Same constructor, run() and get_score() as the reference GPU class:
//   Kmeans(n, d, k, tol, seed, points, deviceProps, init, kernel, level)
//     copies the points to the GPU (and, for a non-linear kernel, builds the
//     n x n kernel matrix K = f(X X^T), src/kmeans.cu:143-211);
//   run(maxiter, check_converged) starts from labels i % k
//     (init_centroids_rand, src/kmeans.cu:365-374) or, with plus_plus and the
//     linear kernel, from greedy k-means++ centroids drawn from *seed
//     (src/kmeans.cu:447-769), iterates assignment and
//     update, stops on |score - last_score| < tol from the second iteration
//     when check_converged (src/kmeans.cu:1063-1073) or after maxiter
//     iterations, writes each point's label back with Point::setCluster
//     (src/kmeans.cu:1101-1103) and returns the converged iteration or maxiter;
//   get_score() is the reference's score, sum_i of the chosen distance without
//     the ||x_i||^2 (K_ii) term (computeClusterCost, src/kmeans.cu:1054-1061).
// An empty cluster gets distance +inf and is never chosen again, as in the
// reference (c~ = 0 -> +inf, src/kernels/distances.cu:588-599).
//
// How the work runs: the linear kernel is plain Lloyd (distance GEMM with
// fused argmin, label-sorted exact centroid update), which assigns exactly as
// the reference's -2 X X^T formulation does without the n x n matrix;
// polynomial (x.y + 1)^2, sigmoid tanh(x.y + 1) and the Gaussian extension
// use the kernel-matrix path (tensor-core K build, V.K, FP64 centroid terms).
// `level` (0..4, src/include/common.h:36-40) chose between the reference's
// implementations of the same arithmetic; every level runs the same code here
// and values outside 0..4 are rejected.  deviceProps is accepted and unused
// (device 0, as the reference's main uses).  plus_plus with a non-linear
// kernel is rejected (KM_ERR_UNSUPPORTED).
//
// Errors: the reference exits the process (src/cuda_utils.cu:10-41); this
// class throws KmeansError carrying the km_status instead, and the gpukmeans
// CLI turns it into the reference's exit codes.
#ifndef KM_KMEANS_HPP
#define KM_KMEANS_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "km.h"
#include "point.hpp"

struct cudaDeviceProp;

class KmeansError : public std::runtime_error {
 public:
  KmeansError(km_status s, const std::string& what)
      : std::runtime_error(what + ": " + km_status_str(s)), status(s) {}
  km_status status;
};

// Extension: kernel parameters; the reference fixes gamma = coef = 1,
// degree = 2 (src/kernels/kernels.cuh:60-118).
struct KmeansKernelParams {
  float gamma = 1.0f;
  float coef = 1.0f;
  int degree = 2;
  float sigma = 1.0f;     // Gaussian exp(-||x-y||^2 / (2 sigma^2))
};

class Kmeans {
 public:
  enum class InitMethod { random, plus_plus };
  enum class Kernel { linear, polynomial, sigmoid, gaussian };
  // Extension: arithmetic of the distance stage (linear) or of the K build.
  // automatic: split-BF16x3 tensor cores with exact re-scoring for the linear
  // kernel (labels identical to fp32, several times faster), fp32 for the K
  // build of the other kernels (K then matches an FP32 build) while the n*n
  // FP32 kernel matrix fits the device; beyond that, where an n*n buffer
  // cannot exist, split-BF16x3 without a stored K (the fused kernel).
  enum class Precision { fp32, bf16, bf16x3, automatic };

  using KernelParams = KmeansKernelParams;

  Kmeans(size_t n, uint32_t d, uint32_t k, float tol, const int* seed, Point<float>** points,
         cudaDeviceProp* deviceProps, InitMethod initMethod = InitMethod::random,
         Kernel kernel = Kernel::linear, int level = 3, Precision precision = Precision::automatic,
         KernelParams kparams = KernelParams());

  // Extension: points given as one row-major n*d array; run() writes the
  // labels to labels_out (n entries) instead of Point objects.
  Kmeans(size_t n, uint32_t d, uint32_t k, float tol, const int* seed, const float* X,
         uint32_t* labels_out, InitMethod initMethod = InitMethod::random,
         Kernel kernel = Kernel::linear, int level = 3, Precision precision = Precision::automatic,
         KernelParams kparams = KernelParams());

  ~Kmeans();
  Kmeans(const Kmeans&) = delete;
  Kmeans& operator=(const Kmeans&) = delete;

  uint64_t run(uint64_t maxiter, bool check_converged);

  float get_score() const { return score; }

  // ---- extensions ----
  const km_result& last_result() const { return result_; }
  const std::vector<uint32_t>& labels() const { return labels_; }
  // Per-stage mean milliseconds of `iters` more iterations after run()
  // (linear kernel only): distance+argmin, refine, label sort, centroid sums,
  // finalize+control.
  std::vector<double> profile_stages(uint64_t iters);

 private:
  void setup(const float* X, const int* seed, InitMethod initMethod, Kernel kernel, int level,
             Precision precision, const KernelParams& kp);

  size_t n;
  uint32_t d, k;
  float tol;
  float score = 0.0f;
  Point<float>** points_ = nullptr;
  uint32_t* labels_out_ = nullptr;
  km_lloyd* lloyd_ = nullptr;
  km_kkm* kkm_ = nullptr;
  km_result result_{};
  std::vector<uint32_t> labels_;
};

#endif  // KM_KMEANS_HPP
