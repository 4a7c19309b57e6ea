// The Kmeans class of kmeans.hpp: host orchestration over the C ABI only.
#include "kmeans.hpp"

#include <vector>

namespace {

void check(km_status s, const char* what) {
  if (s != KM_OK) throw KmeansError(s, what);
}

km_precision to_prec(Kmeans::Precision p, bool linear) {
  switch (p) {
    case Kmeans::Precision::bf16: return KM_PREC_BF16;
    case Kmeans::Precision::bf16x3: return KM_PREC_BF16X3;
    case Kmeans::Precision::automatic: return linear ? KM_PREC_BF16X3 : KM_PREC_FP32;
    default: return KM_PREC_FP32;
  }
}

}  // namespace

Kmeans::Kmeans(size_t n_, uint32_t d_, uint32_t k_, float tol_, const int* seed,
               Point<float>** points, cudaDeviceProp* /*deviceProps*/, InitMethod initMethod,
               Kernel kernel, int level, Precision precision, KernelParams kparams)
    : n(n_), d(d_), k(k_), tol(tol_), points_(points) {
  if (!points || n == 0 || d == 0) throw KmeansError(KM_ERR_ARG, "Kmeans: points");
  // Array-of-points to one row-major buffer (the reference does the same
  // copy into pinned memory, src/kmeans.cu:94-99).
  std::vector<float> X(n * d);
  for (size_t i = 0; i < n; ++i)
    for (uint32_t j = 0; j < d; ++j) X[i * d + j] = points[i]->get(j);
  setup(X.data(), seed, initMethod, kernel, level, precision, kparams);
}

Kmeans::Kmeans(size_t n_, uint32_t d_, uint32_t k_, float tol_, const int* seed,
               const float* X, uint32_t* labels_out, InitMethod initMethod, Kernel kernel,
               int level, Precision precision, KernelParams kparams)
    : n(n_), d(d_), k(k_), tol(tol_), labels_out_(labels_out) {
  if (!X) throw KmeansError(KM_ERR_ARG, "Kmeans: points");
  setup(X, seed, initMethod, kernel, level, precision, kparams);
}

void Kmeans::setup(const float* X, const int* seed, InitMethod initMethod, Kernel kernel, int level,
                   Precision precision, const KernelParams& kp) {
  if (level < 0 || level > 4) throw KmeansError(KM_ERR_ARG, "Kmeans: level must be 0..4");
  if (initMethod == InitMethod::plus_plus && kernel != Kernel::linear)
    throw KmeansError(KM_ERR_UNSUPPORTED, "Kmeans: plus_plus initialisation with a non-linear kernel");
  if (kernel == Kernel::linear) {
    km_lloyd_params p{};
    p.n = n;
    p.d = d;
    p.k = k;
    p.tol = tol;
    p.seed = seed ? *seed : 0;
    p.maxiter = 1;                       // set by run()
    p.init = initMethod == InitMethod::plus_plus ? KM_INIT_PLUSPLUS : KM_INIT_ROUND_ROBIN;
    p.precision = to_prec(precision, kernel == Kernel::linear);
    p.conv = KM_CONV_NONE;
    p.device = 0;
    p.stream = nullptr;
    p.empty = KM_EMPTY_EXCLUDE;
    check(km_lloyd_create(&p, &lloyd_), "km_lloyd_create");
    km_status s = km_lloyd_set_data(lloyd_, X, 0);
    if (s != KM_OK) {
      km_lloyd_destroy(lloyd_);
      lloyd_ = nullptr;
      check(s, "km_lloyd_set_data");
    }
  } else {
    km_kkm_params p{};
    p.n = n;
    p.d = d;
    p.k = k;
    p.tol = tol;
    p.maxiter = 1;                       // set by run()
    p.kernel_fn = kernel == Kernel::polynomial ? KM_KERNEL_POLY
                : kernel == Kernel::sigmoid    ? KM_KERNEL_SIGMOID
                                               : KM_KERNEL_GAUSSIAN;
    p.gamma = kp.gamma;
    p.coef = kp.coef;
    p.sigma = kp.sigma;
    p.degree = kp.degree;
    p.precision = to_prec(precision, kernel == Kernel::linear);
    p.k_bf16 = 0;
    p.check_converged = 0;
    p.device = 0;
    p.stream = nullptr;
    p.panel_rows = KM_KKM_PANEL_AUTO;    // K resident when it fits, else rebuilt in panels
    check(km_kkm_create(&p, &kkm_), "km_kkm_create");
    if (precision == Precision::automatic && p.precision == KM_PREC_FP32) {
      // One decision, the handle's own: when it chose panels (the FP32 n*n
      // kernel matrix does not fit), keep no K at all instead (fused
      // split-BF16x3) rather than rebuild FP32 panels every iteration.
      uint64_t rows = 0;
      if (km_kkm_panel_rows(kkm_, &rows) == KM_OK && rows != 0) {
        km_kkm_destroy(kkm_);
        kkm_ = nullptr;
        p.precision = KM_PREC_BF16X3;
        check(km_kkm_create(&p, &kkm_), "km_kkm_create");
      }
    }
    km_status s = km_kkm_set_data(kkm_, X, 0);
    if (s != KM_OK) {
      km_kkm_destroy(kkm_);
      kkm_ = nullptr;
      check(s, "km_kkm_set_data");
    }
  }
}

Kmeans::~Kmeans() {
  if (lloyd_) km_lloyd_destroy(lloyd_);
  if (kkm_) km_kkm_destroy(kkm_);
}

uint64_t Kmeans::run(uint64_t maxiter, bool check_converged) {
  labels_.resize(n);
  if (lloyd_) {
    check(km_lloyd_configure(lloyd_, maxiter, tol, check_converged ? KM_CONV_SCORE : KM_CONV_NONE),
          "km_lloyd_configure");
    check(km_lloyd_fit(lloyd_, nullptr, labels_.data(), nullptr, &result_), "km_lloyd_fit");
  } else {
    check(km_kkm_configure(kkm_, maxiter, tol, check_converged ? 1 : 0), "km_kkm_configure");
    check(km_kkm_fit(kkm_, nullptr, labels_.data(), &result_), "km_kkm_fit");
  }
  score = static_cast<float>(result_.score);
  if (points_)
    for (size_t i = 0; i < n; ++i) points_[i]->setCluster(labels_[i]);
  if (labels_out_)
    for (size_t i = 0; i < n; ++i) labels_out_[i] = labels_[i];
  return result_.converged_iter;
}

std::vector<double> Kmeans::profile_stages(uint64_t iters) {
  if (!lloyd_) throw KmeansError(KM_ERR_UNSUPPORTED, "Kmeans::profile_stages: linear kernel only");
  std::vector<double> ms(5, 0.0);
  check(km_lloyd_profile(lloyd_, iters, ms.data()), "km_lloyd_profile");
  return ms;
}
