// ORACLE — test infrastructure only.
//
// A CPU restatement of the reference's k-means arithmetic, used by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
// It is never linked into, loaded by or called from the product library.
//
// Two algorithms are restated:
//
//  * Lloyd k-means exactly as the reference's CPU implementation does it
//    (comparisons/CPU_Kmeans/src/kmeans.cpp):
//      - init: mt19937(seed_seq{seed}), uniform_int_distribution<int>(0, n-1),
//        k picks rejecting points equal by value to an earlier pick
//        (kmeans.cpp:22-29, :49-84);
//      - distance: dist = sum_j (x_j - c_j)^2 in float, j ascending, every
//        operation rounded separately (kmeans.cpp:86-98);
//      - argmin: strict '<' from +inf, so the lowest index wins ties, and the
//        counts (kmeans.cpp:106-122);
//      - update: float sums in point order, then *= float(1.0/(double)max(cnt,1));
//        an empty cluster becomes the zero vector (kmeans.cpp:131-148);
//      - stop: from iteration 2 on, when every centroid moved by
//        sqrtf(sum_j (c_j - c_prev_j)^2) <= tol (kmeans.cpp:157-200).
//    The results are bit-identical to the reference's: the per-(row, centroid)
//    distance and per-(cluster, column) sum keep the reference's operation order;
//    rows, centroids and columns are only spread over threads and SIMD lanes.
//    It is pinned against the reference itself (oracle/_ref, built from the
//    reference sources) and against golden fixtures made by it.
//
//  * The same Lloyd iteration in FP64 (distances, sums and the shift test in
//    double): the "FP64 CPU oracle" that reduced-precision results are scored
//    against (label agreement, relative objective error).
//
//  * Kernel k-means in FP64 with the reference GPU path's semantics
//    (src/kmeans.cu:365-444 labels i % k; :772-1073 iteration loop;
//    src/kernels/distances.cu:895-1002 popcorn distances
//    D[i,c] = -2/|c| sum_{j in c} K_ij + ctilde_c, ctilde_c = (1/|c|^2) sum_{a,b in c} K_ab,
//    ctilde_c == 0 -> +inf (distances.cu:588-599); argmin keeps the lowest index
//    on ties from the initial (0, FLT_MAX) pair (kmeans.cu:923-936); score =
//    sum_i D[i, label_i], which leaves out K_ii (kmeans.cu:1054-1061); stop on
//    |score - last| < tol from iteration 2 when checking (kmeans.cu:1064-1073)).
//    Kernel functions follow src/kernels/kernels.cuh:43-118 (stored without the
//    reference's -2 factor) plus the Gaussian kernel.  The reference GPU path
//    cannot be built here (it needs RAFT fetched at configure time), so this
//    part is checked against a second statement of the same math
//    (experiments/knKmeans.m:13-29, restated in numpy in the tests), not against
//    reference outputs.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <thread>
#include <vector>

namespace {

template <class F>
void parallel_for(int nthreads, uint64_t count, F&& f) {
  if (nthreads <= 1 || count < 2) { f(0, (uint64_t)0, count); return; }
  nthreads = (int)std::min<uint64_t>((uint64_t)nthreads, count);
  std::vector<std::thread> th;
  uint64_t chunk = (count + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    uint64_t b = t * chunk, e = std::min(count, b + chunk);
    if (b >= e) break;
    th.emplace_back([&f, t, b, e] { f(t, b, e); });
  }
  for (auto& x : th) x.join();
}

// kmeans.cpp:49-84 — k distinct sample picks (distinct by value).
bool sample_picks(const float* X, uint64_t n, uint32_t d, uint32_t k, int seed,
                  int32_t* picks) {
  std::seed_seq ss{seed};
  std::mt19937 gen(ss);
  std::uniform_int_distribution<int> random_int(0, (int)(n - 1));
  uint32_t i = 0;
  uint64_t guard = 0;
  while (i < k) {
    if (++guard > 1000ull * (k + 16) + 100000ull) return false;  // fewer than k distinct points
    int p = random_int(gen);
    // Point::operator== compares element-wise with float '!=' (point.hpp:64-70):
    // +0 equals -0 and a NaN never equals anything.
    bool found = false;
    for (uint32_t q = 0; q < i && !found; ++q) {
      bool eq = true;
      for (uint32_t j = 0; j < d && eq; ++j)
        eq = X[(uint64_t)picks[q] * d + j] == X[(uint64_t)p * d + j];
      found = eq;
    }
    if (!found) picks[i++] = p;
  }
  return true;
}

// Distances of one row to all centroids, CPU order (kmeans.cpp:86-98).  Ct is
// the centroid matrix transposed (d x k) so that the loop over centroids is a
// plain element-wise update the compiler can vectorise without reassociating
// any single (row, centroid) sum.
inline void row_dists_f32(const float* x, const float* Ct, uint32_t d, uint32_t k, float* dist) {
  for (uint32_t c = 0; c < k; ++c) dist[c] = 0.0f;
  for (uint32_t j = 0; j < d; ++j) {
    const float xj = x[j];
    const float* cj = Ct + (uint64_t)j * k;
    for (uint32_t c = 0; c < k; ++c) {
      float t = xj - cj[c];
      float sq = t * t;
      dist[c] = dist[c] + sq;
    }
  }
}

inline void row_dists_f64(const float* x, const double* Ct, uint32_t d, uint32_t k, double* dist) {
  for (uint32_t c = 0; c < k; ++c) dist[c] = 0.0;
  for (uint32_t j = 0; j < d; ++j) {
    const double xj = x[j];
    const double* cj = Ct + (uint64_t)j * k;
    for (uint32_t c = 0; c < k; ++c) {
      double t = xj - cj[c];
      dist[c] += t * t;
    }
  }
}

// kmeans.cpp:106-122 — strict '<' from +inf.
template <class T>
inline uint32_t argmin_strict(const T* dist, uint32_t k) {
  T m = std::numeric_limits<T>::infinity();
  uint32_t idx = 0;
  for (uint32_t c = 0; c < k; ++c)
    if (dist[c] < m) { m = dist[c]; idx = c; }
  return idx;
}

struct LloydF32 {
  const float* X; uint64_t n; uint32_t d, k; int nthreads;
  std::vector<float> C, Cprev, Ct;
  std::vector<uint32_t> labels, counts;

  void assign() {
    Ct.assign((uint64_t)d * k, 0.0f);
    for (uint32_t c = 0; c < k; ++c)
      for (uint32_t j = 0; j < d; ++j) Ct[(uint64_t)j * k + c] = C[(uint64_t)c * d + j];
    parallel_for(nthreads, n, [&](int, uint64_t b, uint64_t e) {
      std::vector<float> dist(k);
      for (uint64_t i = b; i < e; ++i) {
        row_dists_f32(X + i * d, Ct.data(), d, k, dist.data());
        labels[i] = argmin_strict(dist.data(), k);
      }
    });
    std::fill(counts.begin(), counts.end(), 0u);
    for (uint64_t i = 0; i < n; ++i) counts[labels[i]]++;
  }

  // kmeans.cpp:131-148: per (cluster, column) float sums in point order.  Columns
  // are split over threads; every thread walks all rows in order.
  void update() {
    std::fill(C.begin(), C.end(), 0.0f);
    parallel_for(nthreads, d, [&](int, uint64_t jb, uint64_t je) {
      for (uint64_t i = 0; i < n; ++i) {
        float* cr = C.data() + (uint64_t)labels[i] * d;
        const float* xr = X + i * d;
        for (uint64_t j = jb; j < je; ++j) cr[j] = cr[j] + xr[j];
      }
    });
    for (uint32_t c = 0; c < k; ++c) {
      uint32_t count = counts[c] > 1 ? counts[c] : 1;
      float scale = (float)(1.0 / (double)count);
      for (uint32_t j = 0; j < d; ++j) C[(uint64_t)c * d + j] *= scale;
    }
  }

  // kmeans.cpp:190-200
  bool shift_ok(float tol) const {
    for (uint32_t c = 0; c < k; ++c) {
      float s = 0.0f;
      for (uint32_t j = 0; j < d; ++j) {
        float t = C[(uint64_t)c * d + j] - Cprev[(uint64_t)c * d + j];
        float sq = t * t;
        s = s + sq;
      }
      if (std::sqrt(s) > tol) return false;
    }
    return true;
  }
};

}  // namespace

extern "C" {

// Seeded k distinct sample picks exactly as the reference CPU k-means draws them.
// Returns 0 on success, 1 if fewer than k distinct points exist.
int orc_sample_picks(const float* X, uint64_t n, uint32_t d, uint32_t k, int seed, int32_t* picks) {
  return sample_picks(X, n, d, k, seed, picks) ? 0 : 1;
}

// Exact (reference-CPU-order) assignment of n rows to k centroids.
void orc_assign_f32(const float* X, const float* C, uint64_t n, uint32_t d, uint32_t k,
                    int nthreads, uint32_t* labels, float* mindist) {
  std::vector<float> Ct((uint64_t)d * k);
  for (uint32_t c = 0; c < k; ++c)
    for (uint32_t j = 0; j < d; ++j) Ct[(uint64_t)j * k + c] = C[(uint64_t)c * d + j];
  parallel_for(nthreads, n, [&](int, uint64_t b, uint64_t e) {
    std::vector<float> dist(k);
    for (uint64_t i = b; i < e; ++i) {
      row_dists_f32(X + i * d, Ct.data(), d, k, dist.data());
      uint32_t l = argmin_strict(dist.data(), k);
      labels[i] = l;
      if (mindist) mindist[i] = dist[l];
    }
  });
}

// Exact (reference-CPU-order) centroid update from labels; counts out.
void orc_update_f32(const float* X, const uint32_t* labels, uint64_t n, uint32_t d, uint32_t k,
                    int nthreads, float* C, uint32_t* counts) {
  LloydF32 L{X, n, d, k, nthreads, {}, {}, {}, {}, {}};
  L.C.assign((uint64_t)k * d, 0.0f);
  L.labels.assign(labels, labels + n);
  L.counts.assign(k, 0u);
  for (uint64_t i = 0; i < n; ++i) L.counts[labels[i]]++;
  L.update();
  std::memcpy(C, L.C.data(), sizeof(float) * k * d);
  if (counts) std::memcpy(counts, L.counts.data(), sizeof(uint32_t) * k);
}

// Reference CPU Lloyd k-means.  If C0 is non-null it gives the initial
// centroids, else the seeded sample picks are used.  Returns the reference's
// Kmeans::run value: the converged iteration, or maxiter.  *executed receives the
// number of iterations actually run.  Returns UINT64_MAX on bad input.
uint64_t orc_lloyd_f32(const float* X, uint64_t n, uint32_t d, uint32_t k, float tol, int seed,
                       uint64_t maxiter, const float* C0, int nthreads,
                       uint32_t* labels_out, float* centroids_out, uint64_t* executed) {
  if (n == 0 || d == 0 || k == 0 || k > n) return UINT64_MAX;
  LloydF32 L{X, n, d, k, nthreads, {}, {}, {}, {}, {}};
  L.C.assign((uint64_t)k * d, 0.0f);
  L.labels.assign(n, 0u);
  L.counts.assign(k, 0u);
  if (C0) {
    std::memcpy(L.C.data(), C0, sizeof(float) * k * d);
  } else {
    std::vector<int32_t> picks(k);
    if (!sample_picks(X, n, d, k, seed, picks.data())) return UINT64_MAX;
    for (uint32_t c = 0; c < k; ++c)
      std::memcpy(L.C.data() + (uint64_t)c * d, X + (uint64_t)picks[c] * d, sizeof(float) * d);
  }
  L.Cprev = L.C;
  uint64_t converged = maxiter, iter = 0;
  while (iter++ < maxiter) {
    L.assign();
    L.update();
    if (iter > 1 && L.shift_ok(tol)) { converged = iter; break; }
    L.Cprev = L.C;
  }
  if (executed) *executed = std::min(iter, maxiter);
  std::memcpy(labels_out, L.labels.data(), sizeof(uint32_t) * n);
  if (centroids_out) std::memcpy(centroids_out, L.C.data(), sizeof(float) * k * d);
  return converged;
}

// The same iteration in FP64 (distances, sums, scale and shift test in double,
// lowest index on ties, empty cluster -> zero vector).  Initial centroids as
// orc_lloyd_f32.  Used as the FP64 oracle for reduced-precision paths.
// objective_out (optional): the FP64 objective sum_i min_c ||x_i - c||^2 of the
// last assignment step (against the centroids that step used).
uint64_t orc_lloyd_f64_obj(const float* X, uint64_t n, uint32_t d, uint32_t k, double tol, int seed,
                           uint64_t maxiter, const float* C0, int nthreads,
                           uint32_t* labels_out, double* centroids_out, uint64_t* executed,
                           double* objective_out) {
  if (n == 0 || d == 0 || k == 0 || k > n) return UINT64_MAX;
  const int nt = std::max(1, nthreads);
  std::vector<double> objpart(nt, 0.0);
  std::vector<double> C((uint64_t)k * d), Cprev, Ct((uint64_t)d * k);
  std::vector<uint32_t> labels(n), counts(k);
  if (C0) {
    for (uint64_t q = 0; q < (uint64_t)k * d; ++q) C[q] = C0[q];
  } else {
    std::vector<int32_t> picks(k);
    if (!sample_picks(X, n, d, k, seed, picks.data())) return UINT64_MAX;
    for (uint32_t c = 0; c < k; ++c)
      for (uint32_t j = 0; j < d; ++j) C[(uint64_t)c * d + j] = X[(uint64_t)picks[c] * d + j];
  }
  Cprev = C;
  uint64_t converged = maxiter, iter = 0;
  while (iter++ < maxiter) {
    for (uint32_t c = 0; c < k; ++c)
      for (uint32_t j = 0; j < d; ++j) Ct[(uint64_t)j * k + c] = C[(uint64_t)c * d + j];
    std::fill(objpart.begin(), objpart.end(), 0.0);
    parallel_for(nthreads, n, [&](int t, uint64_t b, uint64_t e) {
      std::vector<double> dist(k);
      double o = 0.0;
      for (uint64_t i = b; i < e; ++i) {
        row_dists_f64(X + i * d, Ct.data(), d, k, dist.data());
        labels[i] = argmin_strict(dist.data(), k);
        o += dist[labels[i]];
      }
      objpart[t] = o;
    });
    std::fill(counts.begin(), counts.end(), 0u);
    for (uint64_t i = 0; i < n; ++i) counts[labels[i]]++;
    std::fill(C.begin(), C.end(), 0.0);
    parallel_for(nthreads, d, [&](int, uint64_t jb, uint64_t je) {
      for (uint64_t i = 0; i < n; ++i)
        for (uint64_t j = jb; j < je; ++j) C[(uint64_t)labels[i] * d + j] += X[i * d + j];
    });
    for (uint32_t c = 0; c < k; ++c) {
      double s = 1.0 / (double)(counts[c] > 1 ? counts[c] : 1);
      for (uint32_t j = 0; j < d; ++j) C[(uint64_t)c * d + j] *= s;
    }
    if (iter > 1) {
      bool ok = true;
      for (uint32_t c = 0; c < k && ok; ++c) {
        double s = 0.0;
        for (uint32_t j = 0; j < d; ++j) {
          double t = C[(uint64_t)c * d + j] - Cprev[(uint64_t)c * d + j];
          s += t * t;
        }
        ok = std::sqrt(s) <= tol;
      }
      if (ok) { converged = iter; break; }
    }
    Cprev = C;
  }
  if (executed) *executed = std::min(iter, maxiter);
  std::memcpy(labels_out, labels.data(), sizeof(uint32_t) * n);
  if (centroids_out) std::memcpy(centroids_out, C.data(), sizeof(double) * k * d);
  if (objective_out) {
    double o = 0.0;
    for (double v : objpart) o += v;
    *objective_out = o;
  }
  return converged;
}

uint64_t orc_lloyd_f64(const float* X, uint64_t n, uint32_t d, uint32_t k, double tol, int seed,
                       uint64_t maxiter, const float* C0, int nthreads,
                       uint32_t* labels_out, double* centroids_out, uint64_t* executed) {
  return orc_lloyd_f64_obj(X, n, d, k, tol, seed, maxiter, C0, nthreads, labels_out, centroids_out,
                           executed, nullptr);
}

// Seeded greedy k-means++ as the product's device initialisation draws it:
// the reference algorithm (src/kmeans.cu:447-769: first centroid uniform,
// then per round s = 2 + ceil(ln k) candidates drawn with probability
// proportional to the squared distance to the chosen set, raft::random::discrete
// over min_distances :585-588; the candidate with the lowest total cost
// sum_i min(d2_i, ||x_i - cand||^2) is kept, lowest index on equal cost,
// :681-715; d2 updated with its distances, :721-724), with the draws taken
// from std::mt19937_64(seed) instead of std::random_device: the first index
// by uniform_int_distribution<uint64_t>(0, n-1), then (k-1)*s uniforms in
// [0, 1), candidate j of round r using uniform (r-1)*s + j.  A draw u picks the
// first row (ascending, rows with d2 > 0 only) whose FP64 prefix sum of d2
// exceeds u * sum(d2); when every d2 is 0 the pick is floor(u * n).  Squared
// distances are FP32 in the order of the device's warp reduction (per lane l
// an fma chain over columns l, l+32, ..., then a butterfly over 16, 8, 4, 2, 1);
// sums over rows are FP64.  picks receives the k row indices.  Returns 1 when
// s exceeds 16 (the device's limit), else 0.
namespace {
inline float pp_dist32(const float* x, const float* c, uint32_t d) {
  float p[32];
  for (uint32_t l = 0; l < 32; ++l) {
    float a = 0.0f;
    for (uint32_t j = l; j < d; j += 32) {
      const float u = x[j] - c[j];
      a = std::fma(u, u, a);
    }
    p[l] = a;
  }
  for (uint32_t o = 16; o > 0; o >>= 1) {
    float q[32];
    for (uint32_t l = 0; l < 32; ++l) q[l] = p[l] + p[l ^ o];
    for (uint32_t l = 0; l < 32; ++l) p[l] = q[l];
  }
  return p[0];
}
}  // namespace

int orc_plusplus(const float* X, uint64_t n, uint32_t d, uint32_t k, int seed, int nthreads,
                 int64_t* picks) {
  const uint32_t s = 2u + (uint32_t)std::ceil(std::log((double)k));
  if (s > 16 || n == 0 || k == 0) return 1;
  std::mt19937_64 gen((uint64_t)(int64_t)seed);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  const uint64_t first = std::uniform_int_distribution<uint64_t>(0, n - 1)(gen);
  std::vector<double> hu((size_t)(k > 1 ? k - 1 : 1) * s);
  for (auto& v : hu) v = uni(gen);
  std::vector<float> d2(n), D((size_t)n * s);
  parallel_for(nthreads, n, [&](int, uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) d2[i] = pp_dist32(X + i * d, X + first * d, d);
  });
  picks[0] = (int64_t)first;
  std::vector<uint64_t> cand(s);
  const int nt = std::max(1, nthreads);
  for (uint32_t r = 1; r < k; ++r) {
    double tot = 0.0;
    for (uint64_t i = 0; i < n; ++i) tot += (double)d2[i];
    for (uint32_t j = 0; j < s; ++j) {
      const double u = hu[(size_t)(r - 1) * s + j];
      if (!(tot > 0.0)) {
        cand[j] = std::min<uint64_t>(n - 1, (uint64_t)(u * (double)n));
        continue;
      }
      const double target = u * tot;
      double acc = 0.0;
      uint64_t pick = UINT64_MAX, last = 0;
      for (uint64_t i = 0; i < n; ++i) {
        if (!(d2[i] > 0.0f)) continue;
        last = i;
        acc += (double)d2[i];
        if (acc > target) { pick = i; break; }
      }
      cand[j] = pick == UINT64_MAX ? last : pick;
    }
    std::vector<double> part((size_t)nt * s, 0.0);
    parallel_for(nthreads, n, [&](int t, uint64_t b, uint64_t e) {
      for (uint64_t i = b; i < e; ++i)
        for (uint32_t j = 0; j < s; ++j) {
          const float v = pp_dist32(X + i * d, X + cand[j] * d, d);
          D[i * s + j] = v;
          part[(size_t)t * s + j] += (double)std::fmin(v, d2[i]);
        }
    });
    uint32_t best = 0;
    double bestv = 0.0;
    for (uint32_t j = 0; j < s; ++j) {
      double c = 0.0;
      for (int t = 0; t < nt; ++t) c += part[(size_t)t * s + j];
      if (j == 0 || c < bestv) { bestv = c; best = j; }
    }
    picks[r] = (int64_t)cand[best];
    for (uint64_t i = 0; i < n; ++i) d2[i] = std::fmin(d2[i], D[i * s + best]);
  }
  return 0;
}

// FP64 k-means objective sum_i ||x_i - c_{label_i}||^2 for float centroids.
double orc_inertia(const float* X, const uint32_t* labels, const float* C, uint64_t n, uint32_t d,
                   uint32_t k, int nthreads) {
  std::vector<double> part(std::max(1, nthreads), 0.0);
  parallel_for(nthreads, n, [&](int t, uint64_t b, uint64_t e) {
    double s = 0.0;
    for (uint64_t i = b; i < e; ++i) {
      const float* c = C + (uint64_t)labels[i] * d;
      for (uint32_t j = 0; j < d; ++j) { double v = (double)X[i * d + j] - (double)c[j]; s += v * v; }
    }
    part[t] = s;
  });
  double s = 0.0;
  for (double p : part) s += p;
  (void)k;
  return s;
}

// Kernel function kinds: 0 linear x.y; 1 polynomial (gamma x.y + coef)^degree;
// 2 sigmoid tanh(gamma x.y + coef); 3 gaussian exp(-||x-y||^2 / (2 sigma^2)).
// The reference's polynomial is gamma=1, coef=1, degree=2 and its sigmoid
// gamma=1, coef=1 (kernels.cuh:61-111); it stores -2*f, this stores f.
void orc_kernel_matrix(const float* X, uint64_t n, uint32_t d, int kind, double gamma,
                       double coef, int degree, double sigma, int nthreads, double* K) {
  std::vector<double> nrm(n);
  for (uint64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (uint32_t j = 0; j < d; ++j) s += (double)X[i * d + j] * X[i * d + j];
    nrm[i] = s;
  }
  parallel_for(nthreads, n, [&](int, uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i)
      for (uint64_t j = 0; j < n; ++j) {
        double dot = 0.0;
        for (uint32_t q = 0; q < d; ++q) dot += (double)X[i * d + q] * X[j * d + q];
        double v;
        switch (kind) {
          case 0: v = dot; break;
          case 1: v = std::pow(gamma * dot + coef, (double)degree); break;
          case 2: v = std::tanh(gamma * dot + coef); break;
          default: {
            double d2 = nrm[i] + nrm[j] - 2.0 * dot;
            if (d2 < 0) d2 = 0;
            v = std::exp(-d2 / (2.0 * sigma * sigma));
          }
        }
        K[i * n + j] = v;
      }
  });
}

// Kernel k-means with the reference GPU path's semantics (see header), in FP64.
// labels_io holds the initial labels on entry (the reference uses i % k) and the
// final labels on exit.  score_out receives the last score.  Returns the value
// the reference's Kmeans::run returns (converged iteration or maxiter); the
// number of executed iterations goes to *executed.
uint64_t orc_kernel_kmeans(const double* K, uint64_t n, uint32_t k, uint64_t maxiter, double tol,
                           int check_converged, int nthreads, uint32_t* labels_io,
                           double* score_out, uint64_t* executed) {
  std::vector<uint32_t> lab(labels_io, labels_io + n), cnt(k);
  std::vector<double> ct(k), E;
  double score = 0.0, last_score = 0.0;
  uint64_t converged = maxiter, iter = 0;
  std::vector<uint32_t> newlab(n);
  while (iter++ < maxiter) {
    std::fill(cnt.begin(), cnt.end(), 0u);
    for (uint64_t i = 0; i < n; ++i) cnt[lab[i]]++;
    // E[i,c] = sum_{j in c} K_ij
    E.assign(n * k, 0.0);
    parallel_for(nthreads, n, [&](int, uint64_t b, uint64_t e) {
      for (uint64_t i = b; i < e; ++i)
        for (uint64_t j = 0; j < n; ++j) E[i * k + lab[j]] += K[i * n + j];
    });
    // ctilde_c = (1/|c|^2) sum_{i in c} E[i,c]
    std::fill(ct.begin(), ct.end(), 0.0);
    for (uint64_t i = 0; i < n; ++i) ct[lab[i]] += E[i * k + lab[i]];
    for (uint32_t c = 0; c < k; ++c)
      ct[c] = cnt[c] ? ct[c] / ((double)cnt[c] * (double)cnt[c]) : 0.0;
    double sc = 0.0;
    std::vector<double> rowmin(n);
    parallel_for(nthreads, n, [&](int, uint64_t b, uint64_t e) {
      for (uint64_t i = b; i < e; ++i) {
        uint32_t key = 0;
        double val = (double)FLT_MAX;
        for (uint32_t c = 0; c < k; ++c) {
          double add = (ct[c] == 0.0) ? INFINITY : ct[c];
          double v = (cnt[c] ? -2.0 * E[i * k + c] / (double)cnt[c] : 0.0) + add;
          if (v < val) { val = v; key = c; }
        }
        newlab[i] = key;
        rowmin[i] = val;
      }
    });
    for (uint64_t i = 0; i < n; ++i) sc += rowmin[i];
    score = sc;
    lab = newlab;
    if (iter == maxiter) break;
    if (check_converged && iter > 1 && std::fabs(score - last_score) < tol) { converged = iter; break; }
    last_score = score;
  }
  if (executed) *executed = std::min(iter, maxiter);
  std::memcpy(labels_io, lab.data(), sizeof(uint32_t) * n);
  if (score_out) *score_out = score;
  return converged;
}

}  // extern "C"
