// Seeded synthetic Gaussian-blob data (km_synth_blobs in include/km.h).
//
// Deterministic on every platform: a counter-based splitmix64 stream gives the
// uniforms; normals are (u1 + u2 + u3 + u4 - 2) * sqrt(3) (unit variance,
// bounded tails), so only IEEE additions and multiplications are involved
// (compiled with -ffp-contract=off) and x86-64 and aarch64 builds produce the
// same bits.  The only transcendental, pow(), is used for Zipf weights.
//
// Streams: 0 blob centers, 1 blob of each point, 2 noise, 3 per-blob sigma.
// This stands in for the reference's random-input mode (src/include/input_parser.hpp:50-68,
// uniform [-1e5, 1e5]) and its blob generator (py_utils/data_generator.py) with
// the shapes and value distributions the k-means workloads are quoted on.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/km.h"

namespace {

inline uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}

inline uint64_t stream_key(uint64_t seed, uint64_t stream) {
  return mix64(seed * 0x9E3779B97F4A7C15ull + stream * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull);
}

inline double uniform(uint64_t key, uint64_t i) {
  return (double)(mix64(key + (i + 1) * 0x9E3779B97F4A7C15ull) >> 11) * (1.0 / 9007199254740992.0);
}

inline double normal4(uint64_t key, uint64_t i) {
  static const double s3 = std::sqrt(3.0);
  const uint64_t b = 4 * i;
  double s = uniform(key, b);
  s = s + uniform(key, b + 1);
  s = s + uniform(key, b + 2);
  s = s + uniform(key, b + 3);
  return (s - 2.0) * s3;
}

}  // namespace

extern "C" km_status km_synth_blobs(uint64_t n, uint32_t d, uint32_t blobs, double lo, double hi,
                                    double sigma, double sigma_lo, double sigma_hi, double zipf_s,
                                    int32_t round_clip, uint64_t seed, int32_t nthreads,
                                    float* X_out, uint32_t* blob_out) {
  if (n == 0 || d == 0 || blobs == 0 || !X_out || !(hi >= lo)) return KM_ERR_ARG;
  const uint64_t k0 = stream_key(seed, 0), k1 = stream_key(seed, 1), k2 = stream_key(seed, 2),
                 k3 = stream_key(seed, 3);
  std::vector<double> center((size_t)blobs * d), bsig(blobs, sigma);
  for (uint64_t q = 0; q < (uint64_t)blobs * d; ++q) center[q] = lo + (hi - lo) * uniform(k0, q);
  if (sigma_hi > 0)
    for (uint32_t b = 0; b < blobs; ++b) bsig[b] = sigma_lo + (sigma_hi - sigma_lo) * uniform(k3, b);
  std::vector<double> cdf;
  if (zipf_s > 0) {
    cdf.resize(blobs);
    double acc = 0;
    for (uint32_t b = 0; b < blobs; ++b) { acc += std::pow((double)(b + 1), -zipf_s); cdf[b] = acc; }
    for (auto& v : cdf) v /= acc;
  }
  if (nthreads < 1) nthreads = 1;
  auto work = [&](uint64_t b0, uint64_t b1) {
    for (uint64_t i = b0; i < b1; ++i) {
      const double u = uniform(k1, i);
      uint32_t b;
      if (zipf_s > 0) {
        b = (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        if (b >= blobs) b = blobs - 1;
      } else {
        b = (uint32_t)(u * blobs);
        if (b >= blobs) b = blobs - 1;
      }
      if (blob_out) blob_out[i] = b;
      const double* c = center.data() + (size_t)b * d;
      const double sg = bsig[b];
      for (uint32_t j = 0; j < d; ++j) {
        double v = c[j] + sg * normal4(k2, i * d + j);
        if (round_clip) v = std::min(hi, std::max(lo, std::nearbyint(v))) + 0.0;  // -0 -> +0
        X_out[i * d + j] = (float)v;
      }
    }
  };
  const uint64_t T = std::min<uint64_t>((uint64_t)nthreads, (n + 4095) / 4096);
  if (T <= 1) {
    work(0, n);
  } else {
    std::vector<std::thread> th;
    const uint64_t ch = (n + T - 1) / T;
    for (uint64_t t = 0; t < T; ++t) {
      const uint64_t b0 = t * ch, b1 = std::min(n, b0 + ch);
      if (b0 < b1) th.emplace_back(work, b0, b1);
    }
    for (auto& x : th) x.join();
  }
  return KM_OK;
}
