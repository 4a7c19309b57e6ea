// Test infrastructure only: C entry points around the reference's own dataset
// reader/writer (src/include/input_parser.hpp:16-208, src/include/point.hpp),
// so that tests can compare the gpukmeans reader and writer with the
// reference's on the same bytes.  Compiled against the header where it lies
// in the reference tree by oracle/build_ref.sh; nothing of the reference is
// copied here.  Callers must pass inputs the reference reads in bounds:
// exactly n data rows after the header, at most d + 1 CSV columns, SVM indices
// in [1, d].
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>

#include "input_parser.hpp"   // reference: src/include/input_parser.hpp

namespace {
void copy_out(InputParser<float>& p, int d, uint64_t n, float* out) {
  Point<float>** ds = p.get_dataset();
  for (uint64_t i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) out[i * d + j] = ds[i]->get(j);
}
}  // namespace

extern "C" {

// Parses `len` bytes of CSV (svm == 0) or libsvm (svm != 0) text.
void ref_io_read(const char* text, uint64_t len, int svm, int d, uint64_t n, float* out) {
  std::istringstream in(std::string(text, len));
  InputParser<float>::InputFormat f =
      svm ? InputParser<float>::InputFormat::SVM : InputParser<float>::InputFormat::CSV;
  InputParser<float> p(in, d, n, f);
  copy_out(p, d, n, out);
}

// The reference's seeded random points.
void ref_io_random(int seed, int d, uint64_t n, float* out) {
  InputParser<float> p(seed, d, n);
  copy_out(p, d, n, out);
}

// dataset_to_csv of n points with the given labels; returns the byte count
// (the text is written to buf when it fits in cap bytes).
uint64_t ref_io_to_csv(const float* X, const uint32_t* labels, int d, uint64_t n, char* buf,
                       uint64_t cap) {
  InputParser<float> p(0, d, n);
  Point<float>** ds = p.get_dataset();
  for (uint64_t i = 0; i < n; ++i) {
    Point<float> q(const_cast<float*>(X + i * d), d);
    *ds[i] = q;
    ds[i]->setCluster(labels[i]);
  }
  std::ostringstream o;
  p.dataset_to_csv(o);
  const std::string s = o.str();
  if (s.size() <= cap) std::memcpy(buf, s.data(), s.size());
  return s.size();
}

}  // extern "C"
