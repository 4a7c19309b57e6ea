// input_parser.hpp — the reference's dataset reader/writer
// (src/include/input_parser.hpp:16-208), with the same constructors, formats
// and output, over one contiguous row-major float buffer.
//
// Behaviour kept from the reference:
//  * CSV: the first line is a header and is skipped; in every following line
//    the first column is dropped and the next d columns are the coordinates
//    (for a file whose last column is a class label, the label becomes the
//    last coordinate).  Each field is converted as atof() does (strtod of the
//    field, then rounded to float); missing fields are 0; an empty line is a
//    point of zeros.  "READING CSV" is printed when the reader starts.
//  * SVM (libsvm): one point per line, "index:value" pairs with 1-based
//    indices; at most n lines are read.
//  * Random data: mt19937(seed) and uniform_real_distribution<float>(-1e5, 1e5),
//    one draw per coordinate in row-major order.
//  * dataset_to_csv: header "cluster,d0,...,d{d-1}", then "label,v0,...",
//    values with 8 significant digits (the stream default format).
//
// Differences, all in cases where the reference reads or writes out of
// bounds: at most n data rows and d columns are read (the reference writes
// past its arrays on longer input), SVM indices outside [1, d] are ignored,
// and a CSV file with fewer than n data rows is reported through ok() == false
// instead of leaving unset points.  Extensions: CsvColumns::plain keeps every
// column (no label drop); data() exposes the coordinates as one n*d array and
// clusters() the labels, so large inputs need no Point objects; CSV parsing
// and writing run on several threads with byte-identical results.
#ifndef KM_INPUT_PARSER_HPP
#define KM_INPUT_PARSER_HPP

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "point.hpp"

namespace km_io {

// atof() of the field [b, e): strtod on a NUL-terminated copy, so the
// conversion can never run past the field.
inline double field_atof(const char* b, const char* e) {
  char buf[128];
  const size_t len = static_cast<size_t>(e - b);
  if (len < sizeof(buf)) {
    std::memcpy(buf, b, len);
    buf[len] = '\0';
    return std::strtod(buf, nullptr);
  }
  std::string s(b, e);
  return std::strtod(s.c_str(), nullptr);
}

inline unsigned hw_threads() {
  const unsigned t = std::thread::hardware_concurrency();
  return t ? std::min(t, 64u) : 1u;
}

// Runs f(lo, hi) over [0, n) split in contiguous chunks on up to `threads` threads.
template <typename F>
void parallel_ranges(size_t n, unsigned threads, F f) {
  if (n == 0) return;
  threads = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(threads, n / 4096 + 1)));
  if (threads == 1) { f(size_t(0), n); return; }
  std::vector<std::thread> th;
  const size_t step = (n + threads - 1) / threads;
  for (unsigned t = 0; t < threads; ++t) {
    const size_t lo = t * step, hi = std::min(n, lo + step);
    if (lo >= hi) break;
    th.emplace_back([=] { f(lo, hi); });
  }
  for (auto& x : th) x.join();
}

}  // namespace km_io

template <typename T>
class InputParser {
 public:
  enum class InputFormat { CSV, SVM };
  enum class CsvColumns { reference, plain };

  InputParser(std::istream& in, int d, size_t n, InputFormat& format,
              CsvColumns cols = CsvColumns::reference)
      : d_(d), n_(n), X_(static_cast<size_t>(n) * d, T(0)), clusters_(n, 0u) {
    switch (format) {
      case InputFormat::SVM: read_svm(in); break;
      case InputFormat::CSV:
        std::cout << "READING CSV" << std::endl;
        read_csv(in, cols);
        break;
    }
  }

  // Uniform random points in [-1e5, 1e5) from mt19937(seed).
  InputParser(int seed, int d, size_t n)
      : d_(d), n_(n), X_(static_cast<size_t>(n) * d), clusters_(n, 0u), rows_(n) {
    std::mt19937 eng(seed);
    std::uniform_real_distribution<float> distr(-1e5, 1e5);
    for (auto& v : X_) v = distr(eng);
  }

  // Points built from a caller's contiguous n*d buffer (extension).
  InputParser(const T* X, int d, size_t n)
      : d_(d), n_(n), X_(X, X + static_cast<size_t>(n) * d), clusters_(n, 0u), rows_(n) {}

  InputParser(const InputParser&) = delete;
  InputParser& operator=(const InputParser&) = delete;

  // The reference's Point<T>** view.  Built on first use; labels written into
  // these points (Point::setCluster) are what dataset_to_csv prints.
  Point<T>** get_dataset() {
    if (!points_) {
      points_.reset(new std::unique_ptr<Point<T>>[n_]);
      ptrs_.resize(n_);
      for (size_t i = 0; i < n_; ++i) {
        points_[i].reset(new Point<T>(X_.data() + i * d_, static_cast<unsigned>(d_)));
        points_[i]->setCluster(clusters_[i]);
        ptrs_[i] = points_[i].get();
      }
    }
    return ptrs_.data();
  }

  size_t get_dataset_size() { return n_; }

  void dataset_to_csv(std::ostream& o) {
    sync_clusters_from_points();
    o << "cluster,";
    for (int j = 0; j < d_; ++j) {
      o << "d" << j;
      if (j != d_ - 1) o << ",";
    }
    o << "\n";
    // Rows are formatted in parallel blocks and written in order.
    const size_t block = 16384;
    const unsigned threads = km_io::hw_threads();
    std::vector<std::string> buf(threads);
    for (size_t b0 = 0; b0 < n_; b0 += block * threads) {
      auto fmt = [&](unsigned t) {
        std::string& s = buf[t];
        s.clear();
        const size_t r0 = std::min(n_, b0 + t * block), r1 = std::min(n_, r0 + block);
        char num[64];
        for (size_t i = r0; i < r1; ++i) {
          s += std::to_string(clusters_[i]);
          s += ',';
          for (int j = 0; j < d_; ++j) {
            // the stream default float format with precision 8 is %.8g
            const int len = std::snprintf(num, sizeof(num), "%.8g", static_cast<double>(X_[i * d_ + j]));
            s.append(num, static_cast<size_t>(len));
            if (j != d_ - 1) s += ',';
          }
          s += '\n';
        }
      };
      for (auto& s : buf) s.clear();
      std::vector<std::thread> th;
      for (unsigned t = 1; t < threads && b0 + t * block < n_; ++t) th.emplace_back(fmt, t);
      fmt(0);
      for (auto& x : th) x.join();
      for (auto& s : buf) o.write(s.data(), static_cast<std::streamsize>(s.size()));
    }
    o.flush();
  }

  friend std::ostream& operator<<(std::ostream& os, InputParser& p) {
    const int W = 9;
    os << "   i  cluster";
    for (int j = 0; j < p.d_; ++j) {
      std::string s = "d" + std::to_string(j);
      os << std::setw(W) << s;
    }
    os << std::endl;
    auto row = [&](size_t i) {
      os << std::setw(4) << i << std::setw(W) << std::setw(9) << p.cluster_of(i);
      for (int j = 0; j < p.d_; ++j) os << std::setw(9) << std::setprecision(5) << p.X_[i * p.d_ + j];
      os << std::endl;
    };
    for (size_t i = 0; i < std::min<size_t>(p.n_, 5); ++i) row(i);
    if (p.n_ > 5) {
      os << " ..." << std::endl;
      for (size_t i = p.n_ - 5; i < p.n_; ++i) row(i);
    }
    os << std::endl << "[" << p.n_ << " rows x " << p.d_ << " columns]" << std::endl;
    return os;
  }

  // ---- extensions ----
  const T* data() const { return X_.data(); }
  uint32_t* clusters() { return clusters_.data(); }
  int dims() const { return d_; }
  size_t rows_read() const { return rows_; }
  bool ok() const { return rows_ == n_; }

  // Copies labels written into the Point view (if it exists) back to clusters().
  void sync_clusters_from_points() {
    if (!points_) return;
    for (size_t i = 0; i < n_; ++i) clusters_[i] = static_cast<uint32_t>(points_[i]->getCluster());
  }
  // Copies clusters() into the Point view (if it exists).
  void sync_points_from_clusters() {
    if (!points_) return;
    for (size_t i = 0; i < n_; ++i) points_[i]->setCluster(clusters_[i]);
  }

 private:
  uint32_t cluster_of(size_t i) {
    return points_ ? static_cast<uint32_t>(points_[i]->getCluster()) : clusters_[i];
  }

  void read_csv(std::istream& in, CsvColumns cols) {
    const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    // line starts; line 0 is the header
    std::vector<size_t> starts;
    starts.reserve(n_ + 2);
    size_t pos = 0;
    const size_t len = text.size();
    bool header = true;
    while (pos < len && starts.size() < n_) {
      const char* nl = static_cast<const char*>(std::memchr(text.data() + pos, '\n', len - pos));
      const size_t end = nl ? static_cast<size_t>(nl - text.data()) : len;
      if (!header) starts.push_back(pos);
      header = false;
      pos = end + 1;
    }
    rows_ = starts.size();
    const size_t skip = (cols == CsvColumns::reference) ? 1 : 0;
    const char* base = text.data();
    km_io::parallel_ranges(rows_, km_io::hw_threads(), [&](size_t lo, size_t hi) {
      for (size_t i = lo; i < hi; ++i) {
        const char* p = base + starts[i];
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(base + len - p)));
        const char* e = nl ? nl : base + len;
        T* row = X_.data() + i * d_;
        size_t col = 0;
        const char* f = p;
        while (true) {
          const char* c = static_cast<const char*>(std::memchr(f, ',', static_cast<size_t>(e - f)));
          const char* fe = c ? c : e;
          if (col >= skip && col - skip < static_cast<size_t>(d_))
            row[col - skip] = static_cast<T>(km_io::field_atof(f, fe));
          ++col;
          if (!c || col - skip >= static_cast<size_t>(d_)) break;
          f = c + 1;
        }
      }
    });
  }

  void read_svm(std::istream& in) {
    std::string line;
    size_t i = 0;
    while (i < n_ && std::getline(in, line, '\n')) {
      std::istringstream ls(line);
      std::string tok;
      T* row = X_.data() + i * d_;
      while (std::getline(ls, tok, ' ')) {
        const size_t colon = tok.find(':');
        if (colon == std::string::npos || colon + 1 >= tok.size()) continue;  // no "key:value"
        const std::string key = tok.substr(0, colon), val = tok.substr(colon + 1);
        const long idx = std::atol(key.c_str());
        if (idx >= 1 && idx <= d_) row[idx - 1] = static_cast<T>(std::atof(val.c_str()));
      }
      ++i;
    }
    rows_ = i;
  }

  int d_;
  size_t n_;
  std::vector<T> X_;
  std::vector<uint32_t> clusters_;
  size_t rows_ = 0;
  std::unique_ptr<std::unique_ptr<Point<T>>[]> points_;
  std::vector<Point<T>*> ptrs_;
};

#endif  // KM_INPUT_PARSER_HPP
