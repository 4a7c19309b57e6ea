// point.hpp — the reference's per-point carrier, kept for source compatibility
// of callers that build `Point<float>**` arrays (src/include/point.hpp:12-81).
//
// Same public surface and semantics: a point owns a copy of its d coordinates
// and an unsigned cluster id; get(i) past the end exits with status 3 (the
// reference's EXIT_POINT_IOB, src/include/utils.hpp:36); == compares the
// coordinates with float '=='; << prints the cluster and the coordinates in
// width-9 columns with 5 significant digits.  Storage is a std::vector and the
// coordinates are also reachable as one contiguous array through data().
#ifndef KM_POINT_HPP
#define KM_POINT_HPP

#include <cstdlib>
#include <iomanip>
#include <ostream>
#include <vector>

template <typename T>
class Point {
 public:
  Point() = default;

  Point(T* x, unsigned int d) : x_(x, x + d) {}

  // Copy from a pointer, cluster included (reference: Point(Point<T>* const)).
  Point(Point<T>* const p) : x_(p->x_), cluster_(p->cluster_) {}

  Point(const Point&) = default;

  // Assignment copies the coordinates and keeps this point's cluster, as the
  // reference's operator= does.
  Point& operator=(const Point& p) {
    if (this != &p) x_ = p.x_;
    return *this;
  }

  int getCluster() { return static_cast<int>(cluster_); }
  void setCluster(unsigned int c) { cluster_ = c; }

  T get(unsigned int i) {
    if (i >= x_.size()) std::exit(3);
    return x_[i];
  }

  const T* data() const { return x_.data(); }
  unsigned int dims() const { return static_cast<unsigned int>(x_.size()); }

  bool operator==(const Point<T>& p) const {
    if (x_.size() != p.x_.size()) return false;
    for (size_t i = 0; i < x_.size(); ++i)
      if (!(x_[i] == p.x_[i])) return false;
    return true;
  }

  friend std::ostream& operator<<(std::ostream& os, const Point& p) {
    os << std::setw(9) << p.cluster_;
    for (const T& v : p.x_) os << std::setw(9) << std::setprecision(5) << v;
    return os;
  }

 private:
  std::vector<T> x_;
  unsigned int cluster_ = 0;
};

#endif  // KM_POINT_HPP
