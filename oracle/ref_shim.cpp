// Test infrastructure only: a C entry point around the reference's own CPU
// k-means class (comparisons/CPU_Kmeans/include/kmeans.h:10-35,
// comparisons/CPU_Kmeans/src/kmeans.cpp:16-200), so that tests can run the
// unmodified reference algorithm on in-memory data through ctypes.
//
// This file is compiled together with the reference's kmeans.cpp, taken from
// where it lies in the reference tree, by oracle/build_ref.sh.  Nothing of the
// reference is copied here; the wrapper only builds the reference's Point<float>
// objects, calls Kmeans(n,d,k,tol,&seed,points).run(maxiter) and reads back the
// labels the reference wrote with Point::setCluster.
#include <cstdint>
#include <cstddef>

#include "kmeans.h"   // reference: comparisons/CPU_Kmeans/include/kmeans.h

extern "C" {

// Runs the reference CPU k-means.  X is n*d row-major float32.  Returns the
// value of Kmeans::run (converged iteration, or maxiter), labels in labels_out.
uint64_t ref_cpu_kmeans(const float* X, uint64_t n, uint32_t d, uint32_t k,
                        float tol, int seed, uint64_t maxiter,
                        uint32_t* labels_out) {
  Point<float>** pts = new Point<float>*[n];
  for (uint64_t i = 0; i < n; ++i)
    pts[i] = new Point<float>(const_cast<float*>(X + i * d), d);
  uint64_t it;
  {
    Kmeans km(n, d, k, tol, &seed, pts);
    it = km.run(maxiter);
  }
  for (uint64_t i = 0; i < n; ++i) {
    labels_out[i] = (uint32_t)pts[i]->getCluster();
    delete pts[i];
  }
  delete[] pts;
  return it;
}

}
