// Compensated float64 summation (Neumaier's improvement of the Kahan-Babuska sum,
// Z. Angew. Math. Mech. 54 (1974) 39-51): the running sum s and the low-order part c
// that rounding dropped from it; value() = s + c.  Used where one thread adds many
// terms in sequence (the energy and virial sums); the short tree steps that combine
// threads' results stay plain.  Plain C++ so that host tests compile it with g++.
#ifndef SMX_COMPSUM_H
#define SMX_COMPSUM_H

#include <cmath>

#ifdef __CUDACC__
#define SMX_HD __host__ __device__ __forceinline__
#else
#define SMX_HD inline
#endif

namespace smx {

struct CompSum {
  double s = 0.0, c = 0.0;
  SMX_HD void add(double x) {
    const double t = s + x;
    c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  SMX_HD double value() const { return s + c; }
};

}  // namespace smx

#endif  // SMX_COMPSUM_H
