// Lowest eigenpair of the Lanczos tridiagonal matrix T (diagonal a[0..n),
// off-diagonal b[0..n-1)), written once for the device control kernels of
// the Lanczos loop and compiled for the host as well (unit tests).
//
// Replaces ``TridiagGsSolver`` -> ``LAPACKE_dstev`` of gqmps2
// (``lanczos_solver_impl.h:259-313``), which the solver calls for the
// lowest Ritz value after every matvec and for its Ritz vector at the end.
//
// * Eigenvalue: bisection on Sturm counts (the number of negative pivots of
//   the LDL^T factorisation of T - x I equals the number of eigenvalues
//   below x; Golub & Van Loan, Matrix Computations, sec. 8.4.1; the pivot
//   guard of LAPACK's dlaebz), started from the Gershgorin interval.  With
//   `lanes` evaluation points per step (32 on a warp) every step cuts the
//   interval into lanes + 1 parts; it stops when the interval holds no
//   representable point between its ends, or after kMaxSteps steps.
// * Eigenvector: two steps of inverse iteration with the tridiagonal LU
//   factorisation with partial pivoting (the row interchanges of LAPACK's
//   dgttrf / dgttrs) on T - lambda I, from a fixed hashed start vector; normalised
//   to unit length with its largest component positive.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define GQ_HD __host__ __device__
#else
#define GQ_HD
#endif

namespace gq {
namespace tridiag {

#ifndef __CUDACC__
using std::fabs;
using std::fmax;
using std::fmin;
using std::isfinite;
using std::sqrt;
#endif

constexpr int kMaxSteps = 128;
constexpr double kEps = 2.220446049250313e-16;  // 2^-52

// Gershgorin interval [lo, hi] holding every eigenvalue, and the pivot
// guard (smallest admissible |pivot| of the Sturm recurrence).
GQ_HD inline void gershgorin(const double *a, const double *b, int n, double *lo, double *hi,
                             double *pivmin) {
  double l = a[0], h = a[0], bmax2 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < n ? fabs(b[i]) : 0.0);
    l = fmin(l, a[i] - r);
    h = fmax(h, a[i] + r);
    if (i + 1 < n) bmax2 = fmax(bmax2, b[i] * b[i]);
  }
  // widen by a few units of the scale so rounding cannot push an eigenvalue out
  const double scale = fmax(fabs(l), fabs(h));
  l -= 4.0 * kEps * scale + 1e-300;
  h += 4.0 * kEps * scale + 1e-300;
  *lo = l;
  *hi = h;
  *pivmin = fmax(1e-300, 1e-300 * bmax2);
}

// Number of eigenvalues of T below x.
GQ_HD inline int sturm_count(const double *a, const double *b, int n, double x, double pivmin) {
  int cnt = 0;
  double q = a[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0.0) ++cnt;
  for (int i = 1; i < n; ++i) {
    q = (a[i] - x) - (b[i - 1] * b[i - 1]) / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++cnt;
  }
  return cnt;
}

// The j-th of `lanes` interior points of [lo, hi] (j = 0 .. lanes-1).
GQ_HD inline double section_point(double lo, double hi, int j, int lanes) {
  return lo + (hi - lo) * ((double)(j + 1) / (double)(lanes + 1));
}

// One multisection step given the Sturm counts (>= 1 or not) of the
// `lanes` interior points: the new interval is the part that holds the
// lowest eigenvalue.  `first` = the lowest point index whose count is >= 1
// (lanes if none).  Returns false when the interval cannot shrink further.
GQ_HD inline bool section_update(double *lo, double *hi, int first, int lanes) {
  const double l = *lo, h = *hi;
  const double nl = first == 0 ? l : section_point(l, h, first - 1, lanes);
  const double nh = first == lanes ? h : section_point(l, h, first, lanes);
  if (!(nl > l) && !(nh < h)) return false;  // no representable progress
  *lo = nl;
  *hi = nh;
  return true;
}

// Serial form (host tests and single-thread callers): the same points and
// the same decisions as the warp form, one point after another.
GQ_HD inline double lowest_eigenvalue_serial(const double *a, const double *b, int n,
                                             int lanes = 32) {
  if (n == 1) return a[0];
  double lo, hi, pivmin;
  gershgorin(a, b, n, &lo, &hi, &pivmin);
  for (int step = 0; step < kMaxSteps; ++step) {
    int first = lanes;
    for (int j = 0; j < lanes; ++j)
      if (sturm_count(a, b, n, section_point(lo, hi, j, lanes), pivmin) >= 1) {
        first = j;
        break;
      }
    if (!section_update(&lo, &hi, first, lanes)) break;
  }
  return 0.5 * (lo + hi);
}

#ifdef __CUDACC__
// Warp form: lane j evaluates point j; all lanes return the same value.
__device__ inline double lowest_eigenvalue_warp(const double *a, const double *b, int n) {
  if (n == 1) return a[0];
  const int lane = threadIdx.x & 31;
  double lo, hi, pivmin;
  gershgorin(a, b, n, &lo, &hi, &pivmin);
  for (int step = 0; step < kMaxSteps; ++step) {
    const int c = sturm_count(a, b, n, section_point(lo, hi, lane, 32), pivmin);
    const unsigned hit = __ballot_sync(0xffffffffu, c >= 1);
    const int first = hit ? __ffs(hit) - 1 : 32;
    if (!section_update(&lo, &hi, first, 32)) break;
  }
  return 0.5 * (lo + hi);
}
#endif

// Component i of the fixed start vector of the inverse iteration: values
// in [-1, 1) from an integer hash of i (a constant or otherwise structured
// start can be orthogonal to the wanted vector, e.g. the all-ones vector
// and the alternating ground state of a persymmetric T).
GQ_HD inline double start_component(int i) {
  uint32_t h = (uint32_t)i * 2654435761u + 0x9e3779b9u;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return (double)h * (1.0 / 2147483648.0) - 1.0;
}

// Inverse-iteration eigenvector of T for the eigenvalue lambda; work holds
// 5 n doubles and n ints' worth (as doubles).  vec gets n values.
GQ_HD inline void eigenvector(const double *a, const double *b, int n, double lambda,
                              double *work, double *vec) {
  if (n == 1) {
    vec[0] = 1.0;
    return;
  }
  double *dl = work, *dd = work + n, *du = work + 2 * n, *du2 = work + 3 * n, *piv = work + 4 * n;
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i) {
    tnorm = fmax(tnorm, fabs(a[i] - lambda));
    if (i + 1 < n) tnorm = fmax(tnorm, fabs(b[i]));
  }
  const double tiny = fmax(kEps * tnorm, 1e-300);
  for (int i = 0; i < n; ++i) {
    dd[i] = a[i] - lambda;
    if (i + 1 < n) {
      dl[i] = b[i];
      du[i] = b[i];
    }
    du2[i] = 0.0;
    piv[i] = 0.0;
  }
  // LU with partial pivoting (row i and i+1 exchanged when |sub| > |diag|)
  for (int i = 0; i + 1 < n; ++i) {
    if (fabs(dd[i]) >= fabs(dl[i])) {
      if (dd[i] == 0.0) dd[i] = tiny;
      const double l = dl[i] / dd[i];
      dl[i] = l;
      dd[i + 1] -= l * du[i];
    } else {
      const double l = dd[i] / dl[i];
      dd[i] = dl[i];
      dl[i] = l;
      const double t = du[i];
      du[i] = dd[i + 1];
      dd[i + 1] = t - l * dd[i + 1];
      if (i + 2 < n) {
        du2[i] = du[i + 1];
        du[i + 1] = -l * du[i + 1];
      }
      piv[i] = 1.0;
    }
  }
  if (dd[n - 1] == 0.0) dd[n - 1] = tiny;
  for (int i = 0; i < n; ++i) vec[i] = start_component(i);
  for (int it = 0; it < 2; ++it) {
    // forward: apply the interchanges and the multipliers
    for (int i = 0; i + 1 < n; ++i) {
      if (piv[i] != 0.0) {
        const double t = vec[i];
        vec[i] = vec[i + 1];
        vec[i + 1] = t - dl[i] * vec[i + 1];
      } else {
        vec[i + 1] -= dl[i] * vec[i];
      }
    }
    // back substitution with the upper factor (diagonal + two superdiagonals)
    vec[n - 1] /= dd[n - 1];
    vec[n - 2] = (vec[n - 2] - du[n - 2] * vec[n - 1]) / dd[n - 2];
    for (int i = n - 3; i >= 0; --i)
      vec[i] = (vec[i] - du[i] * vec[i + 1] - du2[i] * vec[i + 2]) / dd[i];
    // rescale by the largest component (keeps the next solve in range)
    double big = 0.0;
    for (int i = 0; i < n; ++i) big = fmax(big, fabs(vec[i]));
    if (!(big > 0.0) || !isfinite(big)) big = 1.0;
    for (int i = 0; i < n; ++i) vec[i] /= big;
  }
  int ib = 0;
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) {
    if (fabs(vec[i]) > fabs(vec[ib])) ib = i;
    nrm += vec[i] * vec[i];
  }
  nrm = sqrt(nrm);
  const double f = (vec[ib] < 0.0 ? -1.0 : 1.0) / nrm;
  for (int i = 0; i < n; ++i) vec[i] *= f;
}

}  // namespace tridiag
}  // namespace gq
