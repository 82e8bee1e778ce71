// Lowest eigenpair of the Lanczos tridiagonal matrix.
//
// Replaces ``TridiagGsSolver`` -> ``LAPACKE_dstev`` of gqmps2
// (``lanczos_solver_impl.h:259-313``).  The matrix is at most
// max_iterations x max_iterations (a few hundred), so this runs on the host
// between Lanczos steps.  Method: the implicit QL iteration with Wilkinson
// shifts for symmetric tridiagonal matrices (Wilkinson & Reinsch, Handbook
// for Automatic Computation vol. II, procedure tql2; Golub & Van Loan,
// Matrix Computations, sec. 8.3), written here from that description.
#include <cmath>
#include <vector>

#include "gq_runtime.hpp"

namespace gq {

namespace {
// QL sweeps on (d, e); if z != nullptr accumulate the rotations into the
// row-major n x n matrix z (initialised to the identity) so that column j of
// z is the eigenvector of d[j] on return.
bool ql_implicit(std::vector<double> &d, std::vector<double> &e, int n, double *z) {
  e.resize(n);
  e[n - 1] = 0.0;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      int m = l;
      for (; m < n - 1; ++m) {
        const double scale = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-300 || std::fabs(e[m]) <= 2.220446049250313e-16 * scale) break;
      }
      if (m == l) break;
      if (++iter > 100) return false;
      // Wilkinson shift from the leading 2x2 block
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? r : -r));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = m - 1;
      bool deflated = false;
      for (; i >= l; --i) {
        const double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // underflow: split the matrix here
          d[i + 1] -= p;
          e[m] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        if (z) {
          for (int k = 0; k < n; ++k) {
            const double zk1 = z[k * n + i + 1], zk0 = z[k * n + i];
            z[k * n + i + 1] = s * zk0 + c * zk1;
            z[k * n + i] = c * zk0 - s * zk1;
          }
        }
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  return true;
}
}  // namespace

bool tridiag_lowest(const double *a, const double *b, int n, double *eval, double *vec) {
  if (n <= 0) return false;
  if (n == 1) {
    *eval = a[0];
    if (vec) vec[0] = 1.0;
    return true;
  }
  std::vector<double> d(a, a + n), e(b, b + n - 1);
  std::vector<double> z;
  if (vec) {
    z.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
  }
  if (!ql_implicit(d, e, n, vec ? z.data() : nullptr)) return false;
  int j = 0;
  for (int i = 1; i < n; ++i)
    if (d[i] < d[j]) j = i;
  *eval = d[j];
  if (vec) {
    int big = 0;
    for (int k = 0; k < n; ++k) {
      vec[k] = z[(size_t)k * n + j];
      if (std::fabs(vec[k]) > std::fabs(vec[big])) big = k;
    }
    double nrm = 0.0;
    for (int k = 0; k < n; ++k) nrm += vec[k] * vec[k];
    nrm = std::sqrt(nrm);
    const double sgn = vec[big] < 0.0 ? -1.0 : 1.0;
    for (int k = 0; k < n; ++k) vec[k] *= sgn / nrm;
  }
  return std::isfinite(*eval);
}

}  // namespace gq
