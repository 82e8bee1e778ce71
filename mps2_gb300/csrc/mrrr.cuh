// Eigenpairs of a symmetric positive semi-definite tridiagonal matrix T
// (diagonal d[0..n-1], off-diagonal e[0..n-2]) from one root representation
// L D L^T = T - sigma I, following the relatively robust representation
// method of Dhillon and Parlett (Linear Algebra Appl. 387, 2004) without
// its representation tree:
//   * root_repr      L D L^T of T - sigma I (sigma below the spectrum, so
//                    D > 0 and the representation fixes its eigenvalues to
//                    high relative accuracy);
//   * count_ldl      number of eigenvalues of L D L^T below tau
//                    (stationary qd transform);
//   * eig_ldl        the idx-th eigenvalue by bisection, to relative accuracy;
//   * twisted_vector the eigenvector of an eigenvalue from the twisted
//                    factorisation at the index of the smallest |gamma|.
// Every eigenvalue is independent of the others, so a GPU kernel runs one
// thread (or warp) per eigenvalue.  The functions compile for host and
// device; the host side is what the CPU tests check.  Eigenvalues whose
// relative gaps fall below ~1e-3 give vectors orthogonal only to
// ~n eps / relgap: the caller orthonormalises such clusters (on the DMRG
// Gram spectra they are at most pairs) and finishes with CholeskyQR2.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define GQ_HD __host__ __device__ inline
#else
#define GQ_HD inline
#endif

namespace gq {
namespace mrrr {

constexpr double kEps = 2.220446049250313e-16;  // 2^-52

// Eigenvalues of T below x (Sturm sequence of T - x I).
GQ_HD int sturm_count(const double *d, const double *e, int n, double x) {
  const double tiny = kEps * (fabs(x) + 1e-300);  // an exact zero pivot counts as negative
  int cnt = 0;
  double q = d[0] - x;
  if (q == 0.0) q = -tiny;
  if (q < 0.0) ++cnt;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - e[i - 1] * e[i - 1] / q;
    if (q == 0.0) q = -tiny;
    if (q < 0.0) ++cnt;
  }
  return cnt;
}

// L D L^T = T - sigma I; false when a pivot is not positive (sigma is not
// below the spectrum).
GQ_HD bool root_repr(const double *d, const double *e, int n, double sigma, double *D,
                     double *l) {
  D[0] = d[0] - sigma;
  if (!(D[0] > 0.0)) return false;
  for (int i = 0; i + 1 < n; ++i) {
    l[i] = e[i] / D[i];
    D[i + 1] = d[i + 1] - sigma - l[i] * e[i];
    if (!(D[i + 1] > 0.0)) return false;
  }
  return true;
}

// Eigenvalues of L D L^T below tau: negative pivots of the stationary
// transform L D L^T - tau I = L+ D+ L+^T.
GQ_HD int count_ldl(const double *D, const double *l, int n, double tau) {
  int cnt = 0;
  double s = -tau;
  for (int i = 0; i + 1 < n; ++i) {
    double dp = D[i] + s;
    if (dp == 0.0) dp = -kEps * fabs(tau) - 1e-300;
    if (dp < 0.0) ++cnt;
    const double lp = l[i] * D[i] / dp;
    s = lp * l[i] * s - tau;
  }
  if (D[n - 1] + s < 0.0) ++cnt;
  return cnt;
}

// The idx-th smallest eigenvalue (0-based) of L D L^T inside [lo, hi], by
// bisection down to a relative width of a few ulps.
GQ_HD double eig_ldl(const double *D, const double *l, int n, int idx, double lo, double hi) {
  for (int it = 0; it < 200; ++it) {
    const double m = 0.5 * (lo + hi);
    if (!(m > lo && m < hi)) break;  // the interval cannot shrink any further
    if (count_ldl(D, l, n, m) > idx)
      hi = m;
    else
      lo = m;
    if (hi - lo <= 4.0 * kEps * fmax(fabs(lo), fabs(hi))) break;
  }
  return 0.5 * (lo + hi);
}

// Unit eigenvector z of L D L^T for its eigenvalue tau.  Work arrays of n
// doubles each: s, lp (n-1), p, u (n-1).
GQ_HD void twisted_vector(const double *D, const double *l, int n, double tau, double *s,
                          double *lp, double *p, double *u, double *z) {
  // stationary (top down): L D L^T - tau I = L+ D+ L+^T
  s[0] = -tau;
  for (int i = 0; i + 1 < n; ++i) {
    double dp = D[i] + s[i];
    if (dp == 0.0) dp = -kEps * fabs(tau) - 1e-300;
    lp[i] = l[i] * D[i] / dp;
    s[i + 1] = lp[i] * l[i] * s[i] - tau;
  }
  // progressive (bottom up): L D L^T - tau I = U- D- U-^T
  p[n - 1] = D[n - 1] - tau;
  for (int i = n - 2; i >= 0; --i) {
    double dm = D[i] * l[i] * l[i] + p[i + 1];
    if (dm == 0.0) dm = -kEps * fabs(tau) - 1e-300;
    const double t = D[i] / dm;
    u[i] = l[i] * t;
    p[i] = p[i + 1] * t - tau;
  }
  // twist where |gamma_k| = |s_k + p_k + tau| is smallest
  int r = 0;
  double best = fabs(s[0] + p[0] + tau);
  for (int k = 1; k < n; ++k) {
    const double g = fabs(s[k] + p[k] + tau);
    if (g < best) {
      best = g;
      r = k;
    }
  }
  z[r] = 1.0;
  for (int i = r - 1; i >= 0; --i) z[i] = -lp[i] * z[i + 1];
  for (int i = r; i + 1 < n; ++i) z[i + 1] = -u[i] * z[i];
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) nrm += z[i] * z[i];
  nrm = 1.0 / sqrt(nrm);
  for (int i = 0; i < n; ++i) z[i] *= nrm;
}

}  // namespace mrrr
}  // namespace gq
