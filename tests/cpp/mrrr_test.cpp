// Driver of the MRRR building block (mps2_gb300/csrc/mrrr.cuh) on the host,
// for tests/test_mrrr.py.  Input (binary): repeated [int32 n, n doubles d,
// n-1 doubles e]; output: per matrix [int32 k, double sigma, k doubles
// eigenvalues ascending, n*k doubles eigenvectors column by column] for the
// eigenvalues above floor_rel * lambda_max.
#include "../../mps2_gb300/csrc/mrrr.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace gq::mrrr;

int main(int argc, char **argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s in out floor_rel\n", argv[0]);
    return 2;
  }
  std::FILE *in = std::fopen(argv[1], "rb");
  std::FILE *out = std::fopen(argv[2], "wb");
  const double floor_rel = std::atof(argv[3]);
  if (!in || !out) return 2;
  int n;
  while (std::fread(&n, sizeof(int), 1, in) == 1) {
    std::vector<double> d(n), e(n > 1 ? n - 1 : 1);
    if (std::fread(d.data(), sizeof(double), n, in) != (size_t)n) return 3;
    if (n > 1 && std::fread(e.data(), sizeof(double), n - 1, in) != (size_t)(n - 1)) return 3;
    double tn = 0.0, emax = 0.0;
    for (double x : d) tn = std::fmax(tn, std::fabs(x));
    for (int i = 0; i + 1 < n; ++i) emax = std::fmax(emax, std::fabs(e[i]));
    tn += 2.0 * emax;
    // smallest eigenvalue of T, then a shift just below it
    double lo = -tn, hi = tn;
    for (int it = 0; it < 200; ++it) {
      const double m = 0.5 * (lo + hi);
      if (sturm_count(d.data(), e.data(), n, m) >= 1)
        hi = m;
      else
        lo = m;
    }
    std::vector<double> D(n), l(n > 1 ? n - 1 : 1);
    double margin = 8.0 * n * kEps * tn, sigma = 0.0;
    for (int tries = 0; tries < 60; ++tries, margin *= 4.0) {
      sigma = lo - margin;
      if (root_repr(d.data(), e.data(), n, sigma, D.data(), l.data())) break;
    }
    const double top = eig_ldl(D.data(), l.data(), n, n - 1, 0.0, 2.0 * tn + std::fabs(sigma));
    const double lmax = top + sigma;
    const int first = count_ldl(D.data(), l.data(), n, floor_rel * lmax - sigma);
    const int k = n - first;
    std::vector<double> lam(k), Z((size_t)n * k), s(n), lp(n), p(n), u(n);
    for (int j = 0; j < k; ++j) {
      const double mu = eig_ldl(D.data(), l.data(), n, first + j, 0.0, 2.0 * tn + std::fabs(sigma));
      lam[j] = mu + sigma;
      twisted_vector(D.data(), l.data(), n, mu, s.data(), lp.data(), p.data(), u.data(),
                     Z.data() + (size_t)j * n);
    }
    std::fwrite(&k, sizeof(int), 1, out);
    std::fwrite(&sigma, sizeof(double), 1, out);
    std::fwrite(lam.data(), sizeof(double), k, out);
    std::fwrite(Z.data(), sizeof(double), (size_t)n * k, out);
  }
  std::fclose(in);
  std::fclose(out);
  return 0;
}
