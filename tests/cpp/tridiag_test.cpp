// Driver of the Lanczos tridiagonal solver (mps2_gb300/csrc/tridiag_dev.cuh)
// on the host, for tests/test_tridiag_dev.py.  Input (binary): repeated
// [int32 n, n doubles a, n-1 doubles b]; output per matrix: [double lambda,
// n doubles eigenvector].
#include "../../mps2_gb300/csrc/tridiag_dev.cuh"

#include <cstdio>
#include <vector>

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in out\n", argv[0]);
    return 2;
  }
  std::FILE *in = std::fopen(argv[1], "rb");
  std::FILE *out = std::fopen(argv[2], "wb");
  if (!in || !out) return 2;
  int n;
  while (std::fread(&n, sizeof(int), 1, in) == 1) {
    std::vector<double> a(n), b(n > 1 ? n - 1 : 1), work(5 * n), vec(n);
    if (std::fread(a.data(), sizeof(double), n, in) != (size_t)n) return 3;
    if (n > 1 && std::fread(b.data(), sizeof(double), n - 1, in) != (size_t)(n - 1)) return 3;
    const double lam = gq::tridiag::lowest_eigenvalue_serial(a.data(), b.data(), n);
    gq::tridiag::eigenvector(a.data(), b.data(), n, lam, work.data(), vec.data());
    std::fwrite(&lam, sizeof(double), 1, out);
    std::fwrite(vec.data(), sizeof(double), n, out);
  }
  std::fclose(out);
  return 0;
}
