// Finite-MPS canonicalisation and truncation on the device.
//
// Restates ``FiniteMPS::Centralize`` with ``LeftCanonicalizeTen_`` and
// ``RightCanonicalizeTen_`` and the free function ``TruncateMPS``
// (``one_dim_tn/mps/finite_mps/finite_mps.h:149-300``): each site step is one
// block SVD of the site tensor (untruncated for the canonicalisation, as
// ``mock_gqten::SVD`` at ``utilities.h:26-57`` does) whose orthonormal factor
// stays on the site while S.Vt (or U.S) is contracted into the neighbour.
// The SVD routes and semantics are those of ``svd_truncate``; the tensors
// never leave the device.
#include "gq_runtime.hpp"

namespace gq {

namespace {
// ``mock_gqten::SVD``: Dmin = Dmax = the larger matricised dimension, so
// every value (zeros included) is kept.
int64_t keep_all(const Tensor &t, int ldims) {
  int64_t l = 1, r = 1;
  for (int i = 0; i < t.rank(); ++i) (i < ldims ? l : r) *= t.idx[i].total();
  return std::max(l, r);
}
}  // namespace

void left_canonicalize_ten(std::vector<TensorPtr> &mps, std::vector<int> &cano, int i) {
  GQ_CHECK(i >= 0 && i + 1 < (int)mps.size(), "left canonicalisation: site out of range");
  const Tensor &t = *mps[i];
  const int ldims = i == 0 ? 1 : 2;
  const int64_t D = keep_all(t, ldims);
  SvdOut sv = svd_truncate(t, ldims, t.div, 0.0, D, D, 2);  // U; S.Vt
  mps[i] = sv.u;
  mps[i + 1] = contract(*sv.vt, *mps[i + 1], {1}, {0}, kFP64);
  cano[i] = kCanoLeft;
  cano[i + 1] = kCanoNone;
}

void right_canonicalize_ten(std::vector<TensorPtr> &mps, std::vector<int> &cano, int i) {
  GQ_CHECK(i >= 1 && i < (int)mps.size(), "right canonicalisation: site out of range");
  const Tensor &t = *mps[i];
  QN zero = t.div - t.div;
  const int64_t D = keep_all(t, 1);
  SvdOut sv = svd_truncate(t, 1, zero, 0.0, D, D, 1);  // U.S; Vt
  mps[i] = sv.vt;
  const int axis = i - 1 == 0 ? 1 : 2;
  mps[i - 1] = contract(*mps[i - 1], *sv.u, {axis}, {0}, kFP64);
  cano[i] = kCanoRight;
  cano[i - 1] = kCanoNone;
}

void centralize(std::vector<TensorPtr> &mps, std::vector<int> &cano, int center) {
  const int n = (int)mps.size();
  GQ_CHECK(n >= 2 && (int)cano.size() == n, "centralize: bad MPS");
  GQ_CHECK(center >= 0 && center < n, "centralize: center out of range");
  if (center != 0) {  // LeftCanonicalize_(center - 1)
    const int stop = center - 1;
    int start = -1;
    for (int i = 0; i <= stop; ++i) {
      start = i;
      if (cano[i] != kCanoLeft) break;
      if (i == stop) start = -1;
    }
    if (start >= 0)
      for (int i = start; i <= stop; ++i) left_canonicalize_ten(mps, cano, i);
  }
  if (center != n - 1) {  // RightCanonicalize_(center + 1)
    const int stop = center + 1;
    int start = -1;
    for (int i = n - 1; i >= stop; --i) {
      start = i;
      if (cano[i] != kCanoRight) break;
      if (i == stop) start = -1;
    }
    if (start >= 0)
      for (int i = start; i >= stop; --i) right_canonicalize_ten(mps, cano, i);
  }
}

std::vector<std::pair<double, int64_t>> truncate_mps(std::vector<TensorPtr> &mps,
                                                     std::vector<int> &cano, double trunc_err,
                                                     int64_t dmin, int64_t dmax) {
  const int n = (int)mps.size();
  centralize(mps, cano, 0);
  {  // mps[0].Normalize()
    Tensor &t0 = *mps[0];
    DevBuf red(dot_scratch_elems()), nrm(1);
    dev_dot(t0.data.p, t0.data.p, t0.size(), nrm.p, red.p);
    double h = 0.0;
    GQ_CUDA(cudaMemcpyAsync(&h, nrm.p, sizeof(double), cudaMemcpyDeviceToHost, stream()));
    sync();
    GQ_CHECK(h > 0.0, "TruncateMPS: the MPS has zero norm");
    dev_scale(t0.data.p, t0.size(), 1.0 / std::sqrt(h));
  }
  std::vector<std::pair<double, int64_t>> out;
  for (int i = 0; i + 1 < n; ++i) {
    const Tensor &t = *mps[i];
    SvdOut sv = svd_truncate(t, i == 0 ? 1 : 2, t.div, trunc_err, dmin, dmax, 2);
    out.push_back({sv.trunc_err, sv.D});
    double s2 = 0.0;
    for (double v : sv.s) s2 += v * v;
    GQ_CHECK(s2 > 0.0, "TruncateMPS: zero singular values");
    dev_scale(sv.vt->data.p, sv.vt->size(), 1.0 / std::sqrt(s2));  // S.Normalize()
    mps[i] = sv.u;
    mps[i + 1] = contract(*sv.vt, *mps[i + 1], {1}, {0}, kFP64);
  }
  // the reference writes every site through its non-const accessor, which
  // marks it as not canonical
  for (auto &c : cano) c = kCanoNone;
  return out;
}

}  // namespace gq
