// Truncating block SVD of the two-site ground state.
//
// Replaces gqten's ``SVD(t, ldims, ldiv, trunc_err, Dmin, Dmax, &U, &S, &Vt,
// &err, &D)`` as called at ``two_site_update_finite_vmps_impl.h:258-263``.
// Semantics (shared with the FP64 oracle):
//  * the tensor is matricised with its first `ldims` legs as rows; blocks
//    whose row legs carry the same new-bond charge
//    q = ldiv - sum_{l<ldims} dir_l q_l form one dense matrix (rows: row-leg
//    sector tuples ascending, columns likewise; every allowed block takes
//    part, absent ones are zero);
//  * every group is decomposed in FP64 (cuSOLVER gesvdj, sorted);
//  * values <= 1e-13 * s_max become exact zeros;
//  * global selection: rank all values (ties: earlier group, earlier
//    position); D = smallest count in [Dmin, Dmax] whose discarded weight
//    sum_{i>=D} s_i^2 / sum s^2 <= trunc_err, capped by Dmax and #values;
//  * kept nonzero values use the solver's vectors with the largest-|.|
//    entry of each left vector made positive (right vector follows); kept
//    zero values use the canonical completion of null_completion (a
//    counter-hashed seed matrix projected off the group's nonzero singular
//    vectors, then CholeskyQR2);
//  * new bond sectors: groups with a kept value, ascending charge.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <map>
#include <numeric>

#include "gq_runtime.hpp"

namespace gq {

namespace {
constexpr double kZeroSvRtol = 1e-13;

#define GQ_SOLVER(call)                                                               \
  do {                                                                                \
    cusolverStatus_t s_ = (call);                                                     \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                                \
      ::gq::fail(::gq::kSolverError, std::string(#call) + " failed with status " +    \
                                         std::to_string((int)s_));                    \
  } while (0)

cusolverDnHandle_t solver() {
  auto &c = ctx();
  if (!c.cusolver) {
    cusolverDnHandle_t h;
    GQ_SOLVER(cusolverDnCreate(&h));
    c.cusolver = h;
  }
  auto h = (cusolverDnHandle_t)c.cusolver;
  GQ_SOLVER(cusolverDnSetStream(h, c.stream));
  return h;
}

struct GatherItem { int64_t src_off, dst_off; int rows, cols, ld; };

__global__ void gather_kernel(const GatherItem *__restrict__ items, const double *__restrict__ src,
                              double *__restrict__ dst) {
  const GatherItem it = items[blockIdx.x];
  const int64_t n = (int64_t)it.rows * it.cols;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int64_t i = e / it.cols, j = e % it.cols;
    dst[it.dst_off + i * it.ld + j] = src[it.src_off + e];
  }
}

// Sign convention: column j of `u` (m x *, col-major, ld m): make the first
// entry of largest magnitude positive; flip column j of `v` alongside.
struct SignItem { int64_t u_off, v_off; int m, n; };

__global__ void sign_fix_kernel(const SignItem *__restrict__ items, double *__restrict__ U,
                                double *__restrict__ V) {
  const SignItem it = items[blockIdx.x];
  __shared__ double bv[256];
  __shared__ int bi[256];
  double best = -1.0;
  int besti = 0x7fffffff;
  for (int i = threadIdx.x; i < it.m; i += blockDim.x) {
    const double a = fabs(U[it.u_off + i]);
    if (a > best) { best = a; besti = i; }
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = besti;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double o = bv[threadIdx.x + s];
      const int oi = bi[threadIdx.x + s];
      if (o > bv[threadIdx.x] || (o == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = o;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const bool flip = U[it.u_off + bi[0]] < 0.0;
  __syncthreads();
  if (!flip) return;
  for (int i = threadIdx.x; i < it.m; i += blockDim.x) U[it.u_off + i] = -U[it.u_off + i];
  for (int i = threadIdx.x; i < it.n; i += blockDim.x) V[it.v_off + i] = -V[it.v_off + i];
}

// Output block writer.  mode 0: U block (rows x k, row-major) with
// dst(i,j) = col j of the group's left vectors at row `r0 + i`;
// mode 1: Vt block (k x rows) with dst(j,i) = col j of the right vectors at
// row `r0 + i`.  Columns j < knz come from the SVD, j >= knz from the
// completion.  `scale` multiplies column j by s[j] when set.
struct ScatterItem {
  int64_t dst_off;
  int rows, k, knz, mode, scale;
  int64_t svd_off; int ld_svd;      // col-major vectors, row offset folded in
  int64_t comp_off; int ld_comp;
  int64_t s_off;
};

__global__ void scatter_kernel(const ScatterItem *__restrict__ items,
                               const double *__restrict__ left_svd,
                               const double *__restrict__ right_svd,
                               const double *__restrict__ left_comp,
                               const double *__restrict__ right_comp,
                               const double *__restrict__ svals, double *__restrict__ U,
                               double *__restrict__ Vt) {
  const ScatterItem it = items[blockIdx.x];
  const double *svd = it.mode == 0 ? left_svd : right_svd;
  const double *comp = it.mode == 0 ? left_comp : right_comp;
  double *dst = it.mode == 0 ? U : Vt;
  const int64_t n = (int64_t)it.rows * it.k;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    int i, j;
    if (it.mode == 0) { i = (int)(e / it.k); j = (int)(e % it.k); }
    else { j = (int)(e / it.rows); i = (int)(e % it.rows); }
    double v = j < it.knz ? svd[it.svd_off + i + (int64_t)j * it.ld_svd]
                          : comp[it.comp_off + i + (int64_t)(j - it.knz) * it.ld_comp];
    if (it.scale) v *= svals[it.s_off + j];
    dst[it.dst_off + e] = v;
  }
}

// Counter-based seed matrix for the null-space completion: element (i, j) =
// splitmix64(key ^ (i << 20) ^ j), top 53 bits scaled by 2^-53, minus 0.5.
// Every operation is exact, so the CPU oracle reproduces it bit for bit.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  unsigned long long z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void seed_matrix_kernel(double *__restrict__ w, int dim, int k,
                                   unsigned long long key) {
  const int64_t n = (int64_t)dim * k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long i = (unsigned long long)(e % dim), j = (unsigned long long)(e / dim);
    const unsigned long long z = splitmix64(key ^ (i << 20) ^ j);
    w[e] = (double)(z >> 11) * 0x1p-53 - 0.5;
  }
}

#define GQ_BLAS(call)                                                                 \
  do {                                                                                \
    cublasStatus_t s_ = (call);                                                       \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                  \
      ::gq::fail(::gq::kSolverError, std::string(#call) + " failed with status " +    \
                                         std::to_string((int)s_));                    \
  } while (0)

cublasHandle_t blas() {
  static cublasHandle_t h = nullptr;
  if (!h) GQ_BLAS(cublasCreate(&h));
  GQ_BLAS(cublasSetStream(h, stream()));
  return h;
}

struct Group {
  QN q;
  std::vector<std::vector<int>> rows, cols;
  std::vector<int64_t> rsz, csz, roff, coff;
  int64_t m = 0, n = 0, p = 0;
  int64_t mat_off = 0, lv_off = 0, rv_off = 0, s_off = 0;  // in the work buffers
  int64_t nnz = 0;     // nonzero singular values
  int64_t keep = 0, keep_nz = 0;
  int sector = -1;
  int64_t lc_off = 0, rc_off = 0;  // completion buffers
};

// Canonical completion: k orthonormal columns orthogonal to the r
// orthonormal columns of `vecs` (dim x r, col-major, ld dim), written to
// out (dim x k, col-major).  The seed matrix is projected off `vecs` twice
// (Gram-Schmidt with re-orthogonalisation) and orthonormalised by
// CholeskyQR2; nothing depends on the signs of the columns of `vecs`.
void null_completion(const double *vecs, int64_t dim, int64_t r, int64_t k, int group, int side,
                     double *out) {
  if (k == 0) return;
  auto s = stream();
  const unsigned grid = (unsigned)std::min<int64_t>((dim * k + 255) / 256, 4096);
  const unsigned long long key = (unsigned long long)(2 * group + side) << 40;
  seed_matrix_kernel<<<grid, 256, 0, s>>>(out, (int)dim, (int)k, key);
  GQ_CUDA(cudaGetLastError());
  auto bh = blas();
  const int d = (int)dim, kk = (int)k, rr = (int)r;
  const double one = 1.0, zero = 0.0, mone = -1.0;
  if (r > 0) {
    DevBuf t(r * k);
    for (int pass = 0; pass < 2; ++pass) {
      GQ_BLAS(cublasDgemm(bh, CUBLAS_OP_T, CUBLAS_OP_N, rr, kk, d, &one, vecs, d, out, d, &zero,
                          t.p, rr));
      GQ_BLAS(cublasDgemm(bh, CUBLAS_OP_N, CUBLAS_OP_N, d, kk, rr, &mone, vecs, d, t.p, rr, &one,
                          out, d));
    }
  }
  auto sh = solver();
  DevBuf g(k * k);
  int lw = 0;
  GQ_SOLVER(cusolverDnDpotrf_bufferSize(sh, CUBLAS_FILL_MODE_LOWER, kk, g.p, kk, &lw));
  DevBuf work((int64_t)lw + 1);
  DevArray<int> info;
  info.upload(std::vector<int>(2, 0));
  for (int pass = 0; pass < 2; ++pass) {
    GQ_BLAS(cublasDgemm(bh, CUBLAS_OP_T, CUBLAS_OP_N, kk, kk, d, &one, out, d, out, d, &zero, g.p,
                        kk));
    GQ_SOLVER(cusolverDnDpotrf(sh, CUBLAS_FILL_MODE_LOWER, kk, g.p, kk, work.p, lw,
                               info.p + pass));
    GQ_BLAS(cublasDtrsm(bh, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                        CUBLAS_DIAG_NON_UNIT, d, kk, &one, g.p, kk, out, d));
  }
  int hinfo[2] = {0, 0};
  GQ_CUDA(cudaMemcpyAsync(hinfo, info.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  sync();
  if (hinfo[0] != 0 || hinfo[1] != 0)
    fail(kSolverError, "null-space completion: Cholesky failed");
}
}  // namespace

SvdOut svd_truncate(const Tensor &t_in, int ldims, const QN &ldiv, double trunc_err,
                    int64_t dmin, int64_t dmax, int scale_side) {
  // Every allowed block takes part; embed a sparser tensor first.
  TensorPtr full;
  if ((size_t)t_in.nblocks() != allowed_blocks(t_in.idx, t_in.div).size()) {
    full = lanczos_space(t_in);
    full->allocate();
    embed(t_in, *full);
  }
  const Tensor &t = full ? *full : t_in;
  const int r = t.rank();
  GQ_CHECK(ldims >= 1 && ldims < r, "SVD: ldims must split the legs");
  GQ_CHECK(dmax >= 1 && dmin >= 1, "SVD: Dmin and Dmax must be positive");
  auto s = stream();

  // ---- group the blocks by new-bond charge --------------------------------
  std::map<QN, Group> gmap;
  struct BRef { QN q; std::vector<int> rc, cc; int64_t b; };
  std::vector<BRef> brefs;
  for (int64_t b = 0; b < t.nblocks(); ++b) {
    const int *c = t.block_coords(b);
    QN q = ldiv;
    for (int l = 0; l < ldims; ++l) q = q - t.idx[l].qn[c[l]].scaled(t.idx[l].dir);
    BRef br{q, std::vector<int>(c, c + ldims), std::vector<int>(c + ldims, c + r), b};
    auto &g = gmap[q];
    g.q = q;
    g.rows.push_back(br.rc);
    g.cols.push_back(br.cc);
    brefs.push_back(std::move(br));
  }
  std::vector<Group *> groups;
  int64_t mat_total = 0, lv_total = 0, rv_total = 0, s_total = 0;
  for (auto &kv : gmap) {
    Group &g = kv.second;
    std::sort(g.rows.begin(), g.rows.end());
    g.rows.erase(std::unique(g.rows.begin(), g.rows.end()), g.rows.end());
    std::sort(g.cols.begin(), g.cols.end());
    g.cols.erase(std::unique(g.cols.begin(), g.cols.end()), g.cols.end());
    for (auto &rc : g.rows) {
      int64_t sz = 1;
      for (int l = 0; l < ldims; ++l) sz *= t.idx[l].dim[rc[l]];
      g.roff.push_back(g.m);
      g.rsz.push_back(sz);
      g.m += sz;
    }
    for (auto &cc : g.cols) {
      int64_t sz = 1;
      for (int l = ldims; l < r; ++l) sz *= t.idx[l].dim[cc[l - ldims]];
      g.coff.push_back(g.n);
      g.csz.push_back(sz);
      g.n += sz;
    }
    g.p = std::min(g.m, g.n);
    g.mat_off = mat_total;
    mat_total += g.m * g.n;
    g.lv_off = lv_total;
    lv_total += g.m * g.p;
    g.rv_off = rv_total;
    rv_total += g.n * g.p;
    g.s_off = s_total;
    s_total += g.p;
    groups.push_back(&g);
  }
  GQ_CHECK(!groups.empty(), "SVD of a tensor without blocks");

  // ---- gather each group into a dense row-major m x n matrix --------------
  DevBuf mats(mat_total);
  GQ_CUDA(cudaMemsetAsync(mats.p, 0, sizeof(double) * mat_total, s));
  {
    std::vector<GatherItem> items;
    for (auto &br : brefs) {
      Group &g = gmap[br.q];
      const int64_t ri = std::lower_bound(g.rows.begin(), g.rows.end(), br.rc) - g.rows.begin();
      const int64_t ci = std::lower_bound(g.cols.begin(), g.cols.end(), br.cc) - g.cols.begin();
      GatherItem it{};
      it.src_off = t.offs[br.b];
      it.dst_off = g.mat_off + g.roff[ri] * g.n + g.coff[ci];
      it.rows = (int)g.rsz[ri];
      it.cols = (int)g.csz[ci];
      it.ld = (int)g.n;
      items.push_back(it);
    }
    DevArray<GatherItem> d;
    d.upload(items);
    gather_kernel<<<(unsigned)items.size(), 256, 0, s>>>(d.p, t.data.p, mats.p);
    GQ_CUDA(cudaGetLastError());
  }

  // ---- per-group SVD (the row-major m x n matrix is col-major n x m) -------
  DevBuf lv(lv_total), rv(rv_total), sv(s_total);
  {
    auto h = solver();
    gesvdjInfo_t prm;
    GQ_SOLVER(cusolverDnCreateGesvdjInfo(&prm));
    GQ_SOLVER(cusolverDnXgesvdjSetSortEig(prm, 1));
    int lwork = 0;
    for (Group *g : groups) {
      int lw = 0;
      // X = Theta^T (n x m col-major); X = Ux S Vx^T -> left vectors of
      // Theta are Vx (m x p), right vectors are Ux (n x p).
      GQ_SOLVER(cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)g->n, (int)g->m,
                                             mats.p + g->mat_off, (int)g->n, sv.p + g->s_off,
                                             rv.p + g->rv_off, (int)g->n, lv.p + g->lv_off,
                                             (int)g->m, &lw, prm));
      lwork = std::max(lwork, lw);
    }
    DevBuf work((int64_t)lwork + 1);
    DevArray<int> infos;
    infos.upload(std::vector<int>(groups.size(), 0));
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      Group *g = groups[gi];
      GQ_SOLVER(cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)g->n, (int)g->m,
                                  mats.p + g->mat_off, (int)g->n, sv.p + g->s_off,
                                  rv.p + g->rv_off, (int)g->n, lv.p + g->lv_off, (int)g->m, work.p,
                                  lwork, infos.p + gi, prm));
    }
    std::vector<int> hinfo(groups.size());
    GQ_CUDA(cudaMemcpyAsync(hinfo.data(), infos.p, sizeof(int) * groups.size(),
                            cudaMemcpyDeviceToHost, s));
    sync();
    cusolverDnDestroyGesvdjInfo(prm);
    for (int v : hinfo)
      if (v != 0) fail(kSolverError, "gesvdj did not converge, info=" + std::to_string(v));
  }

  // ---- global truncation on the host (s_total values) --------------------
  std::vector<double> flat(s_total);
  GQ_CUDA(cudaMemcpyAsync(flat.data(), sv.p, sizeof(double) * s_total, cudaMemcpyDeviceToHost, s));
  sync();
  double smax = 0.0;
  for (double v : flat) smax = std::max(smax, v);
  for (double &v : flat)
    if (!(v > kZeroSvRtol * smax)) v = 0.0;
  const int64_t ntot = s_total;
  std::vector<int64_t> order(ntot);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t x, int64_t y) { return flat[x] > flat[y]; });
  int64_t D;
  double err = 0.0;
  if (ntot == 0 || flat[order[0]] <= 0.0) {
    D = std::min<int64_t>(ntot, std::max<int64_t>(1, std::min(dmin, dmax)));
  } else {
    std::vector<double> tail(ntot + 1, 0.0);
    for (int64_t i = ntot - 1; i >= 0; --i) tail[i] = tail[i + 1] + flat[order[i]] * flat[order[i]];
    const double total = tail[0];
    const int64_t dcap = std::min(dmax, ntot);
    D = dcap;
    const int64_t lo = std::max<int64_t>(1, std::min(dmin, dcap));
    for (int64_t d = lo; d <= dcap; ++d)
      if (tail[d] / total <= trunc_err) {
        D = d;
        break;
      }
    err = tail[D] / total;
  }
  std::vector<char> keep(ntot, 0);
  for (int64_t i = 0; i < D; ++i) keep[order[i]] = 1;

  SvdOut out;
  out.D = D;
  out.trunc_err = err;
  std::vector<double> s_kept;        // per kept column, bond order
  std::vector<std::pair<QN, int64_t>> sectors;
  int64_t lc_total = 0, rc_total = 0;
  for (Group *g : groups) {
    for (int64_t j = 0; j < g->p; ++j) {
      const int64_t f = g->s_off + j;
      if (flat[f] > 0.0) g->nnz++;
      if (keep[f]) {
        g->keep++;
        if (flat[f] > 0.0) g->keep_nz++;
      }
    }
    if (g->keep == 0) continue;
    g->sector = (int)sectors.size();
    sectors.push_back({g->q, g->keep});
    const int64_t kz = g->keep - g->keep_nz;
    g->lc_off = lc_total;
    lc_total += g->m * kz;
    g->rc_off = rc_total;
    rc_total += g->n * kz;
  }
  GQ_CHECK(!sectors.empty(), "SVD kept no singular value");

  // ---- sign convention on kept nonzero vectors ----------------------------
  {
    std::vector<SignItem> items;
    for (Group *g : groups)
      for (int64_t j = 0; j < g->keep_nz; ++j)
        items.push_back({g->lv_off + j * g->m, g->rv_off + j * g->n, (int)g->m, (int)g->n});
    if (!items.empty()) {
      DevArray<SignItem> d;
      d.upload(items);
      sign_fix_kernel<<<(unsigned)items.size(), 256, 0, s>>>(d.p, lv.p, rv.p);
      GQ_CUDA(cudaGetLastError());
    }
  }
  // ---- canonical completion for kept zeros ---------------------------------
  DevBuf lcomp(lc_total), rcomp(rc_total);
  for (Group *g : groups) {
    const int64_t kz = g->keep - g->keep_nz;
    if (kz == 0) continue;
    const int gidx = (int)(std::find(groups.begin(), groups.end(), g) - groups.begin());
    null_completion(lv.p + g->lv_off, g->m, g->nnz, kz, gidx, 0, lcomp.p + g->lc_off);
    null_completion(rv.p + g->rv_off, g->n, g->nnz, kz, gidx, 1, rcomp.p + g->rc_off);
  }

  // ---- output tensors --------------------------------------------------------
  Index nb;
  nb.dir = 1;
  for (auto &sq : sectors) {
    nb.qn.push_back(sq.first);
    nb.dim.push_back(sq.second);
  }
  out.new_bond = nb;
  std::vector<Index> uidx(t.idx.begin(), t.idx.begin() + ldims);
  uidx.push_back(nb);
  std::vector<Index> vidx;
  vidx.push_back(nb.inverse());
  vidx.insert(vidx.end(), t.idx.begin() + ldims, t.idx.end());
  std::vector<std::vector<int>> ublocks, vblocks;
  for (Group *g : groups) {
    if (g->keep == 0) continue;
    for (auto &rc : g->rows) {
      auto c = rc;
      c.push_back(g->sector);
      ublocks.push_back(c);
    }
    for (auto &cc : g->cols) {
      std::vector<int> c{g->sector};
      c.insert(c.end(), cc.begin(), cc.end());
      vblocks.push_back(c);
    }
  }
  out.u = make_structure(t.nq, uidx, ldiv, ublocks);
  out.vt = make_structure(t.nq, vidx, t.div - ldiv, vblocks);
  out.u->allocate();
  out.vt->allocate();

  // kept singular values per group (device) for the optional scaling
  std::vector<double> kept_s;
  std::vector<int64_t> ks_off(groups.size(), 0);
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    Group *g = groups[gi];
    ks_off[gi] = (int64_t)kept_s.size();
    for (int64_t j = 0; j < g->keep; ++j) {
      const double v = j < g->keep_nz ? flat[g->s_off + j] : 0.0;
      kept_s.push_back(v);
      out.s.push_back(v);
    }
  }
  DevArray<double> ks;
  ks.upload(kept_s.empty() ? std::vector<double>{0.0} : kept_s);
  {
    std::vector<ScatterItem> items;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      Group *g = groups[gi];
      if (g->keep == 0) continue;
      for (size_t ri = 0; ri < g->rows.size(); ++ri) {
        auto c = g->rows[ri];
        c.push_back(g->sector);
        const int64_t ob = out.u->find(c.data());
        ScatterItem it{};
        it.dst_off = out.u->offs[ob];
        it.rows = (int)g->rsz[ri];
        it.k = (int)g->keep;
        it.knz = (int)g->keep_nz;
        it.mode = 0;
        it.scale = scale_side == 1;
        it.svd_off = g->lv_off + g->roff[ri];
        it.ld_svd = (int)g->m;
        it.comp_off = g->lc_off + g->roff[ri];
        it.ld_comp = (int)g->m;
        it.s_off = ks_off[gi];
        items.push_back(it);
      }
      for (size_t ci = 0; ci < g->cols.size(); ++ci) {
        std::vector<int> c{g->sector};
        c.insert(c.end(), g->cols[ci].begin(), g->cols[ci].end());
        const int64_t ob = out.vt->find(c.data());
        ScatterItem it{};
        it.dst_off = out.vt->offs[ob];
        it.rows = (int)g->csz[ci];
        it.k = (int)g->keep;
        it.knz = (int)g->keep_nz;
        it.mode = 1;
        it.scale = scale_side == 2;
        it.svd_off = g->rv_off + g->coff[ci];
        it.ld_svd = (int)g->n;
        it.comp_off = g->rc_off + g->coff[ci];
        it.ld_comp = (int)g->n;
        it.s_off = ks_off[gi];
        items.push_back(it);
      }
    }
    DevArray<ScatterItem> d;
    d.upload(items);
    scatter_kernel<<<(unsigned)items.size(), 256, 0, s>>>(d.p, lv.p, rv.p, lcomp.p, rcomp.p, ks.p,
                                                         out.u->data.p, out.vt->data.p);
    GQ_CUDA(cudaGetLastError());
  }
  return out;
}

}  // namespace gq
