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
//  * each group has min(m, n) singular values; values <= 1e-13 * s_max
//    (global) are exact zeros;
//  * global selection: rank all values (ties: earlier group, earlier
//    position); D = smallest count in [Dmin, Dmax] whose discarded weight
//    sum_{i>=D} s_i^2 / sum s^2 <= trunc_err, capped by Dmax and #values;
//  * kept nonzero values: the largest-|.| entry of each left vector is made
//    positive (the right vector follows); kept zero values use the
//    canonical completion of null_completion (the unit vectors the group's
//    nonzero singular vectors leave, carried through the Householder
//    reflectors of their QR) -- except on a Gram group solved in full,
//    where the eigenvectors of the below-floor eigenvalues serve (see
//    below);
//  * new bond sectors: groups with a kept value, ascending charge.
//
// Decomposition routes (all FP64):
//  * groups with m, n <= 32: one-sided Jacobi SVD, one CTA per group
//    (small_svd_kernel);
//  * larger groups inside a sweep update: only the factor that becomes the
//    canonical MPS tensor has to be orthonormal, so it is taken from the
//    eigenvectors of the Gram matrix on that side and the other factor comes
//    by projection without dividing by singular values -- 'r' updates: U
//    from Theta Theta^T and S.Vt = U^T Theta; 'l' updates: V from
//    Theta^T Theta and U.S = Theta V.  The Gram matrix first goes through a
//    rank-revealing reduction (pivoted Cholesky with Gram-Schmidt
//    re-orthogonalised columns, pcmgs.cu): a converged state's Gram matrices
//    have a numerical rank far below their dimension, and their eigenpairs
//    above the floor are those of the small matrix T T^T in the basis Q.  A
//    group whose rank exceeds its cap (about 0.3 of the Gram dimension)
//    solves its full Gram matrix instead.  The eigensolves run in size
//    buckets with one batched call per bucket.  On these groups eigenvalues
//    below 1e-14 of the group's largest are the noise floor of the Gram
//    matrix and count as exact zeros (singular values below ~1e-7 of the
//    group's largest);
//  * larger groups of a plain SVD (both factors orthonormal): Jacobi SVD.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <map>
#include <numeric>

#include "gq_runtime.hpp"

namespace gq {

namespace {
constexpr double kZeroSvRtol = 1e-13;
constexpr double kGramZeroRtol = 1e-14;
constexpr int kSmall = 32;
// Rank-revealing reduction of the Gram matrices: stop when the largest
// remaining diagonal entry is 1e-15 of the largest diagonal entry (a decade
// below the eigenvalue floor kGramZeroRtol); Gram matrices of at most 512
// rows run on 4-CTA clusters, larger ones on 16-CTA clusters.
constexpr double kPcTol = 1e-15;
constexpr int64_t kPcSmallRows = 512;
// Eigensolve buckets holding one matrix of at least this size use the
// divide-and-conquer solver instead of the batched one.
constexpr int64_t kSyevdMinRows = 320;

enum Route { kSmallJacobi = 0, kJacobi = 1, kGramLeft = 2, kGramRight = 3 };

#define GQ_SOLVER(call)                                                               \
  do {                                                                                \
    cusolverStatus_t s_ = (call);                                                     \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                                \
      ::gq::fail(::gq::kSolverError, std::string(#call) + " failed with status " +    \
                                         std::to_string((int)s_));                    \
  } while (0)

#define GQ_BLAS(call)                                                                 \
  do {                                                                                \
    cublasStatus_t s_ = (call);                                                       \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                  \
      ::gq::fail(::gq::kSolverError, std::string(#call) + " failed with status " +    \
                                         std::to_string((int)s_));                    \
  } while (0)

// Library handles of this thread's lane, bound to the lane's stream.
cusolverDnHandle_t solver() {
  auto &l = lane();
  if (!l.cusolver) {
    cusolverDnHandle_t h;
    GQ_SOLVER(cusolverDnCreate(&h));
    GQ_SOLVER(cusolverDnSetStream(h, l.stream));
    l.cusolver = h;
  }
  return (cusolverDnHandle_t)l.cusolver;
}

// cuSOLVER handle on the lane's auxiliary stream i.
cusolverDnHandle_t aux_solver(int i) {
  auto &l = lane();
  init_aux(l);
  if (!l.aux_cusolver[i]) {
    cusolverDnHandle_t h;
    GQ_SOLVER(cusolverDnCreate(&h));
    GQ_SOLVER(cusolverDnSetStream(h, l.aux_stream[i]));
    l.aux_cusolver[i] = h;
  }
  return (cusolverDnHandle_t)l.aux_cusolver[i];
}

cublasHandle_t blas() {
  auto &l = lane();
  if (!l.cublas) {
    cublasHandle_t h;
    GQ_BLAS(cublasCreate(&h));
    GQ_BLAS(cublasSetStream(h, l.stream));
    l.cublas = h;
  }
  return (cublasHandle_t)l.cublas;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// Elements [e0, e1) of one block per CTA (blocks are cut into chunks of at
// most kCopyChunk elements, so one large block does not serialise a launch).
constexpr int64_t kCopyChunk = 16384;
struct GatherItem { int64_t src_off, dst_off, e0, e1; int rows, cols, ld; };

__global__ void gather_kernel(const GatherItem *__restrict__ items, const double *__restrict__ src,
                              double *__restrict__ dst) {
  const GatherItem it = items[blockIdx.x];
  for (int64_t e = it.e0 + threadIdx.x; e < it.e1; e += blockDim.x) {
    const int64_t i = e / it.cols, j = e % it.cols;
    dst[it.dst_off + i * it.ld + j] = src[it.src_off + e];
  }
}

// A group matrix X (col-major n x m, ld n) into a zero-padded 32 x 32 slot.
struct PadItem { int64_t src_off, dst_off; int n, m; };

__global__ void pad_small_kernel(const PadItem *__restrict__ items, const double *__restrict__ src,
                                 double *__restrict__ dst) {
  const PadItem it = items[blockIdx.x];
  for (int e = threadIdx.x; e < kSmall * kSmall; e += blockDim.x) {
    const int r = e % kSmall, c = e / kSmall;
    dst[it.dst_off + e] = (r < it.n && c < it.m) ? src[it.src_off + r + (int64_t)c * it.n] : 0.0;
  }
}

// One-sided (Hestenes) Jacobi SVD of every 32 x 32 slot X (column-major),
// one CTA per slot: the columns are rotated in pairs -- 16 disjoint pairs
// per round in round-robin order, one warp per pair, a lane per row --
// until a sweep rotates no pair (|x_p . x_q| <= 1e-15 |x_p| |x_q| for every
// pair, or one of the two columns below 1e-15 of |X|_F: rounding noise left
// by a rank-deficient X, which would otherwise keep rotating) or after
// kSmallSweeps sweeps.  Then X V = W has orthogonal columns:
// sigma_j = |w_j| and u_j = w_j / sigma_j (zero where sigma_j = 0).  Output
// in the layout of the batched library solve it replaces: sigma descending
// (ties: lower column first), U and V column-major 32 x 32.
constexpr int kSmallSweeps = 60;
constexpr double kSmallJacobiTol = 1e-15;

__device__ __forceinline__ double warp_sum_all(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Column at position j of round `round` of the round-robin pairing of nc
// columns (nc even; position 0 fixed, the other nc - 1 rotating).
__device__ __forceinline__ int rr_column(int j, int round, int nc) {
  return j == 0 ? 0 : (j - 1 + round) % (nc - 1) + 1;
}

__global__ void __launch_bounds__(256)
    small_svd_kernel(const double *__restrict__ X, const int *__restrict__ ncols,
                     double *__restrict__ U, double *__restrict__ V, double *__restrict__ S) {
  __shared__ double w[kSmall][kSmall + 1];  // w[column][row]
  __shared__ double v[kSmall][kSmall + 1];
  __shared__ double sig[kSmall];
  __shared__ int perm[kSmall];
  __shared__ int rot[2];
  __shared__ double negligible;
  const int64_t base = (int64_t)blockIdx.x * kSmall * kSmall;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int e = threadIdx.x; e < kSmall * kSmall; e += blockDim.x) {
    const int r = e % kSmall, c = e / kSmall;
    w[c][r] = X[base + e];
    v[c][r] = r == c ? 1.0 : 0.0;
  }
  if (threadIdx.x == 0) rot[0] = rot[1] = 0;
  __syncthreads();
  for (int c = warp; c < kSmall; c += nwarps) {
    const double x = w[c][lane];
    const double n2 = warp_sum_all(x * x);
    if (lane == 0) sig[c] = n2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double f2 = 0.0;
    for (int c = 0; c < kSmall; ++c) f2 += sig[c];
    negligible = 1e-30 * f2;  // (1e-15 |X|_F)^2
  }
  __syncthreads();
  const double neg = negligible;
  // only the slot's own columns take part (the padding columns are zero)
  const int nc = min(kSmall, max(2, (ncols[blockIdx.x] + 1) & ~1));
  for (int sweep = 0; sweep < kSmallSweeps; ++sweep) {
    int mine = 0;
    for (int round = 0; round < nc - 1; ++round) {
      for (int pi = warp; pi < nc / 2; pi += nwarps) {
        const int p = rr_column(pi, round, nc), q = rr_column(nc - 1 - pi, round, nc);
        const double a = w[p][lane], b = w[q][lane];
        const double alpha = warp_sum_all(a * a), beta = warp_sum_all(b * b);
        const double gamma = warp_sum_all(a * b);
        if (gamma != 0.0 && fabs(gamma) > kSmallJacobiTol * sqrt(alpha * beta) &&
            fmin(alpha, beta) > neg) {
          const double zeta = (beta - alpha) / (2.0 * gamma);
          const double t = fabs(zeta) > 1e150
                               ? 0.5 / zeta
                               : (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
          w[p][lane] = c * a - sn * b;
          w[q][lane] = sn * a + c * b;
          const double vp = v[p][lane], vq = v[q][lane];
          v[p][lane] = c * vp - sn * vq;
          v[q][lane] = sn * vp + c * vq;
          mine = 1;
        }
      }
      __syncthreads();
    }
    if (mine && lane == 0) atomicOr(&rot[sweep & 1], 1);
    __syncthreads();
    const int any = rot[sweep & 1];
    if (threadIdx.x == 0) rot[(sweep + 1) & 1] = 0;
    if (!any) break;
  }
  for (int c = warp; c < kSmall; c += nwarps) {
    const double x = w[c][lane];
    const double n2 = warp_sum_all(x * x);
    if (lane == 0) sig[c] = sqrt(n2);
  }
  __syncthreads();
  if (threadIdx.x < kSmall) {
    const int c = threadIdx.x;
    int rank = 0;
    for (int j = 0; j < kSmall; ++j)
      if (sig[j] > sig[c] || (sig[j] == sig[c] && j < c)) ++rank;
    perm[rank] = c;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kSmall * kSmall; e += blockDim.x) {
    const int r = e % kSmall, j = e / kSmall;
    const int c = perm[j];
    const double sc = sig[c];
    U[base + e] = sc > 0.0 ? w[c][r] / sc : 0.0;
    V[base + e] = v[c][r];
  }
  if (threadIdx.x < kSmall) S[(int64_t)blockIdx.x * kSmall + threadIdx.x] = sig[perm[threadIdx.x]];
}

// Gram slot set-up: outside the leading dim x dim block, -1 on the diagonal
// and 0 elsewhere (the leading block is written by the Gram GEMM).
struct PadDiagItem { int64_t off; int bs, dim; };

__global__ void pad_diag_kernel(const PadDiagItem *__restrict__ items, double *__restrict__ buf) {
  const PadDiagItem it = items[blockIdx.x];
  const int64_t n = (int64_t)it.bs * it.bs;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = (int)(e % it.bs), c = (int)(e / it.bs);
    if (r >= it.dim || c >= it.dim) buf[it.off + e] = (r == c) ? -1.0 : 0.0;
  }
}

// A symmetric n x n matrix (leading dimension ld_src) into the top-left of
// an eigensolve slot (leading dimension ld_dst).
struct SlotItem { int64_t src_off, dst_off; int n, ld_src, ld_dst; };

__global__ void slot_copy_kernel(const SlotItem *__restrict__ items, const double *__restrict__ src,
                                 double *__restrict__ dst) {
  const SlotItem it = items[blockIdx.x];
  const int64_t nn = (int64_t)it.n * it.n;
  for (int64_t e = threadIdx.x; e < nn; e += blockDim.x) {
    const int64_t r = e % it.n, c = e / it.n;
    dst[it.dst_off + r + c * it.ld_dst] = src[it.src_off + r + c * it.ld_src];
  }
}

// Column copies: dst[:, dcol] = src[:, scol] * scale over `rows` rows.
struct ColItem { int64_t src_off, dst_off; int rows, ld_src, ld_dst, scol, dcol; double scale; };

__global__ void col_copy_kernel(const ColItem *__restrict__ items, const double *__restrict__ src,
                                double *__restrict__ dst) {
  const ColItem it = items[blockIdx.x];
  const double *s = src + it.src_off + (int64_t)it.scol * it.ld_src;
  double *d = dst + it.dst_off + (int64_t)it.dcol * it.ld_dst;
  for (int r = threadIdx.x; r < it.rows; r += blockDim.x) d[r] = s[r] * it.scale;
}

// Sign convention: column of `u` (m entries): make the first entry of
// largest magnitude positive; flip the matching column of `v` (n entries)
// alongside.
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

// Output blocks.  mode 0: U block (rows x k, row-major), element (i, j) =
// L[r0 + i, j]; mode 1: Vt block (k x rows), element (j, i) = R[r0 + i, j];
// L and R are the group's col-major factors (ld = group m or n).
struct ScatterItem { int64_t dst_off, src_off, e0, e1; int rows, k, ld, mode; };

__global__ void scatter_kernel(const ScatterItem *__restrict__ items, const double *__restrict__ L,
                               const double *__restrict__ R, double *__restrict__ U,
                               double *__restrict__ Vt) {
  const ScatterItem it = items[blockIdx.x];
  const double *src = it.mode == 0 ? L : R;
  double *dst = it.mode == 0 ? U : Vt;
  for (int64_t e = it.e0 + threadIdx.x; e < it.e1; e += blockDim.x) {
    int i, j;
    if (it.mode == 0) { i = (int)(e / it.k); j = (int)(e % it.k); }
    else { j = (int)(e / it.rows); i = (int)(e % it.rows); }
    dst[it.dst_off + e] = src[it.src_off + i + (int64_t)j * it.ld];
  }
}

// Shifted identity: w (dim x k, col-major) = columns r .. r+k-1 of the
// dim x dim identity (the unit vectors the completion starts from).
__global__ void shifted_identity_kernel(double *__restrict__ w, int dim, int k, int r) {
  const int64_t n = (int64_t)dim * k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % dim, j = e / dim;
    w[e] = (i == r + j) ? 1.0 : 0.0;
  }
}

// dst = src with every zero written as +0.0.  A Householder reflector's
// sign follows the sign of its pivot, and LAPACK reads the sign bit of an
// exact zero pivot where the device QR takes it as positive: with signed
// zeros removed the two agree.
__global__ void plus_zero_copy_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                      int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = src[e];
    dst[e] = v == 0.0 ? 0.0 : v;
  }
}

template <typename T>
void launch_items(void (*kern)(const T *, const double *, double *), const std::vector<T> &items,
                  const double *src, double *dst) {
  if (items.empty()) return;
  DevArray<T> d;
  d.upload(items);
  kern<<<(unsigned)items.size(), 256, 0, stream()>>>(d.p, src, dst);
  GQ_CUDA(cudaGetLastError());
}

// Dense FP64 products of the large groups on the FP64-accurate tensor-core
// path: A (a0 x a1) and B (b0 x b1) row-major, contracted over A's axis
// `axa` and B's axis `axb`; C (the two free dimensions, A's first) written
// row-major.  Each operand is a one-block two-leg tensor (trivial charges)
// and goes through the block contraction engine; below ~1e8 flops cuBLAS
// is used instead (kTcMinFlops).
constexpr double kTcMinFlops = 1e8;

TensorPtr dense_tensor(const double *src, int64_t d0, int64_t d1, int dir0, int dir1) {
  Index i0, i1;
  i0.dir = dir0;
  i0.qn = {QN()};
  i0.dim = {d0};
  i1.dir = dir1;
  i1.qn = {QN()};
  i1.dim = {d1};
  auto t = make_structure(1, {i0, i1}, QN(), {{0, 0}});
  t->allocate();
  GQ_CUDA(cudaMemcpyAsync(t->data.p, src, sizeof(double) * d0 * d1, cudaMemcpyDeviceToDevice,
                          stream()));
  return t;
}

// C = contraction of A's axis axa with B's axis axb; the contracted pair
// is given opposite directions, every block is charge-allowed.
void dense_contract_tc(const double *A, int64_t a0, int64_t a1, int axa, const double *B,
                       int64_t b0, int64_t b1, int axb, double *C) {
  auto ta = dense_tensor(A, a0, a1, axa == 0 ? -1 : 1, axa == 1 ? -1 : 1);
  auto tb = dense_tensor(B, b0, b1, axb == 0 ? 1 : -1, axb == 1 ? 1 : -1);
  auto tc = contract(*ta, *tb, {axa}, {axb}, kFP64TC);
  GQ_CUDA(cudaMemcpyAsync(C, tc->data.p, sizeof(double) * tc->size(), cudaMemcpyDeviceToDevice,
                          stream()));
}

// Independent FP64 GEMMs gathered into one grouped batched cuBLAS call
// (each product its own group of one): the per-group products of the block
// SVD are many and mostly small, and one call replaces a library launch
// sequence per group.
struct GemmBatch {
  std::vector<cublasOperation_t> ta, tb;
  std::vector<int> m, n, k, lda, ldb, ldc, size;
  std::vector<double> alpha, beta;
  std::vector<const double *> A, B;
  std::vector<double *> C;
  void add(cublasOperation_t a_op, cublasOperation_t b_op, int m_, int n_, int k_,
           const double *A_, int lda_, const double *B_, int ldb_, double *C_, int ldc_) {
    ta.push_back(a_op);
    tb.push_back(b_op);
    m.push_back(m_);
    n.push_back(n_);
    k.push_back(k_);
    A.push_back(A_);
    lda.push_back(lda_);
    B.push_back(B_);
    ldb.push_back(ldb_);
    C.push_back(C_);
    ldc.push_back(ldc_);
    alpha.push_back(1.0);
    beta.push_back(0.0);
    size.push_back(1);
  }
  void run(cublasHandle_t h) {
    if (A.empty()) return;
    DevArray<const double *> dA, dB;
    DevArray<double *> dC;
    dA.upload(A);
    dB.upload(B);
    dC.upload(C);
    GQ_BLAS(cublasDgemmGroupedBatched(h, ta.data(), tb.data(), m.data(), n.data(), k.data(),
                                      alpha.data(), dA.p, lda.data(), dB.p, ldb.data(),
                                      beta.data(), dC.p, ldc.data(), (int)A.size(),
                                      size.data()));
  }
};

// Canonical completion: k orthonormal columns orthogonal to the r
// orthonormal columns of `vecs` (dim x r, col-major, ld dim), written to
// out (dim x k, col-major, ld dim): columns r .. r+k-1 of the orthogonal
// factor of the complete Householder QR of `vecs` -- the unit vectors
// e_r .. e_{r+k-1} carried through its r reflectors (geqrf, then ormqr on
// the shifted identity; LAPACK's reflector conventions, as the oracle's
// numpy QR, on the vectors with signed zeros made +0.0).  O(dim r (r + k))
// work, exactly orthonormal whatever the overlap of the unit vectors with
// `vecs`.  In two steps: prepare (on the lane's stream: the shifted
// identity, the QR input, the workspace) and factor (geqrf + ormqr with the
// given handle, so that the completions of one SVD can run side by side on
// the lane's auxiliary streams).  The status words of the two calls go to
// info[0..1] (checked later by the caller).
struct Completion {
  DevBuf q;              // the r input vectors (dim x r)
  DevBuf a, tau, work;   // QR input and factors, workspace
  int64_t dim = 0, r = 0, k = 0;
  int lw = 0;
  double *out = nullptr;
  int *info = nullptr;
};

void completion_prepare(Completion &c) {
  if (c.k == 0) return;
  auto s = stream();
  const unsigned grid = (unsigned)std::min<int64_t>((c.dim * c.k + 255) / 256, 4096);
  shifted_identity_kernel<<<grid, 256, 0, s>>>(c.out, (int)c.dim, (int)c.k, (int)c.r);
  GQ_CUDA(cudaGetLastError());
  if (c.r == 0) return;
  auto sh = solver();
  const int d = (int)c.dim, kk = (int)c.k, rr = (int)c.r;
  c.a.alloc(c.dim * c.r);
  c.tau.alloc(c.r);
  plus_zero_copy_kernel<<<(unsigned)std::min<int64_t>((c.dim * c.r + 255) / 256, 4096), 256, 0,
                          s>>>(c.q.p, c.a.p, c.dim * c.r);
  GQ_CUDA(cudaGetLastError());
  int lw1 = 0, lw2 = 0;
  GQ_SOLVER(cusolverDnDgeqrf_bufferSize(sh, d, rr, c.a.p, d, &lw1));
  GQ_SOLVER(cusolverDnDormqr_bufferSize(sh, CUBLAS_SIDE_LEFT, CUBLAS_OP_N, d, kk, rr, c.a.p, d,
                                        c.tau.p, c.out, d, &lw2));
  c.lw = std::max(lw1, lw2);
  c.work.alloc((int64_t)c.lw + 1);
}

void completion_factor(Completion &c, cusolverDnHandle_t sh) {
  if (c.k == 0 || c.r == 0) return;
  const int d = (int)c.dim, kk = (int)c.k, rr = (int)c.r;
  GQ_SOLVER(cusolverDnDgeqrf(sh, d, rr, c.a.p, d, c.tau.p, c.work.p, c.lw, c.info));
  GQ_SOLVER(cusolverDnDormqr(sh, CUBLAS_SIDE_LEFT, CUBLAS_OP_N, d, kk, rr, c.a.p, d, c.tau.p,
                             c.out, d, c.work.p, c.lw, c.info + 1));
}

struct Group {
  QN q;
  std::vector<std::vector<int>> rows, cols;
  std::vector<int64_t> rsz, csz, roff, coff;
  int64_t m = 0, n = 0, p = 0;
  Route route = kJacobi;
  int64_t mat_off = 0;            // row-major m x n (= col-major X, n x m, ld n)
  int64_t lv_off = 0, rv_off = 0; // left (m rows) / right (n rows) singular vectors
  int ld_l = 0, ld_r = 0;
  int64_t sv_off = 0;             // singular values (small: 32 per group, jacobi: p)
  int64_t ev_off = 0, w_off = 0;  // gram: eigenvectors (dim x dim) and eigenvalues
  int64_t dim = 0;
  bool eig_m = true;              // gram: eigensolve on Theta Theta^T (else Theta^T Theta)
  // Gram groups: the Gram matrix (gn x gn) at g_off; rank-revealing
  // reduction (pcmgs.cu) with rank cap rcap: Q at q_off, T T^T at t_off;
  // pc: the eigensolve ran on T T^T (rank r), eigenvectors Q Z at u_off
  int64_t gn = 0, g_off = 0, q_off = 0, t_off = 0, u_off = 0;
  int rcap = 0, r = -1;
  bool pc = false;
  int64_t small_idx = -1;
  std::vector<double> svals;      // p values, descending
  std::vector<int> src_cols;      // source column of each value
  int64_t nnz = 0, keep = 0, keep_nz = 0;
  int sector = -1;
  int64_t L_off = 0, R_off = 0;   // outputs: L (m x keep), R (n x keep)
};
}  // namespace

void destroy_lane_handles(Lane &l) {
  if (l.cusolver) cusolverDnDestroy((cusolverDnHandle_t)l.cusolver);
  if (l.cublas) cublasDestroy((cublasHandle_t)l.cublas);
  l.cusolver = l.cublas = nullptr;
  for (auto &a : l.aux_cusolver) {
    if (a) cusolverDnDestroy((cusolverDnHandle_t)a);
    a = nullptr;
  }
}

SvdOut svd_truncate(const Tensor &t_in, int ldims, const QN &ldiv, double trunc_err,
                    int64_t dmin, int64_t dmax, int scale_side) {
  prof_begin(kProfSvd);
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
  int64_t mat_total = 0, n_small = 0;
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
    if (g.m <= kSmall && g.n <= kSmall) {
      g.route = kSmallJacobi;
      g.small_idx = n_small++;
    } else if (scale_side == 2) {
      g.route = kGramLeft;
      g.eig_m = true;
    } else if (scale_side == 1) {
      g.route = kGramRight;
      g.eig_m = false;
    } else {
      g.route = kJacobi;
    }
    groups.push_back(&g);
  }
  GQ_CHECK(!groups.empty(), "SVD of a tensor without blocks");

  // ---- gather each group into a dense row-major m x n matrix --------------
  prof_begin(kProfSvdGather);
  DevBuf mats(mat_total);
  GQ_CUDA(cudaMemsetAsync(mats.p, 0, sizeof(double) * mat_total, s));
  {
    std::vector<GatherItem> items;
    for (auto &br : brefs) {
      Group &g = gmap[br.q];
      const int64_t ri = std::lower_bound(g.rows.begin(), g.rows.end(), br.rc) - g.rows.begin();
      const int64_t ci = std::lower_bound(g.cols.begin(), g.cols.end(), br.cc) - g.cols.begin();
      const int64_t n = g.rsz[ri] * g.csz[ci];
      for (int64_t e0 = 0; e0 < n; e0 += kCopyChunk)
        items.push_back({t.offs[br.b], g.mat_off + g.roff[ri] * g.n + g.coff[ci], e0,
                         std::min(n, e0 + kCopyChunk), (int)g.rsz[ri], (int)g.csz[ci],
                         (int)g.n});
    }
    launch_items(gather_kernel, items, t.data.p, mats.p);
  }
  prof_end(kProfSvdGather, 0.0, 0.0);

  // ---- decompositions -----------------------------------------------------
  prof_begin(kProfSvdEig);
  auto h = solver();
  auto bh = blas();
  struct JacobiInfo {  // released on every exit path
    gesvdjInfo_t p = nullptr;
    ~JacobiInfo() {
      if (p) cusolverDnDestroyGesvdjInfo(p);
    }
  } jinfo_guard;
  GQ_SOLVER(cusolverDnCreateGesvdjInfo(&jinfo_guard.p));
  gesvdjInfo_t prm = jinfo_guard.p;
  // small groups: one-sided Jacobi SVD on zero-padded 32 x 32 slots of X
  const int64_t slot = kSmall * kSmall;
  DevBuf sbatch(n_small * slot), su(n_small * slot), sv(n_small * slot), ss(n_small * kSmall);
  if (n_small > 0) {
    std::vector<PadItem> items;
    for (Group *g : groups)
      if (g->route == kSmallJacobi)
        items.push_back({g->mat_off, g->small_idx * slot, (int)g->n, (int)g->m});
    launch_items(pad_small_kernel, items, mats.p, sbatch.p);
    std::vector<int> cols(n_small, 0);
    for (Group *g : groups)
      if (g->route == kSmallJacobi) cols[g->small_idx] = (int)g->m;  // columns of X = Theta^T
    DevArray<int> dcols;
    dcols.upload(cols);
    small_svd_kernel<<<(unsigned)n_small, 256, 0, s>>>(sbatch.p, dcols.p, su.p, sv.p, ss.p);
    GQ_CUDA(cudaGetLastError());
    // X = Ux S Vx^T with X = Theta^T: Theta's left vectors are Vx (sv),
    // its right vectors Ux (su)
    for (Group *g : groups)
      if (g->route == kSmallJacobi) {
        g->lv_off = g->rv_off = g->small_idx * slot;
        g->ld_l = g->ld_r = kSmall;
        g->sv_off = g->small_idx * kSmall;
      }
  }
  // larger groups of a plain SVD: Jacobi SVD each (sorted)
  int64_t jl_total = 0, jr_total = 0, js_total = 0;
  for (Group *g : groups)
    if (g->route == kJacobi) {
      g->lv_off = jl_total;
      jl_total += g->m * g->p;
      g->rv_off = jr_total;
      jr_total += g->n * g->p;
      g->sv_off = js_total;
      js_total += g->p;
      g->ld_l = (int)g->m;
      g->ld_r = (int)g->n;
    }
  DevBuf jl(jl_total), jr(jr_total), js(js_total);
  DevArray<int> jinfo;
  if (js_total > 0) {
    GQ_SOLVER(cusolverDnXgesvdjSetSortEig(prm, 1));
    int lwork = 0;
    for (Group *g : groups) {
      if (g->route != kJacobi) continue;
      int lw = 0;
      GQ_SOLVER(cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)g->n, (int)g->m,
                                             mats.p + g->mat_off, (int)g->n, js.p + g->sv_off,
                                             jr.p + g->rv_off, (int)g->n, jl.p + g->lv_off,
                                             (int)g->m, &lw, prm));
      lwork = std::max(lwork, lw);
    }
    DevBuf work((int64_t)lwork + 1);
    jinfo.upload(std::vector<int>(groups.size(), 0));
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      Group *g = groups[gi];
      if (g->route != kJacobi) continue;
      GQ_SOLVER(cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)g->n, (int)g->m,
                                  mats.p + g->mat_off, (int)g->n, js.p + g->sv_off,
                                  jr.p + g->rv_off, (int)g->n, jl.p + g->lv_off, (int)g->m, work.p,
                                  lwork, jinfo.p + gi, prm));
    }
  }
  // Gram groups.  Each group's canonical-side Gram matrix G (gn x gn,
  // eigenvalues in [0, |Theta|^2]) is formed first; the rank-revealing
  // reduction (pcmgs.cu) then finds its numerical range Q (gn x r) with
  // Q^T G Q ~ T T^T.  A group whose rank stays within its cap solves the
  // r x r matrix T T^T (eigenvectors Q Z); the others solve G itself.
  // Either matrix goes into a slot padded to a bucket size with -1 on the
  // extra diagonal, so the padding's eigenpairs sort below the real ones and
  // stay in the padded coordinates; one batched eigensolve per bucket.
  // Bucket sizes: multiples of 32 up to 256, of 64 above (the padding of a
  // matrix to its bucket costs up to (bucket / size)^3 in work: measured
  // over a D=4000 run, one bucket for all of 65..256 padded to the largest
  // of them took 7.5 of 24 s of eigensolves).
  std::vector<Group *> gram;
  int64_t gbuf_total = 0, q_total = 0, t_total = 0;
  for (Group *g : groups)
    if (g->route == kGramLeft || g->route == kGramRight) {
      g->gn = g->eig_m ? g->m : g->n;
      g->g_off = gbuf_total;
      gbuf_total += g->gn * g->gn;
      if (g->gn <= pcmgs_max_rows()) {
        // rank cap: the reduction's cost grows as gn r^2 and the r x r
        // eigensolve's as r^3, so beyond ~0.3 gn solving G directly is
        // cheaper; a group whose smaller side is at most half the Gram
        // dimension can always use its rank bound
        const int64_t p = std::min(g->m, g->n);
        int64_t cap = std::max<int64_t>(32, (3 * g->gn + 9) / 10);
        if (2 * p <= g->gn) cap = std::max(cap, p);
        g->rcap = (int)std::min<int64_t>(std::min<int64_t>(cap, g->gn), pcmgs_max_rank());
        g->q_off = q_total;
        q_total += g->gn * g->rcap;
        g->t_off = t_total;
        t_total += (int64_t)g->rcap * g->rcap;
      }
      gram.push_back(g);
    }
  DevBuf gbuf(gbuf_total), lbuf(q_total), qbuf(q_total), tbuf(t_total), cbuf(t_total);
  prof_begin(kProfSvdGram);
  {
    GemmBatch gb;
    for (Group *g : gram) {
      const int m = (int)g->m, n = (int)g->n, gd = (int)g->gn;
      const double *X = mats.p + g->mat_off;  // col-major n x m
      double *G = gbuf.p + g->g_off;
      if (2.0 * gd * gd * (double)(g->eig_m ? n : m) >= kTcMinFlops) {
        // X is Theta row-major (m x n): Theta Theta^T contracts axis 1,
        // Theta^T Theta axis 0
        const int ax = g->eig_m ? 1 : 0;
        dense_contract_tc(X, m, n, ax, X, m, n, ax, G);
      } else if (g->eig_m) {  // Theta Theta^T = X^T X (m x m)
        gb.add(CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, X, n, X, n, G, m);
      } else {  // Theta^T Theta = X X^T (n x n)
        gb.add(CUBLAS_OP_N, CUBLAS_OP_T, n, n, m, X, n, X, n, G, n);
      }
    }
    gb.run(bh);
  }
  prof_end(kProfSvdGram, 0.0, 0.0);
  prof_begin(kProfSvdReduce);
  {
    std::vector<PcGroup> pcs[2];
    std::vector<Group *> pcg[2];
    for (Group *g : gram) {
      if (g->rcap == 0) continue;
      const int big = g->gn > kPcSmallRows ? 1 : 0;
      pcs[big].push_back({g->g_off, g->q_off, g->t_off, (int)g->gn, g->rcap});
      pcg[big].push_back(g);
    }
    if (!pcs[0].empty() || !pcs[1].empty()) {
      DevArray<PcGroup> dg[2];
      DevArray<int> dr[2];
      for (int b = 0; b < 2; ++b) {
        dg[b].upload(pcs[b]);
        dr[b].upload(std::vector<int>(pcs[b].size(), -1));
      }
      launch_pcmgs(dg[0].p, (int)pcs[0].size(), dg[1].p, (int)pcs[1].size(), gbuf.p, lbuf.p,
                   qbuf.p, tbuf.p, cbuf.p, dr[0].p, dr[1].p, kPcTol);
      GQ_CUDA(cudaGetLastError());
      std::vector<int> hr[2];
      for (int b = 0; b < 2; ++b) {
        hr[b].resize(pcs[b].size());
        if (!hr[b].empty())
          GQ_CUDA(cudaMemcpyAsync(hr[b].data(), dr[b].p, sizeof(int) * hr[b].size(),
                                  cudaMemcpyDeviceToHost, s));
      }
      sync();
      for (int b = 0; b < 2; ++b)
        for (size_t i = 0; i < hr[b].size(); ++i) {
          pcg[b][i]->r = hr[b][i];
          pcg[b][i]->pc = hr[b][i] >= 0;
        }
    }
  }
  prof_end(kProfSvdReduce, 0.0, 0.0);
  auto bucket_of = [](int64_t real) -> int64_t {
    if (real <= 256) return (real + 31) / 32 * 32;
    return (real + 63) / 64 * 64;
  };
  std::map<int64_t, std::vector<Group *>> buckets;
  for (Group *g : gram) g->dim = (g->pc && g->r == 0) ? 0 : bucket_of(g->pc ? g->r : g->gn);
  for (Group *g : gram) {
    if (g->dim == 0) continue;  // a zero matrix: nothing to solve
    buckets[g->dim].push_back(g);
  }
  int64_t ev_total = 0, w_total = 0, n_gram = 0;
  for (auto &kv : buckets)
    for (Group *g : kv.second) {
      g->ev_off = ev_total;
      ev_total += g->dim * g->dim;
      g->w_off = w_total;
      w_total += g->dim;
      ++n_gram;
    }
  DevBuf ev(ev_total), w(w_total);
  DevArray<int> einfo;
  if (n_gram > 0) {
    std::vector<PadDiagItem> pads;
    std::vector<SlotItem> from_g, from_c;
    for (auto &kv : buckets)
      for (Group *g : kv.second) {
        const int real = (int)(g->pc ? g->r : g->gn);
        pads.push_back({g->ev_off, (int)g->dim, real});
        if (g->pc)
          from_c.push_back({g->t_off, g->ev_off, real, g->rcap, (int)g->dim});
        else
          from_g.push_back({g->g_off, g->ev_off, real, (int)g->gn, (int)g->dim});
      }
    {
      DevArray<PadDiagItem> d;
      d.upload(pads);
      pad_diag_kernel<<<(unsigned)pads.size(), 256, 0, s>>>(d.p, ev.p);
      GQ_CUDA(cudaGetLastError());
    }
    launch_items(slot_copy_kernel, from_g, gbuf.p, ev.p);
    launch_items(slot_copy_kernel, from_c, cbuf.p, ev.p);
    // One batched eigensolve per bucket.  The solves are latency-bound (a
    // 1486-row syevd is ~60 ms of small launches), so buckets of different
    // sizes run side by side: largest first, dealt round-robin over the
    // lane's stream and its auxiliary streams, each with its own handle and
    // workspace, joined back before the values are read.  Same calls on the
    // same data as one after another.
    struct Solve {
      int64_t bs, nb, io;
      Group *first;
      int slot;
    };
    std::vector<Solve> solves;
    {
      int64_t io = 0;  // info words in bucket (map) order
      for (auto &kv : buckets) {
        solves.push_back({kv.first, (int64_t)kv.second.size(), io, kv.second[0], 0});
        io += (int64_t)kv.second.size();
      }
    }
    std::stable_sort(solves.begin(), solves.end(),
                     [](const Solve &a, const Solve &b) { return a.bs > b.bs; });
    const int nslot = (int)std::min<size_t>(solves.size(), 1 + Lane::kAux);
    for (size_t k = 0; k < solves.size(); ++k) solves[k].slot = (int)(k % nslot);
    auto handle_of = [&](int slot) { return slot == 0 ? h : aux_solver(slot - 1); };
    struct ParamsSet {  // released on every exit path
      std::vector<cusolverDnParams_t> v;
      ~ParamsSet() {
        for (auto x : v) cusolverDnDestroyParams(x);
      }
    } params;
    for (int k = 0; k < nslot; ++k) {
      cusolverDnParams_t x = nullptr;
      GQ_SOLVER(cusolverDnCreateParams(&x));
      params.v.push_back(x);
    }
    const std::vector<cusolverDnParams_t> &sp = params.v;
    // A bucket holding one large matrix goes to the divide-and-conquer
    // solver: measured over a D=4000 run, the batched call took 10-20 ms for
    // one matrix of 320-960 rows.
    auto single = [](const Solve &v) { return v.nb == 1 && v.bs >= kSyevdMinRows; };
    std::vector<size_t> dws(nslot, 0), hws(nslot, 0);
    for (const Solve &v : solves) {
      size_t d1 = 0, h1 = 0;
      if (single(v))
        GQ_SOLVER(cusolverDnXsyevd_bufferSize(
            handle_of(v.slot), sp[v.slot], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, v.bs,
            CUDA_R_64F, ev.p + v.first->ev_off, v.bs, CUDA_R_64F, w.p + v.first->w_off,
            CUDA_R_64F, &d1, &h1));
      else
        GQ_SOLVER(cusolverDnXsyevBatched_bufferSize(
            handle_of(v.slot), sp[v.slot], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, v.bs,
            CUDA_R_64F, ev.p + v.first->ev_off, v.bs, CUDA_R_64F, w.p + v.first->w_off,
            CUDA_R_64F, &d1, &h1, v.nb));
      dws[v.slot] = std::max(dws[v.slot], d1);
      hws[v.slot] = std::max(hws[v.slot], h1);
    }
    std::vector<DevBuf> dwork;
    std::vector<std::vector<char>> hwork;
    for (int k = 0; k < nslot; ++k) {
      dwork.emplace_back((int64_t)(dws[k] / sizeof(double)) + 2);
      hwork.emplace_back(hws[k] + 16);
    }
    einfo.upload(std::vector<int>(n_gram, 0));
    Lane &ln = lane();
    fork_aux(ln, nslot - 1);  // after the Gram matrices, workspaces and info words
    {
      // the lane's stream waits for every solve before anything here is
      // released -- on an error too, since the workspaces are freed in
      // stream order on the lane's stream
      AuxJoin joined(ln, nslot - 1);
      for (const Solve &v : solves) {
        if (single(v))
          GQ_SOLVER(cusolverDnXsyevd(
              handle_of(v.slot), sp[v.slot], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
              v.bs, CUDA_R_64F, ev.p + v.first->ev_off, v.bs, CUDA_R_64F,
              w.p + v.first->w_off, CUDA_R_64F, dwork[v.slot].p, dws[v.slot],
              hwork[v.slot].data(), hws[v.slot], einfo.p + v.io));
        else
          GQ_SOLVER(cusolverDnXsyevBatched(
              handle_of(v.slot), sp[v.slot], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
              v.bs, CUDA_R_64F, ev.p + v.first->ev_off, v.bs, CUDA_R_64F,
              w.p + v.first->w_off, CUDA_R_64F, dwork[v.slot].p, dws[v.slot],
              hwork[v.slot].data(), hws[v.slot], einfo.p + v.io, v.nb));
      }
    }
  }
  // eigenvectors of the reduced groups: U = Q Z (gn x r), Z the slot's
  // last r columns (ascending eigenvalues, padded coordinates zero)
  int64_t u_total = 0;
  for (Group *g : gram)
    if (g->pc && g->r > 0) {
      g->u_off = u_total;
      u_total += g->gn * g->r;
    }
  DevBuf ubuf(u_total);
  {
    GemmBatch gb;
    for (Group *g : gram) {
      if (!g->pc || g->r == 0) continue;
      const int gd = (int)g->gn, r = g->r, bs = (int)g->dim;
      // Q row-major gn x rcap is col-major rcap x gn: op(A) = A^T
      gb.add(CUBLAS_OP_T, CUBLAS_OP_N, gd, r, r, qbuf.p + g->q_off, g->rcap,
             ev.p + g->ev_off + (int64_t)(bs - r) * bs, bs, ubuf.p + g->u_off, gd);
    }
    gb.run(bh);
  }
  prof_end(kProfSvdEig, 0.0, 0.0);
  // ---- values to the host ---------------------------------------------------
  std::vector<double> hs_small(n_small * kSmall), hs_j(js_total), hw(w_total);
  std::vector<int> hinfo_j(groups.size(), 0), hinfo_e(n_gram, 0);
  if (n_small > 0) {
    GQ_CUDA(cudaMemcpyAsync(hs_small.data(), ss.p, sizeof(double) * hs_small.size(),
                            cudaMemcpyDeviceToHost, s));
  }
  if (js_total > 0) {
    GQ_CUDA(cudaMemcpyAsync(hs_j.data(), js.p, sizeof(double) * js_total, cudaMemcpyDeviceToHost,
                            s));
    GQ_CUDA(cudaMemcpyAsync(hinfo_j.data(), jinfo.p, sizeof(int) * groups.size(),
                            cudaMemcpyDeviceToHost, s));
  }
  if (w_total > 0) {
    GQ_CUDA(cudaMemcpyAsync(hw.data(), w.p, sizeof(double) * w_total, cudaMemcpyDeviceToHost, s));
    GQ_CUDA(cudaMemcpyAsync(hinfo_e.data(), einfo.p, sizeof(int) * n_gram,
                            cudaMemcpyDeviceToHost, s));
  }
  sync();
  for (int v : hinfo_j)
    if (v != 0) fail(kSolverError, "gesvdj did not converge, info=" + std::to_string(v));
  for (int v : hinfo_e)
    if (v != 0) fail(kSolverError, "syevd failed, info=" + std::to_string(v));

  // per-group descending values (p of them) and their source columns
  for (Group *g : groups) {
    g->svals.assign(g->p, 0.0);
    g->src_cols.assign(g->p, 0);
    if (g->route == kSmallJacobi) {
      std::vector<int> idx(kSmall);
      std::iota(idx.begin(), idx.end(), 0);
      const double *sv0 = hs_small.data() + g->sv_off;
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return sv0[a] > sv0[b]; });
      for (int64_t j = 0; j < g->p; ++j) {
        g->src_cols[j] = idx[j];
        g->svals[j] = sv0[idx[j]];
      }
    } else if (g->route == kJacobi) {
      for (int64_t j = 0; j < g->p; ++j) {
        g->src_cols[j] = (int)j;
        g->svals[j] = hs_j[g->sv_off + j];
      }
    } else if (g->pc) {
      // reduced group: r Ritz values (the slot's last r), zeros beyond; the
      // j-th largest has eigenvector column r - 1 - j of U = Q Z
      const int64_t r = g->r;
      const double *lam = r > 0 ? hw.data() + g->w_off : nullptr;  // ascending
      const double lmax = r > 0 ? std::max(lam[g->dim - 1], 0.0) : 0.0;
      for (int64_t j = 0; j < g->p; ++j) {
        if (j < r) {
          g->src_cols[j] = (int)(r - 1 - j);
          const double l = lam[g->dim - 1 - j];
          g->svals[j] = (l > kGramZeroRtol * lmax) ? std::sqrt(l) : 0.0;
        } else {
          g->src_cols[j] = 0;
          g->svals[j] = 0.0;
        }
      }
    } else {
      const double *lam = hw.data() + g->w_off;  // ascending
      const double lmax = std::max(lam[g->dim - 1], 0.0);
      for (int64_t j = 0; j < g->p; ++j) {
        const int64_t c = g->dim - 1 - j;
        g->src_cols[j] = (int)c;
        const double l = lam[c];
        g->svals[j] = (l > kGramZeroRtol * lmax) ? std::sqrt(l) : 0.0;
      }
    }
  }

  // ---- global truncation on the host -----------------------------------------
  std::vector<double> flat;
  for (Group *g : groups) flat.insert(flat.end(), g->svals.begin(), g->svals.end());
  double smax = 0.0;
  for (double v : flat) smax = std::max(smax, v);
  for (double &v : flat)
    if (!(v > kZeroSvRtol * smax)) v = 0.0;
  const int64_t ntot = (int64_t)flat.size();
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
  std::vector<std::pair<QN, int64_t>> sectors;
  int64_t L_total = 0, R_total = 0, pos = 0;
  for (Group *g : groups) {
    for (int64_t j = 0; j < g->p; ++j, ++pos) {
      g->svals[j] = flat[pos];
      if (flat[pos] > 0.0) g->nnz++;
      if (keep[pos]) {
        g->keep++;
        if (flat[pos] > 0.0) g->keep_nz++;
      }
    }
    if (g->keep == 0) continue;
    g->sector = (int)sectors.size();
    sectors.push_back({g->q, g->keep});
    g->L_off = L_total;
    L_total += g->m * g->keep;
    g->R_off = R_total;
    R_total += g->n * g->keep;
  }
  GQ_CHECK(!sectors.empty(), "SVD kept no singular value");

  // ---- factors L (m x keep) and R (n x keep) per group ------------------------
  prof_begin(kProfSvdFactors);
  // 'r' (scale_side 2): L = U, R = (S.Vt)^T; 'l' (1): L = U.S, R = V;
  // plain (0): L = U, R = V.  Columns of kept zero values start at zero.
  DevBuf Lb(L_total), Rb(R_total);
  GQ_CUDA(cudaMemsetAsync(Lb.p, 0, sizeof(double) * L_total, s));
  GQ_CUDA(cudaMemsetAsync(Rb.p, 0, sizeof(double) * R_total, s));
  const bool scale_l = scale_side == 1, scale_r = scale_side == 2;
  std::vector<ColItem> l_small, r_small, l_jac, r_jac, l_ev, r_ev, l_pc, r_pc;
  // A Gram group solved in full supplies the canonical side's columns for
  // kept zero values too: the eigenvectors of the zero (below-floor)
  // eigenvalues are orthonormal and orthogonal to the kept nonzero ones,
  // which is all the completion has to provide.  A reduced group has no
  // such vectors and takes the canonical completion.
  auto eig_is_canonical = [](const Group *g) {
    return !g->pc &&
           ((g->route == kGramLeft && g->eig_m) || (g->route == kGramRight && !g->eig_m));
  };
  for (Group *g : groups) {
    const int64_t ncopy = eig_is_canonical(g) ? g->keep : g->keep_nz;
    for (int64_t j = 0; j < ncopy; ++j) {
      const int sc = g->src_cols[j];
      const double sj = g->svals[j];
      switch (g->route) {
        case kSmallJacobi:
        case kJacobi: {
          auto &vl = g->route == kSmallJacobi ? l_small : l_jac;
          auto &vr = g->route == kSmallJacobi ? r_small : r_jac;
          vl.push_back({g->lv_off, g->L_off, (int)g->m, g->ld_l, (int)g->m, sc, (int)j,
                        scale_l ? sj : 1.0});
          vr.push_back({g->rv_off, g->R_off, (int)g->n, g->ld_r, (int)g->n, sc, (int)j,
                        scale_r ? sj : 1.0});
          break;
        }
        case kGramLeft:
        case kGramRight:
          if (g->pc) {
            if (g->eig_m)
              l_pc.push_back({g->u_off, g->L_off, (int)g->m, (int)g->gn, (int)g->m, sc, (int)j, 1.0});
            else
              r_pc.push_back({g->u_off, g->R_off, (int)g->n, (int)g->gn, (int)g->n, sc, (int)j, 1.0});
          } else if (g->eig_m) {
            l_ev.push_back({g->ev_off, g->L_off, (int)g->m, (int)g->dim, (int)g->m, sc, (int)j, 1.0});
          } else {
            r_ev.push_back({g->ev_off, g->R_off, (int)g->n, (int)g->dim, (int)g->n, sc, (int)j, 1.0});
          }
          break;
      }
    }
  }
  launch_items(col_copy_kernel, l_small, sv.p, Lb.p);
  launch_items(col_copy_kernel, r_small, su.p, Rb.p);
  launch_items(col_copy_kernel, l_jac, jl.p, Lb.p);
  launch_items(col_copy_kernel, r_jac, jr.p, Rb.p);
  launch_items(col_copy_kernel, l_ev, ev.p, Lb.p);
  launch_items(col_copy_kernel, r_ev, ev.p, Rb.p);
  launch_items(col_copy_kernel, l_pc, ubuf.p, Lb.p);
  launch_items(col_copy_kernel, r_pc, ubuf.p, Rb.p);
  // projections for the Gram routes: R = X L (canonical left) or L = X^T R
  // (canonical right)
  {
    GemmBatch gb;
    for (Group *g : groups) {
      if (g->keep_nz == 0 || (g->route != kGramLeft && g->route != kGramRight)) continue;
      const int m = (int)g->m, n = (int)g->n, k = (int)g->keep_nz;
      const double *X = mats.p + g->mat_off;
      double *L = Lb.p + g->L_off, *R = Rb.p + g->R_off;
      const bool tc = 2.0 * m * n * (double)k >= kTcMinFlops;
      // L, R col-major (ld m, n) = row-major k x m, k x n
      auto left_from_right = [&] {  // L = X^T R (m x k): Lrow = Rrow . Theta^T
        if (tc)
          dense_contract_tc(R, k, n, 1, X, m, n, 1, L);
        else
          gb.add(CUBLAS_OP_T, CUBLAS_OP_N, m, k, n, X, n, R, n, L, m);
      };
      auto right_from_left = [&] {  // R = X L (n x k): Rrow = Lrow . Theta
        if (tc)
          dense_contract_tc(L, k, m, 1, X, m, n, 0, R);
        else
          gb.add(CUBLAS_OP_N, CUBLAS_OP_N, n, k, m, X, n, L, m, R, n);
      };
      if (g->route == kGramLeft)
        right_from_left();
      else
        left_from_right();
    }
    gb.run(bh);
  }
  // sign convention on the kept nonzero columns (by the left factor)
  {
    std::vector<SignItem> items;
    for (Group *g : groups)
      for (int64_t j = 0; j < g->keep_nz; ++j)
        items.push_back({g->L_off + j * g->m, g->R_off + j * g->n, (int)g->m, (int)g->n});
    if (!items.empty()) {
      DevArray<SignItem> d;
      d.upload(items);
      sign_fix_kernel<<<(unsigned)items.size(), 256, 0, s>>>(d.p, Lb.p, Rb.p);
      GQ_CUDA(cudaGetLastError());
    }
  }
  // canonical completion of the kept zero values on the orthonormal side(s);
  // their status words are checked once, after the output scatter
  DevArray<int> cinfo;
  {
    int64_t ncomp = 0;
    for (Group *g : groups)
      if (g->keep > g->keep_nz) ncomp += 2;
    cinfo.upload(std::vector<int>(2 * ncomp + 2, 0));
  }
  int64_t cslot = 0;
  std::vector<Completion> comps;
  comps.reserve(2 * groups.size());
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    Group *g = groups[gi];
    const int64_t kz = g->keep - g->keep_nz;
    if (kz == 0) continue;
    auto completion = [&](bool left, double *dst) {
      const int64_t dim = left ? g->m : g->n;
      comps.emplace_back();
      Completion &c = comps.back();
      c.q.alloc(std::max<int64_t>(dim * g->nnz, 1));
      std::vector<ColItem> items;
      const bool gram = g->route == kGramLeft || g->route == kGramRight;
      for (int64_t j = 0; j < g->nnz; ++j)
        items.push_back({gram ? (g->pc ? g->u_off : g->ev_off) : (left ? g->lv_off : g->rv_off),
                         0, (int)dim,
                         gram ? (int)(g->pc ? g->gn : g->dim) : (left ? g->ld_l : g->ld_r),
                         (int)dim, g->src_cols[j], (int)j, 1.0});
      const double *src = gram ? (g->pc ? ubuf.p : ev.p)
                               : g->route == kSmallJacobi ? (left ? sv.p : su.p)
                                                          : (left ? jl.p : jr.p);
      launch_items(col_copy_kernel, items, src, c.q.p);
      c.dim = dim;
      c.r = g->nnz;
      c.k = kz;
      c.out = dst;
      c.info = cinfo.p + cslot;
      completion_prepare(c);
      cslot += 2;
    };
    if (eig_is_canonical(g)) continue;  // zero columns came with the eigenvectors
    if (scale_side != 1) completion(true, Lb.p + g->L_off + g->keep_nz * g->m);
    if (scale_side != 2) completion(false, Rb.p + g->R_off + g->keep_nz * g->n);
  }
  // the factorisations, dealt round-robin over the lane's stream and its
  // auxiliary streams (each with its own handle), joined back before the
  // buffers above are released
  {
    int nfac = 0;
    for (auto &c : comps) nfac += (c.k > 0 && c.r > 0) ? 1 : 0;
    if (nfac > 0) {
      prof_begin(kProfSvdOrtho);
      const int nslot = std::min(nfac, 1 + Lane::kAux);
      Lane &ln = lane();
      fork_aux(ln, nslot - 1);
      {
        AuxJoin joined(ln, nslot - 1);
        int i = 0;
        for (auto &c : comps) {
          if (c.k == 0 || c.r == 0) continue;
          const int slot = i++ % nslot;
          completion_factor(c, slot == 0 ? solver() : aux_solver(slot - 1));
        }
      }
      prof_end(kProfSvdOrtho, 0.0, 0.0);
    }
  }

  prof_end(kProfSvdFactors, 0.0, 0.0);
  // ---- output tensors ---------------------------------------------------------
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
    for (int64_t j = 0; j < g->keep; ++j) out.s.push_back(j < g->keep_nz ? g->svals[j] : 0.0);
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
  {
    std::vector<ScatterItem> items;
    for (Group *g : groups) {
      if (g->keep == 0) continue;
      for (size_t ri = 0; ri < g->rows.size(); ++ri) {
        auto c = g->rows[ri];
        c.push_back(g->sector);
        const int64_t ob = out.u->find(c.data());
        const int64_t n = g->rsz[ri] * g->keep;
        for (int64_t e0 = 0; e0 < n; e0 += kCopyChunk)
          items.push_back({out.u->offs[ob], g->L_off + g->roff[ri], e0,
                           std::min(n, e0 + kCopyChunk), (int)g->rsz[ri], (int)g->keep,
                           (int)g->m, 0});
      }
      for (size_t ci = 0; ci < g->cols.size(); ++ci) {
        std::vector<int> c{g->sector};
        c.insert(c.end(), g->cols[ci].begin(), g->cols[ci].end());
        const int64_t ob = out.vt->find(c.data());
        const int64_t n = g->csz[ci] * g->keep;
        for (int64_t e0 = 0; e0 < n; e0 += kCopyChunk)
          items.push_back({out.vt->offs[ob], g->R_off + g->coff[ci], e0,
                           std::min(n, e0 + kCopyChunk), (int)g->csz[ci], (int)g->keep,
                           (int)g->n, 1});
      }
    }
    DevArray<ScatterItem> d;
    d.upload(items);
    scatter_kernel<<<(unsigned)items.size(), 256, 0, s>>>(d.p, Lb.p, Rb.p, out.u->data.p,
                                                         out.vt->data.p);
    GQ_CUDA(cudaGetLastError());
  }
  if (cslot > 0) {
    std::vector<int> hinfo(cslot, 0);
    GQ_CUDA(cudaMemcpyAsync(hinfo.data(), cinfo.p, sizeof(int) * cslot, cudaMemcpyDeviceToHost,
                            s));
    sync();
    for (int v : hinfo)
      if (v != 0) fail(kSolverError, "QR of a null-space completion failed");
  }
  prof_end(kProfSvd, 0.0, 0.0);
  return out;
}

}  // namespace gq
