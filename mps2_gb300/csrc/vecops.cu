// Lanczos vector kernels (gqten Normalize / LinearCombine / full-contraction
// inner product as used at ``lanczos_solver_impl.h:120, 134-160, 173, 215``).
//
// Every Krylov vector of one solve shares a single block structure, so the
// vector operations are flat streams over contiguous FP64 arrays: pure HBM
// bandwidth work.  Reductions use a fixed grid and a fixed-order second pass,
// so results are bitwise reproducible run to run.
#include "gq_runtime.hpp"
#include "tridiag_dev.cuh"

namespace gq {

namespace {
constexpr int kRedBlocks = 608;  // 4 x 152 SMs
constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[kRedThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < kRedThreads / 32 ? ws[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;  // valid in thread 0
}

__global__ void __launch_bounds__(kRedThreads)
    dot_partial_kernel(const double *__restrict__ x, const double *__restrict__ y, int64_t n,
                       double *__restrict__ partial) {
  double s = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // two independent accumulators for ILP
  double s2 = 0.0;
  for (; i + stride < n; i += 2 * stride) {
    s = fma(x[i], y[i], s);
    s2 = fma(x[i + stride], y[i + stride], s2);
  }
  if (i < n) s = fma(x[i], y[i], s);
  s = block_sum(s + s2);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads)
    finish_sum_kernel(const double *__restrict__ partial, int np, double *__restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
  s = block_sum(s);
  if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kRedThreads)
    gamma_kernel(const double *__restrict__ x, const double *__restrict__ u,
                 const double *__restrict__ a_dev, const double *__restrict__ v,
                 const double *__restrict__ b_dev, int b_is_sq, double *__restrict__ y, int64_t n,
                 double *__restrict__ partial) {
  const double a = u ? *a_dev : 0.0;
  double b = 0.0;
  if (v) b = b_is_sq ? sqrt(*b_dev) : *b_dev;
  double s = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double g = x[i];
    if (u) g = fma(-a, u[i], g);
    if (v) g = fma(-b, v[i], g);
    y[i] = g;
    s = fma(g, g, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void scale_rsqrt_kernel(double *__restrict__ x, int64_t n,
                                   const double *__restrict__ nrm2) {
  const double f = 1.0 / sqrt(*nrm2);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] *= f;
}

__global__ void scale_kernel(double *__restrict__ x, int64_t n, double s) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] *= s;
}

__global__ void block_copy_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                  const int64_t *__restrict__ triples) {
  const int64_t so = triples[3 * blockIdx.x], dof = triples[3 * blockIdx.x + 1],
                n = triples[3 * blockIdx.x + 2];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[dof + i] = src[so + i];
}

// ---------------------------------------------------------------------------
// The Lanczos loop on the device.  The iteration index lives in LzCtl::m and
// the Krylov vectors are reached through a device table of pointers, so the
// same launches serve every iteration: replayed by the body of a CUDA-graph
// while loop, or launched one iteration at a time by the host.  Every
// kernel returns at once when the control block says the loop has stopped.
// ---------------------------------------------------------------------------
__global__ void lz_init_kernel(LzCtl *__restrict__ ctl, const double *__restrict__ a_dev) {
  LzCtl c{};
  c.m = 1;
  c.e0 = a_dev[0];
  *ctl = c;
}

// b[m-1] = sqrt(nrm2[m]); stop on a non-finite norm or an invariant subspace.
__global__ void lz_pre_kernel(LzCtl *__restrict__ ctl, const double *__restrict__ n_dev,
                              double *__restrict__ b_dev) {
  if (ctl->status != kLzRunning) return;
  const int m = ctl->m;
  const double nrm2 = n_dev[m];
  if (!isfinite(nrm2)) {
    ctl->status = kLzBadVector;
    return;
  }
  const double nb = sqrt(nrm2);
  if (nb == 0.0) {  // invariant subspace: the Ritz pair of the m vectors so far
    ctl->status = kLzInvariant;
    ctl->nvec = m;
    ctl->iters = m;
    ctl->energy = ctl->e0;
    return;
  }
  b_dev[m - 1] = nb;
}

// v_m = gamma_m / |gamma_m| in place, also written to xin when given.
__global__ void lz_scale_kernel(double *const *__restrict__ vecs, int64_t n,
                                const double *__restrict__ n_dev, const LzCtl *__restrict__ ctl,
                                double *__restrict__ xin) {
  if (ctl->status != kLzRunning) return;
  const int m = ctl->m;
  double *__restrict__ x = vecs[m];
  const double f = 1.0 / sqrt(n_dev[m]);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double v = x[i] * f;
    x[i] = v;
    if (xin) xin[i] = v;
  }
}

__global__ void __launch_bounds__(kRedThreads)
    lz_dot_partial_kernel(double *const *__restrict__ vecs, const double *__restrict__ y,
                          int64_t n, const LzCtl *__restrict__ ctl,
                          double *__restrict__ partial) {
  if (ctl->status != kLzRunning) return;
  const double *__restrict__ x = vecs[ctl->m];
  double s = 0.0, s2 = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    s = fma(x[i], y[i], s);
    s2 = fma(x[i + stride], y[i + stride], s2);
  }
  if (i < n) s = fma(x[i], y[i], s);
  s = block_sum(s + s2);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// out[m + off] = sum of the partials, unless stopped or m + off >= limit.
__global__ void __launch_bounds__(kRedThreads)
    lz_finish_kernel(const double *__restrict__ partial, int np, double *__restrict__ out,
                     const LzCtl *__restrict__ ctl, int off, int limit) {
  if (ctl->status != kLzRunning || ctl->m + off >= limit) return;
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
  s = block_sum(s);
  if (threadIdx.x == 0) out[ctl->m + off] = s;
}

// gamma_{m+1} = w - a_m v_m - b_{m-1} v_{m-1} into vecs[m+1] (skipped when
// m + 1 == maxit), with its squared norm's partials.
__global__ void __launch_bounds__(kRedThreads)
    lz_gamma_kernel(double *const *__restrict__ vecs, const double *__restrict__ w, int64_t n,
                    const double *__restrict__ a_dev, const double *__restrict__ n_dev,
                    const LzCtl *__restrict__ ctl, int maxit, double *__restrict__ partial) {
  if (ctl->status != kLzRunning) return;
  const int m = ctl->m;
  if (m + 1 >= maxit) return;
  double *__restrict__ y = vecs[m + 1];
  const double *__restrict__ u = vecs[m];
  const double *__restrict__ v = vecs[m - 1];
  const double a = a_dev[m];
  const double b = sqrt(n_dev[m]);
  double s = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double g = w[i];
    g = fma(-a, u[i], g);
    g = fma(-b, v[i], g);
    y[i] = g;
    s = fma(g, g, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Convergence test of iteration m (one warp): the lowest eigenvalue of the
// (m+1) x (m+1) tridiagonal matrix, the reference's stopping rule
// (E_old - E_new < error, m == eff_dim, m == max_iterations - 1), and the
// loop condition of the graph (0 once stopped or after `cap` iterations).
__global__ void lz_post_kernel(LzCtl *__restrict__ ctl, const double *__restrict__ a_dev,
                               const double *__restrict__ b_dev, int maxit, int64_t dim,
                               double error, int cap, int set_cond,
                               cudaGraphConditionalHandle cond) {
  LzCtl c = *ctl;
  if (c.status == kLzRunning) {
    const int m = c.m;
    if (!isfinite(a_dev[m])) {
      c.status = kLzBadCoefficient;
    } else {
      const double e_new = tridiag::lowest_eigenvalue_warp(a_dev, b_dev, m + 1);
      if (!isfinite(e_new)) {
        c.status = kLzBadCoefficient;
      } else if ((c.e0 - e_new) < error || m == dim || m == maxit - 1) {
        c.status = kLzConverged;
        c.nvec = m + 1;
        c.iters = m;
        c.energy = e_new;
      } else {
        c.e0 = e_new;
        c.m = m + 1;
      }
    }
  }
  c.guard += 1;
  if (c.status == kLzRunning && c.guard >= cap) c.status = kLzCapped;
  if (threadIdx.x == 0) {
    *ctl = c;
    if (set_cond) cudaGraphSetConditional(cond, c.status == kLzRunning ? 1u : 0u);
  }
}

// Ritz vector coefficients c[0..nvec) of the stopped loop (one thread).
__global__ void lz_ritz_kernel(const LzCtl *__restrict__ ctl, const double *__restrict__ a_dev,
                               const double *__restrict__ b_dev, double *__restrict__ c_dev,
                               double *__restrict__ work) {
  const LzCtl c = *ctl;
  if (c.status != kLzConverged && c.status != kLzInvariant) return;
  const double lam = tridiag::lowest_eigenvalue_warp(a_dev, b_dev, c.nvec);
  if (threadIdx.x == 0) tridiag::eigenvector(a_dev, b_dev, c.nvec, lam, work, c_dev);
}

// out = sum_{k < nvec} c_k v_k.
__global__ void lz_combine_kernel(double *const *__restrict__ vecs, const double *__restrict__ c,
                                  const LzCtl *__restrict__ ctl, double *__restrict__ out,
                                  int64_t n) {
  const int m = ctl->status == kLzConverged || ctl->status == kLzInvariant ? ctl->nvec : 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double s = 0.0;
    for (int k = 0; k < m; ++k) s = fma(c[k], vecs[k][i], s);
    out[i] = s;
  }
}

unsigned stream_grid(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 4 * 152 * 4) g = 4 * 152 * 4;
  if (g < 1) g = 1;
  return (unsigned)g;
}
}  // namespace

int64_t dot_scratch_elems() { return kRedBlocks; }

void dev_dot(const double *x, const double *y, int64_t n, double *out_dev, double *scratch) {
  prof_begin(kProfVector);
  dot_partial_kernel<<<kRedBlocks, kRedThreads, 0, stream()>>>(x, y, n, scratch);
  finish_sum_kernel<<<1, kRedThreads, 0, stream()>>>(scratch, kRedBlocks, out_dev);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, 2.0 * n, 16.0 * n);
}

void dev_lanczos_gamma(const double *x, const double *u, const double *a_dev, const double *v,
                       const double *b_dev, bool b_is_sq, double *y, int64_t n,
                       double *nrm2_out_dev, double *scratch) {
  prof_begin(kProfVector);
  gamma_kernel<<<kRedBlocks, kRedThreads, 0, stream()>>>(x, u, a_dev, v, b_dev, b_is_sq ? 1 : 0,
                                                         y, n, scratch);
  finish_sum_kernel<<<1, kRedThreads, 0, stream()>>>(scratch, kRedBlocks, nrm2_out_dev);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, 6.0 * n, 8.0 * n * (2 + (u ? 1 : 0) + (v ? 1 : 0)));
}

void dev_scale_rsqrt(double *x, int64_t n, const double *nrm2_dev) {
  prof_begin(kProfVector);
  scale_rsqrt_kernel<<<stream_grid(n), 256, 0, stream()>>>(x, n, nrm2_dev);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, (double)n, 16.0 * n);
}

void dev_scale(double *x, int64_t n, double s) {
  scale_kernel<<<stream_grid(n), 256, 0, stream()>>>(x, n, s);
  GQ_CUDA(cudaGetLastError());
}

void lz_init(LzCtl *ctl, const double *a_dev) {
  lz_init_kernel<<<1, 1, 0, stream()>>>(ctl, a_dev);
  GQ_CUDA(cudaGetLastError());
}

void lz_iteration(const LzLoop &L, const MatvecFn &matvec, bool set_cond,
                  cudaGraphConditionalHandle cond) {
  auto s = stream();
  prof_begin(kProfVector);
  lz_pre_kernel<<<1, 1, 0, s>>>(L.ctl, L.n_dev, L.b_dev);
  lz_scale_kernel<<<stream_grid(L.n), 256, 0, s>>>(L.vecs, L.n, L.n_dev, L.ctl, L.xin);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, (double)L.n, 16.0 * L.n);
  matvec();
  prof_begin(kProfVector);
  lz_dot_partial_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(L.vecs, L.w, L.n, L.ctl, L.red);
  lz_finish_kernel<<<1, kRedThreads, 0, s>>>(L.red, kRedBlocks, L.a_dev, L.ctl, 0, L.maxit);
  lz_gamma_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(L.vecs, L.w, L.n, L.a_dev, L.n_dev, L.ctl,
                                                     L.maxit, L.red);
  lz_finish_kernel<<<1, kRedThreads, 0, s>>>(L.red, kRedBlocks, L.n_dev, L.ctl, 1, L.maxit);
  lz_post_kernel<<<1, 32, 0, s>>>(L.ctl, L.a_dev, L.b_dev, L.maxit, L.dim, L.error, L.cap,
                                  set_cond ? 1 : 0, cond);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, 8.0 * L.n, 8.0 * L.n * 7);
}

void lz_ritz_vector(const LzLoop &L, double *out) {
  auto s = stream();
  prof_begin(kProfVector);
  lz_ritz_kernel<<<1, 32, 0, s>>>(L.ctl, L.a_dev, L.b_dev, L.c_dev, L.work);
  lz_combine_kernel<<<stream_grid(L.n), 256, 0, s>>>(L.vecs, L.c_dev, L.ctl, out, L.n);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, 2.0 * L.n, 8.0 * L.n * 4);
}

void dev_block_copy(const double *src, double *dst, const std::vector<int64_t> &triples) {
  const int64_t nb = (int64_t)triples.size() / 3;
  if (nb == 0) return;
  DevArray<int64_t> d;
  d.upload(triples);
  block_copy_kernel<<<(unsigned)nb, 256, 0, stream()>>>(src, dst, d.p);
  GQ_CUDA(cudaGetLastError());
}

}  // namespace gq
