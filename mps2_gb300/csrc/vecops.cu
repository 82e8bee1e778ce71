// Lanczos vector kernels (gqten Normalize / LinearCombine / full-contraction
// inner product as used at ``lanczos_solver_impl.h:120, 134-160, 173, 215``).
//
// Every Krylov vector of one solve shares a single block structure, so the
// vector operations are flat streams over contiguous FP64 arrays: pure HBM
// bandwidth work.  Reductions use a fixed grid and a fixed-order second pass,
// so results are bitwise reproducible run to run.
#include "gq_runtime.hpp"

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

__global__ void combine_kernel(const double *const *__restrict__ bases,
                               const double *__restrict__ c, int m, double *__restrict__ out,
                               int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double s = 0.0;
    for (int k = 0; k < m; ++k) s = fma(c[k], bases[k][i], s);
    out[i] = s;
  }
}

__global__ void block_copy_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                  const int64_t *__restrict__ triples) {
  const int64_t so = triples[3 * blockIdx.x], dof = triples[3 * blockIdx.x + 1],
                n = triples[3 * blockIdx.x + 2];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[dof + i] = src[so + i];
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

void dev_combine(const std::vector<const double *> &bases, const std::vector<double> &c,
                 double *out, int64_t n) {
  const int m = (int)bases.size();
  DevArray<const double *> dp;
  DevArray<double> dc;
  dp.upload(bases);
  dc.upload(c);
  prof_begin(kProfVector);
  combine_kernel<<<stream_grid(n), 256, 0, stream()>>>(dp.p, dc.p, m, out, n);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfVector, 2.0 * n * m, 8.0 * n * (m + 1));
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
