// Rank-revealing reduction of Gram matrices for the block SVD.
//
// A converged two-site state has a steeply graded Schmidt spectrum: at the
// centre of the L=64 Hubbard chain with D=4000, 523 of its 12779 singular
// values lie above 1e-7 of the largest.  A full eigensolve of each group's
// Gram matrix G = X X^T (n x n) therefore spends almost all of its work on
// the noise floor.  This kernel finds G's numerical range first:
//
//   pivoted Cholesky  G ~ L L^T  (left-looking, largest remaining diagonal
//   first, stopped when that diagonal falls to `tol` times G's largest
//   diagonal), with every new column of L orthogonalised against the
//   previous ones by modified Gram-Schmidt with one re-orthogonalisation:
//   L = Q T with Q (n x r) orthonormal and T (r x r) upper triangular.
//
// Then Q^T G Q ~ T T^T (the neglected Schur complement has all its
// diagonal entries below tol * max diag G), whose r x r eigen-decomposition
// Z Lambda Z^T gives G's eigenpairs above the floor as (Lambda, Q Z).  The
// eigenvalue floor of the Gram routes (1e-14 of the largest) sits a decade
// above the stopping tolerance.  Method: pivoted Cholesky for positive
// semi-definite matrices (Higham, "Analysis of the Cholesky decomposition of
// a semi-definite matrix", 1990; LAPACK dpstrf) with Gram-Schmidt
// re-orthogonalisation (Giraud, Langou, Rozloznik, "twice is enough", 2005).
//
// Parallel layout: one thread-block cluster per group; the cluster's CTAs
// split the rows of G, L and Q; the cluster-wide argmax, dot products and
// norms go through distributed shared memory with one cluster barrier each
// (four per column).  L and Q are row-major (n x rcap) so that the per-row
// dot products read contiguous memory.  Every loop is bounded by rcap.
#include <cooperative_groups.h>

#include "gq_runtime.hpp"

namespace cg = cooperative_groups;

namespace gq {

namespace {
constexpr int kPcThreads = 256;
constexpr int kPcMaxRows = 512;    // rows of one CTA (n / cluster size)
constexpr int kPcMaxRank = 768;    // rcap limit (partial-sum buffers)

struct PcArgs {
  const PcGroup *groups;
  const double *G;
  double *L, *Q, *T, *C;
  int *r_out;
  double tol;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int CS>
__global__ void __launch_bounds__(kPcThreads) pcmgs_kernel(PcArgs a) {
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank();
  const int gid = blockIdx.x / CS;
  const PcGroup grp = a.groups[gid];
  const int n = grp.n, rcap = grp.rcap;
  const double *G = a.G + grp.g_off;
  double *L = a.L + grp.q_off, *Q = a.Q + grp.q_off;
  double *T = a.T + grp.t_off, *C = a.C + grp.t_off;
  const int row0 = (int)((int64_t)n * crank / CS), row1 = (int)((int64_t)n * (crank + 1) / CS);
  const int nr = row1 - row0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = kPcThreads / 32;

  __shared__ double d[kPcMaxRows];      // remaining diagonal of own rows (-1: pivoted)
  __shared__ double v[kPcMaxRows];      // the new column, own rows
  __shared__ double lp[kPcMaxRank];     // pivot row of L
  __shared__ double c1[kPcMaxRank], c2[kPcMaxRank];   // Gram-Schmidt coefficients
  __shared__ double part1[kPcMaxRank], part2[kPcMaxRank];  // own partial dots
  __shared__ double am_val[1];          // own argmax candidate
  __shared__ int am_idx[1];
  __shared__ double nrm_part[1];
  __shared__ double red_v[kPcThreads / 32];
  __shared__ int red_i[kPcThreads / 32];
  __shared__ double s_piv_d, s_d0, s_norm;
  __shared__ int s_piv, s_stop;

  for (int i = tid; i < nr; i += kPcThreads) d[i] = G[(int64_t)(row0 + i) * n + row0 + i];
  __syncthreads();

  int j = 0;
  for (; j <= rcap; ++j) {
    // ---- cluster-wide argmax of the remaining diagonal --------------------
    double bv = -1.0;
    int bi = 0x7fffffff;
    for (int i = tid; i < nr; i += kPcThreads) {
      const double x = d[i];
      if (x > bv) { bv = x; bi = row0 + i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < nwarp; ++w)
        if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < bi)) { bv = red_v[w]; bi = red_i[w]; }
      am_val[0] = bv;
      am_idx[0] = bi;
    }
    cluster.sync();
    if (tid == 0) {
      double gv = -1.0;
      int gi = 0x7fffffff;
      for (int c = 0; c < CS; ++c) {
        const double ov = *cluster.map_shared_rank(&am_val[0], c);
        const int oi = *cluster.map_shared_rank(&am_idx[0], c);
        if (ov > gv || (ov == gv && oi < gi)) { gv = ov; gi = oi; }
      }
      if (j == 0) s_d0 = gv;
      s_piv_d = gv;
      s_piv = gi;
      s_stop = (!(gv > a.tol * s_d0) || j == rcap) ? 1 : 0;
    }
    __syncthreads();
    if (s_stop) break;
    const int p = s_piv;
    const double dp = s_piv_d, sq = sqrt(dp);
    // ---- new column of L on own rows ------------------------------------------
    // row p may belong to another CTA of the cluster: read it from L2
    for (int k = tid; k < j; k += kPcThreads) lp[k] = __ldcg(&L[(int64_t)p * rcap + k]);
    __syncthreads();
    for (int i = warp; i < nr; i += nwarp) {
      const double *Li = L + (int64_t)(row0 + i) * rcap;
      double acc = 0.0;
      for (int k = lane; k < j; k += 32) acc = fma(Li[k], lp[k], acc);
      acc = warp_sum(acc);
      if (lane == 0) {
        double x;
        if (row0 + i == p) x = sq;
        else if (d[i] < 0.0) x = 0.0;  // already pivoted: zero in exact arithmetic
        else x = (G[(int64_t)(row0 + i) * n + p] - acc) / sq;
        v[i] = x;
        L[(int64_t)(row0 + i) * rcap + j] = x;
        if (row0 + i == p) d[i] = -1.0;
        else if (d[i] >= 0.0) d[i] = fmax(d[i] - x * x, 0.0);
      }
    }
    __syncthreads();
    // ---- Gram-Schmidt against Q[:, 0:j], twice ---------------------------------
    for (int pass = 0; pass < 2; ++pass) {
      double *part = pass == 0 ? part1 : part2;
      double *cf = pass == 0 ? c1 : c2;
      for (int k = tid; k < j; k += kPcThreads) {
        double acc = 0.0;
        for (int i = 0; i < nr; ++i) acc = fma(Q[(int64_t)(row0 + i) * rcap + k], v[i], acc);
        part[k] = acc;
      }
      cluster.sync();
      for (int k = tid; k < j; k += kPcThreads) {
        double s = 0.0;
        for (int c = 0; c < CS; ++c) s += *cluster.map_shared_rank(&part[k], c);
        cf[k] = s;
      }
      __syncthreads();
      for (int i = warp; i < nr; i += nwarp) {
        const double *Qi = Q + (int64_t)(row0 + i) * rcap;
        double acc = 0.0;
        for (int k = lane; k < j; k += 32) acc = fma(Qi[k], cf[k], acc);
        acc = warp_sum(acc);
        if (lane == 0) v[i] -= acc;
      }
      __syncthreads();
    }
    // ---- normalise ------------------------------------------------------------
    double ss = 0.0;
    for (int i = tid; i < nr; i += kPcThreads) ss = fma(v[i], v[i], ss);
    ss = warp_sum(ss);
    if (lane == 0) red_v[warp] = ss;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < nwarp; ++w) s += red_v[w];
      nrm_part[0] = s;
    }
    cluster.sync();
    if (tid == 0) {
      double s = 0.0;
      for (int c = 0; c < CS; ++c) s += *cluster.map_shared_rank(&nrm_part[0], c);
      s_norm = sqrt(s);
    }
    __syncthreads();
    const double nv = s_norm;
    const double inv = nv > 0.0 ? 1.0 / nv : 0.0;
    for (int i = tid; i < nr; i += kPcThreads) Q[(int64_t)(row0 + i) * rcap + j] = v[i] * inv;
    if (crank == 0) {
      for (int k = tid; k < j; k += kPcThreads) T[(int64_t)k * rcap + j] = c1[k] + c2[k];
      if (tid == 0) T[(int64_t)j * rcap + j] = nv;
    }
    __syncthreads();
  }
  const int r = j;
  const bool exceeded = j == rcap && s_piv_d > a.tol * s_d0;
  if (crank == 0 && tid == 0) a.r_out[gid] = exceeded ? -1 : r;
  // every remote shared-memory read of this cluster is done before any CTA
  // exits, and T's columns (written by rank 0) are visible to the cluster
  cluster.sync();
  if (exceeded) return;
  // ---- C = T T^T (r x r, row-major, ld rcap); T upper triangular ----------
  const int64_t rr = (int64_t)r * r;
  for (int64_t e = (int64_t)crank * kPcThreads + tid; e < rr; e += (int64_t)CS * kPcThreads) {
    const int x = (int)(e / r), y = (int)(e % r);
    if (y < x) continue;
    double acc = 0.0;
    for (int k = y; k < r; ++k)
      acc = fma(__ldcg(&T[(int64_t)x * rcap + k]), __ldcg(&T[(int64_t)y * rcap + k]), acc);
    C[(int64_t)x * rcap + y] = acc;
    C[(int64_t)y * rcap + x] = acc;
  }
}

template <int CS>
void launch_cs(const PcGroup *dgroups, int ngroups, const PcArgs &base, cudaStream_t s) {
  if (ngroups == 0) return;
  PcArgs a = base;
  a.groups = dgroups;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ngroups * CS));
  cfg.blockDim = dim3(kPcThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GQ_CUDA(cudaLaunchKernelEx(&cfg, pcmgs_kernel<CS>, a));
}

// Cluster size for the large Gram matrices: 16 CTAs (a non-portable size)
// when the device can schedule such a cluster of this kernel, else 8.
int big_cluster_size() {
  static const int cs = [] {
    if (cudaFuncSetAttribute(pcmgs_kernel<16>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1) != cudaSuccess) {
      cudaGetLastError();
      return 8;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kPcThreads);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, pcmgs_kernel<16>, &cfg) != cudaSuccess) {
      cudaGetLastError();
      return 8;
    }
    return nclusters > 0 ? 16 : 8;
  }();
  return cs;
}
}  // namespace

int pcmgs_max_rows() { return kPcMaxRows * big_cluster_size(); }
int pcmgs_max_rank() { return kPcMaxRank; }

void launch_pcmgs(const PcGroup *groups_small, int n_small, const PcGroup *groups_big, int n_big,
                  const double *G, double *L, double *Q, double *T, double *C, int *r_small,
                  int *r_big, double tol) {
  auto s = stream();
  PcArgs base{nullptr, G, L, Q, T, C, nullptr, tol};
  base.r_out = r_small;
  launch_cs<4>(groups_small, n_small, base, s);
  base.r_out = r_big;
  if (big_cluster_size() == 16)
    launch_cs<16>(groups_big, n_big, base, s);
  else
    launch_cs<8>(groups_big, n_big, base, s);
}

}  // namespace gq
