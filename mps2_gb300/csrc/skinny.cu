// Tall-skinny block contractions: C = A . B where B is an MPO tensor.
//
// In the matvec (``lanczos_solver_impl.h:232-233, 243``) and in the
// environment growth (``two_site_update_finite_vmps_impl.h:297, 315``) the
// MPO-tensor contractions have a huge free dimension on the A side and only
// a handful of contracted (k) and B-free (n) values: m ~ 10^5-10^6, k and n
// of a few units, spread over many small blocks.  A 64x64 GEMM tile wastes
// almost all of its work on such shapes, and permuting A into matrix form
// costs a full extra pass, so these contractions get their own kernel:
//  * one thread per output row: consecutive threads take consecutive rows,
//    whose A elements are consecutive along A's last free leg, so a warp's
//    loads of A are contiguous (A is read in place through its leg strides,
//    no permute);
//  * the plan lists, for every contributing block pair, the A offsets of its
//    contracted indices and the B offsets of its (k, j) values, so a thread's
//    work per pair is K loads of A and K x N multiply-adds with the B values
//    read through the cache (the same address across the CTA), with no
//    staging and no barrier;
//  * every output column (up to 32 per pass) is accumulated in registers in
//    one pass over A;
//  * the CTA's output rows form one contiguous stretch of C and are written
//    back through shared memory in full, coalesced lines.
// Memory-bound by construction: A is read once per contributing block pair
// and C written once.  Sums run over pairs, then contracted indices, in plan
// order.
#include "gq_runtime.hpp"

namespace gq {

namespace {
constexpr int kSkRows = 256;    // output rows per CTA, one per thread
constexpr int kSkPool = 4096;   // output staging (doubles)

template <int JB>
__global__ void __launch_bounds__(kSkRows)
    skinny_kernel(const SkinnyItem *__restrict__ items, int nitems,
                  const SkinnyPair *__restrict__ pairs,
                  const int64_t *__restrict__ koffs, const int *__restrict__ bidx,
                  const double *__restrict__ A, const double *__restrict__ B,
                  double *__restrict__ C) {
  __shared__ double pool[kSkPool];
  // this CTA's output block: the last item whose first CTA is <= blockIdx.x
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (items[mid].cta0 <= (int)blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  const SkinnyItem it = items[lo];
  const int row0 = ((int)blockIdx.x - it.cta0) * kSkRows;
  const int tid = threadIdx.x;
  const int i = row0 + tid;
  const bool live = i < it.M;
  // the row's coordinates along A's free legs
  int fc[kSkMaxFree];
  {
    int rem = live ? i : 0;
#pragma unroll
    for (int t = kSkMaxFree - 1; t >= 0; --t) {
      fc[t] = 0;
      if (t < it.nfa) {
        fc[t] = rem % it.fa_dims[t];
        rem /= it.fa_dims[t];
      }
    }
  }
  const int N = it.N;
  for (int j0 = 0; j0 < N; j0 += JB) {
    const int jn = min(JB, N - j0);
    double acc[JB];
#pragma unroll
    for (int j = 0; j < JB; ++j) acc[j] = 0.0;
    if (live) {
      for (int p = it.pair_begin; p < it.pair_end; ++p) {
        const SkinnyPair P = pairs[p];
        int64_t ai = P.a_off;
#pragma unroll
        for (int t = 0; t < kSkMaxFree; ++t) ai += (int64_t)fc[t] * P.fa_str[t];
        const int64_t *__restrict__ ko = koffs + P.koff;
        const int *__restrict__ bi = bidx + P.bidx + j0;
#pragma unroll 2
        for (int k = 0; k < P.K; ++k) {
          const double av = __ldg(A + ai + __ldg(ko + k));
          const int *bk = bi + k * N;
#pragma unroll
          for (int j = 0; j < JB; ++j)
            if (j < jn) acc[j] = fma(av, __ldg(B + __ldg(bk + j)), acc[j]);
        }
      }
    }
    const int nrows = min(kSkRows, it.M - row0);
    if (jn == N) {
      // one pass holds every column: the CTA's rows are one contiguous
      // stretch of C, written through shared memory in full lines
      const int per = kSkPool / N;  // rows per round
      for (int r0 = 0; r0 < nrows; r0 += per) {
        const int rn = min(per, nrows - r0);
        if (tid >= r0 && tid < r0 + rn) {
#pragma unroll
          for (int j = 0; j < JB; ++j)
            if (j < jn) pool[(tid - r0) * N + j] = acc[j];
        }
        __syncthreads();
        double *c = C + it.c_off + (int64_t)(row0 + r0) * N;
        for (int e = tid; e < rn * N; e += kSkRows) c[e] = pool[e];
        __syncthreads();
      }
    } else if (live) {
      double *c = C + it.c_off + (int64_t)i * N + j0;
#pragma unroll
      for (int j = 0; j < JB; ++j)
        if (j < jn) c[j] = acc[j];
    }
  }
}
}  // namespace

bool skinny_eligible_sizes(int64_t a_elems, int64_t b_elems) {
  return b_elems <= 16384 && 32 * b_elems <= a_elems;
}

bool skinny_eligible(const Tensor &b, int64_t max_k, int64_t max_n) {
  return b.size() <= 16384 && max_k <= kSkMaxK && max_n <= 256;
}

int skinny_max_free_legs() { return kSkMaxFree; }

void launch_skinny(const ContractPlan &p, const double *A, const double *B, double *C) {
  if (p.sk_nitems == 0) return;
  prof_begin(kProfSkinny);
  auto s = stream();
  const unsigned grid = (unsigned)p.sk_nctas;
  const int ni = (int)p.sk_nitems;
  const int64_t *ko = p.sk_koffs.p;
  const int *bi = p.sk_bidx.p;
  switch (p.sk_jb) {
    case 2:
      skinny_kernel<2><<<grid, kSkRows, 0, s>>>(p.sk_items.p, ni, p.sk_pairs.p, ko, bi, A, B, C);
      break;
    case 4:
      skinny_kernel<4><<<grid, kSkRows, 0, s>>>(p.sk_items.p, ni, p.sk_pairs.p, ko, bi, A, B, C);
      break;
    case 8:
      skinny_kernel<8><<<grid, kSkRows, 0, s>>>(p.sk_items.p, ni, p.sk_pairs.p, ko, bi, A, B, C);
      break;
    case 16:
      skinny_kernel<16><<<grid, kSkRows, 0, s>>>(p.sk_items.p, ni, p.sk_pairs.p, ko, bi, A, B, C);
      break;
    default:
      skinny_kernel<32><<<grid, kSkRows, 0, s>>>(p.sk_items.p, ni, p.sk_pairs.p, ko, bi, A, B, C);
  }
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfSkinny, p.flops, 8.0 * (double)(p.a_elems + p.b_elems + p.out->size()));
}

int skinny_rows_per_cta() { return kSkRows; }

}  // namespace gq
