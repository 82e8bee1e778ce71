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
//  * the contributing block pairs of an output block are staged in shared
//    memory a chunk at a time (up to 16 pairs: their A offsets and strides,
//    the A offsets of every contracted index, and the B values), so the
//    per-pair work of a thread is a few multiply-adds with no barrier;
//  * every output column (up to 32) is accumulated in registers in one
//    pass over A;
//  * the CTA's output rows form one contiguous stretch of C and are written
//    back through shared memory in full, coalesced lines.
// Memory-bound by construction: A is read once per contributing block pair
// and C written once.
#include "gq_runtime.hpp"

namespace gq {

namespace {
constexpr int kSkRows = 256;     // output rows per CTA, one per thread
constexpr int kSkChunk = 16;     // block pairs staged per round
constexpr int kSkPoolK = 1024;   // staged contracted-index offsets per round
constexpr int kSkPoolB = 4096;   // staged B values per round (also the output staging)
constexpr int kSkMaxFree = 4;    // free legs of A

template <int JB>
__global__ void __launch_bounds__(kSkRows)
    skinny_kernel(const SkinnyItem *__restrict__ items, const SkinnyPair *__restrict__ pairs,
                  const double *__restrict__ A, const double *__restrict__ B,
                  double *__restrict__ C) {
  const SkinnyItem it = items[blockIdx.x];
  __shared__ int64_t s_aoff[kSkChunk];
  __shared__ int64_t s_fstr[kSkChunk][kSkMaxFree];
  __shared__ int s_K[kSkChunk], s_kb[kSkChunk];
  __shared__ int s_cnt, s_nfa;
  __shared__ int s_fdims[kSkMaxFree];
  __shared__ int64_t koff[kSkPoolK];
  __shared__ double pool[kSkPoolB];
  const int tid = threadIdx.x, lane = tid & 31;
  const int i = it.row0 + tid;
  const bool live = i < it.M;
  const bool any = it.pair_end > it.pair_begin;
  // the row's coordinates along A's free legs (the same dims for every
  // contributing pair of this output block)
  if (tid == 0) s_nfa = any ? pairs[it.pair_begin].nfa : 0;
  if (tid < kSkMaxFree) s_fdims[tid] = any ? pairs[it.pair_begin].fa_dims[tid] : 1;
  __syncthreads();
  const int nfa = s_nfa;
  int fc[kSkMaxFree];
  {
    int rem = live ? i : 0;
#pragma unroll
    for (int t = kSkMaxFree - 1; t >= 0; --t) {
      fc[t] = 0;
      if (t < nfa) {
        fc[t] = rem % s_fdims[t];
        rem /= s_fdims[t];
      }
    }
  }
  for (int j0 = 0; j0 < it.N; j0 += JB) {
    const int jn = min(JB, it.N - j0);
    double acc[JB];
#pragma unroll
    for (int j = 0; j < JB; ++j) acc[j] = 0.0;
    for (int p0 = it.pair_begin; p0 < it.pair_end;) {
      // ---- the chunk: leading pairs whose k offsets and B values fit -------
      if (tid < 32) {
        const int q = p0 + lane;
        const int K = (lane < kSkChunk && q < it.pair_end) ? pairs[q].K : 0;
        int sk = K;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, sk, o);
          if (lane >= o) sk += y;
        }
        const bool fits = lane < kSkChunk && q < it.pair_end && sk <= kSkPoolK &&
                          sk * JB <= kSkPoolB;
        const unsigned m = __ballot_sync(0xffffffffu, fits);
        if (fits) {
          s_K[lane] = K;
          s_kb[lane] = sk - K;
        }
        if (lane == 0) s_cnt = __ffs(~m) - 1;  // leading run of pairs that fit
      }
      __syncthreads();
      const int cnt = s_cnt;  // >= 1: one pair needs at most kSkMaxK offsets
      const int ktot = s_kb[cnt - 1] + s_K[cnt - 1];
      for (int e = tid; e < cnt * (1 + kSkMaxFree); e += kSkRows) {
        const int q = e / (1 + kSkMaxFree), t = e % (1 + kSkMaxFree);
        if (t == 0) s_aoff[q] = pairs[p0 + q].a_off;
        else s_fstr[q][t - 1] = t - 1 < nfa ? pairs[p0 + q].fa_str[t - 1] : 0;
      }
      for (int e = tid; e < ktot; e += kSkRows) {
        int q = 0;
        while (q + 1 < cnt && s_kb[q + 1] <= e) ++q;
        const SkinnyPair &P = pairs[p0 + q];
        int rem = e - s_kb[q];
        int64_t oa = 0;
        for (int t = P.nk - 1; t >= 0; --t) {
          oa += (int64_t)(rem % P.k_dims[t]) * P.ka_str[t];
          rem /= P.k_dims[t];
        }
        koff[e] = oa;
      }
      for (int e = tid; e < ktot * JB; e += kSkRows) {
        const int kk = e / JB, j = e % JB;
        int q = 0;
        while (q + 1 < cnt && s_kb[q + 1] <= kk) ++q;
        double val = 0.0;
        if (j < jn) {
          const SkinnyPair &P = pairs[p0 + q];
          int rem = kk - s_kb[q];
          int64_t ob = P.b_off;
          for (int t = P.nk - 1; t >= 0; --t) {
            ob += (int64_t)(rem % P.k_dims[t]) * P.kb_str[t];
            rem /= P.k_dims[t];
          }
          rem = j0 + j;
          for (int t = P.nfb - 1; t >= 0; --t) {
            ob += (int64_t)(rem % P.fb_dims[t]) * P.fb_str[t];
            rem /= P.fb_dims[t];
          }
          val = B[ob];
        }
        pool[e] = val;
      }
      __syncthreads();
      if (live) {
        for (int q = 0; q < cnt; ++q) {
          int64_t ai = s_aoff[q];
#pragma unroll
          for (int t = 0; t < kSkMaxFree; ++t) ai += (int64_t)fc[t] * s_fstr[q][t];
          const int kb = s_kb[q], K = s_K[q];
          for (int k = 0; k < K; ++k) {
            const double av = __ldg(A + ai + koff[kb + k]);
            const double *bv = pool + (kb + k) * JB;
#pragma unroll
            for (int j = 0; j < JB; ++j) acc[j] = fma(av, bv[j], acc[j]);
          }
        }
      }
      __syncthreads();  // the next chunk reuses the staging arrays
      p0 += cnt;
    }
    const int nrows = min(kSkRows, it.M - it.row0);
    if (jn == it.N) {
      // one pass holds every column: the CTA's rows are one contiguous
      // stretch of C, written through shared memory in full lines
      const int per = kSkPoolB / it.N;  // rows per round
      for (int r0 = 0; r0 < nrows; r0 += per) {
        const int rn = min(per, nrows - r0);
        if (tid >= r0 && tid < r0 + rn) {
#pragma unroll
          for (int j = 0; j < JB; ++j)
            if (j < jn) pool[(tid - r0) * it.N + j] = acc[j];
        }
        __syncthreads();
        double *c = C + it.c_off + (int64_t)(it.row0 + r0) * it.N;
        for (int e = tid; e < rn * it.N; e += kSkRows) c[e] = pool[e];
        __syncthreads();
      }
    } else if (live) {
      double *c = C + it.c_off + (int64_t)i * it.N + j0;
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
  const unsigned grid = (unsigned)p.sk_nitems;
  if (p.sk_jb == 8)
    skinny_kernel<8><<<grid, kSkRows, 0, s>>>(p.sk_items.p, p.sk_pairs.p, A, B, C);
  else if (p.sk_jb == 16)
    skinny_kernel<16><<<grid, kSkRows, 0, s>>>(p.sk_items.p, p.sk_pairs.p, A, B, C);
  else
    skinny_kernel<32><<<grid, kSkRows, 0, s>>>(p.sk_items.p, p.sk_pairs.p, A, B, C);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfSkinny, p.flops, 8.0 * (double)(p.a_elems + p.b_elems + p.out->size()));
}

int skinny_rows_per_cta() { return kSkRows; }

}  // namespace gq
