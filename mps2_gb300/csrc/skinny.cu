// Tall-skinny block contractions: C = A . B where B is an MPO tensor.
//
// In the matvec (``lanczos_solver_impl.h:232-233, 243``) and in the
// environment growth (``two_site_update_finite_vmps_impl.h:297, 315``) the
// MPO-tensor contractions have a huge free dimension on the A side and only
// a handful of contracted (k) and B-free (n) values: m ~ 10^5-10^6, k and n
// of a few units.  A 64x64 GEMM tile wastes almost all of its work on such
// shapes, and permuting A into matrix form costs a full extra pass, so these
// contractions get their own kernel: one thread per output row, A read in
// place through its leg strides (no permute), the small B block staged in
// shared memory, FP64 accumulation.  Memory-bound by construction: A is read
// once per contributing block pair and C written once.
#include "gq_runtime.hpp"

namespace gq {

namespace {
constexpr int kSkRows = 256;  // output rows per CTA

template <int JB>
__global__ void __launch_bounds__(kSkRows)
    skinny_kernel(const SkinnyItem *__restrict__ items, const SkinnyPair *__restrict__ pairs,
                  const double *__restrict__ A, const double *__restrict__ B,
                  double *__restrict__ C) {
  const SkinnyItem it = items[blockIdx.x];
  __shared__ SkinnyPair P;
  __shared__ double bsm[kSkMaxK * JB];
  __shared__ int64_t koff[kSkMaxK];
  const int i = it.row0 + threadIdx.x;
  for (int j0 = 0; j0 < it.N; j0 += JB) {
    const int jn = min(JB, it.N - j0);
    double acc[JB];
#pragma unroll
    for (int j = 0; j < JB; ++j) acc[j] = 0.0;
    for (int p = it.pair_begin; p < it.pair_end; ++p) {
      __syncthreads();
      if (threadIdx.x == 0) P = pairs[p];
      __syncthreads();
      for (int k = threadIdx.x; k < P.K; k += blockDim.x) {
        int rem = k;
        int64_t oa = 0;
        for (int t = P.nk - 1; t >= 0; --t) {
          oa += (int64_t)(rem % P.k_dims[t]) * P.ka_str[t];
          rem /= P.k_dims[t];
        }
        koff[k] = oa;
      }
      for (int e = threadIdx.x; e < P.K * JB; e += blockDim.x) {
        const int k = e / JB, j = e % JB;
        double v = 0.0;
        if (j < jn) {
          int rem = k;
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
          v = B[ob];
        }
        bsm[e] = v;
      }
      __syncthreads();
      if (i < it.M) {
        int rem = i;
        int64_t ai = P.a_off;
        for (int t = P.nfa - 1; t >= 0; --t) {
          ai += (int64_t)(rem % P.fa_dims[t]) * P.fa_str[t];
          rem /= P.fa_dims[t];
        }
        for (int k = 0; k < P.K; ++k) {
          const double a = A[ai + koff[k]];
#pragma unroll
          for (int j = 0; j < JB; ++j) acc[j] = fma(a, bsm[k * JB + j], acc[j]);
        }
      }
    }
    if (i < it.M) {
      double *c = C + it.c_off + (int64_t)i * it.N + j0;
      for (int j = 0; j < jn; ++j) c[j] = acc[j];
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
  prof_end(kProfSkinny, p.flops, 8.0 * (double)(p.a_elems + p.b_elems));
}

int skinny_rows_per_cta() { return kSkRows; }

}  // namespace gq
