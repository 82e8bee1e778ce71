// Block-sparse tensor contraction on the GPU.
//
// C = A . B over matching quantum-number sectors of the contracted legs
// (GraceQ/tensor ``Contract`` as called throughout gqmps2, e.g.
// ``lanczos_solver_impl.h:231-254`` and
// ``two_site_update_finite_vmps_impl.h:118-129, 290-317``).  Output legs are
// A's free legs in order, then B's free legs in order.
//
// Execution: every output block is a row-major M x N matrix (M = product of
// A's free dims, N = product of B's free dims).  Each block is cut into
// tiles; one CTA owns one tile and loops over every (A block, B block) pair
// that contributes to it, in a fixed order (output-stationary: no atomics,
// bitwise-reproducible).  A block is used in place when its legs are already
// ordered (free, contracted) or (contracted, free); otherwise one batched
// permute kernel reorders all of its blocks first.
#include <map>

#include "gq_runtime.hpp"

namespace gq {

namespace {

constexpr int kPermChunk = 16384;

bool is_identity(const std::vector<int> &p) {
  for (int i = 0; i < (int)p.size(); ++i)
    if (p[i] != i) return false;
  return true;
}

void build_perm_plan(const Tensor &t, const std::vector<int> &perm, PermPlan &pp) {
  pp.needed = true;
  pp.total = t.size();
  const int r = t.rank();
  std::vector<PermBlock> blocks;
  std::vector<PermChunk> chunks;
  blocks.reserve(t.nblocks());
  for (int64_t b = 0; b < t.nblocks(); ++b) {
    PermBlock pb{};
    pb.src_off = t.offs[b];
    pb.dst_off = t.offs[b];
    pb.n = t.block_size(b);
    pb.rank = r;
    int64_t sdims[kMaxRank], sstr[kMaxRank];
    for (int l = 0; l < r; ++l) sdims[l] = t.block_dim(b, l);
    int64_t s = 1;
    for (int l = r - 1; l >= 0; --l) {
      sstr[l] = s;
      s *= sdims[l];
    }
    for (int j = 0; j < r; ++j) {
      pb.dims[j] = (int)sdims[perm[j]];
      pb.sstride[j] = sstr[perm[j]];
    }
    blocks.push_back(pb);
    for (int64_t e = 0; e < pb.n; e += kPermChunk)
      chunks.push_back({(int)b, e, std::min<int64_t>(pb.n, e + kPermChunk)});
  }
  pp.blocks.upload(blocks);
  pp.chunks.upload(chunks);
  pp.nchunks = (int64_t)chunks.size();
}

__global__ void permute_blocks_kernel(const PermBlock *__restrict__ blocks,
                                      const PermChunk *__restrict__ chunks,
                                      const double *__restrict__ src, double *__restrict__ dst) {
  const PermChunk ch = chunks[blockIdx.x];
  __shared__ PermBlock pb;
  if (threadIdx.x == 0) pb = blocks[ch.block];
  __syncthreads();
  const int r = pb.rank;
  for (int64_t e = ch.begin + threadIdx.x; e < ch.end; e += blockDim.x) {
    int64_t rem = e, so = 0;
    for (int j = r - 1; j >= 0; --j) {
      const int64_t d = pb.dims[j];
      const int64_t i = rem % d;
      rem /= d;
      so += i * pb.sstride[j];
    }
    dst[pb.dst_off + e] = src[pb.src_off + so];
  }
}

void run_perm(const PermPlan &pp, const double *src, double *dst) {
  if (pp.nchunks == 0) return;
  prof_begin(kProfPermute);
  permute_blocks_kernel<<<(unsigned)pp.nchunks, 256, 0, stream()>>>(pp.blocks.p, pp.chunks.p, src,
                                                                      dst);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfPermute, 0.0, 16.0 * (double)pp.total);
}

}  // namespace

std::shared_ptr<ContractPlan> plan_contract(const Tensor &a, const Tensor &b,
                                            const std::vector<int> &axes_a,
                                            const std::vector<int> &axes_b,
                                            const Tensor *target, Precision prec) {
  const int ra = a.rank(), rb = b.rank(), nc = (int)axes_a.size();
  GQ_CHECK(nc == (int)axes_b.size() && nc >= 1, "contraction needs matching, non-empty axes");
  GQ_CHECK(a.nq == b.nq, "operands use different charge counts");
  std::vector<char> ca(ra, 0), cb(rb, 0);
  for (int i = 0; i < nc; ++i) {
    GQ_CHECK(axes_a[i] >= 0 && axes_a[i] < ra && !ca[axes_a[i]], "bad axes for A");
    GQ_CHECK(axes_b[i] >= 0 && axes_b[i] < rb && !cb[axes_b[i]], "bad axes for B");
    ca[axes_a[i]] = cb[axes_b[i]] = 1;
    const Index &ia = a.idx[axes_a[i]], &ib = b.idx[axes_b[i]];
    GQ_CHECK(ia.dir == -ib.dir && ia.same_sectors(ib),
             "contracted legs must carry the same sectors with opposite directions");
  }
  std::vector<int> free_a, free_b;
  for (int i = 0; i < ra; ++i)
    if (!ca[i]) free_a.push_back(i);
  for (int i = 0; i < rb; ++i)
    if (!cb[i]) free_b.push_back(i);
  GQ_CHECK(!free_a.empty() || !free_b.empty(), "full contraction to a scalar is not a GEMM");

  auto plan = std::make_shared<ContractPlan>();
  std::vector<Index> oidx;
  for (int f : free_a) oidx.push_back(a.idx[f]);
  for (int f : free_b) oidx.push_back(b.idx[f]);
  const QN odiv = a.div + b.div;

  // Operand layouts.
  std::vector<int> pa = free_a, pb = axes_b;
  pa.insert(pa.end(), axes_a.begin(), axes_a.end());
  pb.insert(pb.end(), free_b.begin(), free_b.end());
  std::vector<int> pa_t = axes_a, pb_t = free_b;
  pa_t.insert(pa_t.end(), free_a.begin(), free_a.end());
  pb_t.insert(pb_t.end(), axes_b.begin(), axes_b.end());

  // Group B blocks by their contracted-sector key.
  std::unordered_map<std::string, std::vector<int64_t>> bgroups;
  std::vector<int> key(nc);
  for (int64_t j = 0; j < b.nblocks(); ++j) {
    const int *c = b.block_coords(j);
    for (int i = 0; i < nc; ++i) key[i] = c[axes_b[i]];
    bgroups[Tensor::key(key.data(), nc)].push_back(j);
  }
  // Output block -> contributing pairs, in (A block, B block) order.
  struct Contrib { int64_t ablk, bblk; };
  std::map<std::vector<int>, std::vector<Contrib>> out;
  std::vector<int> oc(free_a.size() + free_b.size());
  for (int64_t i = 0; i < a.nblocks(); ++i) {
    const int *c = a.block_coords(i);
    for (int t = 0; t < nc; ++t) key[t] = c[axes_a[t]];
    auto it = bgroups.find(Tensor::key(key.data(), nc));
    if (it == bgroups.end()) continue;
    for (size_t t = 0; t < free_a.size(); ++t) oc[t] = c[free_a[t]];
    for (int64_t j : it->second) {
      const int *d = b.block_coords(j);
      for (size_t t = 0; t < free_b.size(); ++t) oc[free_a.size() + t] = d[free_b[t]];
      out[oc].push_back({i, j});
    }
  }

  if (target) {
    GQ_CHECK(target->idx.size() == oidx.size(), "target structure has the wrong rank");
    for (size_t l = 0; l < oidx.size(); ++l)
      GQ_CHECK(target->idx[l] == oidx[l], "target structure has different legs");
    plan->out = clone_structure(*target);
  } else {
    std::vector<std::vector<int>> blocks;
    blocks.reserve(out.size());
    for (auto &kv : out) blocks.push_back(kv.first);
    plan->out = make_structure(a.nq, oidx, odiv, blocks);
  }
  const Tensor &o = *plan->out;
  const size_t nfa = free_a.size();

  // Kernel choice.  The tensor-core form pads every block to 128 x 128 x 32
  // tiles; it is used when at least 30% of the padded work is useful (the
  // small MPO contractions, with k and n of a few units, stay on the FP64
  // kernel where they are memory-bound anyway).
  if (prec == kTF32x3) {
    double useful = 0.0, padded = 0.0;
    for (auto &kv : out) {
      int64_t m = 1, n = 1;
      for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[kv.first[l]];
      for (size_t l = nfa; l < kv.first.size(); ++l) n *= o.idx[l].dim[kv.first[l]];
      for (auto &cp : kv.second) {
        int64_t k = 1;
        for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
        useful += 2.0 * m * n * k;
        padded += 2.0 * ((m + 127) / 128 * 128.0) * ((n + 127) / 128 * 128.0) *
                  ((k + 31) / 32 * 32.0);
      }
    }
    plan->use_tc = padded > 0.0 && useful >= 0.3 * padded;
    plan->padded_flops = padded;
  }
  if (plan->use_tc) {
    build_tc_pack(a, free_a, axes_a, plan->ta);
    build_tc_pack(b, free_b, axes_b, plan->tb);
  } else {
    if (is_identity(pa)) {
      plan->transA = 0;
    } else if (is_identity(pa_t)) {
      plan->transA = 1;
    } else {
      plan->transA = 0;
      build_perm_plan(a, pa, plan->pa);
    }
    if (is_identity(pb)) {
      plan->transB = 0;
    } else if (is_identity(pb_t)) {
      plan->transB = 1;
    } else {
      plan->transB = 0;
      build_perm_plan(b, pb, plan->pb);
    }
  }

  const Precision kern = plan->use_tc ? kTF32x3 : kFP64;
  const int TM = gemm_tile_m(kern), TN = gemm_tile_n(kern);
  plan->tile_m = TM;
  plan->tile_n = TN;
  std::vector<GemmTile> tiles;
  std::vector<GemmPair> pairs;
  std::vector<char> touched(o.nblocks(), 0);
  for (auto &kv : out) {
    const int64_t ob = o.find(kv.first.data());
    GQ_CHECK(ob >= 0, "contraction produces a block missing from the target structure");
    touched[ob] = 1;
    int64_t m = 1, n = 1;
    for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[kv.first[l]];
    for (size_t l = nfa; l < kv.first.size(); ++l) n *= o.idx[l].dim[kv.first[l]];
    const int pbeg = (int)pairs.size();
    int64_t ksum = 0;
    for (auto &cp : kv.second) {
      int64_t k = 1;
      for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
      GemmPair gp{};
      gp.a_off = plan->use_tc ? plan->ta.base[cp.ablk] : a.offs[cp.ablk];
      gp.b_off = plan->use_tc ? plan->tb.base[cp.bblk] : b.offs[cp.bblk];
      gp.k = (int)k;
      gp.lda = (int)(plan->transA ? m : k);
      gp.ldb = (int)(plan->transB ? k : n);
      pairs.push_back(gp);
      ksum += k;
      plan->flops += 2.0 * (double)m * (double)n * (double)k;
    }
    const int pend = (int)pairs.size();
    for (int64_t r0 = 0; r0 < m; r0 += TM)
      for (int64_t c0 = 0; c0 < n; c0 += TN) {
        GemmTile t{};
        t.c_off = o.offs[ob];
        t.m = (int)m;
        t.n = (int)n;
        t.row0 = (int)r0;
        t.col0 = (int)c0;
        t.pair_begin = pbeg;
        t.pair_end = pend;
        t.work = ksum * std::min<int64_t>(TM, m - r0) * std::min<int64_t>(TN, n - c0);
        tiles.push_back(t);
      }
  }
  // Target blocks without contributions are written as zeros by empty tiles.
  for (int64_t ob = 0; ob < o.nblocks(); ++ob) {
    if (touched[ob]) continue;
    const int *c = o.block_coords(ob);
    int64_t m = 1, n = 1;
    for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[c[l]];
    for (size_t l = nfa; l < o.idx.size(); ++l) n *= o.idx[l].dim[c[l]];
    for (int64_t r0 = 0; r0 < m; r0 += TM)
      for (int64_t c0 = 0; c0 < n; c0 += TN) {
        GemmTile t{};
        t.c_off = o.offs[ob];
        t.m = (int)m;
        t.n = (int)n;
        t.row0 = (int)r0;
        t.col0 = (int)c0;
        t.pair_begin = t.pair_end = 0;
        t.work = 0;
        tiles.push_back(t);
      }
    plan->nzero_blocks++;
  }
  // Longest tiles first so the tail of the grid is short ones.
  std::stable_sort(tiles.begin(), tiles.end(),
                   [](const GemmTile &x, const GemmTile &y) { return x.work > y.work; });
  plan->ntiles = (int64_t)tiles.size();
  plan->tiles.upload(tiles);
  plan->pairs.upload(pairs);
  plan->a_elems = a.size();
  plan->b_elems = b.size();
  return plan;
}

namespace {
int64_t floats_as_doubles(int64_t f) { return (f + 1) / 2 + 8; }  // + slack for alignment
float *align16(double *p) {
  return reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(p) + 15) & ~(uintptr_t)15);
}
}  // namespace

int64_t contract_scratch(const ContractPlan &p) {
  if (p.use_tc)
    return (p.a_cached ? 0 : floats_as_doubles(p.ta.floats)) +
           (p.b_cached ? 0 : floats_as_doubles(p.tb.floats));
  return (p.pa.needed ? p.pa.total : 0) + (p.pb.needed ? p.pb.total : 0);
}

void cache_operand(ContractPlan &p, int which, const double *src) {
  if (!p.use_tc) return;
  if (which == 0) {
    p.a_packed.alloc(floats_as_doubles(p.ta.floats));
    run_tc_pack(p.ta, src, align16(p.a_packed.p));
    p.a_cached = true;
  } else {
    p.b_packed.alloc(floats_as_doubles(p.tb.floats));
    run_tc_pack(p.tb, src, align16(p.b_packed.p));
    p.b_cached = true;
  }
}

void run_contract(const ContractPlan &p, const double *a, const double *b, double *c,
                  double *scratch, Precision) {
  if (p.use_tc) {
    double *s = scratch;
    const float *A, *B;
    if (p.a_cached) {
      A = align16(p.a_packed.p);
    } else {
      run_tc_pack(p.ta, a, align16(s));
      A = align16(s);
      s += floats_as_doubles(p.ta.floats);
    }
    if (p.b_cached) {
      B = align16(p.b_packed.p);
    } else {
      run_tc_pack(p.tb, b, align16(s));
      B = align16(s);
    }
    if (p.ntiles > 0) launch_gemm_tf32x3(p, A, B, c);
    return;
  }
  const double *A = a, *B = b;
  double *s = scratch;
  if (p.pa.needed) {
    run_perm(p.pa, a, s);
    A = s;
    s += p.pa.total;
  }
  if (p.pb.needed) {
    run_perm(p.pb, b, s);
    B = s;
  }
  if (p.ntiles == 0) return;
  launch_gemm_fp64(p, A, B, c);
}

void check_device_errors() {
  int h = 0;
  GQ_CUDA(cudaMemcpyAsync(&h, tc_error_flag(), sizeof(int), cudaMemcpyDeviceToHost, stream()));
  sync();
  if (h != 0) {
    GQ_CUDA(cudaMemsetAsync(tc_error_flag(), 0, sizeof(int), stream()));
    fail(kCudaError, "a tensor-core GEMM hit its wait limit and stopped early");
  }
}

TensorPtr contract(const Tensor &a, const Tensor &b, const std::vector<int> &axes_a,
                   const std::vector<int> &axes_b, Precision prec, double *flops_out) {
  auto plan = plan_contract(a, b, axes_a, axes_b, nullptr, prec);
  auto out = clone_structure(*plan->out);
  out->allocate();
  DevBuf scratch(contract_scratch(*plan));
  run_contract(*plan, a.data.p, b.data.p, out->data.p, scratch.p, prec);
  if (flops_out) *flops_out = plan->flops;
  return out;
}

// ---------------------------------------------------------------------------
// FP64 grouped GEMM (plain form).  64x64 output tile per CTA, 256 threads,
// 4x4 register micro-tile per thread, K staged through shared memory in
// steps of 16.  Ragged edges are zero-filled on load and masked on store.
// ---------------------------------------------------------------------------
namespace {
constexpr int kBM = 64, kBN = 64, kBK = 16;

template <int TA, int TB>
__global__ void __launch_bounds__(256)
    gemm_fp64_kernel(const GemmTile *__restrict__ tiles, const GemmPair *__restrict__ pairs,
                     const double *__restrict__ A, const double *__restrict__ B,
                     double *__restrict__ C) {
  __shared__ double As[kBK][kBM];
  __shared__ double Bs[kBK][kBN];
  const GemmTile t = tiles[blockIdx.x];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int p = t.pair_begin; p < t.pair_end; ++p) {
    const GemmPair pr = pairs[p];
    const double *Ab = A + pr.a_off;
    const double *Bb = B + pr.b_off;
    for (int k0 = 0; k0 < pr.k; k0 += kBK) {
#pragma unroll
      for (int it = 0; it < (kBM * kBK) / 256; ++it) {
        const int i = tid + it * 256;
        int r, kk;
        if (TA == 0) { kk = i % kBK; r = i / kBK; } else { r = i % kBM; kk = i / kBM; }
        const int gr = t.row0 + r, gk = k0 + kk;
        double v = 0.0;
        if (gr < t.m && gk < pr.k)
          v = TA == 0 ? Ab[(int64_t)gr * pr.lda + gk] : Ab[(int64_t)gk * pr.lda + gr];
        As[kk][r] = v;
      }
#pragma unroll
      for (int it = 0; it < (kBN * kBK) / 256; ++it) {
        const int i = tid + it * 256;
        int c, kk;
        if (TB == 0) { c = i % kBN; kk = i / kBN; } else { kk = i % kBK; c = i / kBK; }
        const int gc = t.col0 + c, gk = k0 + kk;
        double v = 0.0;
        if (gc < t.n && gk < pr.k)
          v = TB == 0 ? Bb[(int64_t)gk * pr.ldb + gc] : Bb[(int64_t)gc * pr.ldb + gk];
        Bs[kk][c] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kBK; ++kk) {
        double av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
      }
      __syncthreads();
    }
  }
  double *Cb = C + t.c_off;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = t.row0 + ty + 16 * i;
    if (gr >= t.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gc = t.col0 + tx + 16 * j;
      if (gc < t.n) Cb[(int64_t)gr * t.n + gc] = acc[i][j];
    }
  }
}
}  // namespace

void launch_gemm_fp64(const ContractPlan &p, const double *A, const double *B, double *C) {
  const unsigned grid = (unsigned)p.ntiles;
  auto s = stream();
  prof_begin(kProfGemmFp64);
  if (p.transA == 0 && p.transB == 0)
    gemm_fp64_kernel<0, 0><<<grid, 256, 0, s>>>(p.tiles.p, p.pairs.p, A, B, C);
  else if (p.transA == 0 && p.transB == 1)
    gemm_fp64_kernel<0, 1><<<grid, 256, 0, s>>>(p.tiles.p, p.pairs.p, A, B, C);
  else if (p.transA == 1 && p.transB == 0)
    gemm_fp64_kernel<1, 0><<<grid, 256, 0, s>>>(p.tiles.p, p.pairs.p, A, B, C);
  else
    gemm_fp64_kernel<1, 1><<<grid, 256, 0, s>>>(p.tiles.p, p.pairs.p, A, B, C);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfGemmFp64, p.flops, 8.0 * (double)(p.a_elems + p.b_elems));
}

}  // namespace gq
