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
#include <array>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>

#include "gq_runtime.hpp"

namespace gq {

namespace {

constexpr int kPermChunk = 16384;

bool is_identity(const std::vector<int> &p) {
  for (int i = 0; i < (int)p.size(); ++i)
    if (p[i] != i) return false;
  return true;
}

// Permute the blocks with used[b] != 0 (all if used is null) into the same
// offsets of the destination buffer.
void build_perm_plan(const Tensor &t, const std::vector<int> &perm, PermPlan &pp,
                     const std::vector<char> *used = nullptr) {
  pp.needed = true;
  pp.total = t.size();
  pp.moved = 0;
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
    if (used && !(*used)[b]) continue;
    pp.moved += pb.n;
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
  prof_end(kProfPermute, 0.0, 16.0 * (double)pp.moved);
}

}  // namespace

namespace {
std::shared_ptr<ContractPlan> build_plan(const Tensor &a, const Tensor &b,
                                         const std::vector<int> &axes_a,
                                         const std::vector<int> &axes_b, const Tensor *target,
                                         Precision prec, double tc_frac);

// 128-bit fingerprint of a plan's inputs: two independent 64-bit mixes
// (FNV-1a and a splitmix64 chain) over every structural word.
struct Fingerprint {
  uint64_t h0 = 1469598103934665603ull, h1 = 0x243f6a8885a308d3ull;
  void add(uint64_t x) {
    h0 = (h0 ^ x) * 1099511628211ull;
    uint64_t z = h1 + x + 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    h1 = z ^ (z >> 31);
  }
  void add_tensor(const Tensor &t) {
    add((uint64_t)t.nq);
    add((uint64_t)t.rank());
    for (const Index &ix : t.idx) {
      add((uint64_t)(int64_t)ix.dir);
      add((uint64_t)ix.qn.size());
      for (size_t k = 0; k < ix.qn.size(); ++k) {
        for (int q = 0; q < t.nq; ++q) add((uint64_t)(int64_t)ix.qn[k].v[q]);
        add((uint64_t)ix.dim[k]);
      }
    }
    for (int q = 0; q < t.nq; ++q) add((uint64_t)(int64_t)t.div.v[q]);
    add((uint64_t)t.nblocks());
    for (int c : t.coords) add((uint64_t)(int64_t)c);
  }
};

struct PlanKey {
  uint64_t h0, h1;
  bool operator==(const PlanKey &o) const { return h0 == o.h0 && h1 == o.h1; }
};
struct PlanKeyHash {
  size_t operator()(const PlanKey &k) const { return (size_t)k.h0; }
};

int64_t plan_device_bytes(const ContractPlan &p) {
  auto arr = [](const auto &d) { return d.n * (int64_t)sizeof(*d.p); };
  return arr(p.sk_items) + arr(p.sk_pairs) + arr(p.tiles) + arr(p.pairs) + arr(p.tiles_tc) +
         arr(p.pairs_tc) + arr(p.tiles_oz) + arr(p.pairs_oz) + arr(p.zero_blocks) +
         arr(p.pa.blocks) + arr(p.pa.chunks) + arr(p.pb.blocks) + arr(p.pb.chunks) +
         arr(p.ta.blocks_dev) + arr(p.ta.tasks_dev) + arr(p.tb.blocks_dev) +
         arr(p.tb.tasks_dev) + arr(p.oa.blocks_dev) + arr(p.oa.tasks_dev) +
         arr(p.ob.blocks_dev) + arr(p.ob.tasks_dev);
}

void release_operand_packs(ContractPlan &p) {
  p.a_packed.release();
  p.b_packed.release();
  p.a_oz.release();
  p.b_oz.release();
  p.a_cached = p.b_cached = p.a_oz_cached = p.b_oz_cached = false;
}

constexpr size_t kPlanCacheEntries = 8192;
constexpr int64_t kPlanCacheBytes = int64_t(8) << 30;  // device work lists
}  // namespace

struct PlanCache {
  struct Entry {
    std::shared_ptr<ContractPlan> plan;
    bool in_use = false;
    uint64_t last = 0;
    int64_t bytes = 0;
  };
  std::unordered_map<PlanKey, Entry, PlanKeyHash> map;
  uint64_t tick = 0;
  int64_t bytes = 0;

  // Least recently used entries not in use go first.
  void make_room(int64_t need) {
    while (!map.empty() && (map.size() >= kPlanCacheEntries || bytes + need > kPlanCacheBytes)) {
      auto victim = map.end();
      for (auto it = map.begin(); it != map.end(); ++it)
        if (!it->second.in_use && (victim == map.end() || it->second.last < victim->second.last))
          victim = it;
      if (victim == map.end()) return;
      bytes -= victim->second.bytes;
      map.erase(victim);
    }
  }
};

namespace {
// The holder's handle on a cached plan: when the last copy goes, the plan's
// operand packs are released and the entry may be handed out again.
std::shared_ptr<ContractPlan> lend(const std::shared_ptr<PlanCache> &cache, const PlanKey &key,
                                   PlanCache::Entry &e) {
  e.in_use = true;
  e.last = ++cache->tick;
  std::shared_ptr<ContractPlan> master = e.plan;
  return std::shared_ptr<ContractPlan>(master.get(), [cache, key, master](ContractPlan *p) {
    release_operand_packs(*p);
    auto it = cache->map.find(key);
    if (it != cache->map.end() && it->second.plan.get() == p) it->second.in_use = false;
  });
}

bool plan_cache_on() {
  static const bool off = std::getenv("GQ_NO_PLAN_CACHE") != nullptr;
  return !off;
}
}  // namespace

std::shared_ptr<ContractPlan> plan_contract(const Tensor &a, const Tensor &b,
                                            const std::vector<int> &axes_a,
                                            const std::vector<int> &axes_b,
                                            const Tensor *target, Precision prec,
                                            double tc_frac) {
  struct PlanTimer {  // host planning time, added to the profiler on every exit
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    ~PlanTimer() {
      prof_host(kProfHostPlan,
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
  } plan_timer;
  if (!plan_cache_on()) return build_plan(a, b, axes_a, axes_b, target, prec, tc_frac);
  Fingerprint f;
  f.add(0x706c616e31ull);  // layout version of the key
  f.add_tensor(a);
  f.add_tensor(b);
  f.add(axes_a.size());
  for (int x : axes_a) f.add((uint64_t)(int64_t)x);
  for (int x : axes_b) f.add((uint64_t)(int64_t)x);
  f.add(target ? 1 : 0);
  if (target) f.add_tensor(*target);
  f.add((uint64_t)prec);
  f.add(autotune_on() ? 1 : 0);  // plans carry the autotuner key only when it is on
  uint64_t fb;
  std::memcpy(&fb, &tc_frac, sizeof(fb));
  f.add(fb);
  const PlanKey key{f.h0, f.h1};
  Lane &l = lane();
  if (!l.plan_cache) l.plan_cache = std::make_shared<PlanCache>();
  auto &cache = l.plan_cache;
  auto it = cache->map.find(key);
  if (it != cache->map.end()) {
    if (!it->second.in_use) return lend(cache, key, it->second);
    return build_plan(a, b, axes_a, axes_b, target, prec, tc_frac);  // held: a private plan
  }
  auto p = build_plan(a, b, axes_a, axes_b, target, prec, tc_frac);
  const int64_t bytes = plan_device_bytes(*p);
  cache->make_room(bytes);
  auto &e = cache->map[key];
  e.plan = p;
  e.bytes = bytes;
  cache->bytes += bytes;
  return lend(cache, key, e);
}

namespace {
// Block coordinates packed 16 bits per leg (up to 8 legs), first leg most
// significant: comparing keys compares the coordinates lexicographically.
struct PackedKey {
  uint64_t hi, lo;
  bool operator<(const PackedKey &o) const { return hi != o.hi ? hi < o.hi : lo < o.lo; }
  bool operator==(const PackedKey &o) const { return hi == o.hi && lo == o.lo; }
};
struct Contrib { int64_t ablk, bblk; };
struct IntSpan {
  const int *p;
  size_t n;
  const int *data() const { return p; }
  size_t size() const { return n; }
  int operator[](size_t i) const { return p[i]; }
};
struct ContribSpan {
  const Contrib *b, *e;
  const Contrib *begin() const { return b; }
  const Contrib *end() const { return e; }
  size_t size() const { return (size_t)(e - b); }
  const Contrib &operator[](size_t i) const { return b[i]; }
};
struct OutGroup {  // an output block: its coordinates and its block pairs
  IntSpan first;
  ContribSpan second;
};

std::shared_ptr<ContractPlan> build_plan(const Tensor &a, const Tensor &b,
                                         const std::vector<int> &axes_a,
                                         const std::vector<int> &axes_b, const Tensor *target,
                                         Precision prec, double tc_frac) {
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

  // Block pairs.  B blocks are grouped by their contracted-sector key; every
  // (A block, B block) pair is tagged with its output block's coordinates
  // packed 16 bits per leg, first leg most significant, and the pairs are
  // sorted stably by that tag: output blocks come in ascending coordinate
  // order, the pairs of one block in (A block, B block) order.
  const int ro = (int)(free_a.size() + free_b.size());
  for (const Tensor *t : {&a, &b})
    for (const Index &ix : t->idx)
      GQ_CHECK(ix.nsec() < 65536, "a leg with 65536 or more sectors");
  auto pack = [](const int *c, const int *legs, int n) {
    PackedKey k{0, 0};
    for (int t = 0; t < n; ++t) {
      const uint64_t v = (uint64_t)(legs ? c[legs[t]] : c[t]);
      if (t < 4) k.hi |= v << (48 - 16 * t);
      else k.lo |= v << (48 - 16 * (t - 4));
    }
    return k;
  };
  std::vector<std::pair<PackedKey, int64_t>> bkeys((size_t)b.nblocks());
  for (int64_t j = 0; j < b.nblocks(); ++j) bkeys[j] = {pack(b.block_coords(j), axes_b.data(), nc), j};
  std::stable_sort(bkeys.begin(), bkeys.end(),
                   [](const auto &x, const auto &y) { return x.first < y.first; });
  struct PairRec { PackedKey okey; int64_t ablk, bblk; };
  std::vector<PairRec> prs;
  {
    int oc[kMaxRank];
    for (int64_t i = 0; i < a.nblocks(); ++i) {
      const int *c = a.block_coords(i);
      const PackedKey k = pack(c, axes_a.data(), nc);
      auto lo = std::lower_bound(bkeys.begin(), bkeys.end(), k,
                                 [](const auto &x, const PackedKey &y) { return x.first < y; });
      for (auto it = lo; it != bkeys.end() && it->first == k; ++it) {
        const int *d = b.block_coords(it->second);
        for (size_t t = 0; t < free_a.size(); ++t) oc[t] = c[free_a[t]];
        for (size_t t = 0; t < free_b.size(); ++t) oc[free_a.size() + t] = d[free_b[t]];
        prs.push_back({pack(oc, nullptr, ro), i, it->second});
      }
    }
  }
  std::stable_sort(prs.begin(), prs.end(),
                   [](const PairRec &x, const PairRec &y) { return x.okey < y.okey; });
  // Output blocks: coordinates (flat) and their pair ranges.
  std::vector<Contrib> contribs(prs.size());
  std::vector<int> ocoords;
  std::vector<size_t> obeg;
  for (size_t q = 0; q < prs.size(); ++q) {
    contribs[q] = {prs[q].ablk, prs[q].bblk};
    if (q == 0 || !(prs[q].okey == prs[q - 1].okey)) {
      obeg.push_back(q);
      const int *c = a.block_coords(prs[q].ablk), *d = b.block_coords(prs[q].bblk);
      for (size_t t = 0; t < free_a.size(); ++t) ocoords.push_back(c[free_a[t]]);
      for (size_t t = 0; t < free_b.size(); ++t) ocoords.push_back(d[free_b[t]]);
    }
  }
  obeg.push_back(prs.size());
  std::vector<OutGroup> out(obeg.size() - 1);
  for (size_t g = 0; g + 1 < obeg.size(); ++g)
    out[g] = {IntSpan{ocoords.data() + g * ro, (size_t)ro},
              ContribSpan{contribs.data() + obeg[g], contribs.data() + obeg[g + 1]}};
  { std::vector<PairRec>().swap(prs); }

  if (target) {
    GQ_CHECK(target->idx.size() == oidx.size(), "target structure has the wrong rank");
    for (size_t l = 0; l < oidx.size(); ++l)
      GQ_CHECK(target->idx[l] == oidx[l], "target structure has different legs");
    plan->out = clone_structure(*target);
  } else {
    plan->out = make_structure_sorted(a.nq, oidx, odiv, ocoords);
  }
  const Tensor &o = *plan->out;
  const size_t nfa = free_a.size();

  // Small B (an MPO tensor): the tall-skinny kernel reads A in place.  B
  // must be small in absolute terms and tiny next to A, so a two-site state
  // contracted with an environment never lands here.
  if (skinny_eligible_sizes(a.size(), b.size())) {
    int64_t max_k = 0, max_n = 0, kn = 0;
    for (auto &kv : out) {
      int64_t n = 1;
      for (size_t l = nfa; l < kv.first.size(); ++l) n *= o.idx[l].dim[kv.first[l]];
      max_n = std::max(max_n, n);
      for (auto &cp : kv.second) {
        int64_t k = 1;
        for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
        max_k = std::max(max_k, k);
        kn += k * n;
      }
    }
    // the plan lists every pair's (k, j) B offsets: keep that list small
    if (skinny_eligible(b, max_k, max_n) && (int)free_a.size() <= skinny_max_free_legs() &&
        kn <= (int64_t(1) << 26)) {
      auto strides = [](const Tensor &t, int64_t blk, int64_t *str) {
        int64_t s = 1;
        for (int l = t.rank() - 1; l >= 0; --l) {
          str[l] = s;
          s *= t.block_dim(blk, l);
        }
      };
      std::vector<SkinnyPair> sp;
      std::vector<SkinnyItem> items;
      std::vector<int64_t> koffs;
      std::vector<int> bidx;
      std::vector<char> touched(o.nblocks(), 0);
      const int rows = skinny_rows_per_cta();
      int64_t nctas = 0;
      auto add_items = [&](int64_t c_off, int64_t m, int64_t n, int pb, int pe,
                           const int *fdims, int nf) {
        if (m == 0 || n == 0) return;
        SkinnyItem it{};
        it.c_off = c_off;
        it.M = (int)m;
        it.N = (int)n;
        it.cta0 = (int)nctas;
        it.pair_begin = pb;
        it.pair_end = pe;
        it.nfa = nf;
        for (int t = 0; t < kSkMaxFree; ++t) it.fa_dims[t] = t < nf ? fdims[t] : 1;
        items.push_back(it);
        nctas += (m + rows - 1) / rows;
      };
      const int nfree = (int)free_a.size();
      // The A offsets of the contracted indices depend on the A block only,
      // the B offsets of the (k, j) values on the B block only: listed once
      // per block, shared by its pairs.
      std::vector<int> a_list(a.nblocks(), -1), b_list(b.nblocks(), -1);
      auto a_offsets = [&](int64_t ablk, const int64_t *sa, int K) {
        if (a_list[ablk] < 0) {
          a_list[ablk] = (int)koffs.size();
          for (int e = 0; e < K; ++e) {  // last contracted leg fastest
            int rem = e;
            int64_t oa = 0;
            for (int t = nc - 1; t >= 0; --t) {
              const int d = (int)a.block_dim(ablk, axes_a[t]);
              oa += (int64_t)(rem % d) * sa[axes_a[t]];
              rem /= d;
            }
            koffs.push_back(oa);
          }
        }
        return a_list[ablk];
      };
      auto b_offsets = [&](int64_t bblk, int K, int64_t n) {
        if (b_list[bblk] < 0) {
          int64_t sb[kMaxRank];
          strides(b, bblk, sb);
          b_list[bblk] = (int)bidx.size();
          for (int e = 0; e < K; ++e) {  // j over B's free legs, last fastest
            int rem = e;
            int64_t obk = b.offs[bblk];
            for (int t = nc - 1; t >= 0; --t) {
              const int d = (int)b.block_dim(bblk, axes_b[t]);
              obk += (int64_t)(rem % d) * sb[axes_b[t]];
              rem /= d;
            }
            for (int64_t j = 0; j < n; ++j) {
              int64_t rj = j, o2 = obk;
              for (int t = (int)free_b.size() - 1; t >= 0; --t) {
                const int64_t d = b.block_dim(bblk, free_b[t]);
                o2 += (rj % d) * sb[free_b[t]];
                rj /= d;
              }
              bidx.push_back((int)o2);
            }
          }
        }
        return b_list[bblk];
      };
      for (auto &kv : out) {
        const int64_t ob = o.find(kv.first.data());
        GQ_CHECK(ob >= 0, "contraction produces a block missing from the target structure");
        touched[ob] = 1;
        int64_t m = 1, n = 1;
        for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[kv.first[l]];
        for (size_t l = nfa; l < kv.first.size(); ++l) n *= o.idx[l].dim[kv.first[l]];
        const int pb = (int)sp.size();
        int fdims[kSkMaxFree] = {1, 1, 1, 1};
        for (auto &cp : kv.second) {
          int64_t sa[kMaxRank];
          strides(a, cp.ablk, sa);
          SkinnyPair q{};
          q.a_off = a.offs[cp.ablk];
          q.K = 1;
          for (int t = 0; t < nc; ++t) q.K *= (int)a.block_dim(cp.ablk, axes_a[t]);
          for (int t = 0; t < nfree; ++t) {
            fdims[t] = (int)a.block_dim(cp.ablk, free_a[t]);
            q.fa_str[t] = sa[free_a[t]];
          }
          q.koff = a_offsets(cp.ablk, sa, q.K);
          q.bidx = b_offsets(cp.bblk, q.K, n);
          sp.push_back(q);
          plan->flops += 2.0 * (double)m * (double)n * (double)q.K;
        }
        add_items(o.offs[ob], m, n, pb, (int)sp.size(), fdims, nfree);
      }
      for (int64_t ob = 0; ob < o.nblocks(); ++ob) {
        if (touched[ob]) continue;
        const int *c = o.block_coords(ob);
        int64_t m = 1, n = 1;
        for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[c[l]];
        for (size_t l = nfa; l < o.idx.size(); ++l) n *= o.idx[l].dim[c[l]];
        int fdims[kSkMaxFree] = {1, 1, 1, 1};
        for (int t = 0; t < nfree; ++t) fdims[t] = (int)o.idx[t].dim[c[t]];
        add_items(o.offs[ob], m, n, 0, 0, fdims, nfree);
        plan->nzero_blocks++;
      }
      plan->use_skinny = true;
      plan->sk_jb = max_n <= 2 ? 2 : max_n <= 4 ? 4 : max_n <= 8 ? 8 : max_n <= 16 ? 16 : 32;
      GQ_CHECK(nctas < (int64_t(1) << 31), "tall-skinny launch too large");
      plan->sk_nitems = (int64_t)items.size();
      plan->sk_nctas = nctas;
      plan->sk_items.upload(items);
      plan->sk_pairs.upload(sp);
      plan->sk_koffs.upload(koffs);
      plan->sk_bidx.upload(bidx);
      plan->a_elems = a.size();
      plan->b_elems = b.size();
      return plan;
    }
  }

  // Per output block kernel choice: the FP64 tiles (64 x 64), 3xTF32 tiles
  // (128 x 128) or FP64-accurate tiles (128 x 96), each padding a block to
  // whole tiles (k to multiples of 32 on the tensor cores).
  //  * The form's own tensor-core kernel takes a block when at least 2%
  //    (3xTF32) or 3% (FP64-accurate) of its padded work is useful: those
  //    rates are a few hundred and ~35 times this part's FP64 rate.
  //  * Otherwise (with the default threshold or an autotuner candidate below
  //    1; the candidate above 1 keeps everything else on FP64 tiles) a block
  //    goes to the FP64-accurate kernel when its padded work there costs
  //    less time than the FP64 kernel's padded tiles: thin blocks (a few
  //    rows or columns, long k) waste most of either tile and the FP64 pipe
  //    of this part is ~20x slower.  In the
  //    split form too: there the thin blocks keep FP64 accuracy (moved to
  //    3xTF32 they shift its Lanczos convergence enough to leave the
  //    per-sweep energy parity of 1e-9).
  //  * The rest -- tiny blocks and MPO contractions -- stays on the FP64
  //    kernel, where it is memory-bound anyway.  The FP64-accurate kernel's
  //    exact running sums cover k <= oz_max_k().
  enum Kind : int { kKindFp64 = 0, kKindTf32 = 1, kKindOz = 2 };
  struct OutBlock { int64_t ob, m, n; const ContribSpan *pairs; int kind; };
  std::vector<OutBlock> obs;
  obs.reserve(out.size());
  std::vector<char> touched(o.nblocks(), 0);
  bool any_tf32 = false, any_oz = false, any_fp = false;
  for (auto &kv : out) {
    const int64_t ob = o.find(kv.first.data());
    GQ_CHECK(ob >= 0, "contraction produces a block missing from the target structure");
    touched[ob] = 1;
    int64_t m = 1, n = 1;
    for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[kv.first[l]];
    for (size_t l = nfa; l < kv.first.size(); ++l) n *= o.idx[l].dim[kv.first[l]];
    int kind = kKindFp64;
    if (prec == kTF32x3 || prec == kFP64TC) {
      const int TM = prec == kTF32x3 ? 128 : oz_tile_m();
      const int TN = prec == kTF32x3 ? 128 : oz_tile_n();
      const int OM = oz_tile_m(), ON = oz_tile_n();
      const double frac = tc_frac >= 0.0 ? tc_frac : (prec == kTF32x3 ? 0.02 : 0.03);
      plan->tc_frac = frac;
      double useful = 0.0, padded = 0.0, padded_oz = 0.0, padded_fp64 = 0.0;
      int64_t ksum = 0;
      for (auto &cp : kv.second) {
        int64_t k = 1;
        for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
        const double kp = (k + 31) / 32 * 32.0;
        useful += 2.0 * m * n * k;
        padded += 2.0 * (double)((m + TM - 1) / TM * TM) * (double)((n + TN - 1) / TN * TN) * kp;
        padded_oz += 2.0 * (double)((m + OM - 1) / OM * OM) * (double)((n + ON - 1) / ON * ON) * kp;
        padded_fp64 += 2.0 * (double)((m + 63) / 64 * 64) * (double)((n + 63) / 64 * 64) * k;
        ksum += (k + 31) / 32 * 32;
      }
      const bool oz_ok = ksum <= oz_max_k();
      if (useful >= frac * padded && (prec == kTF32x3 || oz_ok))
        kind = prec == kTF32x3 ? kKindTf32 : kKindOz;
      else if (tc_frac < 1.0 && oz_ok && padded_oz < 20.0 * padded_fp64)
        kind = kKindOz;
      if (kind == kKindTf32) plan->padded_flops += padded;
      if (kind == kKindOz) plan->padded_flops += padded_oz;
    }
    any_tf32 |= kind == kKindTf32;
    any_oz |= kind == kKindOz;
    any_fp |= kind == kKindFp64;
    obs.push_back({ob, m, n, &kv.second, kind});
  }
  // autotuner key: the 16 heaviest output blocks' (log2 m, log2 n, log2 k of
  // their largest pair) and log2 of the block count, hashed (FNV-1a); only
  // the autotuner reads it
  if (autotune_on()) {
    std::vector<std::array<int, 4>> h;
    for (auto &b0 : obs) {
      int64_t kmax = 1;
      for (auto &cp : *b0.pairs) {
        int64_t k = 1;
        for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
        kmax = std::max(kmax, k);
      }
      auto lg = [](int64_t x) { int r = 0; while ((x >>= 1) > 0) ++r; return r; };
      h.push_back({lg(b0.m) + lg(b0.n) + lg(kmax), lg(b0.m), lg(b0.n), lg(kmax)});
    }
    std::sort(h.begin(), h.end(), [](const std::array<int, 4> &x, const std::array<int, 4> &y) {
      return x > y;
    });
    uint64_t hs = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { hs = (hs ^ v) * 1099511628211ull; };
    int nb = 0;
    for (int64_t x = (int64_t)obs.size(); x > 1; x >>= 1) ++nb;
    mix((uint64_t)nb);
    for (size_t i = 0; i < h.size() && i < 16; ++i)
      for (int j = 1; j < 4; ++j) mix((uint64_t)h[i][j]);
    plan->signature = hs;
  }
  // target blocks without contributions are written as zeros by FP64 tiles
  for (int64_t ob = 0; ob < o.nblocks(); ++ob)
    if (!touched[ob]) { any_fp = true; plan->nzero_blocks++; }

  plan->use_tc = any_tf32;
  plan->use_oz = any_oz;
  // operand blocks read by each kernel's tiles: each pack or permute covers
  // only its own
  std::vector<char> a_use[3], b_use[3];
  for (int k = 0; k < 3; ++k) {
    a_use[k].assign(a.nblocks(), 0);
    b_use[k].assign(b.nblocks(), 0);
  }
  for (auto &b0 : obs)
    for (auto &cp : *b0.pairs) {
      a_use[b0.kind][cp.ablk] = 1;
      b_use[b0.kind][cp.bblk] = 1;
    }
  std::vector<char> &a_fp = a_use[kKindFp64], &b_fp = b_use[kKindFp64];
  if (plan->use_tc) {
    build_tc_pack(a, free_a, axes_a, plan->ta, &a_use[kKindTf32]);
    build_tc_pack(b, free_b, axes_b, plan->tb, &b_use[kKindTf32]);
  }
  if (plan->use_oz) {
    build_oz_pack(a, free_a, axes_a, oz_tile_m(), plan->oa, &a_use[kKindOz]);
    build_oz_pack(b, free_b, axes_b, oz_tile_n(), plan->ob, &b_use[kKindOz]);
  }
  if (any_fp) {
    if (is_identity(pa)) {
      plan->transA = 0;
    } else if (is_identity(pa_t)) {
      plan->transA = 1;
    } else {
      plan->transA = 0;
      build_perm_plan(a, pa, plan->pa, &a_fp);
    }
    if (is_identity(pb)) {
      plan->transB = 0;
    } else if (is_identity(pb_t)) {
      plan->transB = 1;
    } else {
      plan->transB = 0;
      build_perm_plan(b, pb, plan->pb, &b_fp);
    }
  }

  std::vector<GemmTile> tiles, tiles_tc;
  std::vector<GemmPair> pairs, pairs_tc;
  std::vector<OzTile> tiles_oz;
  std::vector<OzPair> pairs_oz;
  auto add_tiles = [](std::vector<GemmTile> &dst, int64_t c_off, int64_t m, int64_t n, int pbeg,
                      int pend, int64_t ksum, int TM, int TN) {
    for (int64_t r0 = 0; r0 < m; r0 += TM)
      for (int64_t c0 = 0; c0 < n; c0 += TN) {
        GemmTile t{};
        t.c_off = c_off;
        t.m = (int)m;
        t.n = (int)n;
        t.row0 = (int)r0;
        t.col0 = (int)c0;
        t.pair_begin = pbeg;
        t.pair_end = pend;
        t.work = ksum * std::min<int64_t>(TM, m - r0) * std::min<int64_t>(TN, n - c0);
        dst.push_back(t);
      }
  };
  for (auto &b0 : obs) {
    if (b0.kind == kKindOz) {
      const int pbeg = (int)pairs_oz.size();
      int64_t ksum = 0;
      for (auto &cp : *b0.pairs) {
        int64_t k = 1;
        for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
        pairs_oz.push_back({plan->oa.base[cp.ablk], plan->ob.base[cp.bblk], (int)k, 0});
        ksum += k;
        const double f = 2.0 * (double)b0.m * (double)b0.n * (double)k;
        plan->flops += f;
        plan->flops_oz += f;
      }
      const auto &cp0 = (*b0.pairs)[0];
      const int ar = plan->oa.row_base[cp0.ablk], br = plan->ob.row_base[cp0.bblk];
      const int TM = oz_tile_m(), TN = oz_tile_n();
      for (int64_t r0 = 0; r0 < b0.m; r0 += TM)
        for (int64_t c0 = 0; c0 < b0.n; c0 += TN) {
          OzTile t{};
          t.c_off = o.offs[b0.ob];
          t.m = (int)b0.m;
          t.n = (int)b0.n;
          t.row0 = (int)r0;
          t.col0 = (int)c0;
          t.pair_begin = pbeg;
          t.pair_end = (int)pairs_oz.size();
          t.a_rbase = ar;
          t.b_rbase = br;
          t.work = ksum * std::min<int64_t>(TM, b0.m - r0) * std::min<int64_t>(TN, b0.n - c0);
          tiles_oz.push_back(t);
        }
      continue;
    }
    const bool tc = b0.kind == kKindTf32;
    auto &pl = tc ? pairs_tc : pairs;
    const int pbeg = (int)pl.size();
    int64_t ksum = 0;
    for (auto &cp : *b0.pairs) {
      int64_t k = 1;
      for (int t = 0; t < nc; ++t) k *= a.block_dim(cp.ablk, axes_a[t]);
      GemmPair gp{};
      gp.a_off = tc ? plan->ta.base[cp.ablk] : a.offs[cp.ablk];
      gp.b_off = tc ? plan->tb.base[cp.bblk] : b.offs[cp.bblk];
      gp.k = (int)k;
      gp.lda = (int)(plan->transA ? b0.m : k);
      gp.ldb = (int)(plan->transB ? k : b0.n);
      pl.push_back(gp);
      ksum += k;
      const double f = 2.0 * (double)b0.m * (double)b0.n * (double)k;
      plan->flops += f;
      if (tc) plan->flops_tc += f;
    }
    if (tc)
      add_tiles(tiles_tc, o.offs[b0.ob], b0.m, b0.n, pbeg, (int)pl.size(), ksum,
                gemm_tile_m(kTF32x3), gemm_tile_n(kTF32x3));
    else
      add_tiles(tiles, o.offs[b0.ob], b0.m, b0.n, pbeg, (int)pl.size(), ksum,
                gemm_tile_m(kFP64), gemm_tile_n(kFP64));
  }
  for (int64_t ob = 0; ob < o.nblocks(); ++ob) {
    if (touched[ob]) continue;
    const int *c = o.block_coords(ob);
    int64_t m = 1, n = 1;
    for (size_t l = 0; l < nfa; ++l) m *= o.idx[l].dim[c[l]];
    for (size_t l = nfa; l < o.idx.size(); ++l) n *= o.idx[l].dim[c[l]];
    add_tiles(tiles, o.offs[ob], m, n, 0, 0, 0, gemm_tile_m(kFP64), gemm_tile_n(kFP64));
  }
  // Longest tiles first so the tail of each grid is short ones.
  auto by_work = [](const GemmTile &x, const GemmTile &y) { return x.work > y.work; };
  std::stable_sort(tiles.begin(), tiles.end(), by_work);
  std::stable_sort(tiles_tc.begin(), tiles_tc.end(), by_work);
  std::stable_sort(tiles_oz.begin(), tiles_oz.end(),
                   [](const OzTile &x, const OzTile &y) { return x.work > y.work; });
  plan->ntiles_oz = (int64_t)tiles_oz.size();
  plan->tiles_oz.upload(tiles_oz);
  plan->pairs_oz.upload(pairs_oz);
  plan->tile_m = gemm_tile_m(any_tf32 ? kTF32x3 : kFP64);
  plan->tile_n = gemm_tile_n(any_tf32 ? kTF32x3 : kFP64);
  plan->ntiles = (int64_t)tiles.size();
  plan->tiles.upload(tiles);
  plan->pairs.upload(pairs);
  plan->ntiles_tc = (int64_t)tiles_tc.size();
  plan->tiles_tc.upload(tiles_tc);
  plan->pairs_tc.upload(pairs_tc);
  plan->a_elems = a.size();
  plan->b_elems = b.size();
  return plan;
}
}  // namespace

namespace {
int64_t floats_as_doubles(int64_t f) { return (f + 1) / 2 + 8; }  // + slack for alignment
float *align16(double *p) {
  return reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(p) + 15) & ~(uintptr_t)15);
}
}  // namespace

int64_t contract_scratch(const ContractPlan &p) {
  if (p.use_skinny) return 0;
  int64_t s = (p.pa.needed ? p.pa.total : 0) + (p.pb.needed ? p.pb.total : 0);
  if (p.use_tc)
    s += (p.a_cached ? 0 : floats_as_doubles(p.ta.floats)) +
         (p.b_cached ? 0 : floats_as_doubles(p.tb.floats));
  if (p.use_oz)
    s += (p.a_oz_cached ? 0 : oz_pack_doubles(p.oa)) + (p.b_oz_cached ? 0 : oz_pack_doubles(p.ob));
  return s;
}

void cache_operand(ContractPlan &p, int which, const double *src) {
  if (p.use_skinny) return;
  if (p.use_oz) {
    if (which == 0) {
      p.a_oz.alloc(oz_pack_doubles(p.oa));
      run_oz_pack(p.oa, src, oz_layout(p.oa, p.a_oz.p));
      p.a_oz_cached = true;
    } else {
      p.b_oz.alloc(oz_pack_doubles(p.ob));
      run_oz_pack(p.ob, src, oz_layout(p.ob, p.b_oz.p));
      p.b_oz_cached = true;
    }
  }
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
  if (p.use_skinny) {
    launch_skinny(p, a, b, c);
    return;
  }
  double *s = scratch;
  if (p.use_tc && p.ntiles_tc > 0) {
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
      s += floats_as_doubles(p.tb.floats);
    }
    launch_gemm_tf32x3(p, A, B, c);
  }
  if (p.use_oz && p.ntiles_oz > 0) {
    OzPacked A, B;
    if (p.a_oz_cached) {
      A = oz_layout(p.oa, const_cast<double *>(p.a_oz.p));
    } else {
      A = oz_layout(p.oa, s);
      run_oz_pack(p.oa, a, A);
      s += oz_pack_doubles(p.oa);
    }
    if (p.b_oz_cached) {
      B = oz_layout(p.ob, const_cast<double *>(p.b_oz.p));
    } else {
      B = oz_layout(p.ob, s);
      run_oz_pack(p.ob, b, B);
      s += oz_pack_doubles(p.ob);
    }
    launch_gemm_fp64tc(p, A, B, c);
  }
  if (p.ntiles == 0) return;
  const double *A = a, *B = b;
  if (p.pa.needed) {
    run_perm(p.pa, a, s);
    A = s;
    s += p.pa.total;
  }
  if (p.pb.needed) {
    run_perm(p.pb, b, s);
    B = s;
  }
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

// ---------------------------------------------------------------------------
// Autotuner cache (process-wide; lanes share it)
// ---------------------------------------------------------------------------
namespace {
std::mutex g_tune_mu;
std::map<std::pair<uint64_t, int>, double> g_tune;
bool g_tune_on = false;
}  // namespace

// Tensor-core thresholds tried by the autotuner; the last one (above 1)
// keeps every block on the FP64 kernel.
const double kTuneCandidates[5] = {0.005, 0.02, 0.08, 0.3, 2.0};

void autotune_enable(bool on) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_on = on;
}
bool autotune_on() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_tune_on;
}
bool autotune_lookup(uint64_t sig, Precision prec, double *frac) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find({sig, (int)prec});
  if (it == g_tune.end()) return false;
  *frac = it->second;
  return true;
}
void autotune_store(uint64_t sig, Precision prec, double frac) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[{sig, (int)prec}] = frac;
}

TensorPtr contract(const Tensor &a, const Tensor &b, const std::vector<int> &axes_a,
                   const std::vector<int> &axes_b, Precision prec, double *flops_out) {
  auto plan = plan_contract(a, b, axes_a, axes_b, nullptr, prec);
  double frac;
  if (prec != kFP64 && !plan->use_skinny && autotune_on() &&
      autotune_lookup(plan->signature, prec, &frac) && frac != plan->tc_frac)
    plan = plan_contract(a, b, axes_a, axes_b, nullptr, prec, frac);
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
  prof_end(kProfGemmFp64, p.flops - p.flops_tc - p.flops_oz, 8.0 * (double)(p.a_elems + p.b_elems));
}

}  // namespace gq
