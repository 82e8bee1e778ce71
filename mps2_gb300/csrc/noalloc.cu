// gq_contract_noalloc: the block-sparse contraction (FP64 form) without any
// device allocation.
//
// Who needs it: a caller that owns every byte of device memory itself and
// cannot let a library allocate behind its back -- for example a host
// application that hands this library a fixed memory budget carved out of
// its own pool, a plugin running inside another framework's time step where
// cudaMalloc's implicit device synchronisation would stall unrelated work,
// or a process whose device memory is already fully reserved.  Such a caller
// creates its input and output tensors up front (gq_tensor_create) and then
// contracts them any number of times with this entry point, which only
// launches kernels and copies small work lists into memory that was set
// aside when the library was loaded.
//
// How: the two operands are permuted into matrix form inside a file-scope
// device array (g_na_operands, kNaOperandElems doubles = 16 MiB) and the
// per-call work lists go to three more file-scope arrays (about 6 MiB in
// all).  Every GPU that uses the library keeps these ~22 MiB until the
// process exits.  Host code cannot use the arrays' names as device
// addresses, so a set-up step, once per device and with that device
// current, looks their addresses up with cudaGetSymbolAddress and launches
// each kernel of this file once with no work.  CUDA loads a module's
// device memory and kernels lazily (CUDA_MODULE_LOADING=LAZY is the default
// since CUDA 12.2), and that load can allocate and synchronise; the set-up
// makes it happen there.  gq_init runs the set-up for its device; a caller
// that skips gq_init gets it inside its first call of this entry point on
// that device, and must make that first call before its no-allocation phase
// and before any stream capture.  All calls share the arrays and each call
// rewrites every element it later reads, so nothing needs clearing between
// calls; two calls whose work overlaps on the GPU race on the arrays and
// must not be issued concurrently.  Each call waits for its own GPU work to
// finish before it returns (the work lists are copied from host memory that
// the call owns).
#include <map>
#include <mutex>

#include "gq_runtime.hpp"

namespace gq {
namespace {

constexpr int64_t kNaOperandElems = int64_t(1) << 21;  // 16 MiB of FP64 operands
constexpr int64_t kNaMaxTiles = int64_t(1) << 15;
constexpr int64_t kNaMaxPairs = int64_t(1) << 17;
constexpr int64_t kNaMaxPerm = int64_t(1) << 15;      // permute tasks (chunks)

struct NaTile { int64_t c_off; int m, n, row0, col0, pbeg, pend; };
struct NaPair { int64_t a_off, b_off; int k, pad; };
struct NaPerm {  // one chunk of one block: dst(i...) = src(sum i_l * sstride_l)
  int64_t src_off, dst_off, begin, end;
  int rank, pad;
  int dims[kMaxRank];
  int64_t sstride[kMaxRank];
};

static __device__ __align__(256) double g_na_operands[kNaOperandElems];
static __device__ __align__(256) NaTile g_na_tiles[kNaMaxTiles];
static __device__ __align__(256) NaPair g_na_pairs[kNaMaxPairs];
static __device__ __align__(256) NaPerm g_na_perm[kNaMaxPerm];

struct NaAddrs {
  double *operands = nullptr;
  NaTile *tiles = nullptr;
  NaPair *pairs = nullptr;
  NaPerm *perm = nullptr;
};
std::mutex g_na_mu;
std::map<int, NaAddrs> g_na_addrs;  // per device

__global__ void na_permute_kernel(const NaPerm *__restrict__ tasks, int ntasks,
                                  const double *__restrict__ src, double *__restrict__ dst);
__global__ void na_gemm_kernel(const NaTile *__restrict__ tiles, int ntiles,
                               const NaPair *__restrict__ pairs, const double *__restrict__ A,
                               const double *__restrict__ B, double *__restrict__ C);

// Set-up, once per device, with that device current.
NaAddrs na_addresses() {
  int dev = 0;
  GQ_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_na_mu);
  auto it = g_na_addrs.find(dev);
  if (it != g_na_addrs.end()) return it->second;
  NaAddrs a;
  GQ_CUDA(cudaGetSymbolAddress((void **)&a.operands, g_na_operands));
  GQ_CUDA(cudaGetSymbolAddress((void **)&a.tiles, g_na_tiles));
  GQ_CUDA(cudaGetSymbolAddress((void **)&a.pairs, g_na_pairs));
  GQ_CUDA(cudaGetSymbolAddress((void **)&a.perm, g_na_perm));
  // one launch of each kernel with no work, so that lazy module loading
  // happens here and not inside a later call
  na_permute_kernel<<<1, 32, 0, stream()>>>(a.perm, 0, nullptr, nullptr);
  na_gemm_kernel<<<1, 256, 0, stream()>>>(a.tiles, 0, a.pairs, nullptr, nullptr, nullptr);
  GQ_CUDA(cudaGetLastError());
  GQ_CUDA(cudaStreamSynchronize(stream()));
  g_na_addrs[dev] = a;
  return a;
}

__global__ void na_permute_kernel(const NaPerm *__restrict__ tasks, int ntasks,
                                  const double *__restrict__ src, double *__restrict__ dst) {
  if ((int)blockIdx.x >= ntasks) return;  // ntasks == 0: the set-up's empty launch
  __shared__ NaPerm t;
  if (threadIdx.x == 0) t = tasks[blockIdx.x];
  __syncthreads();
  for (int64_t e = t.begin + threadIdx.x; e < t.end; e += blockDim.x) {
    int64_t rem = e, so = 0;
    for (int j = t.rank - 1; j >= 0; --j) {
      const int64_t d = t.dims[j];
      so += (rem % d) * t.sstride[j];
      rem /= d;
    }
    dst[t.dst_off + e] = src[t.src_off + so];
  }
}

// FP64 tile GEMM on operands already in matrix form: A' row-major m x k,
// B' row-major k x n (the same 64x64 tiling and summation order as the
// allocating path's FP64 kernel).
__global__ void __launch_bounds__(256)
    na_gemm_kernel(const NaTile *__restrict__ tiles, int ntiles, const NaPair *__restrict__ pairs,
                   const double *__restrict__ A, const double *__restrict__ B,
                   double *__restrict__ C) {
  if ((int)blockIdx.x >= ntiles) return;  // ntiles == 0: the set-up's empty launch
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ double As[BK][BM];
  __shared__ double Bs[BK][BN];
  const NaTile t = tiles[blockIdx.x];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int p = t.pbeg; p < t.pend; ++p) {
    const NaPair pr = pairs[p];
    for (int k0 = 0; k0 < pr.k; k0 += BK) {
#pragma unroll
      for (int it = 0; it < (BM * BK) / 256; ++it) {
        const int i = tid + it * 256, kk = i % BK, r = i / BK;
        const int gr = t.row0 + r, gk = k0 + kk;
        As[kk][r] = (gr < t.m && gk < pr.k) ? A[pr.a_off + (int64_t)gr * pr.k + gk] : 0.0;
      }
#pragma unroll
      for (int it = 0; it < (BN * BK) / 256; ++it) {
        const int i = tid + it * 256, c = i % BN, kk = i / BN;
        const int gc = t.col0 + c, gk = k0 + kk;
        Bs[kk][c] = (gc < t.n && gk < pr.k) ? B[pr.b_off + (int64_t)gk * t.n + gc] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
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
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = t.row0 + ty + 16 * i;
    if (gr >= t.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gc = t.col0 + tx + 16 * j;
      if (gc < t.n) C[t.c_off + (int64_t)gr * t.n + gc] = acc[i][j];
    }
  }
}

// Permute tasks that bring every block of `t` into the leg order `perm`,
// writing at the same block offsets shifted by `base`.
void na_perm_tasks(const Tensor &t, const std::vector<int> &perm, int64_t base,
                   std::vector<NaPerm> &out) {
  const int r = t.rank();
  for (int64_t b = 0; b < t.nblocks(); ++b) {
    NaPerm p{};
    p.src_off = t.offs[b];
    p.dst_off = base + t.offs[b];
    p.rank = r;
    int64_t sdims[kMaxRank], sstr[kMaxRank], s = 1;
    for (int l = 0; l < r; ++l) sdims[l] = t.block_dim(b, l);
    for (int l = r - 1; l >= 0; --l) {
      sstr[l] = s;
      s *= sdims[l];
    }
    for (int j = 0; j < r; ++j) {
      p.dims[j] = (int)sdims[perm[j]];
      p.sstride[j] = sstr[perm[j]];
    }
    const int64_t n = t.block_size(b);
    for (int64_t e = 0; e < n; e += 16384) {
      p.begin = e;
      p.end = std::min<int64_t>(n, e + 16384);
      out.push_back(p);
    }
  }
}

}  // namespace

void noalloc_setup() { (void)na_addresses(); }

void contract_noalloc(const Tensor &A, const Tensor &B, const std::vector<int> &xa,
                      const std::vector<int> &xb, Tensor &O) {
  const int ra = A.rank(), rb = B.rank(), nc = (int)xa.size();
  GQ_CHECK(nc >= 1 && nc == (int)xb.size(), "bad axes");
  std::vector<char> ca(ra, 0), cb(rb, 0);
  for (int i = 0; i < nc; ++i) {
    GQ_CHECK(xa[i] >= 0 && xa[i] < ra && !ca[xa[i]], "bad axes for a");
    GQ_CHECK(xb[i] >= 0 && xb[i] < rb && !cb[xb[i]], "bad axes for b");
    ca[xa[i]] = cb[xb[i]] = 1;
    GQ_CHECK(A.idx[xa[i]].dir == -B.idx[xb[i]].dir && A.idx[xa[i]].same_sectors(B.idx[xb[i]]),
             "contracted legs must carry the same sectors with opposite directions");
  }
  std::vector<int> fa, fb;
  for (int i = 0; i < ra; ++i)
    if (!ca[i]) fa.push_back(i);
  for (int i = 0; i < rb; ++i)
    if (!cb[i]) fb.push_back(i);
  GQ_CHECK(O.rank() == (int)(fa.size() + fb.size()), "output tensor has the wrong rank");
  for (size_t l = 0; l < fa.size(); ++l)
    GQ_CHECK(O.idx[l] == A.idx[fa[l]], "output legs must be a's free legs then b's");
  for (size_t l = 0; l < fb.size(); ++l)
    GQ_CHECK(O.idx[fa.size() + l] == B.idx[fb[l]], "output legs must be a's free legs then b's");
  GQ_CHECK(O.div == A.div + B.div, "output divergence must be div(a) + div(b)");
  GQ_CHECK(A.size() + B.size() <= kNaOperandElems,
           "operands exceed the no-allocation scratch: a and b together may hold at most " +
               std::to_string(kNaOperandElems) + " elements");

  // Host work lists: operands permuted to (free, contracted) and
  // (contracted, free); one 64x64 tile list over every output block.
  std::vector<int> pa = fa, pb = xb;
  pa.insert(pa.end(), xa.begin(), xa.end());
  pb.insert(pb.end(), fb.begin(), fb.end());
  std::vector<NaPerm> perm;
  na_perm_tasks(A, pa, 0, perm);
  const size_t na_tasks = perm.size();
  na_perm_tasks(B, pb, A.size(), perm);
  std::map<std::vector<int>, std::vector<int64_t>> bgroups;
  for (int64_t j = 0; j < B.nblocks(); ++j) {
    std::vector<int> key;
    for (int x : xb) key.push_back(B.block_coords(j)[x]);
    bgroups[key].push_back(j);
  }
  std::map<std::vector<int>, std::vector<std::pair<int64_t, int64_t>>> contrib;
  for (int64_t i = 0; i < A.nblocks(); ++i) {
    std::vector<int> key, oc;
    for (int x : xa) key.push_back(A.block_coords(i)[x]);
    auto it = bgroups.find(key);
    if (it == bgroups.end()) continue;
    for (int f : fa) oc.push_back(A.block_coords(i)[f]);
    for (int64_t j : it->second) {
      std::vector<int> c = oc;
      for (int f : fb) c.push_back(B.block_coords(j)[f]);
      contrib[c].push_back({i, j});
    }
  }
  std::vector<NaTile> tiles;
  std::vector<NaPair> pairs;
  for (int64_t ob = 0; ob < O.nblocks(); ++ob) {
    std::vector<int> c(O.block_coords(ob), O.block_coords(ob) + O.rank());
    int64_t m = 1, n = 1;
    for (size_t l = 0; l < fa.size(); ++l) m *= O.idx[l].dim[c[l]];
    for (size_t l = fa.size(); l < c.size(); ++l) n *= O.idx[l].dim[c[l]];
    const int pbeg = (int)pairs.size();
    auto it = contrib.find(c);
    if (it != contrib.end()) {
      for (auto &pr : it->second) {
        int64_t k = 1;
        for (int x : xa) k *= A.block_dim(pr.first, x);
        pairs.push_back({A.offs[pr.first], A.size() + B.offs[pr.second], (int)k, 0});
      }
      contrib.erase(it);
    }
    const int pend = (int)pairs.size();
    for (int64_t r0 = 0; r0 < m; r0 += 64)
      for (int64_t c0 = 0; c0 < n; c0 += 64)
        tiles.push_back({O.offs[ob], (int)m, (int)n, (int)r0, (int)c0, pbeg, pend});
  }
  GQ_CHECK(contrib.empty(), "output tensor lacks a block that the contraction produces");
  GQ_CHECK((int64_t)tiles.size() <= kNaMaxTiles,
           "too many output tiles for the no-allocation work list (max " +
               std::to_string(kNaMaxTiles) + ")");
  GQ_CHECK((int64_t)pairs.size() <= kNaMaxPairs,
           "too many block products for the no-allocation work list (max " +
               std::to_string(kNaMaxPairs) + ")");
  GQ_CHECK((int64_t)perm.size() <= kNaMaxPerm,
           "too many permute tasks for the no-allocation work list (max " +
               std::to_string(kNaMaxPerm) + ")");

  const NaAddrs ad = na_addresses();
  cudaStream_t s = stream();
  if (!perm.empty())
    GQ_CUDA(cudaMemcpyAsync(ad.perm, perm.data(), sizeof(NaPerm) * perm.size(),
                            cudaMemcpyHostToDevice, s));
  if (!pairs.empty())
    GQ_CUDA(cudaMemcpyAsync(ad.pairs, pairs.data(), sizeof(NaPair) * pairs.size(),
                            cudaMemcpyHostToDevice, s));
  if (!tiles.empty())
    GQ_CUDA(cudaMemcpyAsync(ad.tiles, tiles.data(), sizeof(NaTile) * tiles.size(),
                            cudaMemcpyHostToDevice, s));
  if (na_tasks > 0)
    na_permute_kernel<<<(unsigned)na_tasks, 256, 0, s>>>(ad.perm, (int)na_tasks, A.data.p,
                                                         ad.operands);
  if (perm.size() > na_tasks) {
    const int nb_tasks = (int)(perm.size() - na_tasks);
    na_permute_kernel<<<(unsigned)nb_tasks, 256, 0, s>>>(ad.perm + na_tasks, nb_tasks, B.data.p,
                                                         ad.operands);
  }
  GQ_CUDA(cudaGetLastError());
  if (!tiles.empty())
    na_gemm_kernel<<<(unsigned)tiles.size(), 256, 0, s>>>(ad.tiles, (int)tiles.size(), ad.pairs,
                                                           ad.operands, ad.operands, O.data.p);
  GQ_CUDA(cudaGetLastError());
  // the host work lists above are copied from pageable memory; finish
  // before they go out of scope and before the caller reads the output
  GQ_CUDA(cudaStreamSynchronize(s));
}

}  // namespace gq
