// Library runtime: device context, stream-ordered memory, tensor structure.
#include "gq_runtime.hpp"

#include <cstdio>
#include <atomic>
#include <chrono>
#include <cstring>
#include <map>
#include <algorithm>
#include <mutex>
#include <thread>
#include <vector>

namespace gq {

namespace {
Context *g_ctx = nullptr;
std::mutex g_ctx_mu;
}  // namespace

Context &ctx() {
  if (!g_ctx) init_context(-1);
  return *g_ctx;
}

void init_context(int device) {
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  if (g_ctx) {
    if (device >= 0 && device != g_ctx->device)
      fail(kInvalidArgument, "library already initialised on another device");
    return;
  }
  int ndev = 0;
  GQ_CUDA(cudaGetDeviceCount(&ndev));
  if (ndev <= 0) fail(kCudaError, "no CUDA device visible");
  if (device < 0) GQ_CUDA(cudaGetDevice(&device));
  GQ_CUDA(cudaSetDevice(device));
  auto *c = new Context();
  c->device = device;
  GQ_CUDA(cudaGetDeviceProperties(&c->prop, device));
  if (c->prop.major < 10)
    fail(kCudaError, "this library is built for sm_103a (GB300); found sm_" +
                         std::to_string(c->prop.major) + std::to_string(c->prop.minor));
  // Keep freed blocks cached in the pool: tensors are created and released
  // at every two-site update.
  cudaMemPool_t pool;
  GQ_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t thr = UINT64_MAX;
  GQ_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  init_lane(c->main);
  g_ctx = c;
  noalloc_setup();
}

namespace {
thread_local Lane *t_lane = nullptr;
}  // namespace

void init_lane(Lane &l) {
  GQ_CUDA(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking));
  GQ_CUDA(cudaMallocHost((void **)&l.host_scalars, sizeof(double) * 64));
  GQ_CUDA(cudaMallocAsync((void **)&l.dev_scalars, sizeof(double) * 64, l.stream));
  GQ_CUDA(cudaMemsetAsync(l.dev_scalars, 0, sizeof(double) * 64, l.stream));
  GQ_CUDA(cudaStreamSynchronize(l.stream));
}

void init_aux(Lane &l) {
  if (l.fork_event) return;
  for (int i = 0; i < Lane::kAux; ++i) {
    GQ_CUDA(cudaStreamCreateWithFlags(&l.aux_stream[i], cudaStreamNonBlocking));
    GQ_CUDA(cudaEventCreateWithFlags(&l.join_event[i], cudaEventDisableTiming));
  }
  GQ_CUDA(cudaEventCreateWithFlags(&l.fork_event, cudaEventDisableTiming));
}

void fork_aux(Lane &l, int n) {
  if (n <= 0) return;
  init_aux(l);
  GQ_CUDA(cudaEventRecord(l.fork_event, l.stream));
  for (int i = 0; i < n; ++i) GQ_CUDA(cudaStreamWaitEvent(l.aux_stream[i], l.fork_event, 0));
}

void join_aux(Lane &l, int n) {
  for (int i = 0; i < n; ++i) {
    GQ_CUDA(cudaEventRecord(l.join_event[i], l.aux_stream[i]));
    GQ_CUDA(cudaStreamWaitEvent(l.stream, l.join_event[i], 0));
  }
}

Lane &lane() { return t_lane ? *t_lane : ctx().main; }

Lane *lane_create() {
  ctx();
  auto *l = new Lane();
  init_lane(*l);
  return l;
}

void lane_destroy(Lane *l) {
  if (!l) return;
  if (t_lane == l) t_lane = nullptr;
  cudaStreamSynchronize(l->stream);
  destroy_lane_handles(*l);
  cudaFreeAsync(l->dev_scalars, l->stream);
  cudaStreamSynchronize(l->stream);
  cudaFreeHost(l->host_scalars);
  if (l->staging) cudaFreeHost(l->staging);
  for (int k = 0; k < 2; ++k) {
    if (l->xfer[k]) cudaFreeHost(l->xfer[k]);
    if (l->xfer_done[k]) cudaEventDestroy(l->xfer_done[k]);
  }
  if (l->fork_event) {
    for (int i = 0; i < Lane::kAux; ++i) {
      cudaStreamSynchronize(l->aux_stream[i]);
      cudaStreamDestroy(l->aux_stream[i]);
      cudaEventDestroy(l->join_event[i]);
    }
    cudaEventDestroy(l->fork_event);
  }
  cudaStreamDestroy(l->stream);
  delete l;
}

void lane_bind(Lane *l) { t_lane = l; }

bool on_main_lane() { return t_lane == nullptr; }

cudaStream_t stream() { return lane().stream; }

// Work lists (tiles, pairs, pack tasks...) go to the device while kernels
// run.  A cudaMemcpyAsync from pageable memory synchronises the stream
// first, which would drain the GPU at every plan built between two kernels
// (the SVD's projections and the environment growth build several); the
// lists are staged through a pinned ring per lane instead.  Every wait on
// the lane's stream (sync()) empties the ring, since every copy from it has
// then run; between two waits the ring wraps behind a stream
// synchronisation only when it is full -- which, with a Lanczos loop queued
// as one graph, would hold the host until the whole loop has run, so the
// ring is sized to hold an update's work lists.
namespace {
constexpr size_t kStagingBytes = size_t(64) << 20;
}

void upload_async(void *dst, const void *src, size_t bytes) {
  Lane &l = lane();
  if (bytes == 0) return;
  if (bytes > kStagingBytes) {  // rare: plain (synchronising) copy
    GQ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, l.stream));
    return;
  }
  if (!l.staging) {
    GQ_CUDA(cudaMallocHost((void **)&l.staging, kStagingBytes));
    l.staging_head = 0;
  }
  size_t off = (l.staging_head + 255) & ~size_t(255);
  if (off + bytes > kStagingBytes) {
    GQ_CUDA(cudaStreamSynchronize(l.stream));
    off = 0;
  }
  std::memcpy(l.staging + off, src, bytes);
  GQ_CUDA(cudaMemcpyAsync(dst, l.staging + off, bytes, cudaMemcpyHostToDevice, l.stream));
  l.staging_head = off + bytes;
}

namespace {
std::atomic<int64_t> g_host_syncs{0};
}  // namespace

int64_t host_sync_count() { return g_host_syncs.load(); }

namespace {
constexpr size_t kXferBytes = size_t(64) << 20;   // per pinned buffer
constexpr size_t kXferDirect = size_t(1) << 20;   // below: one plain copy
constexpr int kXferThreads = 8;

// Bytes [lo, hi) of the concatenation of the segments (starts pre[i], the
// last entry the total) into dst, split over up to kXferThreads host
// threads for large ranges.
void host_gather(char *dst, const char *const *segs, const std::vector<size_t> &pre, size_t lo,
                 size_t hi) {
  auto part_copy = [&](size_t b, size_t e) {
    size_t i = (size_t)(std::upper_bound(pre.begin(), pre.end(), b) - pre.begin()) - 1;
    while (b < e) {
      const size_t end = std::min(e, pre[i + 1]);
      if (end > b) std::memcpy(dst + (b - lo), segs[i] + (b - pre[i]), end - b);
      b = end;
      ++i;
    }
  };
  const size_t bytes = hi - lo;
  const int nt = bytes >= (size_t(8) << 20) ? kXferThreads : 1;
  if (nt == 1) {
    part_copy(lo, hi);
    return;
  }
  const size_t part = (bytes + nt - 1) / nt;
  std::vector<std::thread> th;
  th.reserve(nt - 1);
  for (int t = 1; t < nt; ++t) {
    const size_t b = lo + std::min(bytes, t * part), e = lo + std::min(bytes, (t + 1) * part);
    if (b < e) th.emplace_back(part_copy, b, e);
  }
  part_copy(lo, lo + std::min(bytes, part));
  for (auto &x : th) x.join();
}

void host_copy(char *dst, const char *src, size_t bytes) {
  const char *seg[1] = {src};
  host_gather(dst, seg, {0, bytes}, 0, bytes);
}

void xfer_setup(Lane &l) {
  for (int k = 0; k < 2; ++k) {
    if (!l.xfer[k]) GQ_CUDA(cudaMallocHost((void **)&l.xfer[k], kXferBytes));
    if (!l.xfer_done[k])
      GQ_CUDA(cudaEventCreateWithFlags(&l.xfer_done[k], cudaEventDisableTiming));
  }
}
}  // namespace

void copy_h2d_gather(void *dst, const void *const *srcs, const size_t *sizes, size_t nseg) {
  Lane &l = lane();
  std::vector<size_t> pre(nseg + 1, 0);
  for (size_t i = 0; i < nseg; ++i) pre[i + 1] = pre[i] + sizes[i];
  const size_t bytes = pre[nseg];
  if (bytes == 0) return;
  const char *const *segs = reinterpret_cast<const char *const *>(srcs);
  char *d = static_cast<char *>(dst);
  if (nseg == 1 && bytes <= kXferDirect) {
    GQ_CUDA(cudaMemcpyAsync(dst, srcs[0], bytes, cudaMemcpyHostToDevice, l.stream));
    sync();
    return;
  }
  xfer_setup(l);
  size_t off = 0;
  for (int c = 0; off < bytes; ++c) {
    const int k = c & 1;
    const size_t b = std::min(kXferBytes, bytes - off);
    GQ_CUDA(cudaEventSynchronize(l.xfer_done[k]));  // its previous DMA is done
    host_gather(l.xfer[k], segs, pre, off, off + b);
    GQ_CUDA(cudaMemcpyAsync(d + off, l.xfer[k], b, cudaMemcpyHostToDevice, l.stream));
    GQ_CUDA(cudaEventRecord(l.xfer_done[k], l.stream));
    off += b;
  }
  sync();
}

void copy_h2d(void *dst, const void *src, size_t bytes) {
  const void *seg[1] = {src};
  copy_h2d_gather(dst, seg, &bytes, 1);
}

void copy_d2h(void *dst, const void *src, size_t bytes) {
  Lane &l = lane();
  if (bytes == 0) return;
  if (bytes <= kXferDirect) {
    GQ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, l.stream));
    sync();
    return;
  }
  xfer_setup(l);
  const char *s = static_cast<const char *>(src);
  char *d = static_cast<char *>(dst);
  const int nchunks = (int)((bytes + kXferBytes - 1) / kXferBytes);
  auto chunk = [&](int c) { return std::min(kXferBytes, bytes - (size_t)c * kXferBytes); };
  auto issue = [&](int c) {
    const int k = c & 1;
    GQ_CUDA(cudaMemcpyAsync(l.xfer[k], s + (size_t)c * kXferBytes, chunk(c),
                            cudaMemcpyDeviceToHost, l.stream));
    GQ_CUDA(cudaEventRecord(l.xfer_done[k], l.stream));
  };
  issue(0);
  for (int c = 0; c < nchunks; ++c) {
    // the buffer of chunk c + 1 held chunk c - 1, whose host copy is done
    if (c + 1 < nchunks) issue(c + 1);
    GQ_CUDA(cudaEventSynchronize(l.xfer_done[c & 1]));
    host_copy(d + (size_t)c * kXferBytes, l.xfer[c & 1], chunk(c));
  }
  sync();
}

void sync() {
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  Lane &l = lane();
  if (!prof_on()) {
    GQ_CUDA(cudaStreamSynchronize(l.stream));
    l.staging_head = 0;  // every staged copy has run
    return;
  }
  const auto t0 = std::chrono::steady_clock::now();
  GQ_CUDA(cudaStreamSynchronize(l.stream));
  l.staging_head = 0;
  prof_host(kProfHostSync,
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
}

void DevBuf::alloc(int64_t elems) {
  release();
  n = elems;
  if (elems <= 0) return;
  GQ_CUDA(cudaMallocAsync((void **)&p, sizeof(double) * elems, stream()));
}

void DevBuf::release() {
  if (p) cudaFreeAsync(p, stream());
  p = nullptr;
  n = 0;
}

// ---------------------------------------------------------------------------
// Kernel profiling
// ---------------------------------------------------------------------------
namespace {
struct ProfRec { int k; cudaEvent_t e0, e1; double flops, bytes; };
struct ProfState {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<ProfRec> pending;
  cudaEvent_t open[kProfCount] = {};
  int64_t launches[kProfCount] = {};
  double ms[kProfCount] = {}, flops[kProfCount] = {}, bytes[kProfCount] = {};
} g_prof;

cudaEvent_t prof_event() {
  if (!g_prof.pool.empty()) {
    auto e = g_prof.pool.back();
    g_prof.pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  GQ_CUDA(cudaEventCreate(&e));
  return e;
}

void prof_drain() {
  if (g_prof.pending.empty()) return;
  sync();
  for (auto &r : g_prof.pending) {
    float t = 0.f;
    GQ_CUDA(cudaEventElapsedTime(&t, r.e0, r.e1));
    g_prof.launches[r.k]++;
    g_prof.ms[r.k] += t;
    g_prof.flops[r.k] += r.flops;
    g_prof.bytes[r.k] += r.bytes;
    g_prof.pool.push_back(r.e0);
    g_prof.pool.push_back(r.e1);
  }
  g_prof.pending.clear();
}
}  // namespace

// The profiler's counters are process-wide and filled from the main lane
// only; work on other lanes is not profiled.
bool prof_on() { return g_prof.on && on_main_lane(); }

void prof_enable(bool on) {
  prof_drain();
  for (int k = 0; k < kProfCount; ++k) {
    g_prof.launches[k] = 0;
    g_prof.ms[k] = g_prof.flops[k] = g_prof.bytes[k] = 0.0;
  }
  g_prof.on = on;
}

void prof_begin(ProfKernel k) {
  if (!prof_on()) return;
  auto e = prof_event();
  GQ_CUDA(cudaEventRecord(e, stream()));
  g_prof.open[k] = e;
}

void prof_end(ProfKernel k, double flops, double bytes) {
  if (!prof_on() || !g_prof.open[k]) return;
  auto e = prof_event();
  GQ_CUDA(cudaEventRecord(e, stream()));
  g_prof.pending.push_back({(int)k, g_prof.open[k], e, flops, bytes});
  g_prof.open[k] = nullptr;
  if (g_prof.pending.size() > 4096) prof_drain();
}

void prof_host(ProfKernel k, double seconds) {
  if (!prof_on()) return;
  g_prof.launches[k]++;
  g_prof.ms[k] += seconds * 1e3;
}

void prof_read(ProfKernel k, int64_t *launches, double *ms, double *flops, double *bytes) {
  prof_drain();
  if (launches) *launches = g_prof.launches[k];
  if (ms) *ms = g_prof.ms[k];
  if (flops) *flops = g_prof.flops[k];
  if (bytes) *bytes = g_prof.bytes[k];
}

// ---------------------------------------------------------------------------
void Tensor::finalize_structure() {
  const int r = rank();
  const int64_t nb = r ? (int64_t)coords.size() / r : 1;
  offs.assign(nb + 1, 0);
  for (int64_t b = 0; b < nb; ++b) {
    int64_t sz = 1;
    for (int l = 0; l < r; ++l) sz *= idx[l].dim[coords[b * r + l]];
    offs[b + 1] = offs[b] + sz;
  }
}

void Tensor::allocate() { data.alloc(size()); }

void Tensor::zero() {
  if (size() > 0) GQ_CUDA(cudaMemsetAsync(data.p, 0, sizeof(double) * size(), stream()));
}

TensorPtr make_structure(int nq, const std::vector<Index> &idx, const QN &div,
                         std::vector<std::vector<int>> blocks) {
  auto t = std::make_shared<Tensor>();
  t->nq = nq;
  t->idx = idx;
  t->div = div;
  std::sort(blocks.begin(), blocks.end());
  blocks.erase(std::unique(blocks.begin(), blocks.end()), blocks.end());
  const int r = (int)idx.size();
  t->coords.reserve(blocks.size() * r);
  for (auto &b : blocks) {
    GQ_CHECK((int)b.size() == r, "block coordinate of wrong rank");
    for (int l = 0; l < r; ++l) {
      GQ_CHECK(b[l] >= 0 && b[l] < idx[l].nsec(), "block coordinate out of range");
      t->coords.push_back(b[l]);
    }
  }
  if (r == 0) t->coords.clear();
  t->finalize_structure();
  return t;
}

TensorPtr make_structure_sorted(int nq, const std::vector<Index> &idx, const QN &div,
                                std::vector<int> coords) {
  auto t = std::make_shared<Tensor>();
  t->nq = nq;
  t->idx = idx;
  t->div = div;
  t->coords = std::move(coords);
  t->finalize_structure();
  return t;
}

std::vector<std::vector<int>> allowed_blocks(const std::vector<Index> &idx, const QN &div) {
  std::vector<std::vector<int>> out;
  const int r = (int)idx.size();
  if (r == 0) return out;
  // Depth-first over legs with the partial charge; prune nothing (sector
  // counts are small), emit in ascending order.
  std::vector<int> c(r, 0);
  std::vector<QN> partial(r + 1);
  int l = 0;
  c[0] = -1;
  while (l >= 0) {
    c[l]++;
    if (c[l] >= idx[l].nsec()) {
      --l;
      continue;
    }
    partial[l + 1] = partial[l] + idx[l].qn[c[l]].scaled(idx[l].dir);
    if (l == r - 1) {
      if (partial[r] == div) out.push_back(c);
    } else {
      ++l;
      c[l] = -1;
    }
  }
  return out;
}

TensorPtr clone_structure(const Tensor &t) {
  auto o = std::make_shared<Tensor>();
  o->nq = t.nq;
  o->idx = t.idx;
  o->div = t.div;
  o->coords = t.coords;
  o->offs = t.offs;
  return o;
}

TensorPtr clone(const Tensor &t) {
  auto o = clone_structure(t);
  o->allocate();
  if (t.size() > 0)
    GQ_CUDA(cudaMemcpyAsync(o->data.p, t.data.p, sizeof(double) * t.size(),
                            cudaMemcpyDeviceToDevice, stream()));
  return o;
}

TensorPtr dag(const Tensor &t) {
  auto o = clone(t);
  for (auto &ix : o->idx) ix.dir = -ix.dir;
  o->div = t.div.scaled(-1);
  return o;
}

}  // namespace gq
