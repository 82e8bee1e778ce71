// Host-side structures shared by the GB300 two-site DMRG library.
//
// A block-sparse tensor (the device counterpart of GraceQ/tensor's
// GQTensor as used by gqmps2) is:
//   * legs (Index): direction OUT=+1 / IN=-1 and ordered (QN, dim) sectors,
//   * a divergence QN: a block with sector coordinates c is allowed when
//     sum_i dir_i * qn_i(c_i) == div,
//   * a list of present blocks sorted ascending by sector coordinates
//     ("block order"), each stored dense row-major at an offset of one
//     contiguous device buffer of doubles.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace gq {

constexpr int kMaxQ = 4;      // U(1)^kMaxQ charges at most
constexpr int kMaxRank = 8;   // legs per tensor (intermediates reach 5)

enum Status : int {
  kOk = 0,
  kInvalidArgument = 1,
  kCudaError = 2,
  kSolverError = 3,
  kNumericalError = 4,
  kOutOfMemory = 5,
  kInternalError = 6,
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error(code, msg); }

#define GQ_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      ::gq::fail(e_ == cudaErrorMemoryAllocation ? ::gq::kOutOfMemory              \
                                                 : ::gq::kCudaError,               \
                 std::string(#call) + ": " + cudaGetErrorString(e_) + " at " +      \
                     __FILE__ + ":" + std::to_string(__LINE__));                   \
  } while (0)

#define GQ_CHECK(cond, msg)                                                        \
  do {                                                                             \
    if (!(cond)) ::gq::fail(::gq::kInvalidArgument, msg);                          \
  } while (0)

struct QN {
  int v[kMaxQ] = {0, 0, 0, 0};
  bool operator==(const QN &o) const { return std::memcmp(v, o.v, sizeof(v)) == 0; }
  bool operator!=(const QN &o) const { return !(*this == o); }
  bool operator<(const QN &o) const {
    for (int i = 0; i < kMaxQ; ++i)
      if (v[i] != o.v[i]) return v[i] < o.v[i];
    return false;
  }
  QN operator+(const QN &o) const {
    QN r;
    for (int i = 0; i < kMaxQ; ++i) r.v[i] = v[i] + o.v[i];
    return r;
  }
  QN operator-(const QN &o) const {
    QN r;
    for (int i = 0; i < kMaxQ; ++i) r.v[i] = v[i] - o.v[i];
    return r;
  }
  QN scaled(int s) const {
    QN r;
    for (int i = 0; i < kMaxQ; ++i) r.v[i] = s * v[i];
    return r;
  }
};

struct Index {
  int dir = 1;                 // +1 OUT, -1 IN
  std::vector<QN> qn;          // per sector
  std::vector<int64_t> dim;    // per sector
  int nsec() const { return (int)dim.size(); }
  int64_t total() const {
    int64_t s = 0;
    for (auto d : dim) s += d;
    return s;
  }
  Index inverse() const {
    Index r = *this;
    r.dir = -dir;
    return r;
  }
  bool same_sectors(const Index &o) const { return qn == o.qn && dim == o.dim; }
  bool operator==(const Index &o) const { return dir == o.dir && same_sectors(o); }
};

// ---------------------------------------------------------------------------
// Device memory: stream-ordered allocations from CUDA's pool allocator.
// ---------------------------------------------------------------------------
cudaStream_t stream();  // the library's compute stream
// Stream-ordered host-to-device copy of a host buffer the caller may reuse
// as soon as this returns (staged through pinned memory; runtime.cu).
void upload_async(void *dst, const void *src, size_t bytes);

struct DevBuf {
  double *p = nullptr;
  int64_t n = 0;  // elements
  DevBuf() = default;
  explicit DevBuf(int64_t elems) { alloc(elems); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(int64_t elems);
  void release();
};

template <typename T>
struct DevArray {  // small typed device arrays for work lists
  T *p = nullptr;
  int64_t n = 0;
  DevArray() = default;
  DevArray(const DevArray &) = delete;
  DevArray &operator=(const DevArray &) = delete;
  DevArray(DevArray &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevArray &operator=(DevArray &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevArray() { release(); }
  void upload(const std::vector<T> &h) { upload(h.data(), (int64_t)h.size()); }
  void upload(const T *h, int64_t count) {
    release();
    n = count;
    if (n == 0) return;
    GQ_CUDA(cudaMallocAsync((void **)&p, sizeof(T) * n, stream()));
    upload_async(p, h, sizeof(T) * n);
  }
  void release() {
    if (p) cudaFreeAsync(p, stream());
    p = nullptr;
    n = 0;
  }
};

// ---------------------------------------------------------------------------
// Block-sparse tensor
// ---------------------------------------------------------------------------
struct Tensor {
  int nq = 1;
  std::vector<Index> idx;
  QN div;
  std::vector<int> coords;        // nblocks x rank, ascending block order
  std::vector<int64_t> offs;      // nblocks + 1 prefix offsets (elements)
  DevBuf data;

  int rank() const { return (int)idx.size(); }
  int64_t nblocks() const { return (int64_t)offs.size() - 1; }
  int64_t size() const { return offs.empty() ? 0 : offs.back(); }
  const int *block_coords(int64_t b) const { return coords.data() + b * rank(); }
  int64_t block_dim(int64_t b, int leg) const { return idx[leg].dim[block_coords(b)[leg]]; }
  int64_t block_size(int64_t b) const { return offs[b + 1] - offs[b]; }

  // Block id of the coordinates c, or -1: binary search over the sorted
  // coordinate list.
  int64_t find(const int *c) const {
    const int r = rank();
    int64_t lo = 0, hi = nblocks();
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      const int *m = coords.data() + mid * r;
      int cmp = 0;
      for (int l = 0; l < r && cmp == 0; ++l)
        if (m[l] != c[l]) cmp = m[l] < c[l] ? -1 : 1;
      if (cmp == 0) return mid;
      if (cmp < 0) lo = mid + 1;
      else hi = mid;
    }
    return -1;
  }
  QN block_div(const int *c) const {
    QN q;
    for (int i = 0; i < rank(); ++i) q = q + idx[i].qn[c[i]].scaled(idx[i].dir);
    return q;
  }
  // Build the offsets from `coords` (must be sorted and unique).
  void finalize_structure();
  // Allocate device storage for the structure (contents undefined).
  void allocate();
  void zero();
};

using TensorPtr = std::shared_ptr<Tensor>;

// Structure helpers
TensorPtr make_structure(int nq, const std::vector<Index> &idx, const QN &div,
                         std::vector<std::vector<int>> blocks /* any order */);
// The same from flat coordinates (nblocks x rank) already sorted and unique.
TensorPtr make_structure_sorted(int nq, const std::vector<Index> &idx, const QN &div,
                                std::vector<int> coords);
// Every block allowed by `div` for these legs.
std::vector<std::vector<int>> allowed_blocks(const std::vector<Index> &idx, const QN &div);
TensorPtr clone_structure(const Tensor &t);
TensorPtr clone(const Tensor &t);   // structure + data copy (device)
TensorPtr dag(const Tensor &t);     // legs inverted, div negated, data copied

}  // namespace gq
