/*
 * gqmps2_gb300.hpp -- header-only C++ front end of libgqmps2_gb300.so with
 * gqmps2's names and signatures, so that a gqmps2 program (or one of its DMRG
 * tests) switches by changing its include and its tensor type:
 *
 *   gqmps2 (v0.2-alpha.0)                          this header
 *   SweepParams (two_site_update_finite_vmps.h:27)  gqmps2::SweepParams (+ precision)
 *   LanczosParams (lanczos_solver.h:27-43)         gqmps2::LanczosParams
 *   SiteVec (site_vec.h:37-132)                    gqmps2::SiteVec
 *   TenVec / MPO (ten_vec.h:30-85, mpo.h:25)       gqmps2::TenVec, gqmps2::MPO
 *   FiniteMPS (finite_mps.h:51-140, mps.h:69-107)  gqmps2::FiniteMPS
 *   DirectStateInitMps (finite_mps_init.h:216)     gqmps2::DirectStateInitMps
 *   TruncateMPS (finite_mps.h:251-300)             gqmps2::TruncateMPS
 *   MeasureOneSiteOp / MeasureTwoSiteOp / MeasureMultiSiteOp / DumpMeasuRes
 *     (finite_mps_measu.h:150-584)                 same names
 *   TwoSiteFiniteVMPS (..._vmps_impl.h:77-101)     gqmps2::TwoSiteFiniteVMPS
 *   LanczosSolver / LanczosRes (lanczos_solver_impl.h:71-226)
 *                                                  gqmps2::LanczosSolver / LanczosRes
 *   gqten Contract (call sites ..._vmps_impl.h:118-129, 243, 272-317)
 *                                                  gqmps2::Contract
 *
 * The tensor type is this library's host block-sparse tensor
 * (gqmps2::GQTensor: real FP64, U(1)^n quantum numbers) in place of gqten's
 * GQTensor<GQTEN_Double, QNT>; it converts to and from device tensors
 * (gqmps2::DeviceTensor) of the C ABI.  Files use the layout that
 * mps2_gb300/finite_mps.py:write_tensor documents ("GQTB", version 1), under
 * the reference's file names (GenMPSTenName mps.h:31-34, GenEnvTenName
 * two_site_update_finite_vmps_impl.h:55-61).
 *
 * Errors: a nonzero status of the C ABI becomes gqmps2::Error carrying
 * gq_last_error(); a malformed file or argument throws the same type.  The
 * reference asserts or exits instead.
 *
 * C++17, POSIX (stat/mkdir for the paths).  Link with -lgqmps2_gb300.
 */
#ifndef GQMPS2_GB300_HPP
#define GQMPS2_GB300_HPP

#include "gqmps2_gb300.h"

#include <sys/stat.h>
#include <sys/types.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gqmps2 {

/* ---------------------------------------------------------------------- */
/* errors                                                                  */
/* ---------------------------------------------------------------------- */
class Error : public std::runtime_error {
 public:
  explicit Error(const std::string &what) : std::runtime_error(what) {}
};

inline void Check(int status) {
  if (status != GQ_OK) {
    const char *msg = gq_last_error();
    throw Error(std::string("libgqmps2_gb300: ") + (msg && *msg ? msg : "error ") +
                (msg && *msg ? "" : std::to_string(status)));
  }
}

/* ---------------------------------------------------------------------- */
/* quantum numbers and legs                                                */
/* ---------------------------------------------------------------------- */
using QN = std::vector<int>;  // U(1)^n charges, n <= 4

inline QN operator+(const QN &a, const QN &b) {
  if (a.size() != b.size()) throw Error("QN: different numbers of charges");
  QN c(a.size());
  for (size_t i = 0; i < a.size(); ++i) c[i] = a[i] + b[i];
  return c;
}
inline QN operator-(const QN &a, const QN &b) {
  if (a.size() != b.size()) throw Error("QN: different numbers of charges");
  QN c(a.size());
  for (size_t i = 0; i < a.size(); ++i) c[i] = a[i] - b[i];
  return c;
}
inline QN operator-(const QN &a) { return QN(a.size(), 0) - a; }

struct QNSector {
  QNSector() = default;
  QNSector(QN q, int64_t d) : qn(std::move(q)), dim(d) {}
  QN qn;
  int64_t dim = 0;
  bool operator==(const QNSector &o) const { return qn == o.qn && dim == o.dim; }
};

constexpr int OUT = GQ_OUT;
constexpr int IN = GQ_IN;

/* A leg: direction plus ordered (QN, degeneracy) sectors. */
struct Index {
  Index() = default;
  Index(std::vector<QNSector> s, int d) : sectors(std::move(s)), dir(d) {
    if (dir != OUT && dir != IN) throw Error("Index: direction must be IN or OUT");
    for (auto &x : sectors)
      if (x.dim <= 0) throw Error("Index: sector dimensions must be positive");
  }
  std::vector<QNSector> sectors;
  int dir = OUT;

  int64_t dim() const {
    int64_t d = 0;
    for (auto &s : sectors) d += s.dim;
    return d;
  }
  size_t nq() const { return sectors.empty() ? 0 : sectors[0].qn.size(); }
  int GetDir() const { return dir; }
  /* (sector, offset inside it) of an actual coordinate */
  std::pair<size_t, int64_t> CoorToSector(int64_t coor) const {
    for (size_t s = 0; s < sectors.size(); ++s) {
      if (coor < sectors[s].dim) return {s, coor};
      coor -= sectors[s].dim;
    }
    throw Error("Index: coordinate out of range");
  }
  const QNSector &GetQNSctFromActualCoor(int64_t coor) const {
    return sectors[CoorToSector(coor).first];
  }
  bool operator==(const Index &o) const { return dir == o.dir && sectors == o.sectors; }
  bool operator!=(const Index &o) const { return !(*this == o); }
};

inline Index InverseIndex(const Index &ix) { return Index(ix.sectors, -ix.dir); }

/* ---------------------------------------------------------------------- */
/* host block-sparse tensor                                                */
/* ---------------------------------------------------------------------- */
class GQTensor {
 public:
  using Coords = std::vector<int>;  // sector coordinate of a block

  GQTensor() = default;
  explicit GQTensor(std::vector<Index> indices) : indices_(std::move(indices)) {}
  GQTensor(std::vector<Index> indices, QN div)
      : indices_(std::move(indices)), div_(std::move(div)), has_div_(true) {}

  const std::vector<Index> &GetIndexes() const { return indices_; }
  size_t Rank() const { return indices_.size(); }
  bool IsDefault() const { return indices_.empty(); }
  size_t nq() const {
    for (auto &ix : indices_)
      if (ix.nq()) return ix.nq();
    return div_.size();
  }
  /* divergence: set by the first stored element, or given at construction */
  QN Div() const { return has_div_ ? div_ : QN(nq(), 0); }

  std::vector<int64_t> BlockShape(const Coords &c) const {
    std::vector<int64_t> s(c.size());
    for (size_t l = 0; l < c.size(); ++l) s[l] = indices_[l].sectors[c[l]].dim;
    return s;
  }
  QN BlockDiv(const Coords &c) const {
    QN q(nq(), 0);
    for (size_t l = 0; l < c.size(); ++l) {
      const QN &s = indices_[l].sectors[c[l]].qn;
      for (size_t k = 0; k < q.size(); ++k) q[k] += indices_[l].dir * s[k];
    }
    return q;
  }

  /* element access by actual coordinates, as gqten's t(i, j, ...) */
  void SetElem(const std::vector<int64_t> &coors, double v) {
    auto [c, off] = Locate(coors);
    auto it = blocks_.find(c);
    if (it == blocks_.end()) {
      QN d = BlockDiv(c);
      if (!has_div_) {
        div_ = d;
        has_div_ = true;
      } else if (d != div_) {
        throw Error("GQTensor: element breaks the tensor's divergence");
      }
      int64_t n = 1;
      for (auto s : BlockShape(c)) n *= s;
      it = blocks_.emplace(c, std::vector<double>(n, 0.0)).first;
    }
    it->second[off] = v;
  }
  double GetElem(const std::vector<int64_t> &coors) const {
    auto [c, off] = Locate(coors);
    auto it = blocks_.find(c);
    return it == blocks_.end() ? 0.0 : it->second[off];
  }

  /* stored blocks in ascending sector-coordinate order ("block order") */
  const std::map<Coords, std::vector<double>> &Blocks() const { return blocks_; }
  std::map<Coords, std::vector<double>> &Blocks() { return blocks_; }

  bool operator==(const GQTensor &o) const {
    return indices_ == o.indices_ && Div() == o.Div() && blocks_ == o.blocks_;
  }
  bool operator!=(const GQTensor &o) const { return !(*this == o); }

  /* file layout: "GQTB", u32 version (1), u32 rank, u32 nq, i32[nq] div;
   * per leg i32 dir, u32 nsec, nsec x (i32[nq] qn, i64 dim); u64 nblocks;
   * nblocks x u32[rank] coordinates; the blocks' float64 data in that order.
   * Little endian (both supported hosts are). */
  void Dump(const std::string &file) const {
    std::ofstream f(file, std::ios::binary);
    if (!f) throw Error("cannot write " + file);
    const uint32_t rank = (uint32_t)Rank(), q = (uint32_t)nq();
    f.write("GQTB", 4);
    Put<uint32_t>(f, 1);
    Put<uint32_t>(f, rank);
    Put<uint32_t>(f, q);
    for (int v : Div()) Put<int32_t>(f, v);
    for (auto &ix : indices_) {
      Put<int32_t>(f, ix.dir);
      Put<uint32_t>(f, (uint32_t)ix.sectors.size());
      for (auto &s : ix.sectors) {
        for (int v : s.qn) Put<int32_t>(f, v);
        Put<int64_t>(f, s.dim);
      }
    }
    Put<uint64_t>(f, blocks_.size());
    for (auto &b : blocks_)
      for (int c : b.first) Put<uint32_t>(f, (uint32_t)c);
    for (auto &b : blocks_)
      f.write(reinterpret_cast<const char *>(b.second.data()),
              (std::streamsize)(b.second.size() * sizeof(double)));
    if (!f) throw Error("write failed: " + file);
  }

  void Load(const std::string &file) {
    std::ifstream f(file, std::ios::binary);
    if (!f) throw Error("cannot read " + file);
    char magic[4];
    f.read(magic, 4);
    if (!f || std::memcmp(magic, "GQTB", 4) != 0) throw Error(file + ": not a tensor file");
    if (Get<uint32_t>(f) != 1) throw Error(file + ": unsupported version");
    const uint32_t rank = Get<uint32_t>(f), q = Get<uint32_t>(f);
    QN div(q);
    for (auto &v : div) v = Get<int32_t>(f);
    std::vector<Index> idx;
    for (uint32_t l = 0; l < rank; ++l) {
      int dir = Get<int32_t>(f);
      uint32_t nsec = Get<uint32_t>(f);
      std::vector<QNSector> secs(nsec);
      for (auto &s : secs) {
        s.qn.resize(q);
        for (auto &v : s.qn) v = Get<int32_t>(f);
        s.dim = Get<int64_t>(f);
      }
      idx.emplace_back(std::move(secs), dir);
    }
    GQTensor t(std::move(idx), div);
    const uint64_t nb = Get<uint64_t>(f);
    std::vector<Coords> coords(nb, Coords(rank));
    for (auto &c : coords)
      for (auto &v : c) {
        v = (int)Get<uint32_t>(f);
      }
    for (auto &c : coords) {
      for (uint32_t l = 0; l < rank; ++l)
        if (c[l] < 0 || (size_t)c[l] >= t.indices_[l].sectors.size())
          throw Error(file + ": block coordinate out of range");
      int64_t n = 1;
      for (auto s : t.BlockShape(c)) n *= s;
      std::vector<double> data(n);
      f.read(reinterpret_cast<char *>(data.data()), (std::streamsize)(n * sizeof(double)));
      t.blocks_.emplace(c, std::move(data));
    }
    if (!f) throw Error(file + ": truncated");
    f.peek();
    if (!f.eof()) throw Error(file + ": trailing bytes");
    *this = std::move(t);
  }

 private:
  std::pair<Coords, int64_t> Locate(const std::vector<int64_t> &coors) const {
    if (coors.size() != Rank()) throw Error("GQTensor: wrong number of coordinates");
    Coords c(Rank());
    int64_t off = 0;
    for (size_t l = 0; l < Rank(); ++l) {
      auto [s, o] = indices_[l].CoorToSector(coors[l]);
      c[l] = (int)s;
      off = off * indices_[l].sectors[s].dim + o;
    }
    return {c, off};
  }
  template <typename T>
  static void Put(std::ofstream &f, T v) {
    f.write(reinterpret_cast<const char *>(&v), sizeof(T));
  }
  template <typename T>
  static T Get(std::ifstream &f) {
    T v{};
    f.read(reinterpret_cast<char *>(&v), sizeof(T));
    if (!f) throw Error("tensor file truncated");
    return v;
  }

  std::vector<Index> indices_;
  QN div_;
  bool has_div_ = false;
  std::map<Coords, std::vector<double>> blocks_;
};

/* ---------------------------------------------------------------------- */
/* device tensors (owning handle of the C ABI)                             */
/* ---------------------------------------------------------------------- */
class DeviceTensor {
 public:
  DeviceTensor() = default;
  explicit DeviceTensor(gq_tensor *h) : h_(h) {}
  DeviceTensor(const DeviceTensor &) = delete;
  DeviceTensor &operator=(const DeviceTensor &) = delete;
  DeviceTensor(DeviceTensor &&o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  DeviceTensor &operator=(DeviceTensor &&o) noexcept {
    std::swap(h_, o.h_);
    return *this;
  }
  ~DeviceTensor() {
    if (h_) gq_tensor_destroy(h_);
  }
  gq_tensor *get() const { return h_; }
  gq_tensor *release() {
    gq_tensor *h = h_;
    h_ = nullptr;
    return h;
  }

  static DeviceTensor FromHost(const GQTensor &t) {
    const int rank = (int)t.Rank(), q = (int)t.nq();
    std::vector<int> dirs, nsecs, qns, div = t.Div(), coords;
    std::vector<int64_t> dims;
    for (auto &ix : t.GetIndexes()) {
      dirs.push_back(ix.dir);
      nsecs.push_back((int)ix.sectors.size());
      for (auto &s : ix.sectors) {
        qns.insert(qns.end(), s.qn.begin(), s.qn.end());
        dims.push_back(s.dim);
      }
    }
    std::vector<double> data;
    for (auto &b : t.Blocks()) {
      coords.insert(coords.end(), b.first.begin(), b.first.end());
      data.insert(data.end(), b.second.begin(), b.second.end());
    }
    gq_tensor *h = nullptr;
    Check(gq_tensor_create(rank, q, dirs.data(), nsecs.data(), qns.data(), dims.data(),
                           div.data(), (int64_t)t.Blocks().size(), coords.data(),
                           data.empty() ? nullptr : data.data(), &h));
    return DeviceTensor(h);
  }

  GQTensor ToHost() const {
    int rank = 0, q = 0;
    int64_t nsec = 0, nb = 0, ne = 0;
    Check(gq_tensor_describe(h_, &rank, &q, &nsec, &nb, &ne));
    std::vector<int> dirs(rank), nsecs(rank), qns(nsec * q + 1), div(q + 1), coords(nb * rank + 1);
    std::vector<int64_t> dims(nsec + 1);
    std::vector<double> data(ne + 1);
    Check(gq_tensor_export(h_, dirs.data(), nsecs.data(), qns.data(), dims.data(), div.data(),
                           coords.data(), data.data()));
    std::vector<Index> idx;
    int64_t so = 0;
    for (int l = 0; l < rank; ++l) {
      std::vector<QNSector> secs;
      for (int s = 0; s < nsecs[l]; ++s, ++so)
        secs.emplace_back(QN(qns.begin() + so * q, qns.begin() + (so + 1) * q), dims[so]);
      idx.emplace_back(std::move(secs), dirs[l]);
    }
    GQTensor t(std::move(idx), QN(div.begin(), div.begin() + q));
    int64_t off = 0;
    for (int64_t b = 0; b < nb; ++b) {
      GQTensor::Coords c(coords.begin() + b * rank, coords.begin() + (b + 1) * rank);
      int64_t n = 1;
      for (auto s : t.BlockShape(c)) n *= s;
      t.Blocks().emplace(c, std::vector<double>(data.begin() + off, data.begin() + off + n));
      off += n;
    }
    return t;
  }

 private:
  gq_tensor *h_ = nullptr;
};

/* gqten Contract(pa, pb, {axes_a, axes_b}, pc) on the GPU (FP64): the
 * result's legs are a's free legs then b's free legs. */
inline void Contract(const GQTensor *pa, const GQTensor *pb,
                     const std::vector<std::vector<size_t>> &axes_set, GQTensor *pc,
                     int precision = GQ_PREC_FP64) {
  if (axes_set.size() != 2 || axes_set[0].size() != axes_set[1].size())
    throw Error("Contract: axes_set must hold two lists of equal length");
  DeviceTensor a = DeviceTensor::FromHost(*pa), b = DeviceTensor::FromHost(*pb);
  std::vector<int> xa(axes_set[0].begin(), axes_set[0].end());
  std::vector<int> xb(axes_set[1].begin(), axes_set[1].end());
  gq_tensor *c = nullptr;
  double flops = 0.0;
  Check(gq_contract(a.get(), b.get(), (int)xa.size(), xa.data(), xb.data(), precision, &c,
                    &flops));
  *pc = DeviceTensor(c).ToHost();
}

/* ---------------------------------------------------------------------- */
/* containers                                                              */
/* ---------------------------------------------------------------------- */
/* Fixed-size vector of optionally present tensors (DuoVector + TenVec). */
template <typename TenT>
class TenVec {
 public:
  explicit TenVec(size_t n = 0) : raw_(n) {}
  TenVec(const TenVec &o) : raw_(o.raw_.size()) {
    for (size_t i = 0; i < o.raw_.size(); ++i)
      if (o.raw_[i]) raw_[i] = std::make_unique<TenT>(*o.raw_[i]);
  }
  TenVec &operator=(const TenVec &o) {
    TenVec c(o);
    raw_.swap(c.raw_);
    return *this;
  }
  TenVec(TenVec &&) noexcept = default;
  TenVec &operator=(TenVec &&) noexcept = default;
  virtual ~TenVec() = default;

  size_t size() const { return raw_.size(); }
  /* setter: allocates a default element if absent (duovector.h:121-126) */
  TenT &operator[](size_t i) {
    if (!raw_.at(i)) raw_[i] = std::make_unique<TenT>();
    return *raw_[i];
  }
  const TenT &operator[](size_t i) const {
    if (!raw_.at(i)) throw Error("TenVec: element " + std::to_string(i) + " is not allocated");
    return *raw_[i];
  }
  const TenT *operator()(size_t i) const { return raw_.at(i).get(); }
  void alloc(size_t i) {
    if (!raw_.at(i)) raw_[i] = std::make_unique<TenT>();
  }
  void dealloc(size_t i) { raw_.at(i).reset(); }
  void clear() {
    for (auto &p : raw_) p.reset();
  }
  bool empty() const {
    for (auto &p : raw_)
      if (p) return false;
    return true;
  }
  void LoadTen(size_t i, const std::string &file) { (*this)[i].Load(file); }
  void DumpTen(size_t i, const std::string &file, bool release_mem = false) {
    (*this)[i].Dump(file);
    if (release_mem) dealloc(i);
  }

 private:
  std::vector<std::unique_ptr<TenT>> raw_;
};

template <typename TenT = GQTensor>
using MPO = TenVec<TenT>;

/* identity operator on one site: legs (IN, OUT) (site_vec.h:47-53) */
inline GQTensor GenIdOp(const Index &pb_out) {
  GQTensor op({InverseIndex(pb_out), pb_out});
  for (int64_t i = 0; i < pb_out.dim(); ++i) op.SetElem({i, i}, 1.0);
  return op;
}

struct SiteVec {
  SiteVec(size_t n, const Index &pb) : sites(n, pb.dir == OUT ? pb : InverseIndex(pb)) {
    Fill();
  }
  explicit SiteVec(const std::vector<Index> &pbs) {
    for (auto &ix : pbs) sites.push_back(ix.dir == OUT ? ix : InverseIndex(ix));
    Fill();
  }
  size_t size = 0;
  std::vector<Index> sites;
  std::vector<GQTensor> id_ops;

 private:
  void Fill() {
    size = sites.size();
    for (auto &ix : sites) id_ops.push_back(GenIdOp(ix));
  }
};

const std::string kMpsPath = "mps";
const std::string kRuntimeTempPath = ".temp";
const std::string kGQTenFileSuffix = "gqten";

inline std::string GenMPSTenName(const std::string &mps_path, size_t idx) {
  return mps_path + "/mps_ten" + std::to_string(idx) + "." + kGQTenFileSuffix;
}
inline std::string GenEnvTenName(const std::string &dir, size_t blk_len,
                                 const std::string &temp_path) {
  return temp_path + "/" + dir + "env" + std::to_string(blk_len) + "." + kGQTenFileSuffix;
}
inline bool IsPathExist(const std::string &path) {
  struct stat st;
  return stat(path.c_str(), &st) == 0;
}
inline void CreatPath(const std::string &path) {
  if (mkdir(path.c_str(), 0755) != 0 && !IsPathExist(path))
    throw Error("cannot create directory " + path);
}

enum MPSTenCanoType { NONE = GQ_CANO_NONE, LEFT = GQ_CANO_LEFT, RIGHT = GQ_CANO_RIGHT };
const long kUncentralizedCenterIdx = -1;

class FiniteMPS : public TenVec<GQTensor> {
 public:
  explicit FiniteMPS(const SiteVec &sv)
      : TenVec<GQTensor>(sv.size), tens_cano_type_(sv.size, NONE), site_vec_(sv) {}
  /* write access marks the site non-canonical and the MPS uncentralised, as
   * the reference's non-const accessor does (finite_mps.h:67-75) */
  GQTensor &operator[](size_t i) {
    tens_cano_type_.at(i) = NONE;
    center_ = kUncentralizedCenterIdx;
    return TenVec<GQTensor>::operator[](i);
  }
  const GQTensor &operator[](size_t i) const { return TenVec<GQTensor>::operator[](i); }
  const SiteVec &GetSitesInfo() const { return site_vec_; }
  std::vector<MPSTenCanoType> GetTensCanoType() const { return tens_cano_type_; }
  MPSTenCanoType GetTenCanoType(size_t i) const { return tens_cano_type_.at(i); }
  long GetCenter() const { return center_; }
  void Dump(const std::string &mps_path = kMpsPath, bool release_mem = false) {
    CreatPath(mps_path);
    for (size_t i = 0; i < size(); ++i) DumpTen(i, GenMPSTenName(mps_path, i), release_mem);
  }
  void Load(const std::string &mps_path = kMpsPath) {
    for (size_t i = 0; i < size(); ++i) LoadTen(i, GenMPSTenName(mps_path, i));
  }
  /* FiniteMPS::Centralize (finite_mps.h:149-248) on the GPU: every site must
   * be loaded; the tensors are replaced by the canonicalised ones. */
  void Centralize(long target_center) {
    const int n = (int)size();
    std::vector<int> cano(tens_cano_type_.begin(), tens_cano_type_.end());
    const FiniteMPS &self = *this;  // reads leave the canonical types alone
    std::vector<DeviceTensor> d;
    std::vector<gq_tensor *> h;
    for (int i = 0; i < n; ++i) {
      d.push_back(DeviceTensor::FromHost(self[i]));
      h.push_back(d.back().get());
    }
    Check(gq_mps_centralize(h.data(), n, (int)target_center, cano.data()));
    for (int i = 0; i < n; ++i) {  // the handles' tensors were rewritten in place
      (*this)[i] = d[i].ToHost();
      tens_cano_type_[i] = (MPSTenCanoType)cano[i];
    }
    center_ = target_center;
  }
  std::vector<MPSTenCanoType> tens_cano_type_;
  long center_ = kUncentralizedCenterIdx;

 private:
  SiteVec site_vec_;
};

/* TruncateMPS (finite_mps.h:251-300) on the GPU: centralise at 0, normalise
 * the head, then one truncating SVD per bond from the left.  Every site must
 * be loaded.  Optionally returns each bond's truncation error and dimension
 * (the reference prints them). */
inline void TruncateMPS(FiniteMPS &mps, double trunc_err, size_t Dmin, size_t Dmax,
                        std::vector<double> *errs = nullptr,
                        std::vector<int64_t> *dims = nullptr) {
  const int n = (int)mps.size();
  if (n < 2) throw Error("TruncateMPS: at least two sites");
  std::vector<int> cano(mps.tens_cano_type_.begin(), mps.tens_cano_type_.end());
  const FiniteMPS &cm = mps;
  std::vector<DeviceTensor> d;
  std::vector<gq_tensor *> h;
  for (int i = 0; i < n; ++i) {
    d.push_back(DeviceTensor::FromHost(cm[i]));
    h.push_back(d.back().get());
  }
  std::vector<double> e(n - 1);
  std::vector<int64_t> D(n - 1);
  Check(gq_mps_truncate(h.data(), n, cano.data(), trunc_err, (int64_t)Dmin, (int64_t)Dmax,
                        e.data(), D.data()));
  for (int i = 0; i < n; ++i) {  // the handles' tensors were rewritten in place
    mps[i] = d[i].ToHost();
    mps.tens_cano_type_[i] = (MPSTenCanoType)cano[i];
  }
  if (errs) *errs = e;
  if (dims) *dims = D;
}

/* finite_mps_init.h:216-262: bond-dimension-1 product state; the result is
 * already right-canonical (what the reference's trailing Centralize(0)
 * gives for it). */
inline void DirectStateInitMps(FiniteMPS &mps, const std::vector<size_t> &stat_labs,
                               const QN &zero_div) {
  const size_t N = mps.size();
  if (N != stat_labs.size()) throw Error("DirectStateInitMps: one label per site");
  if (N < 2) throw Error("DirectStateInitMps: at least two sites");
  const auto &pb = mps.GetSitesInfo().sites;
  std::vector<QN> qs;
  for (size_t i = 0; i < N; ++i) qs.push_back(pb[i].GetQNSctFromActualCoor(stat_labs[i]).qn);
  QN div = qs[0];
  for (size_t i = 1; i < N; ++i) div = div + qs[i];
  Index rvb({QNSector(div - qs[0], 1)}, OUT);
  GQTensor t0({pb[0], rvb});
  t0.SetElem({(int64_t)stat_labs[0], 0}, 1.0);
  mps[0] = t0;
  for (size_t i = 1; i + 1 < N; ++i) {
    Index lvb = InverseIndex(rvb);
    rvb = Index({QNSector(zero_div - qs[i] + lvb.sectors[0].qn, 1)}, OUT);
    GQTensor t({lvb, pb[i], rvb});
    t.SetElem({0, (int64_t)stat_labs[i], 0}, 1.0);
    mps[i] = t;
  }
  GQTensor tl({InverseIndex(rvb), pb[N - 1]});
  tl.SetElem({0, (int64_t)stat_labs[N - 1]}, 1.0);
  mps[N - 1] = tl;
  mps.tens_cano_type_.assign(N, RIGHT);
  mps.tens_cano_type_[0] = NONE;
  mps.center_ = 0;
}

/* ---------------------------------------------------------------------- */
/* parameters                                                              */
/* ---------------------------------------------------------------------- */
struct LanczosParams {
  LanczosParams(double err, size_t max_iter) : error(err), max_iterations(max_iter) {}
  LanczosParams(double err) : LanczosParams(err, 200) {}
  LanczosParams() : LanczosParams(1.0E-7, 200) {}
  double error;
  size_t max_iterations;
  /* split form only: arithmetic of the Rayleigh-quotient energy */
  int rayleigh = GQ_PREC_FP64;
};

struct SweepParams {
  SweepParams(size_t sweeps, size_t dmin, size_t dmax, double trunc_err,
              const LanczosParams &lancz_params, const std::string mps_path = kMpsPath,
              const std::string temp_path = kRuntimeTempPath)
      : sweeps(sweeps), Dmin(dmin), Dmax(dmax), trunc_err(trunc_err),
        lancz_params(lancz_params), mps_path(mps_path), temp_path(temp_path) {}
  size_t sweeps;
  size_t Dmin;
  size_t Dmax;
  double trunc_err;
  LanczosParams lancz_params;
  std::string mps_path;
  std::string temp_path;
  /* not in the reference: arithmetic of the contractions (GQ_PREC_*) and the
   * per-update log line */
  int precision = GQ_PREC_FP64;
  int verbose = 1;

  gq_sweep_params ToC() const {
    gq_sweep_params p{};
    p.sweeps = (int64_t)sweeps;
    p.dmin = (int64_t)Dmin;
    p.dmax = (int64_t)Dmax;
    p.trunc_err = trunc_err;
    p.lanczos.error = lancz_params.error;
    p.lanczos.max_iterations = (int64_t)lancz_params.max_iterations;
    p.lanczos.rayleigh = lancz_params.rayleigh;
    p.precision = precision;
    p.verbose = verbose;
    return p;
  }
};

/* ---------------------------------------------------------------------- */
/* measurement (finite_mps_measu.h:150-584)                                */
/* ---------------------------------------------------------------------- */
struct MeasuResElem {
  std::vector<size_t> sites;
  double avg = 0.0;
};
using MeasuRes = std::vector<MeasuResElem>;
using MeasuResSet = std::vector<MeasuRes>;

/* DumpMeasuRes (:556-584): "[\n  [[i, j], avg],\n  ...]" in <basename>.json,
 * averages with 12 significant digits in a 14-wide field. */
inline void DumpMeasuRes(const MeasuRes &res, const std::string &basename) {
  std::FILE *f = std::fopen((basename + ".json").c_str(), "w");
  if (!f) throw Error("cannot write " + basename + ".json");
  std::fputs("[\n", f);
  for (size_t n = 0; n < res.size(); ++n) {
    std::fputs("  [[", f);
    for (size_t k = 0; k < res[n].sites.size(); ++k)
      std::fprintf(f, k ? ", %zu" : "%zu", res[n].sites[k]);
    std::fprintf(f, "], %14.12g", res[n].avg);
    std::fputs(n + 1 == res.size() ? "]\n" : "],\n", f);
  }
  std::fputs("]", f);
  std::fclose(f);
}

namespace measu_detail {

inline DeviceTensor Contract(const DeviceTensor &a, const DeviceTensor &b,
                             const std::vector<int> &xa, const std::vector<int> &xb) {
  gq_tensor *c = nullptr;
  double flops = 0.0;
  Check(gq_contract(a.get(), b.get(), (int)xa.size(), xa.data(), xb.data(), GQ_PREC_FP64, &c,
                    &flops));
  return DeviceTensor(c);
}

inline DeviceTensor Dag(const DeviceTensor &a) {
  gq_tensor *c = nullptr;
  Check(gq_tensor_dag(a.get(), &c));
  return DeviceTensor(c);
}

/* every leg of a (in order xa) against every leg of b (in order xb), on the
 * host: the last contraction of each event reduces two site-sized tensors to
 * one number */
inline double FullContract(const GQTensor &a, const GQTensor &b, const std::vector<int> &xa,
                           const std::vector<int> &xb) {
  const size_t r = a.Rank();
  if (b.Rank() != r || xa.size() != r || xb.size() != r)
    throw Error("full contraction: every leg must be contracted");
  double acc = 0.0;
  for (auto &ba : a.Blocks()) {
    GQTensor::Coords cb(r);
    for (size_t k = 0; k < r; ++k) cb[xb[k]] = ba.first[xa[k]];
    auto it = b.Blocks().find(cb);
    if (it == b.Blocks().end()) continue;
    const auto sa = a.BlockShape(ba.first), sb = b.BlockShape(cb);
    std::vector<int64_t> strb(r, 1), step(r, 0);  // b's stride along each of a's legs
    for (int j = (int)r - 2; j >= 0; --j) strb[j] = strb[j + 1] * sb[j + 1];
    for (size_t k = 0; k < r; ++k) step[xa[k]] = strb[xb[k]];
    std::vector<int64_t> idx(r, 0);
    int64_t ob = 0;
    for (double va : ba.second) {  // a's elements in row-major order
      acc += va * it->second[ob];
      for (int l = (int)r - 1; l >= 0; --l) {  // odometer over a's legs
        if (++idx[l] < sa[l]) {
          ob += step[l];
          break;
        }
        ob -= step[l] * (sa[l] - 1);
        idx[l] = 0;
      }
    }
  }
  return acc;
}

/* the MPS on the device with the reference's canonical-type bookkeeping */
struct DeviceMPS {
  explicit DeviceMPS(FiniteMPS &m) : host(m), n((int)m.size()) {
    cano.assign(m.tens_cano_type_.begin(), m.tens_cano_type_.end());
    const FiniteMPS &cm = m;
    for (int i = 0; i < n; ++i) t.push_back(DeviceTensor::FromHost(cm[i]));
    center = m.GetCenter();
  }
  void Centralize(int c) {
    std::vector<gq_tensor *> h;
    for (auto &x : t) h.push_back(x.get());
    Check(gq_mps_centralize(h.data(), n, c, cano.data()));
    center = c;
  }
  void WriteBack() {
    for (int i = 0; i < n; ++i) {
      host[i] = t[i].ToHost();
      host.tens_cano_type_[i] = (MPSTenCanoType)cano[i];
    }
    host.center_ = center;
  }
  FiniteMPS &host;
  int n;
  std::vector<DeviceTensor> t;
  std::vector<int> cano;
  long center = -1;
};

/* OneSiteOpAvg (:366-402) */
inline double OneSiteOpAvg(const DeviceTensor &cent, const DeviceTensor &op, int site, int n) {
  std::vector<int> x1, y1{0}, x2, y2;
  if (site == 0) {
    x1 = {0}; x2 = {0, 1}; y2 = {1, 0};
  } else if (site == n - 1) {
    x1 = {1}; x2 = {0, 1}; y2 = {0, 1};
  } else {
    x1 = {1}; x2 = {0, 2, 1}; y2 = {0, 1, 2};
  }
  DeviceTensor temp = Contract(cent, op, x1, y1);
  return FullContract(temp.ToHost(), Dag(cent).ToHost(), x2, y2);
}

/* CtrctMidTen (:528-554) */
inline DeviceTensor CtrctMidTen(DeviceMPS &dm, int site, const GQTensor &op,
                                const GQTensor &id_op, const DeviceTensor &t) {
  const DeviceTensor &a = dm.t[site];
  if (op == id_op) {
    DeviceTensor temp = Contract(a, t, {0}, {0});
    return Contract(temp, Dag(a), {0, 2}, {1, 0});
  }
  DeviceTensor temp1 = Contract(a, t, {0}, {0});
  DeviceTensor temp2 = Contract(temp1, DeviceTensor::FromHost(op), {0}, {0});
  return Contract(temp2, Dag(a), {1, 2}, {0, 1});
}

/* OpsVecAvg (:462-526): the MPS is centralised at `head` */
inline double OpsVecAvg(DeviceMPS &dm, const std::vector<GQTensor> &ops, int head, int tail) {
  if ((int)ops.size() != tail - head + 1) throw Error("measurement: one operator per site");
  const auto &id_ops = dm.host.GetSitesInfo().id_ops;
  std::vector<int> a1, a2, a3;
  if (head == 0) {
    a1 = {0}; a2 = {1}; a3 = {0};
  } else {
    a1 = {1}; a2 = {0, 2}; a3 = {0, 1};
  }
  const DeviceTensor &h = dm.t[head];
  DeviceTensor temp0 = Contract(h, DeviceTensor::FromHost(ops[0]), a1, {0});
  DeviceTensor t = Contract(temp0, Dag(h), a2, a3);
  for (int i = head + 1; i < tail; ++i) t = CtrctMidTen(dm, i, ops[i - head], id_ops[i], t);
  std::vector<int> b1, b2;
  if (tail == dm.n - 1) {
    b1 = {0, 1}; b2 = {0, 1};
  } else {
    b1 = {0, 1, 2}; b2 = {2, 0, 1};
  }
  const DeviceTensor &tl = dm.t[tail];
  DeviceTensor temp2 = Contract(tl, t, {0}, {0});
  DeviceTensor temp3 = Contract(temp2, DeviceTensor::FromHost(ops.back()), {0}, {0});
  return FullContract(temp3.ToHost(), Dag(tl).ToHost(), b1, b2);
}

/* MultiSiteOpAvg (:404-437): A, inserts, B, inserts, ..., and an optional
 * tail string after the last physical operator */
inline MeasuResElem MultiSiteOpAvg(DeviceMPS &dm, const std::vector<GQTensor> &phys_ops,
                                   const std::vector<std::vector<GQTensor>> &inst_ops_set,
                                   const std::vector<size_t> &sites) {
  const size_t ni = inst_ops_set.size(), np = phys_ops.size();
  if (!(np == ni + 1 || np == ni)) throw Error("measurement: wrong number of insert lists");
  std::vector<GQTensor> ops;
  for (size_t i = 0; i + 1 < np; ++i) {
    ops.push_back(phys_ops[i]);
    ops.insert(ops.end(), inst_ops_set[i].begin(), inst_ops_set[i].end());
  }
  ops.push_back(phys_ops.back());
  if (ni == np) ops.insert(ops.end(), inst_ops_set.back().begin(), inst_ops_set.back().end());
  const int head = (int)sites[0];
  const int tail = head + (int)ops.size() - 1;
  return MeasuResElem{sites, OpsVecAvg(dm, ops, head, tail)};
}

inline void CheckSites(const std::vector<size_t> &sites) {
  if (sites.size() < 2) throw Error("measurement: at least two sites per event");
  for (size_t k = 1; k < sites.size(); ++k)
    if (sites[k] < sites[k - 1]) throw Error("measurement: sites must be ascending");
}

}  // namespace measu_detail

/* MeasureOneSiteOp (:150-214), a list of operators: one result per operator
 * and site; the MPS ends centralised at its last site. */
inline MeasuResSet MeasureOneSiteOp(FiniteMPS &mps, const std::vector<GQTensor> &ops,
                                    const std::vector<std::string> &res_file_basenames) {
  if (ops.size() != res_file_basenames.size())
    throw Error("MeasureOneSiteOp: one file name per operator");
  measu_detail::DeviceMPS dm(mps);
  std::vector<DeviceTensor> dops;
  for (auto &o : ops) dops.push_back(DeviceTensor::FromHost(o));
  MeasuResSet res(ops.size(), MeasuRes(dm.n));
  for (int i = 0; i < dm.n; ++i) {
    dm.Centralize(i);
    for (size_t j = 0; j < ops.size(); ++j)
      res[j][i] = MeasuResElem{{(size_t)i}, measu_detail::OneSiteOpAvg(dm.t[i], dops[j], i, dm.n)};
  }
  dm.WriteBack();
  for (size_t j = 0; j < ops.size(); ++j) DumpMeasuRes(res[j], res_file_basenames[j]);
  return res;
}

inline MeasuRes MeasureOneSiteOp(FiniteMPS &mps, const GQTensor &op,
                                 const std::string &res_file_basename) {
  return MeasureOneSiteOp(mps, std::vector<GQTensor>{op},
                          std::vector<std::string>{res_file_basename})[0];
}

/* MeasureMultiSiteOp (:300-340): inst_ops_set[e][g] lists the insert
 * operators of gap g of event e. */
inline MeasuRes MeasureMultiSiteOp(FiniteMPS &mps,
                                   const std::vector<std::vector<GQTensor>> &phys_ops_set,
                                   const std::vector<std::vector<std::vector<GQTensor>>> &inst_ops_set,
                                   const std::vector<std::vector<size_t>> &sites_set,
                                   const std::string &res_file_basename) {
  if (phys_ops_set.size() != sites_set.size() || inst_ops_set.size() != sites_set.size())
    throw Error("MeasureMultiSiteOp: one operator list per event");
  measu_detail::DeviceMPS dm(mps);
  MeasuRes res;
  for (size_t e = 0; e < sites_set.size(); ++e) {
    measu_detail::CheckSites(sites_set[e]);
    dm.Centralize((int)sites_set[e][0]);
    res.push_back(measu_detail::MultiSiteOpAvg(dm, phys_ops_set[e], inst_ops_set[e], sites_set[e]));
  }
  dm.WriteBack();
  DumpMeasuRes(res, res_file_basename);
  return res;
}

/* MeasureMultiSiteOp (:342-364): one insert operator repeated across each gap */
inline MeasuRes MeasureMultiSiteOp(FiniteMPS &mps,
                                   const std::vector<std::vector<GQTensor>> &phys_ops_set,
                                   const std::vector<std::vector<GQTensor>> &inst_ops_set,
                                   const std::vector<std::vector<size_t>> &sites_set,
                                   const std::string &res_file_basename) {
  std::vector<std::vector<std::vector<GQTensor>>> full;
  for (size_t e = 0; e < sites_set.size(); ++e) {
    measu_detail::CheckSites(sites_set[e]);
    if (phys_ops_set.at(e).size() != inst_ops_set.at(e).size() + 1)
      throw Error("MeasureMultiSiteOp: one insert operator per gap");
    std::vector<std::vector<GQTensor>> gaps;
    for (size_t g = 0; g < inst_ops_set[e].size(); ++g)
      gaps.emplace_back(sites_set[e][g + 1] - sites_set[e][g] - 1, inst_ops_set[e][g]);
    full.push_back(std::move(gaps));
  }
  return MeasureMultiSiteOp(mps, phys_ops_set, full, sites_set, res_file_basename);
}

/* MeasureTwoSiteOp (:216-259): <A_i O ... O B_j> with its own list of insert
 * operators for each event */
inline MeasuRes MeasureTwoSiteOp(FiniteMPS &mps, const std::vector<GQTensor> &phys_ops,
                                 const std::vector<std::vector<GQTensor>> &inst_ops_set,
                                 const std::vector<std::vector<size_t>> &sites_set,
                                 const std::string &res_file_basename) {
  if (phys_ops.size() != 2) throw Error("MeasureTwoSiteOp: two physical operators");
  if (inst_ops_set.size() != sites_set.size())
    throw Error("MeasureTwoSiteOp: one insert list per event");
  std::vector<std::vector<GQTensor>> phys(sites_set.size(), phys_ops);
  std::vector<std::vector<std::vector<GQTensor>>> inst;
  for (size_t e = 0; e < sites_set.size(); ++e) {
    if (sites_set[e].size() != 2 || sites_set[e][1] - sites_set[e][0] - 1 != inst_ops_set[e].size())
      throw Error("MeasureTwoSiteOp: one insert operator per site between the pair");
    inst.push_back({inst_ops_set[e]});
  }
  return MeasureMultiSiteOp(mps, phys, inst, sites_set, res_file_basename);
}

/* MeasureTwoSiteOp (:261-298): the same insert operator on every site between */
inline MeasuRes MeasureTwoSiteOp(FiniteMPS &mps, const std::vector<GQTensor> &phys_ops,
                                 const GQTensor &inst_op,
                                 const std::vector<std::vector<size_t>> &sites_set,
                                 const std::string &res_file_basename) {
  if (phys_ops.size() != 2) throw Error("MeasureTwoSiteOp: two physical operators");
  std::vector<std::vector<GQTensor>> phys(sites_set.size(), phys_ops);
  std::vector<std::vector<GQTensor>> inst(sites_set.size(), std::vector<GQTensor>{inst_op});
  return MeasureMultiSiteOp(mps, phys, inst, sites_set, res_file_basename);
}

/* ---------------------------------------------------------------------- */
/* the solver                                                              */
/* ---------------------------------------------------------------------- */
/* two_site_update_finite_vmps_impl.h:77-101.  The MPS comes from
 * <mps_path>/mps_ten<i> (right-canonical, as DirectStateInitMps + Dump
 * leave it); the right environments are built on the GPU if <temp_path> does
 * not exist, else read from <temp_path>/renv<len> (resume).  Afterwards the
 * MPS and the right environments are written back and `mps` is empty, as
 * the reference leaves it.  Returns the energy of the last update.
 * Optionally appends one record per update to *stats. */
inline double TwoSiteFiniteVMPS(FiniteMPS &mps, const MPO<GQTensor> &mpo,
                                const SweepParams &sp,
                                std::vector<gq_update_stats> *stats = nullptr) {
  const size_t N = mps.size();
  if (N != mpo.size()) throw Error("TwoSiteFiniteVMPS: mps.size() != mpo.size()");
  if (N < 2) throw Error("TwoSiteFiniteVMPS: at least two sites");
  std::vector<DeviceTensor> dm, dw;
  std::vector<gq_tensor *> hm, hw;
  for (size_t i = 0; i < N; ++i) {
    mps.LoadTen(i, GenMPSTenName(sp.mps_path, i));
    dm.push_back(DeviceTensor::FromHost(mps[i]));
    mps.dealloc(i);
    dw.push_back(DeviceTensor::FromHost(mpo[i]));
    hm.push_back(dm.back().get());
    hw.push_back(dw.back().get());
  }
  gq_dmrg *raw = nullptr;
  Check(gq_dmrg_create((int)N, hm.data(), hw.data(), &raw));
  std::unique_ptr<gq_dmrg, int (*)(gq_dmrg *)> d(raw, gq_dmrg_destroy);
  dm.clear();
  dw.clear();
  if (!IsPathExist(sp.temp_path)) {
    CreatPath(sp.temp_path);
    Check(gq_dmrg_init_envs(d.get(), sp.precision));
  } else {
    for (size_t len = 1; len + 1 < N; ++len) {
      GQTensor env;
      env.Load(GenEnvTenName("r", len, sp.temp_path));
      DeviceTensor de = DeviceTensor::FromHost(env);
      Check(gq_dmrg_set_env(d.get(), 'r', (int)len, de.get()));
    }
  }
  gq_sweep_params p = sp.ToC();
  p.sweeps = 1;
  double e0 = 0.0;
  std::vector<gq_update_stats> rec(2 * (N - 1));
  for (size_t s = 1; s <= sp.sweeps; ++s) {
    if (sp.verbose) std::printf("sweep %zu\n", s);
    Check(gq_dmrg_sweep(d.get(), &p, rec.data(), &e0));
    if (stats) stats->insert(stats->end(), rec.begin(), rec.end());
  }
  for (size_t i = 0; i < N; ++i) {
    gq_tensor *h = nullptr;
    Check(gq_dmrg_get_mps(d.get(), (int)i, &h));
    DeviceTensor(h).ToHost().Dump(GenMPSTenName(sp.mps_path, i));
  }
  for (size_t len = 1; len + 1 < N; ++len) {
    gq_tensor *h = nullptr;
    Check(gq_dmrg_get_env(d.get(), 'r', (int)len, &h));
    DeviceTensor(h).ToHost().Dump(GenEnvTenName("r", len, sp.temp_path));
  }
  mps.clear();
  return e0;
}

template <typename TenT>
struct LanczosRes {
  size_t iters;
  double gs_eng;
  TenT *gs_vec;  // caller deletes
};

/* lanczos_solver_impl.h:79-226: eff_ham = {L, W_l, W_r, R} with L or R null
 * at the chain ends; where = "lend" | "cent" | "rend".  Like the reference,
 * the solver takes ownership of (and deletes) the initial state. */
inline LanczosRes<GQTensor> LanczosSolver(const std::vector<GQTensor *> &eff_ham,
                                          GQTensor *init_state, const LanczosParams &params,
                                          const std::string &where,
                                          int precision = GQ_PREC_FP64) {
  std::unique_ptr<GQTensor> init(init_state);
  if (eff_ham.size() != 4) throw Error("LanczosSolver: eff_ham must hold {L, Wl, Wr, R}");
  const int w = where == "lend" ? GQ_WHERE_LEND
                : where == "cent" ? GQ_WHERE_CENT
                : where == "rend" ? GQ_WHERE_REND
                                  : -1;
  if (w < 0) throw Error("LanczosSolver: where must be lend, cent or rend");
  DeviceTensor d[4];
  for (int i = 0; i < 4; ++i)
    if (eff_ham[i]) d[i] = DeviceTensor::FromHost(*eff_ham[i]);
  DeviceTensor x = DeviceTensor::FromHost(*init);
  gq_lanczos_params lp{params.error, (int64_t)params.max_iterations, params.rayleigh};
  int64_t iters = 0;
  double e = 0.0;
  gq_tensor *gs = nullptr;
  Check(gq_lanczos(d[0].get(), d[1].get(), d[2].get(), d[3].get(), w, x.get(), &lp, precision,
                   &iters, &e, &gs));
  LanczosRes<GQTensor> res;
  res.iters = (size_t)iters;
  res.gs_eng = e;
  res.gs_vec = new GQTensor(DeviceTensor(gs).ToHost());
  return res;
}

}  // namespace gqmps2

#endif /* GQMPS2_GB300_HPP */
