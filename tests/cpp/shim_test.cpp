// Test program of the header-only C++ front end (include/gqmps2_gb300.hpp),
// driven by tests/test_cpp_shim.py.
//
//   shim_test host <dir>   host-only checks (no GPU call):
//       reads <dir>/in.gqten and writes it back to <dir>/out.gqten;
//       DirectStateInitMps on a 6-site spin-1/2 chain, dumped to <dir>/mps;
//       SiteVec identity operators, parameter defaults, TenVec dump/load
//       (test_ten_vec.cc:27-60).  Prints "host ok".
//   shim_test dmrg <dir>   the reference's 1DHeisenberg case
//       (test_two_site_update_finite_vmps.cc:186-220) as written there, with
//       the MPO read from <dir>/mpo/mpo_ten<i>.gqten: two TwoSiteFiniteVMPS
//       calls (the second resumes from the environments on disk), then a
//       LanczosSolver on the left end of the result, FiniteMPS::Centralize,
//       and one sweep in the split form.  Prints "key value" lines.
#include "gqmps2_gb300.hpp"

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

using namespace gqmps2;

namespace {

int failures = 0;

void expect(bool ok, const std::string &what) {
  if (!ok) {
    std::printf("FAIL %s\n", what.c_str());
    ++failures;
  }
}

Index spin_half_out() { return Index({QNSector({1}, 1), QNSector({-1}, 1)}, OUT); }

bool is_id_op(const GQTensor &t) {
  const auto &ix = t.GetIndexes();
  if (ix.size() != 2 || ix[0].dir != IN || InverseIndex(ix[0]) != ix[1]) return false;
  for (int64_t i = 0; i < ix[0].dim(); ++i)
    for (int64_t j = 0; j < ix[1].dim(); ++j)
      if (t.GetElem({i, j}) != (i == j ? 1.0 : 0.0)) return false;
  return true;
}

// deterministic fill for the TenVec check
GQTensor rand_ten(const Index &in, const Index &out, int div, unsigned &state) {
  GQTensor t({in, out}, QN{div});
  for (size_t a = 0; a < in.sectors.size(); ++a)
    for (size_t b = 0; b < out.sectors.size(); ++b) {
      GQTensor::Coords c{(int)a, (int)b};
      if (t.BlockDiv(c) != QN{div}) continue;
      std::vector<double> v(in.sectors[a].dim * out.sectors[b].dim);
      for (auto &x : v) {
        state = state * 1664525u + 1013904223u;
        x = (double)(state >> 8) / (double)(1u << 24) - 0.5;
      }
      t.Blocks().emplace(c, v);
    }
  return t;
}

int run_host(const std::string &dir) {
  GQTensor t;
  t.Load(dir + "/in.gqten");
  t.Dump(dir + "/out.gqten");

  SiteVec sv(6, spin_half_out());
  expect(sv.size == 6, "SiteVec size");
  for (auto &op : sv.id_ops) expect(is_id_op(op), "SiteVec identity operator");
  SiteVec sv_in(3, InverseIndex(spin_half_out()));
  expect(sv_in.sites[0] == spin_half_out(), "SiteVec stores OUT legs");

  FiniteMPS mps(sv);
  std::vector<size_t> labs;
  for (size_t i = 0; i < 6; ++i) labs.push_back(i % 2);
  DirectStateInitMps(mps, labs, QN{0});
  expect(mps.GetTensCanoType()[0] == NONE && mps.GetTensCanoType()[1] == RIGHT,
         "canonical types after DirectStateInitMps");
  {  // finite_mps.h:67-75: write access marks the site non-canonical, the MPS uncentralised
    FiniteMPS m2 = mps;
    const FiniteMPS &c2 = m2;
    (void)c2[2];
    expect(m2.GetTenCanoType(2) == RIGHT && m2.GetCenter() == 0, "const access keeps the types");
    m2[2] = c2[2];
    expect(m2.GetTenCanoType(2) == NONE && m2.GetCenter() == kUncentralizedCenterIdx,
           "write access resets the canonical type and the center");
  }
  mps.Dump(dir + "/mps", true);
  expect(mps.empty(), "Dump with release empties the MPS");

  LanczosParams lp;
  expect(lp.error == 1.0E-7 && lp.max_iterations == 200, "LanczosParams defaults");
  SweepParams sp(4, 8, 16, 1.0E-9, LanczosParams(1.0E-8, 50));
  expect(sp.mps_path == kMpsPath && sp.temp_path == kRuntimeTempPath, "SweepParams paths");
  gq_sweep_params c = sp.ToC();
  expect(c.sweeps == 4 && c.dmin == 8 && c.dmax == 16 && c.lanczos.max_iterations == 50 &&
             c.lanczos.error == 1.0E-8 && c.precision == GQ_PREC_FP64,
         "SweepParams to the C struct");

  // test_ten_vec.cc:27-60
  Index idx_out({QNSector({0}, 2), QNSector({1}, 2)}, OUT);
  Index idx_in = InverseIndex(idx_out);
  unsigned st = 7;
  GQTensor t0 = rand_ten(idx_in, idx_out, 0, st), t1 = rand_ten(idx_in, idx_out, 1, st),
           t2 = rand_ten(idx_in, idx_out, -1, st);
  TenVec<GQTensor> tv(3);
  tv[0] = t0;
  tv[1] = t1;
  tv[2] = t2;
  tv.DumpTen(0, dir + "/ten0.gqten");
  tv.DumpTen(1, dir + "/ten1.gqten", true);
  tv.DumpTen(2, dir + "/ten2.gqten", false);
  tv.dealloc(0);
  tv.dealloc(2);
  expect(tv.empty(), "TenVec empty after dealloc");
  tv.LoadTen(0, dir + "/ten2.gqten");
  tv.LoadTen(1, dir + "/ten0.gqten");
  tv.LoadTen(2, dir + "/ten1.gqten");
  expect(tv[0] == t2 && tv[1] == t0 && tv[2] == t1, "TenVec load after dump");

  // test_mpo.cc:42-67: an MPO of N default tensors; element access
  {
    MPO<GQTensor> empty_mpo(0);
    expect(empty_mpo.size() == 0, "MPO of size 0");
    MPO<GQTensor> mpo(5);
    bool all_default = mpo.size() == 5;
    for (size_t i = 0; i < mpo.size(); ++i) all_default = all_default && mpo[i] == GQTensor();
    expect(all_default, "MPO elements start as default tensors");
    MPO<GQTensor> m3(3);
    m3[0] = t0;
    m3[1] = t1;
    m3[2] = t2;
    expect(m3[0] == t0 && m3[1] == t1 && m3[2] == t2, "MPO element assignment");
    m3[1] = t2;
    expect(m3[1] == t2, "MPO element reassignment");
  }

  // test_duovector.cc: copies own their elements, moves take them over
  TenVec<GQTensor> copy(tv);
  expect(copy.size() == 3 && copy[0] == tv[0] && copy(0) != tv(0), "TenVec copy is deep");
  const GQTensor *p0 = tv(0);
  TenVec<GQTensor> moved(std::move(tv));
  expect(moved(0) == p0 && moved[0] == copy[0], "TenVec move keeps the elements");
  TenVec<GQTensor> assigned(1);
  assigned = copy;
  expect(assigned.size() == 3 && assigned[2] == copy[2] && assigned(2) != copy(2),
         "TenVec copy assignment is deep");
  assigned.dealloc(1);
  expect(assigned(1) == nullptr && assigned(0) != nullptr, "TenVec dealloc of one element");

  // the host-side full contraction of the measurements against an explicit
  // element sum: a(i, j, k) b(k, i, j), legs matched a0-b1, a1-b2, a2-b0
  {
    Index p({QNSector({0}, 2), QNSector({1}, 3)}, OUT), q({QNSector({0}, 1), QNSector({1}, 2)}, OUT);
    Index r({QNSector({0}, 2), QNSector({-1}, 2)}, IN);
    unsigned st2 = 11;
    auto rnd = [&] {
      st2 = st2 * 1664525u + 1013904223u;
      return (double)(st2 >> 8) / (double)(1u << 24) - 0.5;
    };
    GQTensor a({p, q, InverseIndex(r)}), b({r, InverseIndex(p), InverseIndex(q)});
    for (int64_t i = 0; i < p.dim(); ++i)
      for (int64_t j = 0; j < q.dim(); ++j)
        for (int64_t k = 0; k < r.dim(); ++k) {
          QN qa = a.BlockDiv({(int)p.CoorToSector(i).first, (int)q.CoorToSector(j).first,
                              (int)r.CoorToSector(k).first});
          if (qa == QN{1}) {
            a.SetElem({i, j, k}, rnd());
            b.SetElem({k, i, j}, rnd());
          }
        }
    double want = 0.0;
    for (int64_t i = 0; i < p.dim(); ++i)
      for (int64_t j = 0; j < q.dim(); ++j)
        for (int64_t k = 0; k < r.dim(); ++k) want += a.GetElem({i, j, k}) * b.GetElem({k, i, j});
    double got = measu_detail::FullContract(a, b, {0, 1, 2}, {1, 2, 0});
    expect(std::fabs(got - want) <= 1e-14 * (1.0 + std::fabs(want)), "full contraction");
    MeasuRes mr{MeasuResElem{{0}, 0.25}, MeasuResElem{{1, 4}, -0.125}};
    DumpMeasuRes(mr, dir + "/measu");
  }

  bool threw = false;
  try {
    GQTensor bad;
    bad.Load(dir + "/missing.gqten");
  } catch (const Error &) {
    threw = true;
  }
  expect(threw, "loading a missing file throws");
  if (failures == 0) std::printf("host ok\n");
  return failures ? 1 : 0;
}

int run_dmrg(const std::string &dir) {
  const size_t N = 6;
  QN qn0{0};
  SiteVec dsite_vec_6(N, spin_half_out());
  MPO<GQTensor> dmpo(N);
  for (size_t i = 0; i < N; ++i) dmpo.LoadTen(i, dir + "/mpo/mpo_ten" + std::to_string(i) + ".gqten");

  FiniteMPS dmps(dsite_vec_6);
  auto sweep_params = SweepParams(4, 8, 8, 1.0E-9, LanczosParams(1.0E-7), dir + "/mps",
                                  dir + "/.temp");
  sweep_params.verbose = 0;
  std::vector<size_t> stat_labs;
  for (size_t i = 0; i < N; ++i) stat_labs.push_back(i % 2);
  DirectStateInitMps(dmps, stat_labs, qn0);
  dmps.Dump(sweep_params.mps_path, true);
  double e0 = TwoSiteFiniteVMPS(dmps, dmpo, sweep_params);
  std::printf("e0 %.17g\n", e0);
  expect(dmps.empty(), "MPS empty after the call");

  // Continue simulation test
  dmps.clear();
  std::vector<gq_update_stats> stats;
  double e0_resume = TwoSiteFiniteVMPS(dmps, dmpo, sweep_params, &stats);
  std::printf("e0_resume %.17g\n", e0_resume);
  std::printf("updates %zu\n", stats.size());

  // LanczosSolver on the left end: init = A_0 A_1, eff_ham = {-, W_0, W_1, R_4}
  dmps.Load(sweep_params.mps_path);
  GQTensor renv;
  renv.Load(GenEnvTenName("r", N - 2, sweep_params.temp_path));
  auto *init = new GQTensor;
  Contract(&dmps[0], &dmps[1], {{1}, {0}}, init);
  std::vector<GQTensor *> eff_ham = {nullptr, &dmpo[0], &dmpo[1], &renv};
  auto res = LanczosSolver(eff_ham, init, LanczosParams(1.0E-9), "lend");
  std::printf("lanczos_e %.17g\n", res.gs_eng);
  std::printf("lanczos_iters %zu\n", res.iters);
  expect(res.gs_vec != nullptr && res.gs_vec->Rank() == 3, "Lanczos ground state (s1, s2, r)");
  delete res.gs_vec;

  // Centralize on the GPU, then A^dag A = 1 on the left-canonical sites
  dmps.Centralize(3);
  std::printf("center %ld\n", dmps.GetCenter());
  auto cano = dmps.GetTensCanoType();
  std::printf("cano");
  for (auto c : cano) std::printf(" %d", (int)c);
  std::printf("\n");
  double worst = 0.0;
  for (size_t i = 0; i < 3; ++i) {
    GQTensor a = dmps[i], ad, m;
    // Dag for real tensors: legs inverted, divergence negated, same data
    std::vector<Index> inv;
    for (auto &ix : a.GetIndexes()) inv.push_back(InverseIndex(ix));
    ad = GQTensor(inv, -a.Div());
    ad.Blocks() = a.Blocks();
    if (i == 0)
      Contract(&a, &ad, {{0}, {0}}, &m);
    else
      Contract(&a, &ad, {{0, 1}, {0, 1}}, &m);
    const int64_t D = m.GetIndexes()[0].dim();
    for (int64_t x = 0; x < D; ++x)
      for (int64_t y = 0; y < D; ++y)
        worst = std::fmax(worst, std::fabs(m.GetElem({x, y}) - (x == y ? 1.0 : 0.0)));
  }
  std::printf("left_canonical_err %.3g\n", worst);

  // measurements on the converged state; the same MPS is dumped for the
  // Python side to measure too
  {
    dmps.Dump(dir + "/mps_meas");
    GQTensor sz({InverseIndex(spin_half_out()), spin_half_out()});
    sz.SetElem({0, 0}, 0.5);
    sz.SetElem({1, 1}, -0.5);
    auto r1 = MeasureOneSiteOp(dmps, sz, dir + "/sz");
    std::vector<std::vector<size_t>> pairs = {{0, 1}, {0, 3}, {2, 5}, {1, 4}};
    auto r2 = MeasureTwoSiteOp(dmps, {sz, sz}, dsite_vec_6.id_ops[0], pairs, dir + "/szsz");
    std::printf("meas_one %zu\n", r1.size());
    std::printf("meas_two %zu\n", r2.size());
    std::printf("meas_center %ld\n", dmps.GetCenter());
  }

  // TruncateMPS to D = 2: every bond at most 2, the state stays normalised
  {
    FiniteMPS tm = dmps;
    std::vector<double> errs;
    std::vector<int64_t> dims;
    TruncateMPS(tm, 0.0, 1, 2, &errs, &dims);
    int64_t dmax_seen = 0;
    for (auto x : dims) dmax_seen = x > dmax_seen ? x : dmax_seen;
    std::printf("truncate_dmax %lld\n", (long long)dmax_seen);
    std::printf("truncate_bonds %zu\n", dims.size());
    double nrm = 0.0;  // <psi|psi> from the left-canonical tensors: |A_{N-1}|^2
    for (auto &b : tm[N - 1].Blocks())
      for (double v : b.second) nrm += v * v;
    std::printf("truncate_norm %.17g\n", nrm);
  }

  // the split form, one sweep from the converged state (right-canonical again)
  dmps.Centralize(0);
  dmps.Dump(sweep_params.mps_path, true);
  sweep_params.precision = GQ_PREC_TF32X3;
  sweep_params.lancz_params.rayleigh = GQ_PREC_FP64TC;
  sweep_params.sweeps = 1;
  sweep_params.temp_path = dir + "/.temp_split";  // absent: environments built anew
  double e_split = TwoSiteFiniteVMPS(dmps, dmpo, sweep_params);
  std::printf("e0_split %.17g\n", e_split);
  std::printf("failures %d\n", failures);
  return failures ? 1 : 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s host|dmrg <dir>\n", argv[0]);
    return 2;
  }
  try {
    const std::string mode = argv[1], dir = argv[2];
    if (mode == "host") return run_host(dir);
    if (mode == "dmrg") return run_dmrg(dir);
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
  } catch (const Error &e) {
    std::printf("ERROR %s\n", e.what());
    return 3;
  }
}
