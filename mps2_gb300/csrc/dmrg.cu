// Two-site finite DMRG sweep with the whole state resident in HBM.
//
// Restates two_site_update_finite_vmps_impl.h: InitEnvs (104-135),
// TwoSiteFiniteVMPSSweep (143-161) and TwoSiteFiniteVMPSUpdate (164-340).
// The reference loads/dumps one tensor file per step (LoadRelatedTens /
// DumpRelatedTens, 343-494); here the MPS and every environment stay on the
// device and the files are written only at call boundaries by the host
// wrapper.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>

#include "gq_dmrg.hpp"

namespace gq {

// Arithmetic of the environment contractions.  An environment's error goes
// into every later energy at first order (E = <psi|L W W R|psi>), so the
// split form grows its environments FP64-accurately, on the tensor cores;
// only the matvec, whose error reaches the energy at second order through
// the Rayleigh quotient, runs in 3xTF32.
Precision env_precision(Precision prec) { return prec == kTF32x3 ? kFP64TC : prec; }

void Dmrg::init_envs(Precision prec_in) {
  const Precision prec = env_precision(prec_in);
  const int Nn = N();
  GQ_CHECK(Nn >= 2, "DMRG needs at least two sites");
  TensorPtr renv;
  for (int i = 1; i <= Nn - 2; ++i) {
    const Tensor &A = *mps[Nn - i];
    auto Ad = dag(A);
    if (i == 1) {
      auto temp = contract(A, *mpo[Nn - 1], {1}, {0}, prec);
      renv = contract(*temp, *Ad, {2}, {1}, prec);
    } else {
      auto t1 = contract(A, *renv, {2}, {0}, prec);
      auto t2 = contract(*t1, *mpo[Nn - i], {1, 2}, {1, 3}, prec);
      renv = contract(*t2, *Ad, {3, 1}, {1, 2}, prec);
    }
    envs[{'r', i}] = renv;
  }
}

namespace {
struct Classified {
  int ls, rs, lenv_len, renv_len, ldims;
  Where where;
  std::vector<int> ia, ib;
};

Classified classify(int N, char dir, int target) {
  Classified c{};
  if (dir == 'r') {
    c.ls = target;
    c.rs = target + 1;
    c.lenv_len = target;
    c.renv_len = N - (target + 2);
    if (target == 0) { c.where = kLend; c.ldims = 1; c.ia = {1}; c.ib = {0}; }
    else if (target == N - 2) { c.where = kRend; c.ldims = 2; c.ia = {2}; c.ib = {0}; }
    else { c.where = kCent; c.ldims = 2; c.ia = {2}; c.ib = {0}; }
  } else {
    c.ls = target - 1;
    c.rs = target;
    c.lenv_len = target - 1;
    c.renv_len = N - target - 1;
    if (target == N - 1) { c.where = kRend; c.ldims = 2; c.ia = {2}; c.ib = {0}; }
    else if (target == 1) { c.where = kLend; c.ldims = 1; c.ia = {1}; c.ib = {0}; }
    else { c.where = kCent; c.ldims = 2; c.ia = {2}; c.ib = {0}; }
  }
  return c;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

double measure_ee(const std::vector<double> &s) {
  double ee = 0.0;
  for (double v : s) {
    const double p = v * v;
    if (p > 0.0) ee += -p * std::log(p);
  }
  return ee;
}
}  // namespace

Dmrg::~Dmrg() {
  for (auto &e : env_ev)
    if (e) cudaEventDestroy(e);
}

void Dmrg::resolve_env_time() {
  if (env_pending && env_ev[1]) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, env_ev[0], env_ev[1]) == cudaSuccess) *env_pending = ms * 1e-3;
  }
  env_pending = nullptr;
}

UpdateStatsC Dmrg::update(const SweepParamsC &prm, char dir, int target, bool overlap) {
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  const int Nn = N();
  const Precision prec = prm.precision;
  const Precision envp = env_precision(prec);
  const Classified c = classify(Nn, dir, target);
  UpdateStatsC st{};
  st.site = target;
  st.dir = dir;

  EffHam h;
  h.where = c.where;
  h.Wl = mpo[c.ls].get();
  h.Wr = mpo[c.rs].get();
  if (c.where != kLend) {
    auto it = envs.find({'l', c.lenv_len});
    GQ_CHECK(it != envs.end(), "missing left environment " + std::to_string(c.lenv_len));
    h.L = it->second.get();
  }
  if (c.where != kRend) {
    auto it = envs.find({'r', c.renv_len});
    GQ_CHECK(it != envs.end(), "missing right environment " + std::to_string(c.renv_len));
    h.R = it->second.get();
  }
  // Two-site state, embedded in the Lanczos space (all allowed blocks).
  auto theta = contract(*mps[c.ls], *mps[c.rs], c.ia, c.ib, prec);
  auto space = lanczos_space(*theta);
  space->allocate();
  embed(*theta, *space);
  theta.reset();
  st.theta_size = space->size();

  const auto tl = clk::now();
  LanczosParamsC lp;
  lp.error = prm.lanczos.error;
  lp.max_iterations = prm.lanczos.max_iterations;
  lp.rayleigh = prm.lanczos.rayleigh;
  auto res = lanczos(h, *space, lp, prec);
  sync();
  resolve_env_time();  // the previous update's growth is done by now
  st.lanczos_seconds = seconds_since(tl);
  st.iters = res.iters;
  st.e0 = res.energy;
  st.matvecs = res.matvecs;
  st.matvec_flops = res.matvec_flops;
  space.reset();

  const auto ts = clk::now();
  auto sv = svd_truncate(*res.gs, c.ldims, mps[c.ls]->div, prm.trunc_err, prm.dmin, prm.dmax,
                         dir == 'r' ? 2 : 1);
  res.gs.reset();
  sync();
  st.svd_seconds = seconds_since(ts);
  st.trunc_err = sv.trunc_err;
  st.D = sv.D;
  st.ee = measure_ee(sv.s);
  mps[c.ls] = sv.u;   // 'l': U.S
  mps[c.rs] = sv.vt;  // 'r': S.Vt

  const auto te = clk::now();
  if (overlap) {
    for (auto &e : env_ev)
      if (!e) GQ_CUDA(cudaEventCreate(&e));
    GQ_CUDA(cudaEventRecord(env_ev[0], stream()));
  }
  double f1 = 0, f2 = 0, f3 = 0;
  if (dir == 'r') {
    if (target != Nn - 2) {
      const Tensor &A = *mps[target];
      auto Ad = dag(A);
      if (target == 0) {
        auto temp = contract(A, *mpo[target], {0}, {0}, envp, &f1);
        envs[{'l', c.lenv_len + 1}] = contract(*temp, *Ad, {2}, {0}, envp, &f2);
      } else {
        auto t1 = contract(*h.L, A, {0}, {0}, envp, &f1);
        auto t2 = contract(*t1, *mpo[target], {0, 2}, {0, 1}, envp, &f2);
        envs[{'l', c.lenv_len + 1}] = contract(*t2, *Ad, {0, 2}, {0, 1}, envp, &f3);
      }
    }
  } else {
    if (target != 1) {
      const Tensor &A = *mps[target];
      auto Ad = dag(A);
      if (target == Nn - 1) {
        auto temp = contract(A, *mpo[target], {1}, {0}, envp, &f1);
        envs[{'r', c.renv_len + 1}] = contract(*temp, *Ad, {2}, {1}, envp, &f2);
      } else {
        auto t1 = contract(A, *h.R, {2}, {0}, envp, &f1);
        auto t2 = contract(*t1, *mpo[target], {1, 2}, {1, 3}, envp, &f2);
        envs[{'r', c.renv_len + 1}] = contract(*t2, *Ad, {3, 1}, {1, 2}, envp, &f3);
      }
    }
  }
  if (overlap) {
    GQ_CUDA(cudaEventRecord(env_ev[1], stream()));  // env_seconds: filled in later
  } else {
    sync();
    st.env_seconds = seconds_since(te);
    check_device_errors();
  }
  st.env_flops = f1 + f2 + f3;
  st.update_seconds = seconds_since(t0);
  if (prm.verbose) {
    // the reference's stream state: fixed, precision 16 for E0, 2 after the
    // scientific TruncErr, 7 for S
    std::printf("Site %4d E0 = %20.16f TruncErr = %.2e D = %5lld Iter = %3lld LanczT = %8.2f "
                "TotT = %8.2f S = %10.7f\n",
                target, st.e0, st.trunc_err, (long long)st.D, (long long)st.iters,
                st.lanczos_seconds, st.update_seconds, st.ee);
    std::fflush(stdout);
  }
  return st;
}

double Dmrg::sweep(const SweepParamsC &prm, std::vector<UpdateStatsC> *stats) {
  const int Nn = N();
  double e0 = 0.0;
  // the pending environment time points into `stats`: no reallocation
  // during the sweep, and no pointer left behind on any exit
  struct PendingReset {
    Dmrg &d;
    ~PendingReset() { d.env_pending = nullptr; }
  } reset{*this};
  if (stats) stats->reserve(stats->size() + 2 * (size_t)std::max(Nn - 1, 0));
  auto one = [&](char dir, int i) {
    auto st = update(prm, dir, i, true);
    e0 = st.e0;
    if (stats) {
      stats->push_back(st);
      env_pending = &stats->back().env_seconds;
    }
  };
  for (int i = 0; i < Nn - 1; ++i) one('r', i);
  for (int i = Nn - 1; i > 0; --i) one('l', i);
  sync();
  resolve_env_time();
  check_device_errors();  // the tensor-core error word, once per sweep
  return e0;
}

}  // namespace gq
