// Device-resident two-site DMRG state (see dmrg.cu).
#pragma once

#include <map>
#include <utility>
#include <vector>

#include "gq_runtime.hpp"

namespace gq {

struct SweepParamsC {
  int64_t sweeps = 1;
  int64_t dmin = 1, dmax = 1;
  double trunc_err = 0.0;
  LanczosParamsC lanczos;
  Precision precision = kFP64;
  int verbose = 0;
};

struct UpdateStatsC {
  int site = 0;
  int dir = 'r';
  double e0 = 0, trunc_err = 0;
  int64_t D = 0, iters = 0;
  double ee = 0;
  double lanczos_seconds = 0, update_seconds = 0, svd_seconds = 0, env_seconds = 0;
  int64_t matvecs = 0;
  double matvec_flops = 0, env_flops = 0;
  int64_t theta_size = 0;
};

struct Dmrg {
  std::vector<TensorPtr> mps, mpo;
  std::map<std::pair<char, int>, TensorPtr> envs;
  // Inside a sweep an update does not wait for its environment growth: the
  // next update's host work (contraction plans, graph build) runs while the
  // growth's kernels do.  The growth's device time is taken with two events
  // and written to *env_pending once a later wait has seen them.
  cudaEvent_t env_ev[2] = {nullptr, nullptr};
  double *env_pending = nullptr;
  Dmrg() = default;
  Dmrg(const Dmrg &) = delete;
  Dmrg &operator=(const Dmrg &) = delete;
  ~Dmrg();
  int N() const { return (int)mps.size(); }
  void init_envs(Precision prec);
  // overlap: return without waiting for the environment growth (sweeps)
  UpdateStatsC update(const SweepParamsC &prm, char dir, int target, bool overlap = false);
  double sweep(const SweepParamsC &prm, std::vector<UpdateStatsC> *stats);
  void resolve_env_time();  // after a wait on the stream
};

}  // namespace gq
