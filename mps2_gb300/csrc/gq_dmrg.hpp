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
  int N() const { return (int)mps.size(); }
  void init_envs(Precision prec);
  UpdateStatsC update(const SweepParamsC &prm, char dir, int target);
  double sweep(const SweepParamsC &prm, std::vector<UpdateStatsC> *stats);
};

}  // namespace gq
