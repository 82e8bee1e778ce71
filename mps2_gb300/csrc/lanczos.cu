// Effective-Hamiltonian matvec and Lanczos ground-state solver.
//
// Restates ``LanczosSolver`` (``lanczos_solver_impl.h:79-226``) with the
// Krylov vectors resident in HBM: no re-orthogonalisation, every basis
// vector kept, stop on ``E_old - E_new < error`` or ``m == eff_dim`` or
// ``m == max_iterations - 1``; breakdown handled as at ``:163-180``.  The
// matvec follows ``eff_ham_mul_state_{cent,lend,rend}`` (``:228-256``)
// contraction for contraction; its work lists are planned once per update
// and replayed every iteration.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>

#include "gq_runtime.hpp"

namespace gq {

struct MatvecStep {
  std::shared_ptr<ContractPlan> plan;
  int a_src, b_src;   // -1: the input vector x; >=0: intermediate id; -2: constant
  const Tensor *a_const = nullptr, *b_const = nullptr;
  int out;            // intermediate id, or -1 for the output vector
};

struct MatvecPlan {
  EffHam h;
  Precision prec = kFP64;
  std::vector<MatvecStep> steps;
  std::vector<TensorPtr> inter;
  DevBuf scratch;
  double flops = 0.0;
  // The matvec's launch sequence is fixed for a whole Lanczos solve, so it
  // is captured once as a CUDA graph reading a fixed input buffer and
  // replayed every further iteration (captured lazily, for one (x, y) pair).
  cudaGraphExec_t exec = nullptr;
  const double *graph_x = nullptr;
  double *graph_y = nullptr;
  ~MatvecPlan() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

namespace {
// Graph replay of the matvec on the main lane, unless the kernel profiler
// is on (it times every launch with its own events) or GQ_NO_GRAPHS is set.
// Not on the lanes of a batched run: there every solve's capture and
// instantiation contend across the host threads (64 XXZ chains: 26.2 s with
// graphs, 19.3 s without; one chain after another: 107 s vs 109 s).
bool graphs_enabled() {
  static const bool off = std::getenv("GQ_NO_GRAPHS") != nullptr;
  return !off && !prof_on() && on_main_lane();
}

void run_matvec_graph(MatvecPlan &p, const double *x, double *y, double *xin, int64_t n) {
  auto s = stream();
  if (!p.exec || p.graph_x != xin || p.graph_y != y) {
    if (p.exec) {
      GQ_CUDA(cudaGraphExecDestroy(p.exec));
      p.exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    GQ_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      run_matvec(p, xin, y);
    } catch (...) {
      cudaGraph_t dead = nullptr;
      cudaStreamEndCapture(s, &dead);
      if (dead) cudaGraphDestroy(dead);
      throw;
    }
    GQ_CUDA(cudaStreamEndCapture(s, &g));
    const cudaError_t e = cudaGraphInstantiate(&p.exec, g, 0);
    cudaGraphDestroy(g);
    GQ_CUDA(e);
    p.graph_x = xin;
    p.graph_y = y;
  }
  if (x != xin)
    GQ_CUDA(cudaMemcpyAsync(xin, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  GQ_CUDA(cudaGraphLaunch(p.exec, s));
}
}  // namespace

int64_t eff_ham_dim(const EffHam &h) {
  switch (h.where) {
    case kCent:
      return h.L->idx[0].total() * h.Wl->idx[1].total() * h.Wr->idx[1].total() *
             h.R->idx[0].total();
    case kLend:
      return h.Wl->idx[0].total() * h.Wr->idx[1].total() * h.R->idx[0].total();
    default:
      return h.L->idx[0].total() * h.Wl->idx[1].total() * h.Wr->idx[0].total();
  }
}

namespace {
// Autotuning of one matvec step: every candidate threshold that gives a
// different kernel split is timed (one warm-up run, one timed run, CUDA
// events) on the step's real operands; the fastest is stored under the
// plan's signature and returned.
std::shared_ptr<ContractPlan> tune_step(const Tensor &A, const double *a, bool a_const,
                                        const Tensor &B, const double *b, bool b_const,
                                        const std::vector<int> &xa, const std::vector<int> &xb,
                                        const Tensor *target, Precision prec,
                                        std::shared_ptr<ContractPlan> first) {
  auto s = stream();
  struct Events {  // released on every exit path
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Events() {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } ev;
  GQ_CUDA(cudaEventCreate(&ev.e0));
  GQ_CUDA(cudaEventCreate(&ev.e1));
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  std::shared_ptr<ContractPlan> best;
  float best_ms = 0.f;
  std::vector<std::pair<int64_t, int64_t>> seen;
  DevBuf out(first->out->size());
  for (double frac : kTuneCandidates) {
    auto pl = plan_contract(A, B, xa, xb, target, prec, frac);
    const std::pair<int64_t, int64_t> split{pl->ntiles_tc + pl->ntiles_oz, pl->ntiles};
    if (std::find(seen.begin(), seen.end(), split) != seen.end()) continue;
    seen.push_back(split);
    if (a_const) cache_operand(*pl, 0, a);
    if (b_const) cache_operand(*pl, 1, b);
    DevBuf scratch(contract_scratch(*pl));
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {
      GQ_CUDA(cudaEventRecord(e0, s));
      run_contract(*pl, a, b, out.p, scratch.p, prec);
      GQ_CUDA(cudaEventRecord(e1, s));
      GQ_CUDA(cudaEventSynchronize(e1));
      GQ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    }
    if (!best || ms < best_ms) {
      best = pl;
      best_ms = ms;
    }
  }
  autotune_store(first->signature, prec, best->tc_frac);
  return best;
}
}  // namespace

std::shared_ptr<MatvecPlan> plan_matvec(const EffHam &h, const Tensor &space, Precision prec) {
  auto mp = std::make_shared<MatvecPlan>();
  mp->h = h;
  mp->prec = prec;
  struct S { const Tensor *ca; int as; const Tensor *cb; int bs; std::vector<int> xa, xb; };
  std::vector<S> spec;
  // a/b source: -1 = x, -2 = constant, k>=0 = intermediate k (previous step)
  if (h.where == kCent) {
    spec = {{h.L, -2, nullptr, -1, {0}, {0}},
            {nullptr, 0, h.Wl, -2, {0, 2}, {0, 1}},
            {nullptr, 1, h.Wr, -2, {4, 1}, {0, 1}},
            {nullptr, 2, h.R, -2, {4, 1}, {1, 0}}};
  } else if (h.where == kLend) {
    spec = {{nullptr, -1, h.Wl, -2, {0}, {0}},
            {nullptr, 0, h.Wr, -2, {0, 2}, {1, 0}},
            {nullptr, 1, h.R, -2, {0, 3}, {0, 1}}};
  } else {
    spec = {{nullptr, -1, h.L, -2, {0}, {0}},
            {nullptr, 0, h.Wl, -2, {2, 0}, {0, 1}},
            {nullptr, 1, h.Wr, -2, {3, 0}, {1, 0}}};
  }
  int64_t scratch = 0;
  for (size_t i = 0; i < spec.size(); ++i) {
    const S &s = spec[i];
    const Tensor &A = s.as == -2 ? *s.ca : (s.as == -1 ? space : *mp->inter[s.as]);
    const Tensor &B = s.bs == -2 ? *s.cb : (s.bs == -1 ? space : *mp->inter[s.bs]);
    const bool last = i + 1 == spec.size();
    auto plan = plan_contract(A, B, s.xa, s.xb, last ? &space : nullptr, prec);
    const double *a_data = A.data.p, *b_data = B.data.p;
    const bool tuned = prec != kFP64 && !plan->use_skinny && autotune_on();
    if (tuned) {
      double frac;
      if (autotune_lookup(plan->signature, prec, &frac)) {
        if (frac != plan->tc_frac)
          plan = plan_contract(A, B, s.xa, s.xb, last ? &space : nullptr, prec, frac);
      } else {
        plan = tune_step(A, a_data, s.as == -2, B, b_data, s.bs == -2, s.xa, s.xb,
                         last ? &space : nullptr, prec, plan);
      }
    }
    // Environments and MPO tensors do not change during the solve: pack
    // them for the tensor cores once.
    if (s.as == -2 && !plan->a_cached && !plan->a_oz_cached) cache_operand(*plan, 0, a_data);
    if (s.bs == -2 && !plan->b_cached && !plan->b_oz_cached) cache_operand(*plan, 1, b_data);
    MatvecStep st;
    st.plan = plan;
    st.a_src = s.as;
    st.b_src = s.bs;
    st.a_const = s.as == -2 ? s.ca : nullptr;
    st.b_const = s.bs == -2 ? s.cb : nullptr;
    if (last) {
      st.out = -1;
    } else {
      auto t = clone_structure(*plan->out);
      t->allocate();
      mp->inter.push_back(t);
      st.out = (int)mp->inter.size() - 1;
      if (autotune_on() && prec != kFP64) {
        // the next step is tuned on real data: run this one now
        DevBuf scratch(contract_scratch(*plan));
        run_contract(*plan, a_data, b_data, t->data.p, scratch.p, prec);
      }
    }
    scratch = std::max(scratch, contract_scratch(*plan));
    mp->flops += plan->flops;
    mp->steps.push_back(std::move(st));
  }
  mp->scratch.alloc(scratch);
  return mp;
}

void run_matvec(MatvecPlan &p, const double *x, double *y) {
  for (auto &st : p.steps) {
    const double *a = st.a_src == -2 ? st.a_const->data.p
                      : st.a_src == -1 ? x
                                       : p.inter[st.a_src]->data.p;
    const double *b = st.b_src == -2 ? st.b_const->data.p
                      : st.b_src == -1 ? x
                                       : p.inter[st.b_src]->data.p;
    double *c = st.out == -1 ? y : p.inter[st.out]->data.p;
    run_contract(*st.plan, a, b, c, p.scratch.p, p.prec);
  }
}

double matvec_flops(const MatvecPlan &p) { return p.flops; }

TensorPtr lanczos_space(const Tensor &state) {
  return make_structure(state.nq, state.idx, state.div, allowed_blocks(state.idx, state.div));
}

void embed(const Tensor &src, Tensor &dst) {
  GQ_CHECK(src.idx.size() == dst.idx.size(), "embed: rank mismatch");
  for (size_t l = 0; l < src.idx.size(); ++l)
    GQ_CHECK(src.idx[l] == dst.idx[l], "embed: leg mismatch");
  dst.zero();
  std::vector<int64_t> tr;
  tr.reserve(src.nblocks() * 3);
  for (int64_t b = 0; b < src.nblocks(); ++b) {
    const int64_t d = dst.find(src.block_coords(b));
    GQ_CHECK(d >= 0, "embed: block missing from the destination structure");
    tr.push_back(src.offs[b]);
    tr.push_back(dst.offs[d]);
    tr.push_back(src.block_size(b));
  }
  dev_block_copy(src.data.p, dst.data.p, tr);
}

namespace {
// Copy `count` device scalars to the pinned host area and wait for them.
void fetch(const double *dev, double *host, int count) {
  GQ_CUDA(cudaMemcpyAsync(host, dev, sizeof(double) * count, cudaMemcpyDeviceToHost, stream()));
  sync();
}
}  // namespace

LanczosResult lanczos(const EffHam &h, const Tensor &init, const LanczosParamsC &prm,
                      Precision prec) {
  using clk = std::chrono::steady_clock;
  const int64_t maxit = prm.max_iterations;
  GQ_CHECK(maxit >= 2, "Lanczos needs max_iterations >= 2");
  const int64_t n = init.size();
  GQ_CHECK(n > 0, "empty Lanczos vector");
  const int64_t dim = eff_ham_dim(h);
  auto plan = plan_matvec(h, init, prec);

  LanczosResult res;
  std::vector<DevBuf> bases;
  bases.reserve(maxit);
  DevBuf last(n);
  // device scalars: a[0..maxit), nrm2[0..maxit)
  DevBuf sc(2 * maxit + 2);
  double *a_dev = sc.p, *n_dev = sc.p + maxit;
  DevBuf red(dot_scratch_elems());
  std::vector<double> a(maxit, 0.0), b(maxit, 0.0), N(maxit, 0.0);
  double *hs = lane().host_scalars;
  const bool use_graph = graphs_enabled();
  DevBuf xin(use_graph ? n : 0);

  // A solve that converges within two matvecs (the common case once a
  // sweep has converged) never pays for capturing and instantiating the
  // graph; longer solves replay it from the third matvec on.
  auto matvec = [&](const double *x) {
    if (use_graph && res.matvecs >= 2)
      run_matvec_graph(*plan, x, last.p, xin.p, n);
    else
      run_matvec(*plan, x, last.p);
    res.matvecs++;
    res.matvec_flops += plan->flops;
  };

  // One host round trip per iteration: right after <v_m, H v_m> the next
  // recurrence vector gamma_{m+1} and its squared norm are formed on the
  // device, and both scalars come back together.  If the iteration turns
  // out to be the last one, that speculative vector is simply unused.
  auto gamma_step = [&](int64_t m1) {  // bases[m1] = last - a[m1-1] v_{m1-1} - b v_{m1-2}
    while ((int64_t)bases.size() <= m1) bases.emplace_back(n);
    dev_lanczos_gamma(last.p, bases[m1 - 1].p, a_dev + (m1 - 1),
                      m1 >= 2 ? bases[m1 - 2].p : nullptr, m1 >= 2 ? n_dev + (m1 - 1) : nullptr,
                      true, bases[m1].p, n, n_dev + m1, red.p);
  };
  auto fetch2 = [&](int64_t m_a) {  // a[m_a] and nrm2[m_a + 1] -> hs[0], hs[1]
    GQ_CUDA(cudaMemcpyAsync(hs, a_dev + m_a, sizeof(double), cudaMemcpyDeviceToHost, stream()));
    GQ_CUDA(cudaMemcpyAsync(hs + 1, n_dev + m_a + 1, sizeof(double), cudaMemcpyDeviceToHost,
                            stream()));
    sync();
  };

  // v0 = init / |init|
  bases.emplace_back(n);
  GQ_CUDA(cudaMemcpyAsync(bases[0].p, init.data.p, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                          stream()));
  dev_dot(bases[0].p, bases[0].p, n, n_dev, red.p);
  dev_scale_rsqrt(bases[0].p, n, n_dev);
  matvec(bases[0].p);
  dev_dot(bases[0].p, last.p, n, a_dev, red.p);
  gamma_step(1);
  fetch2(0);
  a[0] = hs[0];
  double nrm2_next = hs[1];
  double energy0 = a[0];

  auto finish = [&](int64_t nvec, int64_t iters, double energy) {
    std::vector<double> c(nvec, 1.0);
    if (nvec > 1) {
      double ev;
      if (!tridiag_lowest(a.data(), b.data(), (int)nvec, &ev, c.data()))
        fail(kNumericalError, "tridiagonal eigensolver did not converge");
    }
    auto gs = clone_structure(init);
    gs->allocate();
    std::vector<const double *> ptrs;
    for (int64_t k = 0; k < nvec; ++k) ptrs.push_back(bases[k].p);
    dev_combine(ptrs, c, gs->data.p, n);
    res.iters = iters;
    res.energy = energy;
    res.ritz_energy = energy;
    res.gs = gs;
    if (prec == kTF32x3 && prm.fp64_rayleigh) {
      // FP64 Rayleigh quotient of the split-precision ground state
      auto p64 = plan_matvec(h, init, prm.rayleigh);
      run_matvec(*p64, gs->data.p, last.p);
      dev_dot(gs->data.p, last.p, n, a_dev, red.p);
      dev_dot(gs->data.p, gs->data.p, n, n_dev, red.p);
      GQ_CUDA(cudaMemcpyAsync(hs, a_dev, sizeof(double), cudaMemcpyDeviceToHost, stream()));
      GQ_CUDA(cudaMemcpyAsync(hs + 1, n_dev, sizeof(double), cudaMemcpyDeviceToHost, stream()));
      sync();
      res.energy = hs[0] / hs[1];
      res.matvecs++;
      res.matvec_flops += p64->flops;
    }
  };

  int64_t m = 0;
  while (true) {
    m += 1;
    const double nrm2 = nrm2_next;
    if (!std::isfinite(nrm2)) fail(kNumericalError, "Lanczos vector became non-finite");
    const double norm_gamma = std::sqrt(nrm2);
    if (norm_gamma == 0.0) {  // invariant subspace found
      finish(m, m, energy0);
      break;
    }
    N[m] = nrm2;
    b[m - 1] = norm_gamma;
    dev_scale_rsqrt(bases[m].p, n, n_dev + m);
    matvec(bases[m].p);
    dev_dot(bases[m].p, last.p, n, a_dev + m, red.p);
    const bool more = m + 1 < maxit;
    if (more) gamma_step(m + 1);
    if (more) {
      fetch2(m);
      nrm2_next = hs[1];
    } else {
      fetch(a_dev + m, hs, 1);
    }
    a[m] = hs[0];
    if (!std::isfinite(a[m])) fail(kNumericalError, "Lanczos coefficient became non-finite");
    double e_new;
    if (!tridiag_lowest(a.data(), b.data(), (int)(m + 1), &e_new, nullptr))
      fail(kNumericalError, "tridiagonal eigensolver did not converge");
    if ((energy0 - e_new) < prm.error || m == dim || m == maxit - 1) {
      finish(m + 1, m, e_new);
      break;
    }
    energy0 = e_new;
  }
  return res;
}

}  // namespace gq
