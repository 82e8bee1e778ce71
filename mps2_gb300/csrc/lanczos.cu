// Effective-Hamiltonian matvec and Lanczos ground-state solver.
//
// Restates ``LanczosSolver`` (``lanczos_solver_impl.h:79-226``) with the
// Krylov vectors resident in HBM: no re-orthogonalisation, every basis
// vector kept, stop on ``E_old - E_new < error`` or ``m == eff_dim`` or
// ``m == max_iterations - 1``; breakdown handled as at ``:163-180``.  The
// matvec follows ``eff_ham_mul_state_{cent,lend,rend}`` (``:228-256``)
// contraction for contraction; its work lists are planned once per update
// and replayed every iteration.
//
// The iteration itself runs on the device: the recurrence scalars, the
// tridiagonal Ritz value (``TridiagGsSolver``, ``:259-313``) and the
// stopping rule are computed by control kernels, so one iteration is a
// fixed sequence of launches.  On the main lane that sequence is the body
// of a CUDA-graph while loop and a whole solve costs one host wait; the
// lanes of a batched run and profiled runs launch it once per iteration and
// read the control block back after each.
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
};

namespace {
// The device loop runs as a CUDA graph on the main lane, unless the kernel
// profiler is on (it times every launch with its own events, which a graph
// body cannot hold) or GQ_NO_GRAPHS is set.  Not on the lanes of a batched
// run: there every solve's graph build would contend across the host
// threads (64 XXZ chains with graphed matvecs: 26.2 s, without: 19.3 s).
bool graphs_enabled() {
  static const bool off = std::getenv("GQ_NO_GRAPHS") != nullptr;
  return !off && !prof_on() && on_main_lane();
}

// A graph solve allocates every Krylov vector it may need up front; above
// this many bytes the solve runs host-driven and allocates them one by one.
constexpr double kGraphKrylovBytes = 48e9;

struct GraphHolder {  // released on every exit path
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
  ~GraphHolder() {
    if (e) cudaGraphExecDestroy(e);
    if (g) cudaGraphDestroy(g);
  }
};
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

LanczosResult lanczos(const EffHam &h, const Tensor &init, const LanczosParamsC &prm,
                      Precision prec) {
  const int64_t maxit = prm.max_iterations;
  GQ_CHECK(maxit >= 2, "Lanczos needs max_iterations >= 2");
  GQ_CHECK(maxit <= (1 << 20), "Lanczos max_iterations above 2^20");
  const int64_t n = init.size();
  GQ_CHECK(n > 0, "empty Lanczos vector");
  const int64_t dim = eff_ham_dim(h);
  auto plan = plan_matvec(h, init, prec);
  // the split form reports the FP64 Rayleigh quotient of its ground state;
  // its matvec is planned while the device iterates
  const bool rayleigh = prec == kTF32x3 && prm.fp64_rayleigh;
  std::shared_ptr<MatvecPlan> p64;
  auto s = stream();

  // Krylov vectors: v_k for k < kmax at most (the loop stops at m == dim or
  // m == maxit - 1 and writes gamma_{m+1} only while m + 1 < maxit).
  const int64_t kmax = std::min<int64_t>(maxit, dim + 2);
  const bool graph = graphs_enabled() && (double)kmax * (double)n * 8.0 <= kGraphKrylovBytes;
  std::vector<DevBuf> vecs;
  vecs.reserve(kmax);
  std::vector<double *> table(kmax, nullptr);
  auto add_vec = [&]() {
    vecs.emplace_back(n);
    table[vecs.size() - 1] = vecs.back().p;
  };
  add_vec();
  add_vec();
  if (graph)
    while ((int64_t)vecs.size() < kmax) add_vec();
  DevArray<double *> tab;
  tab.upload(table);
  DevBuf w(n), xin(graph ? n : 0), red(dot_scratch_elems()), rq(2);
  // device scalars: a (maxit), b (maxit), |gamma|^2 (maxit + 1), Ritz
  // coefficients (maxit), eigenvector scratch (5 maxit), control block
  const int64_t ctl_doubles = (sizeof(LzCtl) + sizeof(double) - 1) / sizeof(double);
  DevBuf sc(9 * maxit + 1 + ctl_doubles);
  LzLoop L;
  L.a_dev = sc.p;
  L.b_dev = L.a_dev + maxit;
  L.n_dev = L.b_dev + maxit;
  L.c_dev = L.n_dev + maxit + 1;
  L.work = L.c_dev + maxit;
  L.ctl = reinterpret_cast<LzCtl *>(L.work + 5 * maxit);
  L.vecs = tab.p;
  L.xin = graph ? xin.p : nullptr;
  L.w = w.p;
  L.n = n;
  L.red = red.p;
  L.maxit = (int)maxit;
  L.dim = dim;
  L.error = prm.error;
  L.cap = (int)maxit + 2;

  LanczosResult res;
  // v0 = init / |init|, w = H v0, a_0, gamma_1 (``lanczos_solver_impl.h:120-160``)
  double *v0 = table[0];
  GQ_CUDA(cudaMemcpyAsync(v0, init.data.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  dev_dot(v0, v0, n, L.n_dev, red.p);
  dev_scale_rsqrt(v0, n, L.n_dev);
  run_matvec(*plan, v0, w.p);
  dev_dot(v0, w.p, n, L.a_dev, red.p);
  dev_lanczos_gamma(w.p, v0, L.a_dev, nullptr, nullptr, true, table[1], n, L.n_dev + 1, red.p);
  lz_init(L.ctl, L.a_dev);

  LzCtl *hc = reinterpret_cast<LzCtl *>(lane().host_scalars);
  if (graph) {
    GraphHolder G;
    GQ_CUDA(cudaGraphCreate(&G.g, 0));
    cudaGraphConditionalHandle cond;
    GQ_CUDA(cudaGraphConditionalHandleCreate(&cond, G.g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    GQ_CUDA(cudaGraphAddNode(&node, G.g, nullptr, nullptr, 0, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    GQ_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    try {
      lz_iteration(L, [&]() { run_matvec(*plan, xin.p, w.p); }, true, cond);
    } catch (...) {
      cudaGraph_t dead = nullptr;
      cudaStreamEndCapture(s, &dead);
      throw;
    }
    cudaGraph_t captured = nullptr;
    GQ_CUDA(cudaStreamEndCapture(s, &captured));
    GQ_CUDA(cudaGraphInstantiate(&G.e, G.g, 0));
    GQ_CUDA(cudaGraphLaunch(G.e, s));
  } else {
    for (int m = 1;; ) {
      // gamma_{m+1} is written this iteration: its vector must exist
      if (m + 1 < kmax && (int64_t)vecs.size() <= m + 1) {
        add_vec();
        upload_async(tab.p + m + 1, &table[m + 1], sizeof(double *));
      }
      double *vm = table[m];
      lz_iteration(L, [&]() { run_matvec(*plan, vm, w.p); }, false, 0);
      GQ_CUDA(cudaMemcpyAsync(hc, L.ctl, sizeof(LzCtl), cudaMemcpyDeviceToHost, s));
      sync();
      if (hc->status != kLzRunning) break;
      m = hc->m;
    }
  }

  // Ritz vector, the Rayleigh quotient, and one read-back of the results
  if (rayleigh) p64 = plan_matvec(h, init, prm.rayleigh);
  auto gs = clone_structure(init);
  gs->allocate();
  lz_ritz_vector(L, gs->data.p);
  if (rayleigh) {
    run_matvec(*p64, gs->data.p, w.p);
    dev_dot(gs->data.p, w.p, n, rq.p, red.p);
    dev_dot(gs->data.p, gs->data.p, n, rq.p + 1, red.p);
  }
  double *hs = lane().host_scalars + ctl_doubles;
  GQ_CUDA(cudaMemcpyAsync(hc, L.ctl, sizeof(LzCtl), cudaMemcpyDeviceToHost, s));
  if (rayleigh)
    GQ_CUDA(cudaMemcpyAsync(hs, rq.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  sync();
  const LzCtl c = *hc;
  switch (c.status) {
    case kLzConverged:
    case kLzInvariant:
      break;
    case kLzBadVector:
      fail(kNumericalError, "Lanczos vector became non-finite");
    case kLzBadCoefficient:
      fail(kNumericalError, "Lanczos coefficient became non-finite");
    default:
      fail(kNumericalError, "Lanczos loop stopped without meeting its stopping rule (status " +
                                std::to_string(c.status) + ")");
  }
  res.iters = c.iters;
  res.energy = c.energy;
  res.ritz_energy = c.energy;
  res.gs = gs;
  res.matvecs = 1 + c.guard;
  res.matvec_flops = plan->flops * (double)(1 + c.guard);
  if (rayleigh) {
    res.energy = hs[0] / hs[1];
    res.matvecs++;
    res.matvec_flops += p64->flops;
  }
  return res;
}

}  // namespace gq
