// C ABI (include/gqmps2_gb300.h) over the library's C++ internals.
#include "../../include/gqmps2_gb300.h"

#include <atomic>
#include <cstdio>
#include <mutex>
#include <string>
#include <thread>

#include "gq_dmrg.hpp"

struct gq_tensor {
  gq::TensorPtr t;
};
struct gq_dmrg {
  gq::Dmrg d;
};

namespace {
thread_local std::string g_err;

template <typename F>
int guarded(F &&f) {
  try {
    f();
    g_err.clear();
    return GQ_OK;
  } catch (const gq::Error &e) {
    g_err = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_err = "host allocation failed";
    return GQ_ERR_OOM;
  } catch (const std::exception &e) {
    g_err = e.what();
    return GQ_ERR_INTERNAL;
  }
}

gq::Precision prec_of(int p) {
  GQ_CHECK(p == GQ_PREC_FP64 || p == GQ_PREC_TF32X3 || p == GQ_PREC_FP64TC, "unknown precision");
  return (gq::Precision)p;
}

gq::Precision rayleigh_of(int p) {
  GQ_CHECK(p == GQ_PREC_FP64 || p == GQ_PREC_FP64TC,
           "the Rayleigh-quotient energy needs an FP64-accurate form");
  return (gq::Precision)p;
}

gq::Where where_of(int w) {
  GQ_CHECK(w >= GQ_WHERE_LEND && w <= GQ_WHERE_REND, "unknown position");
  return (gq::Where)w;
}

gq_tensor *wrap(gq::TensorPtr t) {
  auto *h = new gq_tensor;
  h->t = std::move(t);
  return h;
}

const gq::Tensor &deref(const gq_tensor *h, const char *what) {
  GQ_CHECK(h && h->t, std::string("null tensor: ") + what);
  return *h->t;
}

gq::EffHam eff_ham(const gq_tensor *L, const gq_tensor *Wl, const gq_tensor *Wr,
                   const gq_tensor *R, int where) {
  gq::EffHam h;
  h.where = where_of(where);
  h.Wl = &deref(Wl, "Wl");
  h.Wr = &deref(Wr, "Wr");
  if (h.where != gq::kLend) h.L = &deref(L, "L");
  if (h.where != gq::kRend) h.R = &deref(R, "R");
  return h;
}
}  // namespace

extern "C" {

int gq_init(int device) {
  return guarded([&] { gq::init_context(device); });
}

const char *gq_last_error(void) { return g_err.c_str(); }

int gq_synchronize(void) {
  return guarded([&] { gq::sync(); });
}

namespace {
// Structure of a tensor from the C arrays of gq_tensor_create, validated.
gq::TensorPtr structure_from_c(int rank, int nq, const int *dirs, const int *nsecs,
                               const int *qns, const int64_t *dims, const int *div,
                               int64_t nblocks, const int *coords) {
    GQ_CHECK(rank >= 1 && rank <= gq::kMaxRank, "rank out of range");
    GQ_CHECK(nq >= 1 && nq <= gq::kMaxQ, "nq out of range");
    GQ_CHECK(dirs && nsecs && qns && dims && div, "null structure array");
    GQ_CHECK(nblocks >= 0 && (nblocks == 0 || coords), "bad block list");
    gq::ctx();
    std::vector<gq::Index> idx(rank);
    int64_t qo = 0, dof = 0;
    for (int l = 0; l < rank; ++l) {
      GQ_CHECK(dirs[l] == GQ_OUT || dirs[l] == GQ_IN, "leg direction must be +1 or -1");
      GQ_CHECK(nsecs[l] >= 1, "every leg needs a sector");
      idx[l].dir = dirs[l];
      for (int s = 0; s < nsecs[l]; ++s) {
        gq::QN q;
        for (int k = 0; k < nq; ++k) q.v[k] = qns[qo++];
        GQ_CHECK(dims[dof] >= 1, "sector dimension must be positive");
        idx[l].qn.push_back(q);
        idx[l].dim.push_back(dims[dof++]);
      }
    }
    gq::QN d;
    for (int k = 0; k < nq; ++k) d.v[k] = div[k];
    std::vector<std::vector<int>> blocks(nblocks, std::vector<int>(rank));
    for (int64_t b = 0; b < nblocks; ++b) {
      for (int l = 0; l < rank; ++l) blocks[b][l] = coords[b * rank + l];
      if (b > 0) GQ_CHECK(blocks[b - 1] < blocks[b], "blocks must be in ascending block order");
    }
    auto t = gq::make_structure(nq, idx, d, blocks);
    for (int64_t b = 0; b < t->nblocks(); ++b)
      GQ_CHECK(t->block_div(t->block_coords(b)) == d, "block breaks the tensor's divergence");
    return t;
}
}  // namespace

int gq_tensor_create(int rank, int nq, const int *dirs, const int *nsecs, const int *qns,
                     const int64_t *dims, const int *div, int64_t nblocks, const int *coords,
                     const double *data, gq_tensor **out) {
  return guarded([&] {
    GQ_CHECK(out, "null output handle");
    auto t = structure_from_c(rank, nq, dirs, nsecs, qns, dims, div, nblocks, coords);
    t->allocate();
    if (data) {
      // complete on return: the caller may free `data`
      gq::copy_h2d(t->data.p, data, sizeof(double) * t->size());
    } else {
      t->zero();
    }
    *out = wrap(t);
  });
}

int gq_tensor_create_blocks(int rank, int nq, const int *dirs, const int *nsecs,
                            const int *qns, const int64_t *dims, const int *div,
                            int64_t nblocks, const int *coords, const double *const *blocks,
                            gq_tensor **out) {
  return guarded([&] {
    GQ_CHECK(out, "null output handle");
    GQ_CHECK(blocks || nblocks == 0, "null block pointer array");
    auto t = structure_from_c(rank, nq, dirs, nsecs, qns, dims, div, nblocks, coords);
    t->allocate();
    std::vector<const void *> src((size_t)nblocks);
    std::vector<size_t> sz((size_t)nblocks);
    for (int64_t b = 0; b < nblocks; ++b) {
      GQ_CHECK(blocks[b], "null block data");
      src[b] = blocks[b];
      sz[b] = sizeof(double) * (size_t)t->block_size(b);
    }
    // complete on return: the caller may free the blocks
    gq::copy_h2d_gather(t->data.p, src.data(), sz.data(), (size_t)nblocks);
    *out = wrap(t);
  });
}

int gq_tensor_describe(const gq_tensor *h, int *rank, int *nq, int64_t *nsec_total,
                       int64_t *nblocks, int64_t *nelem) {
  return guarded([&] {
    const gq::Tensor &t = deref(h, "t");
    int64_t ns = 0;
    for (auto &ix : t.idx) ns += ix.nsec();
    if (rank) *rank = t.rank();
    if (nq) *nq = t.nq;
    if (nsec_total) *nsec_total = ns;
    if (nblocks) *nblocks = t.nblocks();
    if (nelem) *nelem = t.size();
  });
}

int gq_tensor_export(const gq_tensor *h, int *dirs, int *nsecs, int *qns, int64_t *dims, int *div,
                     int *coords, double *data) {
  return guarded([&] {
    const gq::Tensor &t = deref(h, "t");
    int64_t qo = 0, dof = 0;
    for (int l = 0; l < t.rank(); ++l) {
      if (dirs) dirs[l] = t.idx[l].dir;
      if (nsecs) nsecs[l] = t.idx[l].nsec();
      for (int s = 0; s < t.idx[l].nsec(); ++s) {
        for (int k = 0; k < t.nq; ++k) {
          if (qns) qns[qo] = t.idx[l].qn[s].v[k];
          ++qo;
        }
        if (dims) dims[dof] = t.idx[l].dim[s];
        ++dof;
      }
    }
    if (div)
      for (int k = 0; k < t.nq; ++k) div[k] = t.div.v[k];
    if (coords) std::copy(t.coords.begin(), t.coords.end(), coords);
    if (data && t.size() > 0) gq::copy_d2h(data, t.data.p, sizeof(double) * t.size());
  });
}

int gq_tensor_destroy(gq_tensor *h) {
  return guarded([&] { delete h; });
}

int gq_tensor_dag(const gq_tensor *t, gq_tensor **out) {
  return guarded([&] {
    GQ_CHECK(out, "null output");
    *out = wrap(gq::dag(deref(t, "t")));
  });
}

int gq_contract(const gq_tensor *a, const gq_tensor *b, int naxes, const int *axes_a,
                const int *axes_b, int precision, gq_tensor **out, double *flops) {
  return guarded([&] {
    GQ_CHECK(out && axes_a && axes_b && naxes >= 1, "bad arguments");
    std::vector<int> xa(axes_a, axes_a + naxes), xb(axes_b, axes_b + naxes);
    double f = 0.0;
    auto c = gq::contract(deref(a, "a"), deref(b, "b"), xa, xb, prec_of(precision), &f);
    gq::check_device_errors();
    if (flops) *flops = f;
    *out = wrap(c);
  });
}

int gq_contract_noalloc(const gq_tensor *a, const gq_tensor *b, int naxes, const int *axes_a,
                        const int *axes_b, gq_tensor *out) {
  return guarded([&] {
    GQ_CHECK(out && out->t && axes_a && axes_b && naxes >= 1, "bad arguments");
    std::vector<int> xa(axes_a, axes_a + naxes), xb(axes_b, axes_b + naxes);
    gq::contract_noalloc(deref(a, "a"), deref(b, "b"), xa, xb, *out->t);
  });
}

int gq_eff_ham_mul_state(const gq_tensor *L, const gq_tensor *Wl, const gq_tensor *Wr,
                         const gq_tensor *R, int where, const gq_tensor *state, int precision,
                         gq_tensor **out, double *flops) {
  return guarded([&] {
    GQ_CHECK(out, "null output handle");
    auto h = eff_ham(L, Wl, Wr, R, where);
    const gq::Tensor &x = deref(state, "state");
    auto space = gq::lanczos_space(x);
    space->allocate();
    gq::embed(x, *space);
    auto plan = gq::plan_matvec(h, *space, prec_of(precision));
    auto y = gq::clone_structure(*space);
    y->allocate();
    gq::run_matvec(*plan, space->data.p, y->data.p);
    gq::check_device_errors();
    if (flops) *flops = gq::matvec_flops(*plan);
    *out = wrap(y);
  });
}

int gq_lanczos(const gq_tensor *L, const gq_tensor *Wl, const gq_tensor *Wr, const gq_tensor *R,
               int where, const gq_tensor *init, const gq_lanczos_params *params, int precision,
               int64_t *iters, double *gs_eng, gq_tensor **gs_vec) {
  return guarded([&] {
    GQ_CHECK(params, "null Lanczos parameters");
    auto h = eff_ham(L, Wl, Wr, R, where);
    const gq::Tensor &x = deref(init, "init");
    auto space = gq::lanczos_space(x);
    space->allocate();
    gq::embed(x, *space);
    gq::LanczosParamsC lp;
    lp.error = params->error;
    lp.max_iterations = params->max_iterations;
    lp.rayleigh = rayleigh_of(params->rayleigh);
    auto res = gq::lanczos(h, *space, lp, prec_of(precision));
    gq::check_device_errors();
    if (iters) *iters = res.iters;
    if (gs_eng) *gs_eng = res.energy;
    if (gs_vec)
      *gs_vec = wrap(res.gs);
  });
}

int gq_svd(const gq_tensor *t, int ldims, const int *ldiv, double trunc_err, int64_t dmin,
           int64_t dmax, int scale_side, gq_tensor **u, gq_tensor **vt, double *s, int64_t s_cap,
           double *actual_trunc_err, int64_t *D) {
  return guarded([&] {
    const gq::Tensor &x = deref(t, "t");
    GQ_CHECK(ldiv, "null ldiv");
    GQ_CHECK(scale_side >= 0 && scale_side <= 2, "scale_side must be 0, 1 or 2");
    gq::QN q;
    for (int k = 0; k < x.nq; ++k) q.v[k] = ldiv[k];
    auto r = gq::svd_truncate(x, ldims, q, trunc_err, dmin, dmax, scale_side);
    gq::sync();
    if (s) {
      GQ_CHECK(s_cap >= (int64_t)r.s.size(), "singular value buffer too small");
      std::copy(r.s.begin(), r.s.end(), s);
    }
    if (actual_trunc_err) *actual_trunc_err = r.trunc_err;
    if (D) *D = r.D;
    if (u) *u = wrap(r.u);
    if (vt) *vt = wrap(r.vt);
  });
}

int gq_dmrg_create(int n_sites, gq_tensor *const *mps, gq_tensor *const *mpo, gq_dmrg **out) {
  return guarded([&] {
    GQ_CHECK(out && mps && mpo && n_sites >= 2, "bad arguments");
    auto *d = new gq_dmrg;
    try {
      for (int i = 0; i < n_sites; ++i) {
        d->d.mps.push_back(gq::clone(deref(mps[i], "mps")));
        d->d.mpo.push_back(gq::clone(deref(mpo[i], "mpo")));
      }
    } catch (...) {
      delete d;
      throw;
    }
    *out = d;
  });
}

int gq_dmrg_init_envs(gq_dmrg *d, int precision) {
  return guarded([&] {
    GQ_CHECK(d, "null dmrg handle");
    d->d.init_envs(prec_of(precision));
    gq::sync();
  });
}

int gq_dmrg_set_env(gq_dmrg *d, int dir, int len, const gq_tensor *env) {
  return guarded([&] {
    GQ_CHECK(d && (dir == 'l' || dir == 'r') && len >= 1, "bad arguments");
    d->d.envs[{(char)dir, len}] = gq::clone(deref(env, "env"));
  });
}

int gq_dmrg_get_env(gq_dmrg *d, int dir, int len, gq_tensor **out) {
  return guarded([&] {
    GQ_CHECK(d && out, "bad arguments");
    auto it = d->d.envs.find({(char)dir, len});
    GQ_CHECK(it != d->d.envs.end(), "no such environment");
    *out = wrap(gq::clone(*it->second));
    gq::sync();
  });
}

namespace {
gq::SweepParamsC sweep_params(const gq_sweep_params *p) {
  GQ_CHECK(p, "null sweep parameters");
  GQ_CHECK(p->sweeps >= 0 && p->dmin >= 1 && p->dmax >= p->dmin, "bad sweep parameters");
  gq::SweepParamsC sp;
  sp.sweeps = p->sweeps;
  sp.dmin = p->dmin;
  sp.dmax = p->dmax;
  sp.trunc_err = p->trunc_err;
  sp.lanczos.error = p->lanczos.error;
  sp.lanczos.max_iterations = p->lanczos.max_iterations;
  sp.precision = prec_of(p->precision);
  sp.verbose = p->verbose;
  sp.lanczos.rayleigh = rayleigh_of(p->lanczos.rayleigh);
  return sp;
}

void export_stats(const gq::UpdateStatsC &x, gq_update_stats &o) {
  o.site = x.site;
  o.dir = x.dir;
  o.e0 = x.e0;
  o.trunc_err = x.trunc_err;
  o.D = x.D;
  o.iters = x.iters;
  o.ee = x.ee;
  o.lanczos_seconds = x.lanczos_seconds;
  o.update_seconds = x.update_seconds;
  o.svd_seconds = x.svd_seconds;
  o.env_seconds = x.env_seconds;
  o.matvecs = x.matvecs;
  o.matvec_flops = x.matvec_flops;
  o.env_flops = x.env_flops;
  o.theta_size = x.theta_size;
}
}  // namespace

int gq_dmrg_sweep(gq_dmrg *d, const gq_sweep_params *p, gq_update_stats *stats, double *e0) {
  return guarded([&] {
    GQ_CHECK(d, "null dmrg handle");
    const gq::SweepParamsC sp = sweep_params(p);
    double e = 0.0;
    std::vector<gq::UpdateStatsC> st;
    for (int64_t s = 0; s < p->sweeps; ++s) {
      if (p->verbose) std::printf("sweep %lld\n", (long long)(s + 1));
      e = d->d.sweep(sp, &st);
    }
    gq::sync();
    if (stats)
      for (size_t i = 0; i < st.size(); ++i) export_stats(st[i], stats[i]);
    if (e0) *e0 = e;
  });
}

namespace {
std::vector<gq::TensorPtr> mps_of(gq_tensor *const *mps, int n) {
  GQ_CHECK(mps && n >= 2, "an MPS needs at least two sites");
  std::vector<gq::TensorPtr> v(n);
  for (int i = 0; i < n; ++i) {
    GQ_CHECK(mps[i] && mps[i]->t, "null MPS tensor");
    v[i] = mps[i]->t;
  }
  return v;
}
}  // namespace

int gq_mps_centralize(gq_tensor *const *mps, int n, int center, int *cano) {
  return guarded([&] {
    auto v = mps_of(mps, n);
    GQ_CHECK(cano, "null canonical-type array");
    std::vector<int> c(cano, cano + n);
    gq::centralize(v, c, center);
    gq::sync();
    for (int i = 0; i < n; ++i) {
      mps[i]->t = v[i];
      cano[i] = c[i];
    }
  });
}

int gq_mps_truncate(gq_tensor *const *mps, int n, int *cano, double trunc_err, int64_t dmin,
                    int64_t dmax, double *errs, int64_t *Ds) {
  return guarded([&] {
    auto v = mps_of(mps, n);
    GQ_CHECK(cano, "null canonical-type array");
    GQ_CHECK(dmin >= 1 && dmax >= dmin, "bad Dmin/Dmax");
    std::vector<int> c(cano, cano + n);
    auto res = gq::truncate_mps(v, c, trunc_err, dmin, dmax);
    gq::sync();
    for (int i = 0; i < n; ++i) {
      mps[i]->t = v[i];
      cano[i] = c[i];
    }
    for (size_t b = 0; b < res.size(); ++b) {
      if (errs) errs[b] = res[b].first;
      if (Ds) Ds[b] = res[b].second;
    }
  });
}

int gq_dmrg_run_batch(gq_dmrg *const *states, int n, const gq_sweep_params *params,
                      int init_envs, int nthreads, double *e0) {
  return guarded([&] {
    GQ_CHECK(n >= 0 && (n == 0 || (states && params)), "bad arguments");
    GQ_CHECK(nthreads >= 1, "nthreads must be positive");
    for (int i = 0; i < n; ++i) {
      GQ_CHECK(states[i], "null dmrg handle");
      sweep_params(&params[i]);  // validate up front
    }
    gq::sync();  // the states were built on this thread's lane
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    std::mutex mu;
    int err_code = GQ_OK;
    std::string err_msg;
    auto worker = [&] {
      gq::Lane *l = nullptr;
      const int rc = guarded([&] {
        l = gq::lane_create();
        gq::lane_bind(l);
        for (int i = next++; i < n && !failed; i = next++) {
          const gq::SweepParamsC sp = sweep_params(&params[i]);
          gq::Dmrg &d = states[i]->d;
          if (init_envs) d.init_envs(sp.precision);
          double e = 0.0;
          for (int64_t s = 0; s < sp.sweeps; ++s) e = d.sweep(sp, nullptr);
          gq::check_device_errors();
          if (e0) e0[i] = e;
        }
      });
      if (rc != GQ_OK) {
        failed = true;
        std::lock_guard<std::mutex> lk(mu);
        if (err_code == GQ_OK) {
          err_code = rc;
          err_msg = gq_last_error();
        }
      }
      if (l) {
        gq::lane_bind(nullptr);
        gq::lane_destroy(l);
      }
    };
    const int nt = std::max(1, std::min(nthreads, n));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    if (n > 0) worker();
    for (auto &th : pool) th.join();
    if (err_code != GQ_OK) throw gq::Error(err_code, "batched run: " + err_msg);
  });
}

int gq_dmrg_update(gq_dmrg *d, const gq_sweep_params *p, int dir, int target,
                   gq_update_stats *stats) {
  return guarded([&] {
    GQ_CHECK(d, "null dmrg handle");
    GQ_CHECK(dir == 'r' || dir == 'l', "dir must be 'r' or 'l'");
    const int N = d->d.N();
    GQ_CHECK(dir == 'r' ? (target >= 0 && target <= N - 2) : (target >= 1 && target <= N - 1),
             "target site out of range");
    auto st = d->d.update(sweep_params(p), (char)dir, target);
    gq::sync();
    if (stats) export_stats(st, *stats);
  });
}

int gq_autotune_enable(int on) {
  return guarded([&] { gq::autotune_enable(on != 0); });
}

int gq_profile_enable(int on) {
  return guarded([&] {
    gq::ctx();
    gq::prof_enable(on != 0);
  });
}

int gq_host_sync_count(int64_t *count) {
  return guarded([&] {
    GQ_CHECK(count != nullptr, "null count");
    *count = gq::host_sync_count();
  });
}

int gq_profile_read(int kernel, int64_t *launches, double *ms, double *flops, double *bytes) {
  return guarded([&] {
    GQ_CHECK(kernel >= 0 && kernel < gq::kProfCount, "unknown kernel id");
    gq::prof_read((gq::ProfKernel)kernel, launches, ms, flops, bytes);
  });
}

int gq_get_stream(void **s) {
  return guarded([&] {
    GQ_CHECK(s, "null output");
    *s = (void *)gq::stream();
  });
}

int gq_dmrg_get_mps(gq_dmrg *d, int i, gq_tensor **out) {
  return guarded([&] {
    GQ_CHECK(d && out && i >= 0 && i < d->d.N(), "bad arguments");
    *out = wrap(gq::clone(*d->d.mps[i]));
    gq::sync();
  });
}

int gq_dmrg_destroy(gq_dmrg *d) {
  return guarded([&] { delete d; });
}

}  // extern "C"
