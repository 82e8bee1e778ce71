/*
 * gqmps2_gb300.h -- C ABI of the GB300 (sm_103a) two-site finite DMRG library
 * (libgqmps2_gb300.so).
 *
 * The reference, gqmps2 v0.2-alpha.0, is a header-only C++ template library;
 * its hot path is
 *   GQTEN_Double TwoSiteFiniteVMPS(FiniteMPS&, const MPO&, const SweepParams&)
 *     (include/gqmps2/algorithm/vmps/two_site_update_finite_vmps_impl.h:77-101)
 * with LanczosSolver(eff_ham, init, LanczosParams, where)
 *     (include/gqmps2/algorithm/lanczos_solver_impl.h:79-226)
 * and GraceQ/tensor's block-sparse Contract / SVD underneath.  This header
 * exposes the same pieces with plain pointers and sizes: device-resident
 * block-sparse tensors, the contraction, the effective-Hamiltonian matvec,
 * the Lanczos solver, the truncating SVD and the sweep driver.
 *
 * Conventions
 *   - Every call returns an int status (GQ_OK == 0); on failure
 *     gq_last_error() describes it.  Nothing exits the process (the
 *     reference calls exit(1) on a dstev failure, lanczos_solver_impl.h:288).
 *   - A quantum number is nq int32 values (U(1)^nq, nq <= 4).
 *   - Leg direction: GQ_OUT (+1) or GQ_IN (-1).  A block with sector
 *     coordinates c is allowed when sum_i dir_i * qn_i(c_i) == div.
 *   - Blocks are dense, row-major float64, exchanged in ascending
 *     lexicographic order of their sector coordinates ("block order").
 *   - One process drives one GPU; the library is not re-entrant (neither is
 *     the reference, which stages through fixed file paths).
 */
#ifndef GQMPS2_GB300_H
#define GQMPS2_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GQ_OK 0
#define GQ_ERR_INVALID 1
#define GQ_ERR_CUDA 2
#define GQ_ERR_SOLVER 3
#define GQ_ERR_NUMERICAL 4
#define GQ_ERR_OOM 5
#define GQ_ERR_INTERNAL 6

#define GQ_OUT 1
#define GQ_IN (-1)

/* Arithmetic of the contractions (matvec, environment growth, two-site
 * state).  Lanczos recurrence, tridiagonal solve and SVD are FP64 always. */
#define GQ_PREC_FP64 0   /* plain form: FP64 end to end */
#define GQ_PREC_TF32X3 1 /* split form: 3xTF32 tcgen05 products, FP64 sums */
#define GQ_PREC_FP64TC 2 /* FP64-accurate tcgen05 products (exact bf16 digits,
                            exact FP32 partial sums, FP64 merge) */

/* Position of the two-site block (the reference's `where` string,
 * lanczos_solver_impl.h:93-112). */
#define GQ_WHERE_LEND 0
#define GQ_WHERE_CENT 1
#define GQ_WHERE_REND 2

typedef struct gq_tensor gq_tensor;
typedef struct gq_dmrg gq_dmrg;

/* LanczosParams (include/gqmps2/algorithm/lanczos_solver.h:34-39). */
typedef struct {
  double error;           /* default 1e-7 */
  int64_t max_iterations; /* default 200 */
  int rayleigh; /* split form only (not in the reference): arithmetic of the
                   Rayleigh-quotient energy of the ground state,
                   GQ_PREC_FP64 (FP64 FMA) or GQ_PREC_FP64TC */
} gq_lanczos_params;

/* SweepParams (include/gqmps2/algorithm/vmps/two_site_update_finite_vmps.h:27-55)
 * minus the two paths, which the host wrapper owns, plus the precision. */
typedef struct {
  int64_t sweeps;
  int64_t dmin;
  int64_t dmax;
  double trunc_err;
  gq_lanczos_params lanczos;
  int precision; /* GQ_PREC_* */
  int verbose;   /* 1: print the reference's per-update log line */
} gq_sweep_params;

/* One two-site update: the fields of the reference's log line
 * (two_site_update_finite_vmps_impl.h:329-338) plus timing and work. */
typedef struct {
  int32_t site;
  int32_t dir; /* 'r' or 'l' */
  double e0;
  double trunc_err;
  int64_t D;
  int64_t iters;
  double ee;
  double lanczos_seconds;
  double update_seconds;
  double svd_seconds;
  double env_seconds;
  int64_t matvecs;
  double matvec_flops; /* sum of 2*m*n*k over the matvec block GEMMs */
  double env_flops;
  int64_t theta_size;  /* elements of the two-site state */
} gq_update_stats;

/* Library ------------------------------------------------------------- */
/* Bind the calling process to `device` (-1: current device).  Optional:
 * every other entry point initialises on first use. */
int gq_init(int device);
/* Description of the last failure in this thread ("" if none). */
const char *gq_last_error(void);
/* Wait for all queued device work. */
int gq_synchronize(void);

/* Tensors --------------------------------------------------------------- *
 * Replaces GQTensor construction + element assignment on the host and the
 * implicit host->device placement (the reference keeps tensors in RAM and
 * on disk: include/gqmps2/one_dim_tn/framework/ten_vec.h:50-85).
 *   dirs[rank]; nsecs[rank]; qns: for each leg, nsecs[l] x nq ints;
 *   dims: for each leg, nsecs[l] int64; div[nq];
 *   coords[nblocks x rank] in ascending block order (each block allowed);
 *   data: the blocks' elements concatenated in that order (NULL: zeros). */
int gq_tensor_create(int rank, int nq, const int *dirs, const int *nsecs, const int *qns,
                     const int64_t *dims, const int *div, int64_t nblocks,
                     const int *coords, const double *data, gq_tensor **out);
/* The same with each block's elements at its own address: blocks[nblocks]
 * (not in the reference; spares the caller gathering the blocks into one
 * buffer).  Both copy through pinned staging and return with the copy
 * complete. */
int gq_tensor_create_blocks(int rank, int nq, const int *dirs, const int *nsecs,
                            const int *qns, const int64_t *dims, const int *div,
                            int64_t nblocks, const int *coords,
                            const double *const *blocks, gq_tensor **out);
/* Sizes needed to export: rank, nq, total sector count over legs, blocks,
 * elements. */
int gq_tensor_describe(const gq_tensor *t, int *rank, int *nq, int64_t *nsec_total,
                       int64_t *nblocks, int64_t *nelem);
/* Export the structure and (if data != NULL) copy the elements to host
 * memory.  Arrays must hold the sizes reported by gq_tensor_describe. */
int gq_tensor_export(const gq_tensor *t, int *dirs, int *nsecs, int *qns, int64_t *dims,
                     int *div, int *coords, double *data);
int gq_tensor_destroy(gq_tensor *t);
/* gqten Dag for real tensors: every leg's direction inverted, divergence
 * negated, data copied (new handle). */
int gq_tensor_dag(const gq_tensor *t, gq_tensor **out);

/* Contraction ------------------------------------------------------------ *
 * gqten Contract(a, b, {axes_a, axes_b}, &c): output legs are a's free
 * legs then b's free legs.  Call sites: two_site_update_finite_vmps_impl.h:
 * 118-129, 243, 272, 276, 290-317; lanczos_solver_impl.h:231-254. */
int gq_contract(const gq_tensor *a, const gq_tensor *b, int naxes, const int *axes_a,
                const int *axes_b, int precision, gq_tensor **out, double *flops);

/* Contraction without device allocation.  This entry point has no
 * counterpart in the reference.  It serves callers that own all device
 * memory themselves and cannot let a library allocate during their work (a
 * host application that lends the library a fixed budget, a plugin inside
 * another framework's time step, where cudaMalloc's device-wide
 * synchronisation would stall unrelated work).  Same result as gq_contract
 * with GQ_PREC_FP64, written into `out`, which the caller creates beforehand
 * (gq_tensor_create) with a's free legs then b's free legs, divergence
 * div(a) + div(b), and every block the contraction produces.  Scratch lives
 * in file-scope device arrays (about 22 MiB on each GPU that uses the
 * library, kept until exit): a and b together may hold at most 2^21
 * elements, with at most 2^15 output tiles of 64 x 64, 2^17 block products
 * and 2^15 permute tasks; larger inputs return GQ_ERR_INVALID.  gq_init
 * looks the arrays up and loads this entry point's kernels on its device
 * (CUDA loads modules lazily, and that load may allocate); without gq_init,
 * the first call on a device does it, so make that first call before the
 * no-allocation phase.  Each call returns after its GPU work has finished
 * (it waits on the library stream, so it cannot be captured into a CUDA
 * graph).  Calls share the arrays: calls that overlap on the GPU race. */
int gq_contract_noalloc(const gq_tensor *a, const gq_tensor *b, int naxes, const int *axes_a,
                        const int *axes_b, gq_tensor *out);

/* Effective Hamiltonian ------------------------------------------------- *
 * eff_ham_mul_state_{cent,lend,rend} (lanczos_solver_impl.h:228-256).
 * L / R may be NULL at the chain ends (where = LEND / REND).  The result
 * lives in the Lanczos space: every block allowed by the state's legs and
 * divergence (blocks the contraction does not reach are zero). */
int gq_eff_ham_mul_state(const gq_tensor *L, const gq_tensor *Wl, const gq_tensor *Wr,
                         const gq_tensor *R, int where, const gq_tensor *state, int precision,
                         gq_tensor **out, double *flops);

/* Lanczos --------------------------------------------------------------- *
 * LanczosSolver (lanczos_solver_impl.h:79-226).  `init` is not modified
 * (the reference consumes it); gs_vec is a new tensor in the Lanczos space
 * that the caller destroys. */
int gq_lanczos(const gq_tensor *L, const gq_tensor *Wl, const gq_tensor *Wr, const gq_tensor *R,
               int where, const gq_tensor *init, const gq_lanczos_params *params, int precision,
               int64_t *iters, double *gs_eng, gq_tensor **gs_vec);

/* Truncating SVD -------------------------------------------------------- *
 * gqten SVD(t, ldims, ldiv, trunc_err, Dmin, Dmax, &u, &s, &vt, &err, &D)
 * (two_site_update_finite_vmps_impl.h:258-263).  s receives the kept
 * singular values in bond order (capacity s_cap; *D tells how many).
 * scale_side: 0 plain U / Vt, 1 return U.S in *u, 2 return S.Vt in *vt. */
int gq_svd(const gq_tensor *t, int ldims, const int *ldiv, double trunc_err, int64_t dmin,
           int64_t dmax, int scale_side, gq_tensor **u, gq_tensor **vt, double *s, int64_t s_cap,
           double *actual_trunc_err, int64_t *D);

/* Two-site DMRG --------------------------------------------------------- *
 * The state of TwoSiteFiniteVMPS kept resident on the device: the MPS, the
 * MPO and the left/right environments that the reference stages through
 * <temp_path>/{l,r}env<len> files (GenEnvTenName, :55-61).  The tensors
 * passed in are copied; the caller keeps ownership of its handles. */
int gq_dmrg_create(int n_sites, gq_tensor *const *mps, gq_tensor *const *mpo, gq_dmrg **out);
/* InitEnvs (two_site_update_finite_vmps_impl.h:104-135): right
 * environments R_1..R_{N-2} from a right-canonical MPS. */
int gq_dmrg_init_envs(gq_dmrg *d, int precision);
/* Install / fetch an environment ('l' or 'r', block length) -- the
 * equivalent of reading / writing an env file, used to resume. */
int gq_dmrg_set_env(gq_dmrg *d, int dir, int len, const gq_tensor *env);
int gq_dmrg_get_env(gq_dmrg *d, int dir, int len, gq_tensor **out);
/* `sweeps` sweeps of TwoSiteFiniteVMPSSweep (:143-161).  stats (may be
 * NULL) receives 2*(N-1) records per sweep.  *e0 = energy of the last
 * update, the reference's return value. */
int gq_dmrg_sweep(gq_dmrg *d, const gq_sweep_params *params, gq_update_stats *stats,
                  double *e0);
/* One two-site update (TwoSiteFiniteVMPSUpdate, :164-340) at `target` in
 * direction 'r' or 'l'; the caller drives the sweep order. */
int gq_dmrg_update(gq_dmrg *d, const gq_sweep_params *params, int dir, int target,
                   gq_update_stats *stats);
/* Copy of the site tensor i (caller destroys). */
int gq_dmrg_get_mps(gq_dmrg *d, int i, gq_tensor **out);
int gq_dmrg_destroy(gq_dmrg *d);

/* Finite-MPS canonicalisation ---------------------------------------------- *
 * FiniteMPS::Centralize (one_dim_tn/mps/finite_mps/finite_mps.h:149-248) and
 * TruncateMPS (:251-300) on device tensors, in place: the n handles of `mps`
 * (site order, the reference's leg orders) are rewritten.  `cano` holds the
 * canonical type of each site (GQ_CANO_*), read and updated as the
 * reference's tens_cano_type_ is. */
#define GQ_CANO_NONE 0
#define GQ_CANO_LEFT 1
#define GQ_CANO_RIGHT 2
int gq_mps_centralize(gq_tensor *const *mps, int n, int center, int *cano);
/* errs[n-1], Ds[n-1] (optional): truncation error and bond dimension of each
 * bond (the reference prints them). */
int gq_mps_truncate(gq_tensor *const *mps, int n, int *cano, double trunc_err, int64_t dmin,
                    int64_t dmax, double *errs, int64_t *Ds);

/* Batched instances ------------------------------------------------------ *
 * Not in the reference (its tests run one chain per process).  Runs n
 * independent DMRG states concurrently: a pool of `nthreads` host threads,
 * each queueing its work on its own CUDA stream, takes the states in index
 * order; for each state it builds the right environments if `init_envs`
 * (in params[i].precision), then sweeps params[i].sweeps times.  e0[i]
 * (optional) receives the energy of state i's last update.  The states must
 * not be used by other calls meanwhile.  On failure the first error is
 * returned; states not yet started are left untouched. */
int gq_dmrg_run_batch(gq_dmrg *const *states, int n, const gq_sweep_params *params,
                      int init_envs, int nthreads, double *e0);

/* Measurement ------------------------------------------------------------ *
 * Not part of the reference (its only instrumentation is the Timer output,
 * lanczos_solver_impl.h:123-132).  CUDA-event timing of each kernel family
 * on the library's stream; enabling resets the counters. */
#define GQ_PROF_GEMM_FP64 0
#define GQ_PROF_GEMM_TF32X3 1
#define GQ_PROF_PERMUTE 2
#define GQ_PROF_VECTOR 3
#define GQ_PROF_SKINNY 4
#define GQ_PROF_GEMM_FP64TC 5
#define GQ_PROF_SVD 6     /* whole SVD, device span including library calls */
#define GQ_PROF_SVD_EIG 7 /* its decompositions */
#define GQ_PROF_SVD_GATHER 8  /* its gather of the groups */
#define GQ_PROF_SVD_FACTORS 9 /* its factor assembly */
#define GQ_PROF_SVD_ORTHO 10  /* of which the QR of null-space completions */
#define GQ_PROF_SVD_GRAM 11   /* of the decompositions: the Gram matrices */
#define GQ_PROF_SVD_REDUCE 12 /* of the decompositions: their rank-revealing
                                 reduction, rank read-back included */
#define GQ_PROF_HOST_PLAN 13  /* host wall time spent planning contractions
                                 (work lists, kernel choice); "launches" counts
                                 the plans */
#define GQ_PROF_HOST_SYNC 14  /* host wall time blocked waiting for the device
                                 (stream synchronisations); "launches" counts
                                 the waits */
int gq_profile_enable(int on);
/* Tile-choice autotuner (not in the reference): with `on`, every matvec
 * contraction whose block-size histogram has not been seen before times the
 * candidate tensor-core thresholds on its real operands and keeps the
 * fastest for all later contractions with that histogram (environment
 * growth included).  Off by default: the fixed thresholds keep results
 * bitwise reproducible from run to run. */
int gq_autotune_enable(int on);
int gq_profile_read(int kernel, int64_t *launches, double *ms, double *flops, double *bytes);
/* The cudaStream_t all library work is queued on. */
int gq_get_stream(void **stream);
/* Diagnostics (not in the reference): the number of times the library has
 * waited on the host for its streams since it was loaded (every thread and
 * lane).  A Lanczos solve on the main lane waits once; driven from the host
 * (batched lanes, profiler on, GQ_NO_GRAPHS set) it waits once more per
 * iteration. */
int gq_host_sync_count(int64_t *count);

#ifdef __cplusplus
}
#endif

#endif /* GQMPS2_GB300_H */
