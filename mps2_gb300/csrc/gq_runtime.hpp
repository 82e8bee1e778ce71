// Declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <functional>

#include <string>
#include <vector>

#include "gq_common.hpp"

namespace gq {

// An execution lane: the stream a host thread's library work is queued on,
// with the scalar buffers and library handles tied to that stream.  Every
// thread uses the context's main lane unless it has bound its own, which
// is how independent DMRG instances run concurrently (one host thread and
// one stream each).
struct PlanCache;  // contract.cu
struct Lane {
  cudaStream_t stream = nullptr;
  double *host_scalars = nullptr;  // pinned, 64 doubles
  double *dev_scalars = nullptr;   // device, 64 doubles; [63] = tensor-core error word
  void *cusolver = nullptr;        // cusolverDnHandle_t, created lazily
  void *cublas = nullptr;          // cublasHandle_t, created lazily
  char *staging = nullptr;         // pinned ring for work-list uploads
  size_t staging_head = 0;
  // Two pinned buffers for large copies of caller memory (copy_h2d/d2h),
  // with the events of their last DMA; allocated on first use.
  char *xfer[2] = {nullptr, nullptr};
  cudaEvent_t xfer_done[2] = {nullptr, nullptr};
  // Auxiliary streams for independent library calls inside one operation
  // (the block SVD's eigensolves of different sizes run side by side),
  // forked from and joined back to `stream` with events; created on first
  // use by init_aux.
  static constexpr int kAux = 3;
  cudaStream_t aux_stream[kAux] = {};
  void *aux_cusolver[kAux] = {};  // cusolverDnHandle_t on aux_stream[i]
  cudaEvent_t fork_event = nullptr;
  cudaEvent_t join_event[kAux] = {};
  // Contraction plans of this lane, kept by structure (contract.cu).
  std::shared_ptr<PlanCache> plan_cache;
};

struct Context {
  int device = 0;
  cudaDeviceProp prop{};
  Lane main;
};

Context &ctx();
void init_context(int device);
void init_lane(Lane &l);
void init_aux(Lane &l);               // the lane's auxiliary streams and events
void fork_aux(Lane &l, int n);        // aux streams 0..n-1 wait for `stream`
void join_aux(Lane &l, int n);        // `stream` waits for aux streams 0..n-1
// Joins aux streams 0..n-1 back into the lane's stream when it goes out of
// scope, on every path (errors are not thrown from the destructor).
struct AuxJoin {
  Lane &l;
  int n;
  AuxJoin(Lane &lane_, int n_) : l(lane_), n(n_) {}
  AuxJoin(const AuxJoin &) = delete;
  AuxJoin &operator=(const AuxJoin &) = delete;
  ~AuxJoin() {
    for (int i = 0; i < n; ++i) {
      cudaEventRecord(l.join_event[i], l.aux_stream[i]);
      cudaStreamWaitEvent(l.stream, l.join_event[i], 0);
    }
  }
};
void destroy_lane_handles(Lane &l);  // cuSOLVER / cuBLAS handles (svd.cu)
Lane &lane();              // this thread's lane
Lane *lane_create();       // a new lane (own non-blocking stream)
void lane_destroy(Lane *l);
void lane_bind(Lane *l);   // bind to this thread (nullptr: the main lane)
bool on_main_lane();
void sync();                // wait for this thread's lane stream (counted)
// Copies of caller (pageable) memory to and from the device on the lane's
// stream, pipelined through the lane's pinned buffers: the host copy of one
// chunk (split over host threads) overlaps the DMA of the other.  Both
// return with the copy complete.
void copy_h2d(void *dst, const void *src, size_t bytes);
// The same for the concatenation of nseg host segments (srcs[i], sizes[i]).
void copy_h2d_gather(void *dst, const void *const *srcs, const size_t *sizes, size_t nseg);
void copy_d2h(void *dst, const void *src, size_t bytes);
int64_t host_sync_count();  // waits by sync() since load, all threads

// Kernel profiling with CUDA events on the library stream (off by default).
enum ProfKernel : int {
  kProfGemmFp64 = 0,   // FP64 grouped GEMM
  kProfGemmTf32 = 1,   // 3xTF32 tcgen05 grouped GEMM
  kProfPermute = 2,    // block permutes feeding the GEMMs
  kProfVector = 3,     // Lanczos vector kernels
  kProfSkinny = 4,     // tall-skinny MPO-tensor contractions
  kProfGemmFp64Tc = 5, // FP64-accurate exact-slice tcgen05 grouped GEMM
  kProfSvd = 6,        // whole truncating SVD (device span, library calls included)
  kProfSvdEig = 7,     // its decompositions (cuSOLVER eigensolves / Jacobi, Gram GEMMs)
  kProfSvdGather = 8,  // its gather of the groups into dense matrices
  kProfSvdFactors = 9, // its factor assembly (copies, projections, sign fix, completion)
  kProfSvdOrtho = 10,  // of which: QR of the null-space completions
  kProfSvdGram = 11,   // of the decompositions: the Gram matrices
  kProfSvdReduce = 12, // of the decompositions: rank-revealing reduction and rank read-back
  kProfHostPlan = 13,  // host wall time of contraction planning (not device time)
  kProfHostSync = 14,  // host wall time blocked in stream synchronisations
  kProfCount = 15,
};
bool prof_on();
void prof_enable(bool on);
void prof_begin(ProfKernel k);
void prof_end(ProfKernel k, double flops, double bytes);
void prof_host(ProfKernel k, double seconds);  // add host wall time to a counter
void prof_read(ProfKernel k, int64_t *launches, double *ms, double *flops, double *bytes);

// Arithmetic of the contractions (matvec, environment growth).
enum Precision : int {
  kFP64 = 0,    // FP64 FMA end to end
  kTF32x3 = 1,  // 3xTF32 split products on tcgen05, FP32 accumulate per
                // K-chunk, FP64 sum of the chunks
  kFP64TC = 2,  // FP64-accurate products on tcgen05: exact bf16 integer
                // digits of the operands, exact FP32 partial sums
};

// ---------------------------------------------------------------------------
// Contraction engine (contract.cu)
// ---------------------------------------------------------------------------
struct GemmTile {       // one output tile of one output block
  int64_t c_off;        // element offset of the output block
  int m, n;             // output block rows / cols
  int row0, col0;       // tile origin inside the block
  int pair_begin, pair_end;
  int64_t work;         // sum over pairs of k (for scheduling)
};
struct GemmPair {       // one contributing (A block, B block) product
  int64_t a_off, b_off; // element offsets in the (possibly permuted) operands
  int k;
  int lda, ldb;
};
struct PermBlock {      // permute one block: dst(i0..ir) = src(sum i_l * sstride_l)
  int64_t src_off, dst_off, n;
  int rank;
  int dims[kMaxRank];       // destination dims
  int64_t sstride[kMaxRank];// source stride of each destination dim
};
struct PermChunk { int block; int64_t begin, end; };

struct PermPlan {
  bool needed = false;
  int64_t total = 0;   // elements of the destination layout
  int64_t moved = 0;   // elements actually permuted
  DevArray<PermBlock> blocks;
  DevArray<PermChunk> chunks;
  int64_t nchunks = 0;
};

// Tall-skinny contraction with a small (MPO) B operand: every contributing
// block pair read in place through leg strides (skinny.cu).  The A offsets
// of a pair's contracted indices and the B offsets of its (k, j) values are
// listed once at plan time.
constexpr int kSkMaxK = 64;
constexpr int kSkMaxFree = 4;  // free legs of A
struct SkinnyPair {
  int64_t a_off;                // A block offset
  int64_t fa_str[kSkMaxFree];   // A strides of the free legs, output-row order
  int K;                        // contracted extent
  int koff;                     // first of its K entries in the A-offset list
  int bidx;                     // first of its K x N entries in the B-offset list
  int pad;
};
struct SkinnyItem {             // one output block, cut into CTAs of 256 rows
  int64_t c_off;
  int M, N, cta0, pair_begin, pair_end, nfa;  // cta0: its first CTA
  int fa_dims[kSkMaxFree];
};

// Packed split-precision operand: every block as 128-row x 32-k tiles of
// TF32 hi then lo, each tile in the tensor-core shared-memory image.
struct TcPackPlan {
  std::vector<int64_t> base;  // float offset of each block's packed tiles
  int64_t floats = 0;
  int64_t ntasks = 0;
  DevArray<char> blocks_dev, tasks_dev;
};

// FP64-accurate tensor-core form (gemm_fp64tc.cu): operands packed as 7
// bf16 digit images per 32-k tile plus one scale exponent per operand row.
struct OzTile {
  int64_t c_off;
  int m, n, row0, col0;
  int pair_begin, pair_end;
  int a_rbase, b_rbase;  // first operand row of the output block in A / B
  int64_t work;
};
struct OzPair { int64_t a_off, b_off; int k, pad; };
struct OzPackPlan {
  std::vector<int64_t> base;  // byte offset of each block's tile images
  std::vector<int> row_base;  // operand row of each block's row 0
  int64_t bytes = 0;
  int nrows = 0;
  int64_t ntasks = 0;
  DevArray<char> blocks_dev, tasks_dev;
};
struct OzPacked { unsigned char *data = nullptr; int *rowexp = nullptr; };

struct ContractPlan {
  TensorPtr out;          // output structure (no data)
  int transA = 0, transB = 0;
  PermPlan pa, pb;
  bool use_skinny = false;  // small-B tall-skinny kernel (skinny.cu)
  DevArray<SkinnyItem> sk_items;
  DevArray<SkinnyPair> sk_pairs;
  DevArray<int64_t> sk_koffs;     // A offsets of the pairs' contracted indices
  DevArray<int> sk_bidx;          // B offsets of the pairs' (k, j) values
  int64_t sk_nitems = 0;   // output blocks
  int64_t sk_nctas = 0;    // CTAs of the launch
  int sk_jb = 8;
  bool use_tc = false;    // 3xTF32 tcgen05 kernel (else the FP64 kernel)
  TcPackPlan ta, tb;
  bool a_cached = false, b_cached = false;  // constant operand packed once
  DevBuf a_packed, b_packed;
  double padded_flops = 0.0;
  DevArray<GemmTile> tiles;       // FP64-kernel tiles (and zero blocks)
  DevArray<GemmPair> pairs;
  int64_t ntiles = 0;
  DevArray<GemmTile> tiles_tc;    // tensor-core tiles (128 x 128)
  DevArray<GemmPair> pairs_tc;    // offsets into the packed operands
  int64_t ntiles_tc = 0;
  double flops_tc = 0.0;
  bool use_oz = false;    // FP64-accurate tcgen05 kernel for some blocks
  OzPackPlan oa, ob;
  bool a_oz_cached = false, b_oz_cached = false;
  DevBuf a_oz, b_oz;
  DevArray<OzTile> tiles_oz;
  DevArray<OzPair> pairs_oz;
  int64_t ntiles_oz = 0;
  double flops_oz = 0.0;
  int64_t nzero_blocks = 0;   // output blocks with no contribution
  DevArray<int64_t> zero_blocks;  // (offset, size) pairs to clear
  double flops = 0.0;         // 2*m*n*k summed over block products
  int64_t a_elems = 0, b_elems = 0;
  int tile_m = 0, tile_n = 0;
  uint64_t signature = 0;     // block-size histogram hash (autotuner key)
  double tc_frac = 0.0;       // threshold the plan was built with
};

// Plan C = A . B over the given axes.  If `target` is non-null the output
// uses its structure (every contributing block must exist there; blocks of
// `target` without contributions are written as zeros).
// `tc_frac` < 0: the default share of useful work at which an output block
// goes to the tensor-core kernel (2% for 3xTF32, 3% for FP64TC); otherwise
// that share (an autotuned value).
//
// Plans are kept per lane and handed out again for a contraction with the
// same block structures, axes, arithmetic and threshold (a sweep at fixed D
// meets every bond's structures again); a plan is never handed to two
// holders at once, and the operand packs of cache_operand are released when
// its holder lets it go.  GQ_NO_PLAN_CACHE turns the cache off.
std::shared_ptr<ContractPlan> plan_contract(const Tensor &a, const Tensor &b,
                                            const std::vector<int> &axes_a,
                                            const std::vector<int> &axes_b,
                                            const Tensor *target, Precision prec,
                                            double tc_frac = -1.0);

// Tile-choice autotuner.  A contraction's signature is a hash of its
// block-size histogram (the output blocks' log2 m, n, k, heaviest first);
// for a new signature the candidate tensor-core thresholds are timed on the
// real operands once and the fastest is kept for every later contraction
// with that signature.  Off by default (the choice then follows fixed
// thresholds and results are bitwise reproducible run to run).
void autotune_enable(bool on);
bool autotune_on();
bool autotune_lookup(uint64_t signature, Precision prec, double *tc_frac);
void autotune_store(uint64_t signature, Precision prec, double tc_frac);
extern const double kTuneCandidates[5];
// Scratch needed by run_contract (elements).
int64_t contract_scratch(const ContractPlan &p);
void run_contract(const ContractPlan &p, const double *a, const double *b, double *c,
                  double *scratch, Precision prec);
TensorPtr contract(const Tensor &a, const Tensor &b, const std::vector<int> &axes_a,
                   const std::vector<int> &axes_b, Precision prec, double *flops_out = nullptr);

// Pack a constant operand of the plan once (which = 0: A, 1: B); later
// run_contract calls ignore that operand's pointer.
void cache_operand(ContractPlan &p, int which, const double *src);

// Tall-skinny kernel (launched by run_contract when use_skinny).
bool skinny_eligible_sizes(int64_t a_elems, int64_t b_elems);
bool skinny_eligible(const Tensor &b, int64_t max_k, int64_t max_n);
int skinny_max_free_legs();  // free legs of A the kernel handles
void launch_skinny(const ContractPlan &p, const double *A, const double *B, double *C);
int skinny_rows_per_cta();

// GEMM kernels (launched by run_contract)
void launch_gemm_fp64(const ContractPlan &p, const double *A, const double *B, double *C);
void launch_gemm_tf32x3(const ContractPlan &p, const float *A, const float *B, double *C);
// The pack plans cover the blocks with used[b] != 0 (every block if used is
// null); the other blocks get no packed image.
void build_oz_pack(const Tensor &t, const std::vector<int> &row_legs,
                   const std::vector<int> &k_legs, int tile_rows, OzPackPlan &pp,
                   const std::vector<char> *used = nullptr);
int64_t oz_pack_doubles(const OzPackPlan &pp);
OzPacked oz_layout(const OzPackPlan &pp, double *buf);
void run_oz_pack(const OzPackPlan &pp, const double *src, const OzPacked &dst);
void launch_gemm_fp64tc(const ContractPlan &p, const OzPacked &A, const OzPacked &B, double *C);
int oz_tile_m();
int oz_tile_n();
int64_t oz_max_k();  // k of one FP64-accurate output tile, summed over its pairs
void build_tc_pack(const Tensor &t, const std::vector<int> &row_legs,
                   const std::vector<int> &k_legs, TcPackPlan &pp,
                   const std::vector<char> *used = nullptr);
void run_tc_pack(const TcPackPlan &pp, const double *src, float *dst);
int gemm_tile_m(Precision prec);
int gemm_tile_n(Precision prec);
// Device-side error word of the tensor-core kernels (bounded waits that ran
// out); check_device_errors() raises and clears it.
int *tc_error_flag();
void check_device_errors();

// FP64 contraction into a caller-created output without any device
// allocation (noalloc.cu).
void contract_noalloc(const Tensor &a, const Tensor &b, const std::vector<int> &axes_a,
                      const std::vector<int> &axes_b, Tensor &out);
// Its once-per-device set-up (array addresses, lazy module load), run by
// init_context for the context's device.
void noalloc_setup();

// ---------------------------------------------------------------------------
// Vector kernels (vecops.cu).  Scalars live in device memory so the Lanczos
// recurrence runs without a host round trip per operation.
// ---------------------------------------------------------------------------
// out = sum_i x_i * y_i  (deterministic two-stage reduction)
void dev_dot(const double *x, const double *y, int64_t n, double *out_dev, double *scratch);
// y = x - a*u - b*v (u or v may be null); out = ||y||^2.  a_dev / b_dev point
// to device scalars (b_dev may be null); b is applied as sqrt(*b_dev) when
// b_is_sq.
void dev_lanczos_gamma(const double *x, const double *u, const double *a_dev,
                       const double *v, const double *b_dev, bool b_is_sq,
                       double *y, int64_t n, double *nrm2_out_dev, double *scratch);
// x *= 1/sqrt(*nrm2_dev)
void dev_scale_rsqrt(double *x, int64_t n, const double *nrm2_dev);
// x *= s
void dev_scale(double *x, int64_t n, double s);
// Block copies between structures: (src_off, dst_off, n) triples.
void dev_block_copy(const double *src, double *dst, const std::vector<int64_t> &triples);
int64_t dot_scratch_elems();

// The Lanczos loop on the device (vecops.cu): its control block, the
// buffers one iteration reads and writes, and the launches of one
// iteration (the same launches for every iteration: they read the
// iteration index from the control block).
enum LzStatus : int {
  kLzRunning = 0,
  kLzConverged = 1,       // the stopping rule was met
  kLzInvariant = 2,       // |gamma| == 0: the Krylov space is invariant
  kLzBadVector = -1,      // non-finite Lanczos vector norm
  kLzBadCoefficient = -2, // non-finite a_m or Ritz value
  kLzCapped = -3,         // iteration cap of the device loop reached
};
struct LzCtl {
  int m = 0;        // current iteration (vector v_m is being formed)
  int status = 0;   // LzStatus
  int nvec = 0;     // once stopped: Krylov vectors in the Ritz vector
  int iters = 0;    // once stopped: iterations, as the reference counts them
  int guard = 0;    // iterations executed by the device loop
  int pad = 0;
  double e0 = 0.0;      // lowest Ritz value of the previous iteration
  double energy = 0.0;  // once stopped: the final Ritz value
};
struct LzLoop {
  LzCtl *ctl = nullptr;
  double *const *vecs = nullptr;  // device table: Krylov vector k at vecs[k]
  double *xin = nullptr;          // copy of v_m for a matvec with a fixed input (or null)
  double *w = nullptr;            // matvec output H v_m
  int64_t n = 0;
  double *a_dev = nullptr, *b_dev = nullptr, *n_dev = nullptr;  // a_m, b_m, |gamma_m|^2
  double *c_dev = nullptr, *work = nullptr, *red = nullptr;     // Ritz coefficients, scratch
  int maxit = 0;
  int64_t dim = 0;
  double error = 0.0;
  int cap = 0;
};
using MatvecFn = std::function<void()>;
void lz_init(LzCtl *ctl, const double *a_dev);  // m = 1, e0 = a_0
// One iteration: b, v_m, w = H v_m (matvec), a_m, gamma_{m+1}, stopping
// test; with set_cond the test also sets the graph's loop condition.
void lz_iteration(const LzLoop &L, const MatvecFn &matvec, bool set_cond,
                  cudaGraphConditionalHandle cond);
// Ritz coefficients of the stopped loop and out = sum_k c_k v_k.
void lz_ritz_vector(const LzLoop &L, double *out);

// ---------------------------------------------------------------------------
// Truncating SVD (svd.cu)
// ---------------------------------------------------------------------------
struct SvdOut {
  TensorPtr u, vt;               // U (row legs..., new OUT), Vt (new IN, col legs...)
  std::vector<double> s;         // kept singular values, bond order
  Index new_bond;                // OUT-directed new bond
  double trunc_err = 0.0;
  int64_t D = 0;
};
// scale_side: 0 none, 1 multiply U columns by s (U.S), 2 multiply Vt rows (S.Vt)
SvdOut svd_truncate(const Tensor &t, int ldims, const QN &ldiv, double trunc_err,
                    int64_t dmin, int64_t dmax, int scale_side);

// Rank-revealing reduction of Gram matrices (pcmgs.cu): pivoted Cholesky
// of G (n x n at g_off) with Gram-Schmidt re-orthogonalised columns,
// G ~ Q T T^T Q^T, stopped when the largest remaining diagonal entry is at
// most tol times G's largest diagonal entry or after rcap columns.  Writes
// L and Q (n x rcap, row-major, at q_off), T and C = T T^T (rcap x rcap,
// row-major, at t_off) and the rank r (-1 when rcap columns did not reach
// the tolerance).  groups_small (at most 512 rows) run on 4-CTA clusters,
// groups_big (up to pcmgs_max_rows() rows) on 16-CTA clusters, or 8-CTA
// ones where the device cannot schedule 16.
struct PcGroup {
  int64_t g_off, q_off, t_off;
  int n, rcap;
};
int pcmgs_max_rows();
int pcmgs_max_rank();
void launch_pcmgs(const PcGroup *groups_small, int n_small, const PcGroup *groups_big, int n_big,
                  const double *G, double *L, double *Q, double *T, double *C, int *r_small,
                  int *r_big, double tol);

// ---------------------------------------------------------------------------
// Finite-MPS canonicalisation and truncation (mps.cu)
// ---------------------------------------------------------------------------
enum CanoType : int { kCanoNone = 0, kCanoLeft = 1, kCanoRight = 2 };
void left_canonicalize_ten(std::vector<TensorPtr> &mps, std::vector<int> &cano, int i);
void right_canonicalize_ten(std::vector<TensorPtr> &mps, std::vector<int> &cano, int i);
void centralize(std::vector<TensorPtr> &mps, std::vector<int> &cano, int center);
// (truncation error, D) per bond
std::vector<std::pair<double, int64_t>> truncate_mps(std::vector<TensorPtr> &mps,
                                                     std::vector<int> &cano, double trunc_err,
                                                     int64_t dmin, int64_t dmax);

// ---------------------------------------------------------------------------
// Effective Hamiltonian and Lanczos (lanczos.cu)
// ---------------------------------------------------------------------------
enum Where : int { kLend = 0, kCent = 1, kRend = 2 };

struct EffHam {
  const Tensor *L = nullptr, *Wl = nullptr, *Wr = nullptr, *R = nullptr;
  Where where = kCent;
};

struct MatvecPlan;  // opaque
std::shared_ptr<MatvecPlan> plan_matvec(const EffHam &h, const Tensor &space, Precision prec);
void run_matvec(MatvecPlan &p, const double *x, double *y);
double matvec_flops(const MatvecPlan &p);

struct LanczosParamsC {
  double error = 1e-7;
  int64_t max_iterations = 200;
  // Split form only: recompute the reported energy as the FP64 Rayleigh
  // quotient <gs|H|gs>/<gs|gs> with one matvec in an FP64-accurate form
  // (kFP64 or kFP64TC).
  bool fp64_rayleigh = true;
  Precision rayleigh = kFP64;
};
struct LanczosResult {
  int64_t iters = 0;
  double energy = 0.0;
  TensorPtr gs;        // in the Lanczos-space structure
  int64_t matvecs = 0;
  double matvec_flops = 0.0;
  double matvec_seconds = 0.0;
  double ritz_energy = 0.0;   // the Lanczos (Ritz) value before any correction
};
// The Lanczos space: every block allowed by the state's legs and div.
TensorPtr lanczos_space(const Tensor &state);
// Copy `src` blocks into `dst` (same legs; dst must contain src's blocks).
void embed(const Tensor &src, Tensor &dst);
LanczosResult lanczos(const EffHam &h, const Tensor &init, const LanczosParamsC &p,
                      Precision prec);
int64_t eff_ham_dim(const EffHam &h);

}  // namespace gq
