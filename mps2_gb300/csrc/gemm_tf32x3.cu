// Split-precision grouped block GEMM on the 5th-generation tensor cores.
//
// C (FP64) = sum over the tile's (A block, B block) pairs of A.B, with every
// FP64 operand split as x = hi + lo (hi, lo TF32) and each product formed as
// hi*hi + hi*lo + lo*hi by tcgen05.mma kind::tf32 (FP32 accumulation in
// TMEM).  Partial sums are merged chunk by chunk into a double-float
// (FP32 hi + FP32 lo, exact TwoSum) accumulator that also lives in TMEM, and
// written out as FP64 at the end (Markidis et al. 2018 / Ootomo & Yokota
// 2022 split products; Dekker/Knuth TwoSum for the accumulation).
//
// Operands are first "packed" by one elementwise pass per contraction: the
// block is permuted into its matricised orientation, split into hi/lo,
// zero-padded to 128-row x 32-column tiles and written in the exact
// shared-memory image the MMA descriptors read (K-major, 128-byte swizzle).
// The GEMM then moves every tile with one bulk asynchronous copy and does no
// per-element work of its own.
//
// CTA layout (192 threads): warps 0-3 merge and write back (warp q owns TMEM
// lanes 32q..32q+31), warp 4 issues the bulk copies, warp 5 allocates TMEM
// and issues the MMAs.  Every mbarrier wait is bounded; on timeout the CTA
// records an error code, drains, frees its TMEM and exits.
#include <cstdint>

#include "exact_convert.cuh"
#include "gq_runtime.hpp"

namespace gq {

namespace tc {
constexpr int BM = 128, BN = 128, BK = 32;      // tile and k-step (fp32 elements)
constexpr int kStages = 3;
constexpr int kTileFloats = BM * BK;             // one 128x32 operand image
constexpr int kTileBytes = kTileFloats * 4;      // 16 KB
constexpr int kStageBytes = 4 * kTileBytes;      // A hi, A lo, B hi, B lo
constexpr int kChunkSteps = 8;                   // k-steps per merged chunk (K <= 256)
constexpr int kThreads = 192;
constexpr uint32_t kTmemCols = 512;              // acc0, acc1, sum_hi, sum_lo
constexpr long long kWaitCycles = 4000000000ll;
}  // namespace tc

// ---------------------------------------------------------------------------
// Packing
// ---------------------------------------------------------------------------
struct PackBlock {
  int64_t src_off;       // element offset of the FP64 block
  int64_t dst_off;       // float offset of the packed image (tile (0,0), hi)
  int rows, cols;        // matricised rows (M or N) and K
  int nrt, nkt;          // row tiles, k tiles
  int rrank, krank;
  int rdims[kMaxRank];
  int64_t rstr[kMaxRank];
  int kdims[kMaxRank];
  int64_t kstr[kMaxRank];
};
struct PackTask { int block, rt, kt; };

// Split x into TF32 hi and lo (FP32 bit patterns) with integer and FP32
// operations only (the FP64 pipe of this part is far slower than its
// integer and FP32 pipes).  hi = round-to-nearest(x) to 11 significant
// bits; lo = the next 11 significant bits of (fl32(x) - hi).  Magnitudes
// below FP32's normal range are flushed to zero.
__device__ __forceinline__ void split_tf32(double x, uint32_t &hi, uint32_t &lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ff);
  const int e32 = e - 1023 + 127;
  if (e == 0 || e32 <= 0) { hi = lo = 0u; return; }
  if (e32 >= 255) { hi = sign | 0x7f7fe000u; lo = 0u; return; }  // clamp (unreachable for DMRG data)
  const unsigned long long mant = b & 0xfffffffffffffull;
  uint32_t m23 = (uint32_t)(mant >> 29);
  uint32_t f = sign | ((uint32_t)e32 << 23) | m23;
  if ((mant >> 28) & 1ull) f += 1u;                      // round half away on the 29 dropped bits
  hi = (f + 0x1000u) & 0xffffe000u;                      // tf32, round half away
  const float r = __uint_as_float(f) - __uint_as_float(hi);  // exact (Sterbenz)
  const uint32_t rb = __float_as_uint(r);
  lo = ((rb & 0x7f800000u) == 0u) ? 0u : ((rb + 0x1000u) & 0xffffe000u);
}

// One CTA per 128x32 tile of one block.  Element (r, k) of the tile goes to
// byte offset r*128 + (((k/4) ^ (r%8)) * 16) + (k%4)*4 of the 16 KB image
// (K-major, 128-byte swizzle, 8-row atoms of 1024 B); lo follows hi.
__global__ void __launch_bounds__(256)
    pack_split_kernel(const PackBlock *__restrict__ blocks, const PackTask *__restrict__ tasks,
                      const double *__restrict__ src, float *__restrict__ dst) {
  const PackTask tk = tasks[blockIdx.x];
  __shared__ PackBlock pb;
  if (threadIdx.x == 0) pb = blocks[tk.block];
  __syncthreads();
  uint32_t *hi = reinterpret_cast<uint32_t *>(dst + pb.dst_off +
                                              ((int64_t)tk.rt * pb.nkt + tk.kt) * 2 * tc::kTileFloats);
  uint32_t *lo = hi + tc::kTileFloats;
  // thread -> (row, k): 8 consecutive k per thread-group for coalescing on
  // K-contiguous sources; 4096 elements, 16 per thread.
  for (int e = threadIdx.x; e < tc::BM * tc::BK; e += blockDim.x) {
    const int r = e / tc::BK, k = e % tc::BK;
    const int gr = tk.rt * tc::BM + r, gk = tk.kt * tc::BK + k;
    uint32_t h = 0u, l = 0u;
    if (gr < pb.rows && gk < pb.cols) {
      int64_t off = pb.src_off;
      int rem = gr;
      for (int j = pb.rrank - 1; j >= 0; --j) {
        const int d = pb.rdims[j];
        off += (int64_t)(rem % d) * pb.rstr[j];
        rem /= d;
      }
      rem = gk;
      for (int j = pb.krank - 1; j >= 0; --j) {
        const int d = pb.kdims[j];
        off += (int64_t)(rem % d) * pb.kstr[j];
        rem /= d;
      }
      split_tf32(src[off], h, l);
    }
    const int w = r * 32 + ((((k >> 2) ^ (r & 7)) << 2) | (k & 3));
    hi[w] = h;
    lo[w] = l;
  }
}

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and *abort set) once about tc::kWaitCycles SM clocks
// (~2 s) have passed, or as soon as another role has aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
  const long long t0 = clock64();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (clock64() - t0 > tc::kWaitCycles) break;
  }
  *abort = 1;
  return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 B apart (SBO), sm100 descriptor version 1.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3fff);
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
#define TC_LD32(taddr, r)                                                                     \
  asm volatile(                                                                               \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"      \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),   \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),            \
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),         \
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),         \
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),         \
        "=r"(r[31])                                                                           \
      : "r"(taddr))
#define TC_ST32(taddr, r)                                                                     \
  asm volatile(                                                                               \
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12," \
      "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::  \
          "r"(taddr),                                                                         \
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), \
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),       \
      "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),     \
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),     \
      "r"(r[29]), "r"(r[30]), "r"(r[31])                                                      \
      : "memory")
__device__ __forceinline__ void tc_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// ---------------------------------------------------------------------------
// The GEMM kernel
// ---------------------------------------------------------------------------
struct TcSmem {
  alignas(1024) unsigned char stage[tc::kStages][tc::kStageBytes];
  uint64_t full[tc::kStages];
  uint64_t empty[tc::kStages];
  uint64_t accfull[2];
  uint64_t accempty[2];
  uint64_t mma_done;
  uint32_t tmem_base;
  int abort;
  int nchunks;
};

__global__ void __launch_bounds__(tc::kThreads, 1)
    gemm_tf32x3_kernel(const GemmTile *__restrict__ tiles, const GemmPair *__restrict__ pairs,
                       const float *__restrict__ Ap, const float *__restrict__ Bp,
                       double *__restrict__ C, int *__restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  TcSmem &sm = *reinterpret_cast<TcSmem *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const GemmTile t = tiles[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int *abort = &sm.abort;

  // chunk count: each pair contributes ceil(ceil(K/32)/kChunkSteps) chunks
  if (threadIdx.x == 0) {
    int nc = 0;
    for (int p = t.pair_begin; p < t.pair_end; ++p) {
      const int nkt = (pairs[p].k + tc::BK - 1) / tc::BK;
      nc += (nkt + tc::kChunkSteps - 1) / tc::kChunkSteps;
    }
    sm.nchunks = nc;
    sm.abort = 0;
    for (int s = 0; s < tc::kStages; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.accfull[b], 1);
      mbar_init(&sm.accempty[b], 128);
    }
    mbar_init(&sm.mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sm.tmem_base)),
                 "r"(tc::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.tmem_base;
  const int nchunks = sm.nchunks;

  if (warp == 4) {
    // ---------------- producer: one bulk copy per packed operand pair -----
    if (lane == 0) {
      int stage = 0;
      for (int p = t.pair_begin; p < t.pair_end && !*abort; ++p) {
        const GemmPair pr = pairs[p];
        const int nkt = (pr.k + tc::BK - 1) / tc::BK;
        const float *a = Ap + pr.a_off + (int64_t)(t.row0 / tc::BM) * nkt * 2 * tc::kTileFloats;
        const float *b = Bp + pr.b_off + (int64_t)(t.col0 / tc::BN) * nkt * 2 * tc::kTileFloats;
        for (int kt = 0; kt < nkt; ++kt, ++stage) {
          const int s = stage % tc::kStages;
          const uint32_t ph = (uint32_t)(stage / tc::kStages) & 1u;
          if (!mbar_wait(&sm.empty[s], ph ^ 1u, abort)) break;
          mbar_arrive_expect_tx(&sm.full[s], 4 * tc::kTileBytes);
          bulk_g2s(sm.stage[s], a + (int64_t)kt * 2 * tc::kTileFloats, 2 * tc::kTileBytes,
                   &sm.full[s]);
          bulk_g2s(sm.stage[s] + 2 * tc::kTileBytes, b + (int64_t)kt * 2 * tc::kTileFloats,
                   2 * tc::kTileBytes, &sm.full[s]);
        }
      }
      // Drain: the last copies into each stage must have landed before the
      // CTA may exit (normally the MMA side already waited for them).
      for (int st = stage - tc::kStages; st < stage; ++st) {
        if (st < 0) continue;
        volatile int no_abort = 0;
        mbar_wait(&sm.full[st % tc::kStages], (uint32_t)(st / tc::kStages) & 1u, &no_abort);
      }
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer ---------------------------------------------
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc(tc::BM, tc::BN);
      int stage = 0, chunk = 0;
      for (int p = t.pair_begin; p < t.pair_end && !*abort; ++p) {
        const int nkt = (pairs[p].k + tc::BK - 1) / tc::BK;
        for (int k0 = 0; k0 < nkt && !*abort; k0 += tc::kChunkSteps, ++chunk) {
          const int buf = chunk & 1;
          if (!mbar_wait(&sm.accempty[buf], ((uint32_t)(chunk >> 1) & 1u) ^ 1u, abort)) break;
          fence_after_sync();
          const uint32_t dacc = tmem + (uint32_t)(buf * tc::BN);
          const int kend = min(nkt, k0 + tc::kChunkSteps);
          for (int kt = k0; kt < kend; ++kt, ++stage) {
            const int s = stage % tc::kStages;
            if (!mbar_wait(&sm.full[s], (uint32_t)(stage / tc::kStages) & 1u, abort)) break;
            fence_after_sync();
            const uint32_t base = smem_u32(sm.stage[s]);
            const uint64_t ahi = make_desc(base), alo = make_desc(base + tc::kTileBytes);
            const uint64_t bhi = make_desc(base + 2 * tc::kTileBytes);
            const uint64_t blo = make_desc(base + 3 * tc::kTileBytes);
#pragma unroll
            for (int ks = 0; ks < tc::BK / 8; ++ks) {
              const uint64_t adv = (uint64_t)((ks * 32) >> 4);  // 8 tf32 = 32 bytes
              const uint32_t first = (kt == k0 && ks == 0) ? 0u : 1u;
              mma_tf32(dacc, ahi + adv, bhi + adv, idesc, first);
              mma_tf32(dacc, ahi + adv, blo + adv, idesc, 1u);
              mma_tf32(dacc, alo + adv, bhi + adv, idesc, 1u);
            }
            mma_commit(&sm.empty[s]);  // frees the stage once these MMAs are done
          }
          mma_commit(&sm.accfull[buf]);
        }
      }
      // Drain every MMA issued by this thread before TMEM is released.
      mma_commit(&sm.mma_done);
      volatile int no_abort = 0;
      mbar_wait(&sm.mma_done, 0u, &no_abort);
    }
  } else {
    // ---------------- merge warps 0-3: lane quarter q = warp -------------------
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const uint32_t sum_hi = tmem + lane_base + 2 * tc::BN;
    const uint32_t sum_lo = tmem + lane_base + 3 * tc::BN;
    for (int c = 0; c < nchunks; ++c) {
      const int buf = c & 1;
      if (!mbar_wait(&sm.accfull[buf], (uint32_t)(c >> 1) & 1u, abort)) break;
      fence_after_sync();
      const uint32_t acc = tmem + lane_base + (uint32_t)(buf * tc::BN);
#pragma unroll 1
      for (int cb = 0; cb < tc::BN / 32; ++cb) {
        uint32_t pv[32], hv[32], lv[32];
        TC_LD32(acc + cb * 32, pv);
        if (c > 0) {
          TC_LD32(sum_hi + cb * 32, hv);
          TC_LD32(sum_lo + cb * 32, lv);
        }
        tc_wait_ld();
        if (c == 0) {
#pragma unroll
          for (int j = 0; j < 32; ++j) { hv[j] = pv[j]; lv[j] = 0u; }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float a = __uint_as_float(hv[j]), b = __uint_as_float(pv[j]);
            const float s = __fadd_rn(a, b);
            const float bb = __fsub_rn(s, a);
            const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
            const float l = __fadd_rn(__uint_as_float(lv[j]), e);
            const float s2 = __fadd_rn(s, l);   // renormalise (fast TwoSum, |s| >= |l|)
            hv[j] = __float_as_uint(s2);
            lv[j] = __float_as_uint(__fsub_rn(l, __fsub_rn(s2, s)));
          }
        }
        TC_ST32(sum_hi + cb * 32, hv);
        TC_ST32(sum_lo + cb * 32, lv);
        tc_wait_st();
      }
      fence_before_sync();
      mbar_arrive(&sm.accempty[buf]);
    }
    // ---------------- write back the FP64 tile ---------------------------------
    const int row = t.row0 + warp * 32 + lane;
    double *crow = C + t.c_off + (int64_t)row * t.n;
    if (!*abort) {
      if (nchunks == 0) {
        if (row < t.m)
          for (int j = 0; j < tc::BN && t.col0 + j < t.n; ++j) crow[t.col0 + j] = 0.0;
      } else {
#pragma unroll 1
        for (int cb = 0; cb < tc::BN / 32; ++cb) {
          uint32_t hv[32], lv[32];
          TC_LD32(sum_hi + cb * 32, hv);
          TC_LD32(sum_lo + cb * 32, lv);
          tc_wait_ld();
          if (row < t.m) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int col = t.col0 + cb * 32 + j;
              if (col < t.n)
                // hi and lo as doubles from their bits (exact_convert.cuh), one FP64 add
                crow[col] = xconv::f32_bits_to_f64(hv[j]) + xconv::f32_bits_to_f64(lv[j]);
            }
          }
        }
      }
    }
  }

  fence_before_sync();
  __syncthreads();
  if (warp == 5) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(tc::kTmemCols)
                 : "memory");
  }
  if (threadIdx.x == 0 && sm.abort) atomicExch(err, 1);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
int gemm_tile_m(Precision prec) { return prec == kTF32x3 ? tc::BM : 64; }
int gemm_tile_n(Precision prec) { return prec == kTF32x3 ? tc::BN : 64; }

namespace {
int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Rows/k-tiles layout of one matricised block: legs `rl` (rows) and `kl`
// (contracted) of block b of tensor t.
PackBlock pack_block(const Tensor &t, int64_t b, const std::vector<int> &rl,
                     const std::vector<int> &kl, int64_t dst_off) {
  PackBlock pb{};
  const int r = t.rank();
  int64_t str[kMaxRank];
  int64_t s = 1;
  for (int l = r - 1; l >= 0; --l) {
    str[l] = s;
    s *= t.block_dim(b, l);
  }
  pb.src_off = t.offs[b];
  pb.dst_off = dst_off;
  int64_t rows = 1, cols = 1;
  pb.rrank = (int)rl.size();
  for (size_t j = 0; j < rl.size(); ++j) {
    pb.rdims[j] = (int)t.block_dim(b, rl[j]);
    pb.rstr[j] = str[rl[j]];
    rows *= pb.rdims[j];
  }
  pb.krank = (int)kl.size();
  for (size_t j = 0; j < kl.size(); ++j) {
    pb.kdims[j] = (int)t.block_dim(b, kl[j]);
    pb.kstr[j] = str[kl[j]];
    cols *= pb.kdims[j];
  }
  pb.rows = (int)rows;
  pb.cols = (int)cols;
  pb.nrt = (int)ceil_div(rows, tc::BM);
  pb.nkt = (int)ceil_div(cols, tc::BK);
  return pb;
}
}  // namespace

void build_tc_pack(const Tensor &t, const std::vector<int> &row_legs,
                   const std::vector<int> &k_legs, TcPackPlan &pp,
                   const std::vector<char> *used) {
  std::vector<PackBlock> blocks;
  std::vector<PackTask> tasks;
  pp.base.assign(t.nblocks(), 0);
  blocks.reserve(t.nblocks());
  int64_t off = 0;
  for (int64_t b = 0; b < t.nblocks(); ++b) {
    PackBlock pb = pack_block(t, b, row_legs, k_legs, off);
    pp.base[b] = off;
    if (used && !(*used)[b]) {  // no image: keep the entry, no space, no tasks
      pb.nrt = pb.nkt = 0;
      blocks.push_back(pb);
      continue;
    }
    off += (int64_t)pb.nrt * pb.nkt * 2 * tc::kTileFloats;
    for (int rt = 0; rt < pb.nrt; ++rt)
      for (int kt = 0; kt < pb.nkt; ++kt) tasks.push_back({(int)b, rt, kt});
    blocks.push_back(pb);
  }
  pp.floats = off;
  pp.ntasks = (int64_t)tasks.size();
  pp.blocks_dev.upload(reinterpret_cast<const char *>(blocks.data()),
                       (int64_t)(blocks.size() * sizeof(blocks[0])));
  pp.tasks_dev.upload(reinterpret_cast<const char *>(tasks.data()),
                      (int64_t)(tasks.size() * sizeof(tasks[0])));
}

void run_tc_pack(const TcPackPlan &pp, const double *src, float *dst) {
  if (pp.ntasks == 0) return;
  prof_begin(kProfPermute);
  pack_split_kernel<<<(unsigned)pp.ntasks, 256, 0, stream()>>>(
      reinterpret_cast<const PackBlock *>(pp.blocks_dev.p),
      reinterpret_cast<const PackTask *>(pp.tasks_dev.p), src, dst);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfPermute, 0.0, (double)pp.ntasks * tc::kTileFloats * 16.0);
}

void launch_gemm_tf32x3(const ContractPlan &p, const float *A, const float *B, double *C) {
  const size_t smem = sizeof(TcSmem) + 1024;
  // once per process, whichever lane launches first
  static const cudaError_t attr = cudaFuncSetAttribute(
      gemm_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  GQ_CUDA(attr);
  int *err = tc_error_flag();
  prof_begin(kProfGemmTf32);
  gemm_tf32x3_kernel<<<(unsigned)p.ntiles_tc, tc::kThreads, smem, stream()>>>(
      p.tiles_tc.p, p.pairs_tc.p, A, B, C, err);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfGemmTf32, p.flops_tc, 8.0 * (double)(p.a_elems + p.b_elems));
}

int *tc_error_flag() { return reinterpret_cast<int *>(lane().dev_scalars + 63); }

}  // namespace gq
