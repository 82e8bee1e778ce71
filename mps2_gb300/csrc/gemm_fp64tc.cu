// FP64-accurate grouped block GEMM on the 5th-generation tensor cores.
//
// Exact integer slicing (the error-free splitting of Ozaki, Ogita, Oishi and
// Rump, "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication", Numer. Algorithms 59 (2012)), mapped
// onto tcgen05.mma kind::f16 with bf16 operands and FP32 accumulation:
//
//  * every row i of the matricised A (over all of its K blocks) gets a scale
//    exponent E_i with max|a_i.| < 2^E_i, every column j of B likewise F_j;
//  * a = 2^(E_i - 7) * sum_{s<7} d_s 2^(-8s) with signed integer digits
//    |d_s| <= 128 (55 bits of the row maximum), held as bf16 values
//    d_s 2^(-8s) -- exact, since a digit has at most 8 significant bits;
//  * the products of digit pairs (s, t) with s + t <= 6 (28 MMAs per
//    k-step) are accumulated in FP32 in TMEM, one accumulator per order
//    g = s + t for g = 0..3 and one shared by g = 4..6.  A product of two
//    digits is an integer below 2^14 times 2^(-8g); with at most
//    (g + 1) * 256 of them per accumulator between two read-outs, every
//    partial sum of the g <= 3 accumulators is an integer below 2^24 times
//    2^(-8g), i.e. exact in FP32.  The shared g >= 4 accumulator rounds at
//    2^-24 of a value already 2^-32 below the leading one;
//  * every 256 k the accumulators are read out and folded into an exact
//    64-bit integer running sum on the grid 2^-30 (in units of the leading
//    digit product): the orders 0..3 are integers times 2^(-8g), so their
//    values times 2^30 are exact integers; the shared order 4..6
//    accumulator is rounded to that grid (2^-31, below FP64 rounding of the
//    result).  No FP64 arithmetic happens per chunk -- GB300's FP64 rate
//    would make the merge, not the tensor cores, the bottleneck -- only one
//    conversion per output element at the end, where the tile is scaled by
//    2^(E_i + F_j - 14) and written once, through shared memory in whole
//    rows.  A tile's k (summed over its block pairs) is at most 2^16, so the
//    integer sum stays below 2^63.
// Result: error about 2^-55 * max|a_i.| * max|b_.j| per product term, the
// same order as an FP64 GEMM's.
//
// Tiles are 128 x 96 (5 accumulators x 96 columns = 480 of TMEM's 512), the
// k-step is 32 bf16 (64-byte rows, 64-byte swizzle), two pipeline stages of
// 7 A and 7 B slice images (98 KB each).  CTA layout: warps 0-7 merge and
// write back (warp w reads TMEM lanes 32 (w % 4) .. +31, columns
// 48 (w / 4) .. +47), warp 8 issues bulk copies, warp 9 owns TMEM and
// issues the MMAs; every wait is bounded.
#include <cstdint>
#include <map>

#include <unordered_map>

#include "exact_convert.cuh"
#include "gq_runtime.hpp"

namespace gq {

namespace oz {
constexpr int BM = 128, BN = 96, BK = 32;     // tile and k-step (bf16 elements)
constexpr int kSlices = 7;
constexpr int kAcc = 5;                       // orders 0..3 exact, 4..6 shared
constexpr int kStages = 2;
constexpr int kRowBytes = BK * 2;             // 64 B per tile row
constexpr int kATile = BM * kRowBytes;        // one A slice image: 8 KB
constexpr int kBTile = BN * kRowBytes;        // one B slice image: 6 KB
constexpr int kAStage = kSlices * kATile;     // 56 KB
constexpr int kBStage = kSlices * kBTile;     // 42 KB
constexpr int kStageBytes = kAStage + kBStage;
constexpr int kChunkSteps = 8;                // 256 k between read-outs

// The merge turns the FP32 accumulator values into int64 running sums and
// the write-back the sums into doubles, both with the integer and FP32
// pipes only (exact_convert.cuh).
constexpr int kThreads = 320;          // 8 merge warps, producer, MMA issuer
constexpr int kMergeThreads = 256;
// k of one tile, summed over its pairs: per k the running sum grows by at
// most sum_g (g+1) 2^14 2^(-8g) 2^30 < 1.008 * 2^44 (digit products below
// 2^14 on the 2^-30 grid), so 2^18 of k stay below 2^62.02 < 2^63.
constexpr int kMaxK = 1 << 18;
constexpr uint32_t kTmemCols = 512;
constexpr long long kWaitCycles = 4000000000ll;
constexpr int kNoExp = -(1 << 30);            // column outside the tile
// Row exponents start below this (memset 0xc0: about -1.06e9); a valid one
// is at least -1021.
__host__ __device__ constexpr bool valid_exp(int e) { return e > -5000; }
}  // namespace oz

// ---------------------------------------------------------------------------
// Packing
// ---------------------------------------------------------------------------
struct OzPackBlock {
  int64_t src_off;       // element offset of the FP64 block
  int64_t dst_off;       // byte offset of the block's first tile image set
  int rows, cols;        // matricised rows and K
  int nrt, nkt;
  int row_base;          // index of the block's row 0 among the operand's rows
  int tile_rows;         // 128 (A) or 96 (B)
  int rrank, krank;
  int rdims[kMaxRank];
  int64_t rstr[kMaxRank];
  int kdims[kMaxRank];
  int64_t kstr[kMaxRank];
};
struct OzPackTask { int block, rt, kt; };

namespace {
__device__ __forceinline__ int64_t oz_src_offset(const OzPackBlock &pb, int gr, int gk) {
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
  return off;
}

// Exponent e with |x| < 2^e from the FP64 bits (subnormals and zeros: none).
__device__ __forceinline__ int oz_exponent(double x, bool &nonzero) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  nonzero = ef != 0;
  return ef - 1022;
}

// Row maxima: rowexp[row] = max over the row's elements of the exponent.
__global__ void __launch_bounds__(256)
    oz_rowexp_kernel(const OzPackBlock *__restrict__ blocks, const OzPackTask *__restrict__ tasks,
                     const double *__restrict__ src, int *__restrict__ rowexp) {
  const OzPackTask tk = tasks[blockIdx.x];
  __shared__ OzPackBlock pb;
  if (threadIdx.x == 0) pb = blocks[tk.block];
  __syncthreads();
  const int n = pb.tile_rows * oz::BK;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = e / oz::BK, k = e % oz::BK;
    const int gr = tk.rt * pb.tile_rows + r, gk = tk.kt * oz::BK + k;
    if (gr < pb.rows && gk < pb.cols) {
      bool nz;
      const int ex = oz_exponent(src[oz_src_offset(pb, gr, gk)], nz);
      if (nz) atomicMax(rowexp + pb.row_base + gr, ex);
    }
  }
}

// Digits of x for a row of exponent E, as bf16 bit patterns d_s 2^(-8s).
// Integer arithmetic only: Y = round(|x| 2^(55 - E)) < 2^55, then signed
// base-256 digits from the least significant one up.
__device__ __forceinline__ void oz_digits(double x, int E, uint16_t *out) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7ff);
#pragma unroll
  for (int s = 0; s < oz::kSlices; ++s) out[s] = 0;
  if (ef == 0 || !oz::valid_exp(E)) return;
  const unsigned long long mant = (b & 0xfffffffffffffull) | (1ull << 52);
  const int sh = E - ef + 1020;  // >= -2 because |x| < 2^E
  long long Y;
  if (sh < 0) Y = (long long)(mant << (-sh));
  else if (sh > 60) Y = 0;
  else if (sh == 0) Y = (long long)mant;
  else Y = (long long)((mant + (1ull << (sh - 1))) >> sh);
  int d[oz::kSlices];
#pragma unroll
  for (int s = oz::kSlices - 1; s >= 1; --s) {
    int v = (int)(Y & 255);
    if (v >= 128) v -= 256;
    d[s] = v;
    Y = (Y - v) >> 8;
  }
  d[0] = (int)Y;
  const bool neg = (b >> 63) != 0;
#pragma unroll
  for (int s = 0; s < oz::kSlices; ++s) {
    const int v = neg ? -d[s] : d[s];
    // v * 2^(-8s) is exact in FP32 and in bf16 (|v| <= 128): take the top
    // 16 bits of the FP32 pattern
    const float f = __int2float_rn(v) * __uint_as_float((uint32_t)(127 - 8 * s) << 23);
    out[s] = (uint16_t)(__float_as_uint(f) >> 16);
  }
}

// One CTA per (tile_rows x 32) tile of one block: 7 slice images, each in
// the K-major 64-byte-swizzle layout: element (r, k) at byte
// r*64 + (((k/8) ^ ((r/2)%4)) * 16) + (k%8)*2.
__global__ void __launch_bounds__(256)
    oz_pack_kernel(const OzPackBlock *__restrict__ blocks, const OzPackTask *__restrict__ tasks,
                   const double *__restrict__ src, const int *__restrict__ rowexp,
                   unsigned char *__restrict__ dst) {
  const OzPackTask tk = tasks[blockIdx.x];
  __shared__ OzPackBlock pb;
  if (threadIdx.x == 0) pb = blocks[tk.block];
  __syncthreads();
  const int img = pb.tile_rows * oz::kRowBytes;
  unsigned char *base =
      dst + pb.dst_off + ((int64_t)tk.rt * pb.nkt + tk.kt) * (int64_t)oz::kSlices * img;
  const int n = pb.tile_rows * oz::BK;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = e / oz::BK, k = e % oz::BK;
    const int gr = tk.rt * pb.tile_rows + r, gk = tk.kt * oz::BK + k;
    uint16_t dg[oz::kSlices];
    if (gr < pb.rows && gk < pb.cols) {
      oz_digits(src[oz_src_offset(pb, gr, gk)], rowexp[pb.row_base + gr], dg);
    } else {
#pragma unroll
      for (int s = 0; s < oz::kSlices; ++s) dg[s] = 0;
    }
    const int byte = r * oz::kRowBytes + ((((k >> 3) ^ ((r >> 1) & 3)) << 4) | ((k & 7) << 1));
#pragma unroll
    for (int s = 0; s < oz::kSlices; ++s)
      *reinterpret_cast<uint16_t *>(base + (int64_t)s * img + byte) = dg[s];
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
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
  const long long t0 = clock64();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (clock64() - t0 > oz::kWaitCycles) break;
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
// Shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row groups
// 512 B apart (SBO), sm100 descriptor version 1, layout type 4 (64 B).
__device__ __forceinline__ uint64_t make_desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3fff);
  d |= (uint64_t)(512 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;
  return d;
}
// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t make_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
#define OZ_LD16(taddr, r)                                                                     \
  asm volatile(                                                                               \
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15}, [%16];"                                                                      \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),   \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),            \
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])                                                 \
      : "r"(taddr))
__device__ __forceinline__ void tc_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---------------------------------------------------------------------------
// The GEMM kernel
// ---------------------------------------------------------------------------
struct OzSmem {
  alignas(1024) unsigned char stage[oz::kStages][oz::kStageBytes];
  uint64_t full[oz::kStages];
  uint64_t empty[oz::kStages];
  uint64_t accfull;
  uint64_t accempty;
  uint64_t mma_done;
  uint32_t tmem_base;
  int abort;
  int nchunks;
  int nsteps;
  int colexp[oz::BN];
};

__global__ void __launch_bounds__(oz::kThreads, 1)
    gemm_fp64tc_kernel(const OzTile *__restrict__ tiles, const OzPair *__restrict__ pairs,
                       const unsigned char *__restrict__ Ap, const unsigned char *__restrict__ Bp,
                       const int *__restrict__ rowexp_a, const int *__restrict__ rowexp_b,
                       double *__restrict__ C, int *__restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  OzSmem &sm = *reinterpret_cast<OzSmem *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const OzTile t = tiles[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int *abort = &sm.abort;

  if (threadIdx.x == 0) {
    int ns = 0;
    for (int p = t.pair_begin; p < t.pair_end; ++p) ns += (pairs[p].k + oz::BK - 1) / oz::BK;
    sm.nsteps = ns;
    sm.nchunks = (ns + oz::kChunkSteps - 1) / oz::kChunkSteps;
    sm.abort = 0;
    for (int s = 0; s < oz::kStages; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.accfull, 1);
    mbar_init(&sm.accempty, oz::kMergeThreads);
    mbar_init(&sm.mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int j = threadIdx.x; j < oz::BN; j += blockDim.x)
    sm.colexp[j] = (t.col0 + j < t.n) ? rowexp_b[t.b_rbase + t.col0 + j] : oz::kNoExp;
  if (warp == 9) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sm.tmem_base)),
                 "r"(oz::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.tmem_base;
  const int nchunks = sm.nchunks, nsteps = sm.nsteps;

  if (warp == 8) {
    // ---------------- producer -------------------------------------------------
    if (lane == 0) {
      int stage = 0;
      for (int p = t.pair_begin; p < t.pair_end && !*abort; ++p) {
        const OzPair pr = pairs[p];
        const int nkt = (pr.k + oz::BK - 1) / oz::BK;
        const unsigned char *a = Ap + pr.a_off + (int64_t)(t.row0 / oz::BM) * nkt * oz::kAStage;
        const unsigned char *b = Bp + pr.b_off + (int64_t)(t.col0 / oz::BN) * nkt * oz::kBStage;
        for (int kt = 0; kt < nkt; ++kt, ++stage) {
          const int s = stage % oz::kStages;
          const uint32_t ph = (uint32_t)(stage / oz::kStages) & 1u;
          if (!mbar_wait(&sm.empty[s], ph ^ 1u, abort)) break;
          mbar_arrive_expect_tx(&sm.full[s], oz::kStageBytes);
          bulk_g2s(sm.stage[s], a + (int64_t)kt * oz::kAStage, oz::kAStage, &sm.full[s]);
          bulk_g2s(sm.stage[s] + oz::kAStage, b + (int64_t)kt * oz::kBStage, oz::kBStage,
                   &sm.full[s]);
        }
      }
      for (int st = stage - oz::kStages; st < stage; ++st) {
        if (st < 0) continue;
        volatile int no_abort = 0;
        mbar_wait(&sm.full[st % oz::kStages], (uint32_t)(st / oz::kStages) & 1u, &no_abort);
      }
    }
  } else if (warp == 9) {
    // ---------------- MMA issuer -------------------------------------------------
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc_bf16(oz::BM, oz::BN);
      int stage = 0, chunk = 0, in_chunk = 0;
      bool ok = true;
      for (int p = t.pair_begin; p < t.pair_end && ok && !*abort; ++p) {
        const int nkt = (pairs[p].k + oz::BK - 1) / oz::BK;
        for (int kt = 0; kt < nkt; ++kt, ++stage) {
          if (in_chunk == 0) {
            if (!mbar_wait(&sm.accempty, ((uint32_t)chunk & 1u) ^ 1u, abort)) { ok = false; break; }
            fence_after_sync();
          }
          const int s = stage % oz::kStages;
          if (!mbar_wait(&sm.full[s], (uint32_t)(stage / oz::kStages) & 1u, abort)) {
            ok = false;
            break;
          }
          fence_after_sync();
          const uint32_t abase = smem_u32(sm.stage[s]);
          const uint32_t bbase = abase + oz::kAStage;
#pragma unroll
          for (int ks = 0; ks < oz::BK / 16; ++ks) {
            const uint64_t adv = (uint64_t)((ks * 32) >> 4);  // 16 bf16 = 32 bytes
#pragma unroll
            for (int g = 0; g < oz::kSlices; ++g) {
              const int acc = g < oz::kAcc - 1 ? g : oz::kAcc - 1;
              const uint32_t dacc = tmem + (uint32_t)(acc * oz::BN);
#pragma unroll
              for (int sa = 0; sa <= g; ++sa) {
                const int sb = g - sa;
                const bool first = in_chunk == 0 && ks == 0 && sa == 0 && g <= oz::kAcc - 1;
                mma_bf16(dacc, make_desc_sw64(abase + sa * oz::kATile) + adv,
                         make_desc_sw64(bbase + sb * oz::kBTile) + adv, idesc, first ? 0u : 1u);
              }
            }
          }
          mma_commit(&sm.empty[s]);
          ++in_chunk;
          const bool last = stage + 1 == nsteps;
          if (in_chunk == oz::kChunkSteps || last) {
            mma_commit(&sm.accfull);
            ++chunk;
            in_chunk = 0;
          }
        }
      }
      mma_commit(&sm.mma_done);
      volatile int no_abort = 0;
      mbar_wait(&sm.mma_done, 0u, &no_abort);
    }
  } else {
    // ---------------- merge warps 0-7 --------------------------------------------
    const int quad = warp & 3, half = warp >> 2;
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    const int lrow = quad * 32 + lane;          // row within the tile
    const int cbase = half * (oz::BN / 2);      // first of this thread's 48 columns
    long long run[oz::BN / 2];
#pragma unroll
    for (int j = 0; j < oz::BN / 2; ++j) run[j] = 0;
    const float two30 = 1073741824.0f;
    bool done = true;
    for (int c = 0; c < nchunks; ++c) {
      if (!mbar_wait(&sm.accfull, (uint32_t)c & 1u, abort)) { done = false; break; }
      fence_after_sync();
#pragma unroll
      for (int cb = 0; cb < oz::BN / 2 / 16; ++cb) {
#pragma unroll 1
        for (int a = 0; a < oz::kAcc; ++a) {
          uint32_t f[16];
          OZ_LD16(tmem + lane_base + (uint32_t)(a * oz::BN + cbase + cb * 16), f);
          tc_wait_ld();
          if (a < oz::kAcc - 1) {
#pragma unroll
            for (int j = 0; j < 16; ++j)  // orders 0..3: x * 2^30 is an exact integer
              run[cb * 16 + j] += xconv::integral_f32_to_i64(__uint_as_float(f[j]) * two30);
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j)  // orders 4..6: rounded to the nearest integer
              run[cb * 16 + j] +=
                  xconv::integral_f32_to_i64(xconv::round_f32(__uint_as_float(f[j]) * two30));
          }
        }
      }
      fence_before_sync();
      mbar_arrive(&sm.accempty);
    }
    // all MMAs are complete (the last chunk's accumulators were read), so
    // the pipeline stages are free: stage the scaled tile there and write
    // whole rows (after an abort copies may still be landing there: nothing
    // is staged)
    double *tile = reinterpret_cast<double *>(sm.stage[0]);  // 128 x 96
    const int row = t.row0 + lrow;
    const int er = (row < t.m) ? rowexp_a[t.a_rbase + row] : oz::kNoExp;
    if (done) {
#pragma unroll
      for (int j = 0; j < oz::BN / 2; ++j) {
        const int cl = cbase + j;
        const int ec = sm.colexp[cl];
        double x = 0.0;
        if (nchunks > 0 && oz::valid_exp(er) && oz::valid_exp(ec)) {
          bool ok;
          x = xconv::scaled_i64_to_f64(run[j], er + ec - 44, ok);
          if (!ok) x = ldexp((double)run[j], er + ec - 44);
        }
        tile[lrow * oz::BN + cl] = x;
      }
    }
    asm volatile("bar.sync 1, %0;" ::"n"(oz::kMergeThreads) : "memory");
    if (done && !*abort) {
      const int rows = min(oz::BM, t.m - t.row0), cols = min(oz::BN, t.n - t.col0);
      for (int e = threadIdx.x; e < rows * cols; e += oz::kMergeThreads) {
        const int r = e / cols, cl = e % cols;
        C[t.c_off + (int64_t)(t.row0 + r) * t.n + t.col0 + cl] = tile[r * oz::BN + cl];
      }
    }
  }

  fence_before_sync();
  __syncthreads();
  if (warp == 9) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(oz::kTmemCols)
                 : "memory");
  }
  if (threadIdx.x == 0 && sm.abort) atomicExch(err, 1);
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
int oz_tile_m() { return oz::BM; }
int oz_tile_n() { return oz::BN; }
int64_t oz_max_k() { return oz::kMaxK; }

void build_oz_pack(const Tensor &t, const std::vector<int> &row_legs,
                   const std::vector<int> &k_legs, int tile_rows, OzPackPlan &pp,
                   const std::vector<char> *used) {
  std::vector<OzPackBlock> blocks;
  std::vector<OzPackTask> tasks;
  pp.base.assign(t.nblocks(), 0);
  pp.row_base.assign(t.nblocks(), 0);
  // operand rows: one range per distinct row-leg sector tuple (the tuple
  // packed 16 bits per leg into two words)
  struct RowKey {
    uint64_t hi, lo;
    bool operator==(const RowKey &o) const { return hi == o.hi && lo == o.lo; }
  };
  struct RowKeyHash {
    size_t operator()(const RowKey &k) const { return (size_t)(k.hi * 0x9e3779b97f4a7c15ull ^ k.lo); }
  };
  std::unordered_map<RowKey, int, RowKeyHash> row_of;
  row_of.reserve((size_t)t.nblocks() * 2);
  GQ_CHECK(row_legs.size() <= 8, "more than 8 row legs");
  for (int l : row_legs) GQ_CHECK(t.idx[l].nsec() < 65536, "a leg with 65536 or more sectors");
  int nrows = 0;
  int64_t off = 0;
  const int r = t.rank();
  blocks.reserve(t.nblocks());
  for (int64_t b = 0; b < t.nblocks(); ++b) {
    OzPackBlock pb{};
    if (used && !(*used)[b]) {  // no image: keep the entry, no rows, no tasks
      pb.dst_off = off;
      pp.base[b] = off;
      blocks.push_back(pb);
      continue;
    }
    int64_t str[kMaxRank];
    int64_t s = 1;
    for (int l = r - 1; l >= 0; --l) {
      str[l] = s;
      s *= t.block_dim(b, l);
    }
    pb.src_off = t.offs[b];
    pb.dst_off = off;
    int64_t rows = 1, cols = 1;
    RowKey key{0, 0};
    pb.rrank = (int)row_legs.size();
    for (size_t j = 0; j < row_legs.size(); ++j) {
      pb.rdims[j] = (int)t.block_dim(b, row_legs[j]);
      pb.rstr[j] = str[row_legs[j]];
      rows *= pb.rdims[j];
      const uint64_t v = (uint64_t)t.block_coords(b)[row_legs[j]];
      if (j < 4) key.hi |= v << (16 * j);
      else key.lo |= v << (16 * (j - 4));
    }
    pb.krank = (int)k_legs.size();
    for (size_t j = 0; j < k_legs.size(); ++j) {
      pb.kdims[j] = (int)t.block_dim(b, k_legs[j]);
      pb.kstr[j] = str[k_legs[j]];
      cols *= pb.kdims[j];
    }
    pb.rows = (int)rows;
    pb.cols = (int)cols;
    pb.tile_rows = tile_rows;
    pb.nrt = (int)ceil_div(rows, tile_rows);
    pb.nkt = (int)ceil_div(cols, oz::BK);
    auto it = row_of.find(key);
    if (it == row_of.end()) {
      it = row_of.emplace(key, nrows).first;
      nrows += (int)rows;
    }
    pb.row_base = it->second;
    pp.base[b] = off;
    pp.row_base[b] = pb.row_base;
    off += (int64_t)pb.nrt * pb.nkt * oz::kSlices * tile_rows * oz::kRowBytes;
    for (int rt = 0; rt < pb.nrt; ++rt)
      for (int kt = 0; kt < pb.nkt; ++kt) tasks.push_back({(int)b, rt, kt});
    blocks.push_back(pb);
  }
  pp.bytes = off;
  pp.nrows = nrows;
  pp.ntasks = (int64_t)tasks.size();
  pp.blocks_dev.upload(reinterpret_cast<const char *>(blocks.data()),
                       (int64_t)(blocks.size() * sizeof(blocks[0])));
  pp.tasks_dev.upload(reinterpret_cast<const char *>(tasks.data()),
                      (int64_t)(tasks.size() * sizeof(tasks[0])));
}

int64_t oz_pack_doubles(const OzPackPlan &pp) {
  // packed images, then the row exponents, with 128-byte alignment slack
  return (pp.bytes + 7) / 8 + (pp.nrows + 1) / 2 + 32;
}

OzPacked oz_layout(const OzPackPlan &pp, double *buf) {
  OzPacked o;
  o.data = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(buf) + 127) &
                                             ~(uintptr_t)127);
  o.rowexp = reinterpret_cast<int *>(o.data + ((pp.bytes + 127) & ~(int64_t)127));
  return o;
}

void run_oz_pack(const OzPackPlan &pp, const double *src, const OzPacked &dst) {
  if (pp.ntasks == 0) return;
  prof_begin(kProfPermute);
  auto s = stream();
  GQ_CUDA(cudaMemsetAsync(dst.rowexp, 0xc0, sizeof(int) * (size_t)std::max(pp.nrows, 1), s));
  const auto *blocks = reinterpret_cast<const OzPackBlock *>(pp.blocks_dev.p);
  const auto *tasks = reinterpret_cast<const OzPackTask *>(pp.tasks_dev.p);
  oz_rowexp_kernel<<<(unsigned)pp.ntasks, 256, 0, s>>>(blocks, tasks, src, dst.rowexp);
  GQ_CUDA(cudaGetLastError());
  oz_pack_kernel<<<(unsigned)pp.ntasks, 256, 0, s>>>(blocks, tasks, src, dst.rowexp, dst.data);
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfPermute, 0.0, (double)pp.bytes * 2.0);
}

void launch_gemm_fp64tc(const ContractPlan &p, const OzPacked &A, const OzPacked &B, double *C) {
  if (p.ntiles_oz == 0) return;
  const size_t smem = sizeof(OzSmem) + 1024;
  // once per process, whichever lane launches first
  static const cudaError_t attr = cudaFuncSetAttribute(
      gemm_fp64tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  GQ_CUDA(attr);
  prof_begin(kProfGemmFp64Tc);
  gemm_fp64tc_kernel<<<(unsigned)p.ntiles_oz, oz::kThreads, smem, stream()>>>(
      p.tiles_oz.p, p.pairs_oz.p, A.data, B.data, A.rowexp, B.rowexp, C, tc_error_flag());
  GQ_CUDA(cudaGetLastError());
  prof_end(kProfGemmFp64Tc, p.flops_oz, 8.0 * (double)(p.a_elems + p.b_elems));
}

}  // namespace gq
