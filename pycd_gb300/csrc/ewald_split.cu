// Split-precision Ewald contraction on tcgen05 tensor cores (sm_103a).
//
// A_fourier = F F^T with F the N x 2K FP64 feature rows
// [sqrt(w_k) cos(k.r_i), sqrt(w_k) sin(k.r_i)].  F is split as F = Fh + Fl
// (BF16 or TF32 parts) and
//     A_fourier ~= Fh Fh^T + Fh Fl^T + Fl Fh^T
// is accumulated in FP32 in tensor memory over chunks of the K dimension;
// the chunks are summed without loss (below) and the FP64 result is added
// to the real-space and self terms.
//
// Work units.  The upper triangle is covered by 256 x 256 super-tiles; a
// unit is one 128-row half of a super-tile: 128 rows x 256 columns, one
// tcgen05.mma of M = 128, N = 256 per K step.  Per 128-byte K slice a unit
// reads 2 x 16 KB of A rows and 2 x 32 KB of B rows for 12 MMAs, i.e. 64
// operand bytes per MMA cycle (128 x 128 tiles need 85).  The L2-to-SM
// operand stream is what bounds this contraction, so bytes per MMA cycle
// set its speed.  Off-diagonal super-tiles write each entry and its mirror;
// diagonal super-tiles are computed whole and each entry is written once,
// by the half that owns its row.
//
// Schedule.  One persistent CTA per SM takes units from a global counter in
// a blocked order (raster x raster super-tiles at a time, the block rows of
// the upper triangle in turn; raster from PycdEwaldDesc.split_raster).  The
// units in flight at one time then share few operand panels and advance
// along K together, so each K slice of a panel is read from DRAM about once
// and reused from L2.  Tensor memory stays allocated from unit to unit and
// the barrier phases carry over, so the next unit's first loads overlap one
// unit's last epilogue.
//
// Sum over chunks.  The tensor core's FP32 accumulation truncates, so one
// accumulation covers at most kChunkCols K columns (a chunk).  The
// epilogue adds each finished chunk x to a running FP32 sum s kept in its
// registers with Knuth's TwoSum (s + x = s' + e exactly) and writes the
// rounding error e back into the chunk's TMEM accumulator; the next chunk
// issued into that accumulator adds its products on top of e, so no error
// is dropped.  A unit's last chunk goes into the same accumulator as the
// one before it, whose fold also adds in the other accumulator's pending
// error and then stores s in that other accumulator.  The last chunk's
// epilogue reads s and x_last from tensor memory in a loop (the running
// sums in registers need a fully unrolled, instruction-cache-heavy body)
// and writes s + x_last; the next unit starts once it is done, with both
// accumulators free.
//
// A CTA-pair form (ewald_split_pair_kernel, below) computes whole
// super-tiles on 2-CTA clusters with 256-row MMAs and is used where the
// device can place such clusters; the single-CTA form is the fallback.
//
// Warp roles (320 threads):
//   warp 8      scheduler and TMA producer: takes units from the counter,
//               hands them to the other warps through a 4-entry ring, loads
//               Ah, Al (unit rows) and Bh, Bl (super-tile columns) in
//               128-byte K slices, SWIZZLE_128B, 2-stage ring of 96 KB
//   warp 9      MMA issuer: one thread issues tcgen05.mma (M=128, N=256)
//               into one of two 256-column TMEM accumulators
//   warps 0-7   epilogue: warp w reads TMEM lanes 32(w%4).. (unit rows) and
//               columns 128(w/4)..+127; TwoSum fold per chunk; FP64 writes
//               into A[i][j] and, off the diagonal, the mirror A[j][i]
//               (built from FP32 pairs with integer operations: GB300's
//               FP64 rate is far too low for a conversion per entry)
// Every mbarrier wait is bounded; on time-out the CTA records an error,
// stops issuing, waits (bounded) for its own copies and MMAs, frees its
// tensor memory and returns.
#include <atomic>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace pycd {

constexpr int kRows = 128;                  // unit rows (MMA M)
constexpr int kCols = 256;                  // unit columns, super-tile side (MMA N)
constexpr int kSlice = 128;                 // K bytes per operand row per stage
constexpr int kABytes = kRows * kSlice;     // 16 KB
constexpr int kBBytes = kCols * kSlice;     // 32 KB
constexpr int kBoxRows = 128;               // rows per TMA box
constexpr int kStageBytes = 2 * kABytes + 2 * kBBytes;  // Ah, Al, Bh, Bl: 96 KB
constexpr int kStages = 2;
constexpr int kTmemCols = 512;              // two 256-column FP32 accumulators
// K columns accumulated in FP32 per chunk: the tensor core's FP32
// accumulation truncates, so its error grows with the MMA steps per chunk
constexpr int kChunkCols = 256;
constexpr int kRing = 4;                    // units handed out ahead
constexpr int kEpiWarps = 8;
constexpr int kThreads = 32 * (kEpiWarps + 2);
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr uint32_t kWaitLimit = 1u << 24;   // bounded try_wait iterations
constexpr int kRasterDefault = 8;           // super-tiles per raster block side
// Final-phase staging: per epilogue warp a 32 x 16 tile of 8-byte values
// (4 KB), XOR-swizzled so that row-wise and column-wise accesses are free
// of bank conflicts; placed after the barrier block.
constexpr int kStageTileBytes = 32 * 16 * 8;
constexpr int kBarrierBytes = 256;
constexpr size_t kSmemBytes =
    (size_t)kStages * kStageBytes + kBarrierBytes + kEpiWarps * kStageTileBytes + 1024;

// (row ti, column tj) of super-tile t in the blocked order: block rows of
// `raster` super-tile rows in turn; within one, the diagonal block's upper
// triangle (row-major), then the blocks to its right (row-major inside each)
__device__ __forceinline__ bool super_tile(int t, int nt, int raster, int& ti, int& tj) {
  for (int r0 = 0; r0 < nt; r0 += raster) {
    const int h = min(raster, nt - r0);
    const int nd = h * (h + 1) / 2;
    if (t < nd) {
      int r = 0;
      while (t >= h - r) { t -= h - r; ++r; }
      ti = r0 + r;
      tj = r0 + r + t;
      return true;
    }
    t -= nd;
    for (int c0 = r0 + h; c0 < nt; c0 += raster) {
      const int w = min(raster, nt - c0);
      if (t < h * w) {
        ti = r0 + t / w;
        tj = c0 + t % w;
        return true;
      }
      t -= h * w;
    }
  }
  return false;
}

// TMEM accumulator of chunk c of a unit of n chunks: chunks alternate from
// accumulator 0, and the last chunk reuses the second-to-last's
__device__ __forceinline__ int chunk_acc(int c, int n) {
  return n == 1 ? 0 : ((c < n - 1 ? c : n - 2) & 1);
}
// first chunk of the unit in its accumulator (starts from zero)
__device__ __forceinline__ bool chunk_fresh(int c, int n) {
  return c == 0 || (c == 1 && n > 2);
}

struct SplitErr {
  int* flag;  // device int, set non-zero on a timed-out wait
  int* next;  // device int, zero at launch: next unit to hand out
};

// Real-space + self terms of a translation-invariant supercell: rows holds
// the first nb rows of that part (cell 0, basis sites 0..nb-1, all n
// columns) as FP32 pairs hi + lo of the FP64 values (table_split_kernel);
// entry (i, j) is rows[b_i][offset(c_j - c_i) * nb + b_j] with site
// i = c_i nb + b_i and cell offsets taken modulo (s0, s1, s2).  With
// rows == nullptr the output already holds those terms and the epilogue
// adds to it.
struct RealTable {
  const float2* rows;
  int nb, s0, s1, s2;
};

// s + e exactly for FP32 a + b (Knuth's TwoSum)
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

// The double nearest below |a + c| (same sign) for an FP32 pair with
// |c| <= ulp(a) / 2, built with integer operations only: GB300 issues one
// FP64 warp instruction per 64 cycles per SM sub-partition, too slow for
// one conversion per output entry.  a's 24 bits fill the top of the 53-bit
// significand, c is added at its place below them (bits of c under
// 2^-29 ulp(a) are dropped: a relative error under 2^-52), and a borrow
// below the leading bit is renormalised.  |a| below 2^-126 gives 0; an
// infinite or NaN a is converted as is.
__device__ __forceinline__ double pair_to_double(float a, float c) {
  const uint32_t ua = __float_as_uint(a), uc = __float_as_uint(c);
  const int ea = (int)((ua >> 23) & 0xffu);
  if (ea == 0) return 0.0;
  if (ea == 0xff) return (double)a;
  uint64_t m = (uint64_t)((ua & 0x7fffffu) | 0x800000u) << 29;
  const int ec = (int)((uc >> 23) & 0xffu);
  if (ec != 0) {
    const uint64_t mc = (uc & 0x7fffffu) | 0x800000u;
    const int sh = ec - ea + 29;  // <= 5: |c| <= ulp(a) / 2
    const uint64_t cm = sh >= 0 ? (mc << sh) : (sh > -25 ? (mc >> -sh) : 0ull);
    if ((ua ^ uc) >> 31) m -= cm; else m += cm;
  }
  int e = ea - 127 + 1023;
  if (m < (1ull << 52)) { m <<= 1; --e; }
  return __longlong_as_double((long long)(((uint64_t)(ua >> 31) << 63) |
                                          ((uint64_t)e << 52) | (m & ((1ull << 52) - 1))));
}

// (basis, cell x, y, z) of site i in the layout of RealTable
__device__ __forceinline__ void site_cell(const RealTable& rt, int64_t i, int& b, int& x,
                                          int& y, int& z) {
  const int64_t c = i / rt.nb;
  b = (int)(i - c * rt.nb);
  const int64_t yz = (int64_t)rt.s1 * rt.s2;
  x = (int)(c / yz);
  const int64_t r = c - (int64_t)x * yz;
  y = (int)(r / rt.s2);
  z = (int)(r - (int64_t)y * rt.s2);
}

// (basis, cell x, y, z) of site i (32-bit arithmetic, i < 2^31)
__device__ __forceinline__ void site_cell32(const RealTable& rt, int i, int& b, int& x, int& y,
                                            int& z) {
  const int c = i / rt.nb;
  b = i - c * rt.nb;
  const int yz = rt.s1 * rt.s2;
  x = c / yz;
  const int r = c - x * yz;
  y = r / rt.s2;
  z = r - y * rt.s2;
}

// slot of element (r, c) of a 32 x 16 staging tile
__device__ __forceinline__ int stage_slot(int r, int c) { return r * 16 + (c ^ (r & 15)); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; also gives up early once another role has aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* abort_flag) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && *abort_flag) return false;
  }
  return false;
}

// Bounded wait that ignores the abort flag (used to drain own operations).
__device__ __forceinline__ bool mbar_wait_drain(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Warp-wide bounded wait: lane 0 polls, the warp takes its answer.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity,
                                         volatile int* abort_flag) {
  bool got = false;
  if ((threadIdx.x & 31) == 0) got = mbar_wait(bar, parity, abort_flag);
  return __shfl_sync(0xffffffffu, got, 0);
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map,
                                            uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 bytes (stride-dimension byte offset 1024), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused here) = 16 B
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset = 1024 B
  d |= (uint64_t)1 << 46;             // fixed 0b001
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}

// Instruction descriptor: D = F32, A/B K-major, M = kRows, N = kCols;
// operand format 1 = BF16 (kind::f16) or 2 = TF32 (kind::tf32).
__host__ __device__ constexpr uint32_t idesc(uint32_t ab_format) {
  return (1u << 4) | (ab_format << 7) | (ab_format << 10) |
         ((uint32_t)(kCols >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);
}

template <bool TF32>
__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b,
                                     uint32_t acc) {
  if (TF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc(2)), "r"(acc));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc(1)), "r"(acc));
  }
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive TMEM columns of this thread's lane (no wait)
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
        "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]),
      "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]),
      "r"(r[14]), "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// 8 consecutive TMEM columns of this thread's lane (no wait)
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
      : "memory");
}

constexpr int kEpiCols = kCols / 2;  // columns per epilogue thread

// s += x (Knuth TwoSum) over this thread's kEpiCols columns of the chunk in
// t_acc; the rounding errors, plus with take_other the pending errors held
// in t_oth, are written back into t_acc for the next chunk to build on, and
// with save_sum the new sums go to t_oth.
__device__ __forceinline__ void fold_chunk(uint32_t t_acc, uint32_t t_oth, bool take_other,
                                           bool save_sum, float (&s)[kEpiCols]) {
#pragma unroll
  for (int g = 0; g < kEpiCols / 8; ++g) {
    uint32_t x[8], o[8];
    tmem_ld8_nowait(t_acc + (uint32_t)(g * 8), x);
    if (take_other) tmem_ld8_nowait(t_oth + (uint32_t)(g * 8), o);
    tmem_ld_wait();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float e;
      s[g * 8 + q] = two_sum(s[g * 8 + q], __uint_as_float(x[q]), e);
      if (take_other) e = __fadd_rn(e, __uint_as_float(o[q]));
      x[q] = __float_as_uint(e);
    }
    tmem_st8(t_acc + (uint32_t)(g * 8), x);
    if (save_sum) {
#pragma unroll
      for (int q = 0; q < 8; ++q) o[q] = __float_as_uint(s[g * 8 + q]);
      tmem_st8(t_oth + (uint32_t)(g * 8), o);
    }
  }
  tmem_st_wait();
}

// Last chunk of a unit: writes s + x (x in t_x, s in t_s; s = 0 for a
// one-chunk unit) plus the real-space table for this thread's row `row` and
// columns col0 .. col0 + kEpiCols - 1, and with `mirror` the transposed
// entries.  The diagonal is F_i . F_i = sum_k w_k (cos^2 + sin^2) =
// sum_k w_k exactly, taken from the FP64 weight sum.  With a real-space
// table the entry (and its mirror) is written once as table value + Fourier
// value, summed as FP32 pairs (relative error ~2^-47); otherwise it is
// added to the real and self terms already in the output.
__device__ __forceinline__ void write_unit(uint32_t t_x, uint32_t t_s, int n_chunks,
                                           int64_t row, int64_t col0, bool mirror, int64_t n,
                                           double* __restrict__ out, const RealTable& rt,
                                           double diag_value, float2* tile) {
  const int lane = threadIdx.x & 31;
  // Each 16-column group goes through this warp's staging tile: s + x is
  // formed with lane = row (the TMEM layout), the table value is added
  // and the entry stored with 16 lanes along a row (contiguous table
  // reads and row stores), and the mirror is stored with lane = row
  // again (contiguous column stores).
  const int nn = (int)n;
  const int row0 = (int)(row - lane);       // first row of this warp
  // this lane's row and, in the row-wise step, its column offset
  int rpack0 = 0, rpack1 = 0;               // (basis, x) and (y, z) of row
  if (rt.rows && row < n) {
    int rb = 0, rx = 0, ry = 0, rz = 0;
    site_cell32(rt, (int)row, rb, rx, ry, rz);
    rpack0 = (rb << 16) | rx;
    rpack1 = (ry << 16) | rz;
  }
  double* tiled = reinterpret_cast<double*>(tile);
  const int cc = lane & 15, rsub = lane >> 4;
#pragma unroll 1
  for (int g = 0; g < kEpiCols / 16; ++g) {
    uint32_t x[16], sv[16];
    tmem_ld16_nowait(t_x + (uint32_t)(g * 16), x);
    if (n_chunks >= 2) {
      tmem_ld16_nowait(t_s + (uint32_t)(g * 16), sv);
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) sv[q] = 0u;
    }
    tmem_ld_wait();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float l;
      const float h = two_sum(__uint_as_float(sv[q]), __uint_as_float(x[q]), l);
      tile[stage_slot(lane, q)] = make_float2(h, l);
    }
    __syncwarp();
    // row-wise: lanes 0-15 take row 2k, lanes 16-31 row 2k + 1
    const int gcol = (int)col0 + g * 16 + cc;
    int cbs = 0, cx = 0, cy = 0, cz = 0;
    if (rt.rows && gcol < nn) site_cell32(rt, gcol, cbs, cx, cy, cz);
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const int rr = 2 * k + rsub;
      const int grow = row0 + rr;
      const int slot = stage_slot(rr, cc);
      const float2 hl = tile[slot];
      const int p0 = __shfl_sync(0xffffffffu, rpack0, rr);
      const int p1 = __shfl_sync(0xffffffffu, rpack1, rr);
      double a = 0.0;
      if (grow < nn && gcol < nn) {
        double* at = out + (int64_t)grow * n + gcol;
        if (rt.rows) {
          int dx = cx - (p0 & 0xffff), dy = cy - (p1 >> 16), dz = cz - (p1 & 0xffff);
          if (dx < 0) dx += rt.s0;
          if (dy < 0) dy += rt.s1;
          if (dz < 0) dz += rt.s2;
          const int o = ((dx * rt.s1 + dy) * rt.s2 + dz) * rt.nb + cbs;
          const float2 t = __ldg(rt.rows + (int64_t)(p0 >> 16) * n + o);
          if (gcol == grow) {
            a = __dadd_rn(__dadd_rn((double)t.x, (double)t.y), diag_value);
          } else {
            // table + Fourier in FP32 pairs, then one conversion
            float e1, e2;
            const float w1 = two_sum(hl.x, t.x, e1);
            const float w2 = two_sum(w1, __fadd_rn(__fadd_rn(hl.y, t.y), e1), e2);
            a = pair_to_double(w2, e2);
          }
          *at = a;
        } else {
          a = gcol == grow ? diag_value : pair_to_double(hl.x, hl.y);
          *at += a;
        }
      }
      tiled[slot] = a;
    }
    __syncwarp();
    if (mirror && row < n) {
      // A[col][row]: lane = row, 32 consecutive doubles per column
#pragma unroll 4
      for (int q = 0; q < 16; ++q) {
        const int mcol = (int)col0 + g * 16 + q;
        if (mcol < nn) {
          double* at = out + (int64_t)mcol * n + row;
          const double a = tiled[stage_slot(lane, q)];
          if (rt.rows) *at = a; else *at += a;
        }
      }
    }
    __syncwarp();
  }
}

template <bool TF32>
__global__ void __launch_bounds__(kThreads, 1)
    ewald_split_kernel(const __grid_constant__ CUtensorMap map_h,
                       const __grid_constant__ CUtensorMap map_l, int64_t n,
                       int k_blocks, int chunk_blocks, int nt, int raster,
                       double* __restrict__ out, const double* __restrict__ diag_sum,
                       RealTable rt, SplitErr err) {
  const double diag_value = *diag_sum;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* acc_full = empty + kStages;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* ring_full = acc_empty + 2;
  uint64_t* ring_empty = ring_full + kRing;
  uint64_t* unit_free = ring_empty + kRing;
  uint64_t* drain = unit_free + 1;
  volatile int* ring_unit = (volatile int*)(drain + 1);
  volatile uint32_t* tmem_slot = (volatile uint32_t*)(ring_unit + kRing);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  float2* stage_tiles = (float2*)(smem + kStages * kStageBytes + kBarrierBytes);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_chunks = (k_blocks + chunk_blocks - 1) / chunk_blocks;
  const int n_units = nt * (nt + 1);  // two halves of nt (nt + 1) / 2 super-tiles

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kEpiWarps);
    }
    for (int r = 0; r < kRing; ++r) {
      mbar_init(&ring_full[r], 1);
      mbar_init(&ring_empty[r], 1 + kEpiWarps);
    }
    mbar_init(unit_free, kEpiWarps);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kProducerWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32((const void*)tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == kProducerWarp) {
    // ---------------- scheduler + TMA producer ----------------
    if (lane == 0) {
      int last_kb[kStages];
      for (int s = 0; s < kStages; ++s) last_kb[s] = -1;
      int gkb = 0;  // k-blocks loaded by this CTA over all its units
      for (int i = 0;; ++i) {
        // next unit whose rows lie inside the matrix; -1 once none is left
        int u = -1, ti = 0, tj = 0;
        for (;;) {
          const int t = atomicAdd(err.next, 1);
          if (t >= n_units) break;
          if (super_tile(t >> 1, nt, raster, ti, tj) &&
              (int64_t)ti * kCols + (int64_t)(t & 1) * kRows < n) {
            u = t;
            break;
          }
        }
        const int r = i % kRing;
        if (!mbar_wait(&ring_empty[r], ((uint32_t)(i / kRing) & 1u) ^ 1u, abort_flag)) {
          *abort_flag = 1;
          break;
        }
        ring_unit[r] = u;
        mbar_arrive(&ring_full[r]);
        if (u < 0) break;
        const int row_a = ti * kCols + (u & 1) * kRows, row_b = tj * kCols;
        bool ok = true;
        for (int kb = 0; kb < k_blocks; ++kb, ++gkb) {
          const int s = gkb % kStages;
          const uint32_t ph = (uint32_t)(gkb / kStages) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag)) { *abort_flag = 1; ok = false; break; }
          if (*abort_flag) { ok = false; break; }
          uint8_t* st = smem + s * kStageBytes;
          mbar_arrive_expect_tx(&full[s], kStageBytes);
          const int x = kb * (TF32 ? kSlice / 4 : kSlice / 2);
          // rows at or past n (edge units) are read as zeros
          tma_load_2d(st, &map_h, &full[s], x, row_a);
          tma_load_2d(st + kABytes, &map_l, &full[s], x, row_a);
          uint8_t* sb = st + 2 * kABytes;
          for (int h = 0; h < kCols / kBoxRows; ++h) {
            tma_load_2d(sb + h * kBoxRows * kSlice, &map_h, &full[s], x, row_b + h * kBoxRows);
            tma_load_2d(sb + kBBytes + h * kBoxRows * kSlice, &map_l, &full[s], x,
                        row_b + h * kBoxRows);
          }
          last_kb[s] = gkb;
        }
        if (!ok) break;
      }
      // every copy this thread issued has landed before the CTA moves on
      // (already true on the normal path, where the MMA issuer consumed them)
      for (int s = 0; s < kStages; ++s)
        if (last_kb[s] >= 0 &&
            !mbar_wait_drain(&full[s], (uint32_t)(last_kb[s] / kStages) & 1u))
          *abort_flag = 1;
    }
  } else if (warp == kMmaWarp) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const int ksteps = kSlice / 32;  // 32-byte K steps (16 BF16 / 8 TF32)
      int gkb = 0;
      int waits[2] = {0, 0};  // acc_empty completions awaited so far
      bool ok = true;
      for (int i = 0; ok; ++i) {
        const int r = i % kRing;
        if (!mbar_wait(&ring_full[r], (uint32_t)(i / kRing) & 1u, abort_flag)) {
          *abort_flag = 1;
          break;
        }
        const int u = ring_unit[r];
        mbar_arrive(&ring_empty[r]);
        if (u < 0) break;
        // both accumulators free: the previous unit's last epilogue is done
        if (i > 0 && !mbar_wait(unit_free, (uint32_t)(i - 1) & 1u, abort_flag)) {
          *abort_flag = 1;
          break;
        }
        int kb = 0;
        for (int c = 0; c < n_chunks; ++c) {
          const int b = chunk_acc(c, n_chunks);
          const bool fresh = chunk_fresh(c, n_chunks);
          if (!fresh) {
            if (!mbar_wait(&acc_empty[b], (uint32_t)waits[b] & 1u, abort_flag)) {
              *abort_flag = 1; ok = false; break;
            }
            ++waits[b];
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t d = tmem + (uint32_t)(b * kCols);
          const int kb_end = min(k_blocks, (c + 1) * chunk_blocks);
          for (int first = 1; kb < kb_end; ++kb, ++gkb, first = 0) {
            const int s = gkb % kStages;
            const uint32_t ph = (uint32_t)(gkb / kStages) & 1u;
            if (!mbar_wait(&full[s], ph, abort_flag)) { *abort_flag = 1; ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(smem + s * kStageBytes);
            const uint64_t ah = sdesc(sa), al = sdesc(sa + kABytes);
            const uint64_t bh = sdesc(sa + 2 * kABytes), bl = sdesc(sa + 2 * kABytes + kBBytes);
            for (int k = 0; k < ksteps; ++k) {
              const uint64_t o = (uint64_t)(k * 2);  // +32 bytes in the >>4 field
              const uint32_t acc0 = (fresh && first && k == 0) ? 0u : 1u;
              umma<TF32>(d, ah + o, bh + o, acc0);
              umma<TF32>(d, ah + o, bl + o, 1u);
              umma<TF32>(d, al + o, bh + o, 1u);
            }
            umma_commit(&empty[s]);  // stage free once these MMAs complete
          }
          if (!ok) break;
          umma_commit(&acc_full[b]);  // chunk finished
        }
      }
      // drain: every issued MMA has completed once this commit arrives
      umma_commit(drain);
      if (!mbar_wait_drain(drain, 0u)) *abort_flag = 1;
    }
  } else {
    // ---------------- epilogue (warps 0-7) ----------------
    const int quad = warp & 3, half = warp >> 2;
    const uint32_t lane_base =
        tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * kEpiCols);
    float s[kEpiCols];  // running sums of this thread's columns
    int seen[2] = {0, 0};  // acc_full completions consumed so far
    for (int i = 0;; ++i) {
      const int r = i % kRing;
      bool got = false;
      int u = -1;
      if (lane == 0) {
        got = mbar_wait(&ring_full[r], (uint32_t)(i / kRing) & 1u, abort_flag);
        if (got) {
          u = ring_unit[r];
          mbar_arrive(&ring_empty[r]);
        } else {
          *abort_flag = 1;
        }
      }
      got = __shfl_sync(0xffffffffu, got, 0);
      u = __shfl_sync(0xffffffffu, u, 0);
      if (!got || u < 0) break;
      int ti = 0, tj = 0;
      super_tile(u >> 1, nt, raster, ti, tj);
      const int64_t row = (int64_t)ti * kCols + (u & 1) * kRows + quad * 32 + lane;
      const int64_t col0 = (int64_t)tj * kCols + half * kEpiCols;
#pragma unroll
      for (int q = 0; q < kEpiCols; ++q) s[q] = 0.f;
      bool ok = true;
      for (int c = 0; c < n_chunks - 1; ++c) {
        const int b = chunk_acc(c, n_chunks);
        if (!warp_wait(&acc_full[b], (uint32_t)seen[b] & 1u, abort_flag)) {
          if (lane == 0) *abort_flag = 1;
          ok = false;
          break;
        }
        ++seen[b];
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // the second-to-last chunk takes the other accumulator's pending
        // error (left there by chunk n - 3) and leaves s there instead
        const bool last_fold = c == n_chunks - 2;
        fold_chunk(lane_base + (uint32_t)(b * kCols), lane_base + (uint32_t)((b ^ 1) * kCols),
                   last_fold && n_chunks >= 3, last_fold, s);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        // chunk n - 3's accumulator is not used again in this unit
        if (lane == 0 && c != n_chunks - 3) mbar_arrive(&acc_empty[b]);
      }
      if (!ok) break;
      // last chunk: the Fourier part is s + x
      const int b = chunk_acc(n_chunks - 1, n_chunks);
      if (!warp_wait(&acc_full[b], (uint32_t)seen[b] & 1u, abort_flag)) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      ++seen[b];
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      write_unit(lane_base + (uint32_t)(b * kCols), lane_base + (uint32_t)((b ^ 1) * kCols),
                 n_chunks, row, col0, ti != tj, n, out, rt, diag_value,
                 stage_tiles + warp * (kStageTileBytes / 8));
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(unit_free);
    }
  }

  // ---------------- teardown ----------------
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err.flag, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == kProducerWarp) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
}

// ---------------------------------------------------------------------------
// CTA-pair form (tcgen05 cta_group::2).  A cluster of two CTAs computes one
// 256 x 256 super-tile per unit with MMAs of M = 256 (each CTA's TMEM holds
// its 128 rows x 256 columns) and N = 256.  Each CTA loads its own 128 rows
// of A and 128 of the 256 B rows (the pair's MMA reads B from both CTAs'
// shared memory), so a 128-byte K slice costs 64 KB per SM for the same 12
// MMAs per SM as the single-CTA form's 96 KB: 43 operand bytes per MMA
// cycle instead of 64.
//   - Each CTA's TMA loads signal its own full barrier; in the second CTA
//     of the pair (rank 1) warp 9 passes each completed stage on to the
//     first CTA's full barrier, which counts its own arrival plus that one.
//     Every CTA can so wait for its own copies.
//   - One thread of the first CTA issues the MMAs and commits them to the
//     empty / acc_full barriers of both CTAs.
//   - Both CTAs' epilogue warps release accumulators and units through the
//     first CTA's acc_empty / unit_free barriers (16 arrivals each).
//   - Units are taken statically: pair p takes super-tiles p, p + P, ... of
//     the blocked order (all units cost the same).
//   - A time-out in either CTA sets the abort flag of both.
// ---------------------------------------------------------------------------
constexpr int kPairStageBytes = 4 * kABytes;  // Ah, Al, and this CTA's Bh, Bl rows: 64 KB
constexpr int kPairStages = 3;
constexpr size_t kPairSmemBytes = (size_t)kPairStages * kPairStageBytes + kBarrierBytes +
                                  kEpiWarps * kStageTileBytes + 1024;

__host__ __device__ constexpr uint32_t idesc_pair(uint32_t ab_format) {
  return (1u << 4) | (ab_format << 7) | (ab_format << 10) |
         ((uint32_t)(kCols >> 3) << 17) | ((uint32_t)((2 * kRows) >> 4) << 24);
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_index() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// address of this CTA's shared location `saddr` in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_rank(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t caddr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cl(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait with cluster-scope acquire (arrivals from the other CTA)
__device__ __forceinline__ bool mbar_wait_cl(uint64_t* bar, uint32_t parity,
                                             volatile int* abort_flag) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    if (mbar_try_wait_cl(bar, parity)) return true;
    if ((i & 1023) == 1023 && *abort_flag) return false;
  }
  return false;
}
__device__ __forceinline__ bool warp_wait_cl(uint64_t* bar, uint32_t parity,
                                            volatile int* abort_flag) {
  bool got = false;
  if ((threadIdx.x & 31) == 0) got = mbar_wait_cl(bar, parity, abort_flag);
  return __shfl_sync(0xffffffffu, got, 0);
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void st_remote_u32(uint32_t caddr, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(caddr), "r"(v) : "memory");
}

template <bool TF32>
__device__ __forceinline__ void umma_pair(uint32_t d_tmem, uint64_t a, uint64_t b,
                                          uint32_t acc) {
  if (TF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc_pair(2)), "r"(acc));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc_pair(1)), "r"(acc));
  }
}
// arrive on the barrier at this offset in both CTAs once the MMAs issued so
// far have completed
__device__ __forceinline__ void umma_commit_both(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(smem_u32(bar)),
      "h"((uint16_t)3)
      : "memory");
}
__device__ __forceinline__ void umma_commit_own(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

template <bool TF32>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 1)
    ewald_split_pair_kernel(const __grid_constant__ CUtensorMap map_h,
                            const __grid_constant__ CUtensorMap map_l, int64_t n,
                            int k_blocks, int chunk_blocks, int nt, int raster,
                            double* __restrict__ out, const double* __restrict__ diag_sum,
                            RealTable rt, SplitErr err) {
  const double diag_value = *diag_sum;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + kPairStages * kPairStageBytes);
  uint64_t* empty = full + kPairStages;
  uint64_t* acc_full = empty + kPairStages;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* unit_free = acc_empty + 2;
  uint64_t* drain = unit_free + 1;
  volatile uint32_t* tmem_slot = (volatile uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  float2* stage_tiles = (float2*)(smem + kPairStages * kPairStageBytes + kBarrierBytes);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const bool leader = rank == 0;
  const int pair = (int)cluster_index(), n_pairs = (int)cluster_count();
  const int n_chunks = (k_blocks + chunk_blocks - 1) / chunk_blocks;
  const int n_tiles = nt * (nt + 1) / 2;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kPairStages; ++s) {
      mbar_init(&full[s], leader ? 2 : 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 2 * kEpiWarps);
    }
    mbar_init(unit_free, 2 * kEpiWarps);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kProducerWarp) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32((const void*)tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  cluster_sync();  // both CTAs' barriers are initialised before any remote use
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // the first CTA's barriers and the other CTA's abort flag, cluster-wide
  const uint32_t lead_full = map_rank(smem_u32(full), 0);
  const uint32_t lead_acc_empty = map_rank(smem_u32(acc_empty), 0);
  const uint32_t lead_unit_free = map_rank(smem_u32(unit_free), 0);
  const uint32_t other_abort = map_rank(smem_u32((const void*)abort_flag), rank ^ 1u);
  auto set_abort = [&]() {
    *abort_flag = 1;
    st_remote_u32(other_abort, 1u);
  };

  if (warp == kProducerWarp) {
    // ---------------- TMA producer (both CTAs) ----------------
    if (lane == 0) {
      int last_kb[kPairStages];
      for (int s = 0; s < kPairStages; ++s) last_kb[s] = -1;
      int gkb = 0;
      bool ok = true;
      for (int t = pair; t < n_tiles && ok; t += n_pairs) {
        int ti = 0, tj = 0;
        super_tile(t, nt, raster, ti, tj);
        const int row_a = ti * kCols + (int)rank * kRows;
        const int row_b = tj * kCols + (int)rank * kRows;
        for (int kb = 0; kb < k_blocks; ++kb, ++gkb) {
          const int s = gkb % kPairStages;
          const uint32_t ph = (uint32_t)(gkb / kPairStages) & 1u;
          if (!mbar_wait_cl(&empty[s], ph ^ 1u, abort_flag)) { set_abort(); ok = false; break; }
          if (*abort_flag) { ok = false; break; }
          uint8_t* st = smem + s * kPairStageBytes;
          mbar_arrive_expect_tx(&full[s], kPairStageBytes);
          const int x = kb * (TF32 ? kSlice / 4 : kSlice / 2);
          // rows at or past n are read as zeros
          tma_load_2d(st, &map_h, &full[s], x, row_a);
          tma_load_2d(st + kABytes, &map_l, &full[s], x, row_a);
          tma_load_2d(st + 2 * kABytes, &map_h, &full[s], x, row_b);
          tma_load_2d(st + 3 * kABytes, &map_l, &full[s], x, row_b);
          last_kb[s] = gkb;
        }
      }
      // this CTA's copies have landed before it moves on (in the first CTA
      // the barrier also waits for the other CTA's hand-over)
      for (int s = 0; s < kPairStages; ++s)
        if (last_kb[s] >= 0 &&
            !mbar_wait_drain(&full[s], (uint32_t)(last_kb[s] / kPairStages) & 1u))
          set_abort();
    }
  } else if (warp == kMmaWarp && !leader) {
    // ---------------- hand-over of loaded stages (second CTA) ----------------
    if (lane == 0) {
      int gkb = 0;
      bool ok = true;
      for (int t = pair; t < n_tiles && ok; t += n_pairs) {
        for (int kb = 0; kb < k_blocks; ++kb, ++gkb) {
          const int s = gkb % kPairStages;
          if (!mbar_wait(&full[s], (uint32_t)(gkb / kPairStages) & 1u, abort_flag)) {
            set_abort(); ok = false; break;
          }
          mbar_arrive_remote(lead_full + (uint32_t)(s * 8));
        }
      }
    }
  } else if (warp == kMmaWarp) {
    // ---------------- MMA issuer (first CTA) ----------------
    if (lane == 0) {
      const int ksteps = kSlice / 32;
      int gkb = 0, ui = 0;
      int waits[2] = {0, 0};
      bool ok = true;
      for (int t = pair; t < n_tiles && ok; t += n_pairs, ++ui) {
        // both accumulators free in both CTAs: the previous unit is written
        if (ui > 0 && !mbar_wait_cl(unit_free, (uint32_t)(ui - 1) & 1u, abort_flag)) {
          set_abort();
          break;
        }
        int kb = 0;
        for (int c = 0; c < n_chunks; ++c) {
          const int b = chunk_acc(c, n_chunks);
          const bool fresh = chunk_fresh(c, n_chunks);
          if (!fresh) {
            if (!mbar_wait_cl(&acc_empty[b], (uint32_t)waits[b] & 1u, abort_flag)) {
              set_abort(); ok = false; break;
            }
            ++waits[b];
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t d = tmem + (uint32_t)(b * kCols);
          const int kb_end = min(k_blocks, (c + 1) * chunk_blocks);
          for (int first = 1; kb < kb_end; ++kb, ++gkb, first = 0) {
            const int s = gkb % kPairStages;
            const uint32_t ph = (uint32_t)(gkb / kPairStages) & 1u;
            if (!mbar_wait_cl(&full[s], ph, abort_flag)) { set_abort(); ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(smem + s * kPairStageBytes);
            const uint64_t ah = sdesc(sa), al = sdesc(sa + kABytes);
            const uint64_t bh = sdesc(sa + 2 * kABytes), bl = sdesc(sa + 3 * kABytes);
            for (int k = 0; k < ksteps; ++k) {
              const uint64_t o = (uint64_t)(k * 2);  // +32 bytes in the >>4 field
              const uint32_t acc0 = (fresh && first && k == 0) ? 0u : 1u;
              umma_pair<TF32>(d, ah + o, bh + o, acc0);
              umma_pair<TF32>(d, ah + o, bl + o, 1u);
              umma_pair<TF32>(d, al + o, bh + o, 1u);
            }
            umma_commit_both(&empty[s]);  // both CTAs' stage s free after these
          }
          if (!ok) break;
          umma_commit_both(&acc_full[b]);  // chunk finished in both CTAs
        }
      }
      umma_commit_own(drain);
      if (!mbar_wait_drain(drain, 0u)) set_abort();
    }
  } else if (warp < kEpiWarps) {
    // ---------------- epilogue (warps 0-7 of both CTAs) ----------------
    const int quad = warp & 3, half = warp >> 2;
    const uint32_t lane_base =
        tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * kEpiCols);
    float s[kEpiCols];
    int seen[2] = {0, 0};
    bool ok = true;
    for (int t = pair; t < n_tiles && ok; t += n_pairs) {
      int ti = 0, tj = 0;
      super_tile(t, nt, raster, ti, tj);
      const int64_t row = (int64_t)ti * kCols + (int64_t)rank * kRows + quad * 32 + lane;
      const int64_t col0 = (int64_t)tj * kCols + half * kEpiCols;
#pragma unroll
      for (int q = 0; q < kEpiCols; ++q) s[q] = 0.f;
      for (int c = 0; c < n_chunks - 1; ++c) {
        const int b = chunk_acc(c, n_chunks);
        if (!warp_wait_cl(&acc_full[b], (uint32_t)seen[b] & 1u, abort_flag)) {
          if (lane == 0) set_abort();
          ok = false;
          break;
        }
        ++seen[b];
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const bool last_fold = c == n_chunks - 2;
        fold_chunk(lane_base + (uint32_t)(b * kCols), lane_base + (uint32_t)((b ^ 1) * kCols),
                   last_fold && n_chunks >= 3, last_fold, s);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0 && c != n_chunks - 3) mbar_arrive_remote(lead_acc_empty + (uint32_t)(b * 8));
      }
      if (!ok) break;
      const int b = chunk_acc(n_chunks - 1, n_chunks);
      if (!warp_wait_cl(&acc_full[b], (uint32_t)seen[b] & 1u, abort_flag)) {
        if (lane == 0) set_abort();
        break;
      }
      ++seen[b];
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      write_unit(lane_base + (uint32_t)(b * kCols), lane_base + (uint32_t)((b ^ 1) * kCols),
                 n_chunks, row, col0, ti != tj, n, out, rt, diag_value,
                 stage_tiles + warp * (kStageTileBytes / 8));
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive_remote(lead_unit_free);
    }
  }

  // ---------------- teardown ----------------
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err.flag, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  cluster_sync();  // no MMA of the pair touches either CTA's memory after this
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == kProducerWarp) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
}

// The real-space table rewritten in place as FP32 pairs: entry i becomes
// (hi, lo) = (RN(v), RN(v - hi)), v - hi - lo below 2^-48 |v|.
__global__ void table_split_kernel(double* __restrict__ rows, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const double v = rows[i];
  const float hi = __double2float_rn(v);
  const float lo = __double2float_rn(__dsub_rn(v, (double)hi));
  reinterpret_cast<float2*>(rows)[i] = make_float2(hi, lo);
}

// sum_k w_k = F_i . F_i, with w_k = 2 c_k / (k^2 eps) as in the feature rows
__global__ void weight_sum_kernel(const double* __restrict__ k2,
                                  const double* __restrict__ ck, int64_t K,
                                  double eps, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t k = threadIdx.x; k < K; k += blockDim.x) s += 2.0 * ck[k] / (k2[k] * eps);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Float-float numbers (hi, lo) with |lo| <= ulp(hi)/2, about 44 bits:
// FP32 instructions only (GB300's FP32 pipe runs ~60x its FP64 pipe), with
// every rounding explicit so that no contraction changes the error terms.
__device__ __forceinline__ float2 ff_from(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(__dsub_rn(v, (double)h)));
}
// a * b: the exact product of the high parts (FMA), the cross terms, one
// renormalisation; relative error ~2^-46
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  const float e = fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.x, b.x, -p)));
  const float s = __fadd_rn(p, e);
  return make_float2(s, __fsub_rn(e, __fsub_rn(s, p)));
}
// a + b: TwoSum of the high parts plus the low parts, one renormalisation
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  float e;
  const float s = two_sum(a.x, b.x, e);
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  const float r = __fadd_rn(s, e);
  return make_float2(r, __fsub_rn(e, __fsub_rn(r, s)));
}
// complex float-float: (re.hi, re.lo, im.hi, im.lo)
__device__ __forceinline__ float4 ffc_mul(float4 a, float4 b) {
  const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
  const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
  const float2 re = ff_add(ff_mul(ar, br), ff_mul(ai, make_float2(-bi.x, -bi.y)));
  const float2 im = ff_add(ff_mul(ar, bi), ff_mul(ai, br));
  return make_float4(re.x, re.y, im.x, im.y);
}

// Feature rows F_i = [sqrt(w_k) cos(k.r_i), sqrt(w_k) sin(k.r_i)]_k,
// w_k = 2 c_k / (k^2 eps), written directly as the hi + lo operands of the
// split contraction (no FP64 copy of F), zero-padded to `ld` columns.
// As in the FP64 feature kernel, every k is m0 b0 + m1 b1 + m2 b2, so
// e^{i k.r} is the product of per-site tables e^{i m phi_d}, phi_d = b_d . r,
// built with FP64 sincos.  The BF16 split keeps ~16 bits of each feature,
// so its two complex products run in FP32 (accurate to ~2e-7, far inside
// the split); the TF32 split keeps ~22 bits and takes them in float-float
// (~44 bits, FP32 instructions only).  A block whose tables would not fit
// evaluates sincos(k . r) in FP64.
constexpr int kSfSites = 16;
constexpr int kSfThreads = 256;
constexpr int kSfSmem = 96 * 1024;

template <bool TF32>
__global__ void __launch_bounds__(kSfThreads)
split_features_direct_kernel(const double* __restrict__ cart, int64_t n,
                             const int32_t* __restrict__ kv, Mat3 recip,
                             const double* __restrict__ kc, const double* __restrict__ k2,
                             const double* __restrict__ ck, int64_t K, double eps,
                             int64_t ld, void* __restrict__ hi, void* __restrict__ lo) {
  // [kSfSites][T]: float-float complex entries (float4) for TF32, float2
  // for BF16
  extern __shared__ float4 tab[];
  __shared__ int mmax[3];
  __shared__ double phi[kSfSites][3];
  const int tid = threadIdx.x;
  const int64_t site0 = (int64_t)blockIdx.x * kSfSites;
  const int ns = (int)min((int64_t)kSfSites, n - site0);
  if (tid < 3) mmax[tid] = 0;
  if (tid < kSfSites * 3) {
    const int si = tid / 3, d = tid % 3;
    double v = 0.0;
    if (si < ns) {
      const double* r = cart + (site0 + si) * 3;
      v = fma(recip.m[d * 3 + 2], r[2], fma(recip.m[d * 3 + 1], r[1], __dmul_rn(recip.m[d * 3], r[0])));
    }
    phi[si][d] = v;
  }
  __syncthreads();
  for (int64_t k = tid; k < K; k += kSfThreads) {
    atomicMax(&mmax[0], abs(kv[k * 3]));
    atomicMax(&mmax[1], abs(kv[k * 3 + 1]));
    atomicMax(&mmax[2], abs(kv[k * 3 + 2]));
  }
  __syncthreads();
  const int M0 = mmax[0], M1 = mmax[1], M2 = mmax[2];
  const int off1 = 2 * M0 + 1, off2 = off1 + 2 * M1 + 1, T = off2 + 2 * M2 + 1;
  const int64_t esz = TF32 ? sizeof(float4) : sizeof(float2);
  const bool use_tab = (int64_t)T * kSfSites * esz <= kSfSmem;
  float2* tabf = (float2*)tab;
  if (use_tab) {
    for (int e = tid; e < kSfSites * T; e += kSfThreads) {
      const int si = e / T, j = e - si * T;
      const int d = j < off1 ? 0 : (j < off2 ? 1 : 2);
      const int m = j - (d == 0 ? M0 : (d == 1 ? off1 + M1 : off2 + M2));
      double sv, cv;
      sincos(__dmul_rn((double)m, phi[si][d]), &sv, &cv);
      if (TF32) {
        const float2 c2 = ff_from(cv), s2 = ff_from(sv);
        tab[e] = make_float4(c2.x, c2.y, s2.x, s2.y);
      } else {
        tabf[e] = make_float2((float)cv, (float)sv);
      }
    }
  }
  __syncthreads();
  for (int64_t k = tid; 2 * k < ld; k += kSfThreads) {
    const int64_t c = 2 * k;
    const bool live = k < K;
    double w = 0.0;
    int m0 = 0, m1 = 0, m2 = 0;
    if (live) {
      w = sqrt(2.0 * ck[k] / (k2[k] * eps));
      m0 = kv[k * 3];
      m1 = kv[k * 3 + 1];
      m2 = kv[k * 3 + 2];
    }
    for (int si = 0; si < ns; ++si) {
      const int64_t at = (site0 + si) * ld + c;
      if (TF32) {
        float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        if (live) {
          if (use_tab) {
            const float4* t = tab + si * T;
            z = ffc_mul(ffc_mul(t[M0 + m0], t[off1 + M1 + m1]), t[off2 + M2 + m2]);
          } else {
            const double* r = cart + (site0 + si) * 3;
            double sv, cv;
            sincos(kc[k * 3] * r[0] + kc[k * 3 + 1] * r[1] + kc[k * 3 + 2] * r[2], &sv, &cv);
            const float2 c2 = ff_from(cv), s2 = ff_from(sv);
            z = make_float4(c2.x, c2.y, s2.x, s2.y);
          }
        }
        const float2 wf = ff_from(w);
        const float2 f0 = ff_mul(wf, make_float2(z.x, z.y));
        const float2 f1 = ff_mul(wf, make_float2(z.z, z.w));
        // hi = TF32(f), lo = TF32(f - hi); f.hi - hi is exact in FP32
        uint32_t h0, h1, l0, l1;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h0) : "f"(f0.x));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h1) : "f"(f1.x));
        const float r0 = __fadd_rn(__fsub_rn(f0.x, __uint_as_float(h0)), f0.y);
        const float r1 = __fadd_rn(__fsub_rn(f1.x, __uint_as_float(h1)), f1.y);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l0) : "f"(r0));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l1) : "f"(r1));
        // c is even and ld a multiple of 32: 8-byte aligned pairs
        *(float2*)((float*)hi + at) = make_float2(__uint_as_float(h0), __uint_as_float(h1));
        *(float2*)((float*)lo + at) = make_float2(__uint_as_float(l0), __uint_as_float(l1));
      } else {
        float2 z = make_float2(0.f, 0.f);
        if (live) {
          if (use_tab) {
            const float2* t = tabf + si * T;
            z = cmulf(cmulf(t[M0 + m0], t[off1 + M1 + m1]), t[off2 + M2 + m2]);
          } else {
            const double* r = cart + (site0 + si) * 3;
            double sv, cv;
            sincos(kc[k * 3] * r[0] + kc[k * 3 + 1] * r[1] + kc[k * 3 + 2] * r[2], &sv, &cv);
            z = make_float2((float)cv, (float)sv);
          }
        }
        const float wf = (float)w;
        const float f0 = wf * z.x, f1 = wf * z.y;
        const __nv_bfloat16 h0 = __float2bfloat16_rn(f0), h1 = __float2bfloat16_rn(f1);
        const __nv_bfloat16 l0 = __float2bfloat16_rn(f0 - __bfloat162float(h0));
        const __nv_bfloat16 l1 = __float2bfloat16_rn(f1 - __bfloat162float(h1));
        // c is even and ld a multiple of 64: 4-byte aligned pairs
        *(__nv_bfloat162*)((__nv_bfloat16*)hi + at) = __halves2bfloat162(h0, h1);
        *(__nv_bfloat162*)((__nv_bfloat16*)lo + at) = __halves2bfloat162(l0, l1);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t,
                                  void*, const cuuint64_t*, const cuuint64_t*,
                                  const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int get_encode(EncodeTiledFn* fn) {
  static EncodeTiledFn cached = nullptr;
  if (!cached) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p,
                                                     12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
      set_error("cuTensorMapEncodeTiled is not available from the driver");
      return PYCD_ERR_CUDA;
    }
    cached = (EncodeTiledFn)p;
  }
  *fn = cached;
  return PYCD_OK;
}

static int64_t split_ld(int64_t kdim, bool tf32) {
  const int64_t per = tf32 ? kSlice / 4 : kSlice / 2;  // elements per K block
  return ((kdim + per - 1) / per) * per;
}

static size_t align256s(size_t b) { return (b + 255) & ~(size_t)255; }

// hi and lo operands, the time-out flag and the weight sum; the real-space
// table (when used) is laid out by ewald.cu
size_t ewald_split_workspace_bytes(const PycdEwaldDesc* d, int mode) {
  const bool tf32 = mode == PYCD_EWALD_TF32X3;
  const int64_t kdim = 2 * d->n_kvec;
  const int64_t ld = split_ld(kdim, tf32);
  const size_t es = tf32 ? 4 : 2;
  return 2 * align256s(es * (size_t)d->n_sites * (size_t)ld) + 256;
}

int ewald_build_split(const PycdEwaldDesc* d, int mode, double* out,
                      const double* kc, const double* k2, const double* ck,
                      double* real_rows, void* ws, size_t ws_bytes, cudaStream_t s) {
  const bool tf32 = mode == PYCD_EWALD_TF32X3;
  const int64_t n = d->n_sites, K = d->n_kvec, kdim = 2 * K;
  const int64_t ld = split_ld(kdim, tf32);
  const size_t es = tf32 ? 4 : 2;
  if (ws_bytes < ewald_split_workspace_bytes(d, mode)) {
    set_error("split workspace too small");
    return PYCD_ERR_WORKSPACE;
  }
  char* p = (char*)ws;
  void* hi = p;
  p += align256s(es * (size_t)n * (size_t)ld);
  void* lo = p;
  p += align256s(es * (size_t)n * (size_t)ld);
  int* flag = (int*)p;       // time-out flag
  int* next = flag + 1;      // unit counter of the persistent schedule
  double* diag_sum = (double*)(p + 8);
  PYCD_REQUIRE(((uintptr_t)hi & 15) == 0 && ((uintptr_t)lo & 15) == 0,
               "split operands must be 16-byte aligned");
  Mat3 recip;
  for (int c = 0; c < 9; ++c) recip.m[c] = d->recip[c];
  weight_sum_kernel<<<1, 256, 0, s>>>(k2, ck, K, d->dielectric, diag_sum);
  PYCD_CUDA(cudaGetLastError());
  const unsigned fblocks = (unsigned)((n + kSfSites - 1) / kSfSites);
  if (tf32) {
    PYCD_CUDA(cudaFuncSetAttribute(split_features_direct_kernel<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, kSfSmem));
    split_features_direct_kernel<true><<<fblocks, kSfThreads, kSfSmem, s>>>(
        d->d_cart, n, d->d_kvec, recip, kc, k2, ck, K, d->dielectric, ld, hi, lo);
  } else {
    PYCD_CUDA(cudaFuncSetAttribute(split_features_direct_kernel<false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, kSfSmem));
    split_features_direct_kernel<false><<<fblocks, kSfThreads, kSfSmem, s>>>(
        d->d_cart, n, d->d_kvec, recip, kc, k2, ck, K, d->dielectric, ld, hi, lo);
  }
  PYCD_CUDA(cudaGetLastError());
  PYCD_CUDA(cudaMemsetAsync(flag, 0, 2 * sizeof(int), s));
  RealTable rt{};
  if (real_rows) {
    const int64_t count = (int64_t)d->basis_sites * n;
    table_split_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(
        real_rows, count);
    PYCD_CUDA(cudaGetLastError());
    rt.rows = reinterpret_cast<const float2*>(real_rows);
    rt.nb = d->basis_sites;
    rt.s0 = d->supercell[0];
    rt.s1 = d->supercell[1];
    rt.s2 = d->supercell[2];
  }

  EncodeTiledFn enc;
  int rc = get_encode(&enc);
  if (rc) return rc;
  CUtensorMap mh, ml;
  const cuuint64_t gdim[2] = {(cuuint64_t)ld, (cuuint64_t)n};
  const cuuint64_t gstride[1] = {(cuuint64_t)(ld * es)};
  const cuuint32_t box[2] = {(cuuint32_t)(kSlice / es), (cuuint32_t)kBoxRows};
  const cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt =
      tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  CUresult r1 = enc(&mh, dt, 2, hi, gdim, gstride, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  CUresult r2 = enc(&ml, dt, 2, lo, gdim, gstride, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r1 != CUDA_SUCCESS || r2 != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d, %d)", (int)r1, (int)r2);
    return PYCD_ERR_CUDA;
  }
  const int k_blocks = (int)(ld / (kSlice / es));
  const int chunk_blocks = (int)(kChunkCols / (kSlice / es));
  const size_t smem = kSmemBytes;
  // super-tiles per side; each of the nt (nt + 1) / 2 upper-triangle
  // super-tiles is two units, taken by one persistent CTA per SM
  const int nt = (int)((n + kCols - 1) / kCols);
  const int n_units = nt * (nt + 1);
  SplitErr err{flag, next};
  const int raster = d->split_raster > 0 ? d->split_raster : kRasterDefault;
  // CTA-pair form when 2-CTA clusters of this size can be co-resident
  const int n_tiles = nt * (nt + 1) / 2;
  const void* pair_fn = tf32 ? (const void*)ewald_split_pair_kernel<true>
                             : (const void*)ewald_split_pair_kernel<false>;
  int pairs = 0;
  if (d->split_form != 2 &&
      cudaFuncSetAttribute(pair_fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kPairSmemBytes) == cudaSuccess) {
    // the count depends on the kernel, its block and its shared memory alone:
    // asked once per device and variant (stored as count + 1)
    static std::atomic<int> known[kMaxDevices][2];
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    const bool keep = dev >= 0 && dev < kMaxDevices;
    const int k = keep ? known[dev][tf32 ? 1 : 0].load(std::memory_order_relaxed) : 0;
    if (k > 0) {
      pairs = k - 1;
    } else {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * (unsigned)n_tiles);
      cfg.blockDim = dim3(kThreads);
      cfg.dynamicSmemBytes = kPairSmemBytes;
      cfg.stream = s;
      if (cudaOccupancyMaxActiveClusters(&pairs, pair_fn, &cfg) != cudaSuccess) pairs = 0;
      if (keep && pairs >= 0)
        known[dev][tf32 ? 1 : 0].store(pairs + 1, std::memory_order_relaxed);
    }
  }
  (void)cudaGetLastError();  // a device without such clusters takes single CTAs
  if (pairs > 0) {
    const unsigned grid = 2u * (unsigned)(pairs < n_tiles ? pairs : n_tiles);
    if (tf32)
      ewald_split_pair_kernel<true><<<grid, kThreads, kPairSmemBytes, s>>>(
          mh, ml, n, k_blocks, chunk_blocks, nt, raster, out, diag_sum, rt, err);
    else
      ewald_split_pair_kernel<false><<<grid, kThreads, kPairSmemBytes, s>>>(
          mh, ml, n, k_blocks, chunk_blocks, nt, raster, out, diag_sum, rt, err);
  } else {
    int dev = 0, sms = 0;
    PYCD_CUDA(cudaGetDevice(&dev));
    PYCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned ctas = (unsigned)(n_units < sms ? n_units : sms);
    if (tf32) {
      PYCD_CUDA(cudaFuncSetAttribute(ewald_split_kernel<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      ewald_split_kernel<true><<<ctas, kThreads, smem, s>>>(
          mh, ml, n, k_blocks, chunk_blocks, nt, raster, out, diag_sum, rt, err);
    } else {
      PYCD_CUDA(cudaFuncSetAttribute(ewald_split_kernel<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      ewald_split_kernel<false><<<ctas, kThreads, smem, s>>>(
          mh, ml, n, k_blocks, chunk_blocks, nt, raster, out, diag_sum, rt, err);
    }
  }
  PYCD_CUDA(cudaGetLastError());
  int h_flag = 0;
  PYCD_CUDA(cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  PYCD_CUDA(cudaStreamSynchronize(s));
  if (h_flag) {
    set_error("split-precision Ewald kernel timed out waiting on a barrier");
    return PYCD_ERR_CUDA;
  }
  return PYCD_OK;
}

}  // namespace pycd
