// Split-precision Ewald contraction on tcgen05 tensor cores (sm_103a).
//
// A_fourier = F F^T with F the N x 2K FP64 feature rows
// [sqrt(w_k) cos(k.r_i), sqrt(w_k) sin(k.r_i)].  F is split as F = Fh + Fl
// (BF16 or TF32 parts) and
//     A_fourier ~= Fh Fh^T + Fh Fl^T + Fl Fh^T
// is accumulated in FP32 in tensor memory over chunks of the K dimension;
// each finished chunk is added in FP64 to the output, which already holds
// the real-space and self terms, so the cross-chunk sum is FP64.
//
// Tile order: the grid is 1-D over blocks of kRaster x kRaster tiles, blocks
// taken along the upper triangle row by row and tiles row-major inside a
// block.  The CTAs resident at one time (one per SM) then cover about two
// blocks, i.e. ~16-24 distinct 128-row operand panels per K slice, and each
// slice of a panel is read from DRAM once and reused from L2 by the CTAs of
// its block row / column (a row-major walk over the whole triangle touches
// one new B panel per CTA).
//
// Kernel layout (one persistent CTA per SM; each walks its share of the
// 128 x 128 upper-triangle output tiles in raster order, with TMEM held and
// the barrier phases carried from tile to tile, so one tile's final
// epilogue overlaps the next tile's first loads and MMAs):
//   warp 4      TMA producer: Ah, Al (tile rows) and Bh, Bl (tile columns),
//               128-byte K slices, SWIZZLE_128B, 3-stage ring
//   warp 5      MMA issuer: one thread issues tcgen05.mma (M=128, N=128)
//               into one of two TMEM accumulators (double buffered)
//   warps 0-3   epilogue: tcgen05.ld of a finished chunk (warp w reads TMEM
//               lanes 32w..32w+31 = tile rows), FP64 add into A[i][j] and,
//               for off-diagonal tiles, into the mirror A[j][i]
// Every mbarrier wait is bounded; on time-out the CTA records an error,
// stops issuing, waits (bounded) for its own copies and MMAs, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace pycd {

constexpr int kTile = 128;               // output tile rows / columns
constexpr int kRowBytes = 128;           // one K slice per row (swizzle span)
constexpr int kTileBytes = kTile * kRowBytes;  // 16 KB
constexpr int kStages = 3;
constexpr int kStageBytes = 4 * kTileBytes;    // Ah, Al, Bh, Bl
// TMEM: two 128-column FP32 accumulators, then the hi and lo halves of the
// cross-chunk sum (128 columns each)
constexpr int kTmemCols = 512;
// K columns accumulated in FP32 per chunk: the tensor core's FP32
// accumulation truncates, so its error grows with the MMA steps per chunk
constexpr int kChunkCols = 256;
constexpr uint32_t kWaitLimit = 1u << 24;      // bounded try_wait iterations
constexpr int kRaster = 8;                     // tiles per raster block side

// (bi, bj) of CTA `cta` in the blocked upper-triangle order; false for the
// CTAs of diagonal and edge blocks that fall below the diagonal or outside
__device__ __forceinline__ bool raster_tile(int cta, int nb, int& bi, int& bj) {
  const int nbb = (nb + kRaster - 1) / kRaster;   // blocks per side
  int blk = cta / (kRaster * kRaster);
  const int loc = cta - blk * (kRaster * kRaster);
  int I = 0;
  while (I < nbb && blk >= nbb - I) { blk -= nbb - I; ++I; }
  if (I >= nbb) return false;
  const int J = I + blk;
  bi = I * kRaster + loc / kRaster;
  bj = J * kRaster + loc % kRaster;
  return bi < nb && bj < nb && bi <= bj;
}

struct SplitErr {
  int* flag;  // device int, set non-zero on a timed-out wait
};

// Real-space + self terms of a translation-invariant supercell: rows holds
// the first nb rows of that part (cell 0, basis sites 0..nb-1, all n
// columns); entry (i, j) is rows[b_i][offset(c_j - c_i) * nb + b_j] with
// site i = c_i nb + b_i and cell offsets taken modulo (s0, s1, s2).  With
// rows == nullptr the output already holds those terms and the epilogue
// adds to it.
struct RealTable {
  const double* rows;
  int nb, s0, s1, s2;
};

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

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -__dmul_rn(a.y, b.y)), fma(a.x, b.y, __dmul_rn(a.y, b.x)));
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

// Instruction descriptor: D = F32, A/B K-major, M = 128, N = 128;
// operand format 1 = BF16 (kind::f16) or 2 = TF32 (kind::tf32).
__host__ __device__ constexpr uint32_t idesc(uint32_t ab_format) {
  return (1u << 4) | (ab_format << 7) | (ab_format << 10) |
         ((uint32_t)(kTile >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
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

template <bool TF32>
__global__ void __launch_bounds__(192, 1)
    ewald_split_kernel(const __grid_constant__ CUtensorMap map_h,
                       const __grid_constant__ CUtensorMap map_l, int64_t n,
                       int k_blocks, int chunk_blocks, int nb, int n_slots,
                       double* __restrict__ out, const double* __restrict__ diag_sum,
                       RealTable rt, SplitErr err) {
  const double diag_value = *diag_sum;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* acc_full = empty + kStages;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* drain = acc_empty + 2;
  volatile uint32_t* tmem_slot = (volatile uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_chunks = (k_blocks + chunk_blocks - 1) / chunk_blocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32((const void*)tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 4) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int last_kb[kStages];
      for (int s = 0; s < kStages; ++s) last_kb[s] = -1;
      int gkb = 0;  // k-blocks loaded by this CTA over all its tiles
      bool ok = true;
      for (int slot = blockIdx.x; slot < n_slots && ok; slot += gridDim.x) {
        int bi = 0, bj = 0;
        if (!raster_tile(slot, nb, bi, bj)) continue;
        for (int kb = 0; kb < k_blocks; ++kb, ++gkb) {
          const int s = gkb % kStages;
          const uint32_t ph = (uint32_t)(gkb / kStages) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag)) { *abort_flag = 1; ok = false; break; }
          if (*abort_flag) { ok = false; break; }
          uint8_t* st = smem + s * kStageBytes;
          mbar_arrive_expect_tx(&full[s], kStageBytes);
          const int x = kb * (TF32 ? kRowBytes / 4 : kRowBytes / 2);
          tma_load_2d(st, &map_h, &full[s], x, bi * kTile);
          tma_load_2d(st + kTileBytes, &map_l, &full[s], x, bi * kTile);
          tma_load_2d(st + 2 * kTileBytes, &map_h, &full[s], x, bj * kTile);
          tma_load_2d(st + 3 * kTileBytes, &map_l, &full[s], x, bj * kTile);
          last_kb[s] = gkb;
        }
      }
      // every copy this thread issued has landed before the CTA moves on
      // (already true on the normal path, where the MMA issuer consumed them)
      for (int s = 0; s < kStages; ++s)
        if (last_kb[s] >= 0 &&
            !mbar_wait_drain(&full[s], (uint32_t)(last_kb[s] / kStages) & 1u))
          *abort_flag = 1;
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const int ksteps = TF32 ? kRowBytes / 32 : kRowBytes / 32;  // 32-byte K steps
      int gkb = 0, gc = 0;  // k-blocks and chunks of this CTA over all its tiles
      bool ok = true;
      for (int slot = blockIdx.x; slot < n_slots && ok; slot += gridDim.x) {
        int bi = 0, bj = 0;
        if (!raster_tile(slot, nb, bi, bj)) continue;
        int kb = 0;
        for (int c = 0; c < n_chunks && ok; ++c, ++gc) {
          const int b = gc & 1;
          if (!mbar_wait(&acc_empty[b], ((uint32_t)(gc >> 1) & 1u) ^ 1u, abort_flag)) {
            *abort_flag = 1; ok = false; break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t d = tmem + (uint32_t)(b * kTile);
          const int kb_end = min(k_blocks, (c + 1) * chunk_blocks);
          for (int first = 1; kb < kb_end; ++kb, ++gkb, first = 0) {
            const int s = gkb % kStages;
            const uint32_t ph = (uint32_t)(gkb / kStages) & 1u;
            if (!mbar_wait(&full[s], ph, abort_flag)) { *abort_flag = 1; ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(smem + s * kStageBytes);
            const uint64_t ah = sdesc(base), al = sdesc(base + kTileBytes);
            const uint64_t bh = sdesc(base + 2 * kTileBytes), bl = sdesc(base + 3 * kTileBytes);
            for (int k = 0; k < ksteps; ++k) {
              const uint64_t o = (uint64_t)(k * 2);  // +32 bytes in the >>4 field
              const uint32_t acc0 = (first && k == 0) ? 0u : 1u;
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
    // ---------------- epilogue (warps 0-3) ----------------
    // Cross-chunk sum per output element as an unevaluated pair hi + lo of
    // FP32 values kept in TMEM columns [256, 384) and [384, 512): each chunk
    // is added with Knuth's error-free TwoSum, the rounding error going to
    // lo, so the pair carries ~48 significant bits; the FP64 result
    // (double)hi + (double)lo is written once per tile.
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t t_hi = lane_base + 2u * kTile, t_lo = lane_base + 3u * kTile;
    bool ok = true;
    int gc = 0;  // chunks of this CTA over all its tiles
    for (int slot = blockIdx.x; slot < n_slots && ok; slot += gridDim.x) {
    int bi = 0, bj = 0;
    if (!raster_tile(slot, nb, bi, bj)) continue;
    const int64_t row = (int64_t)bi * kTile + warp * 32 + lane;
    for (int c = 0; c < n_chunks; ++c, ++gc) {
      const int b = gc & 1;
      bool got = false;
      if (lane == 0) got = mbar_wait(&acc_full[b], (uint32_t)(gc >> 1) & 1u, abort_flag);
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) {
        if (lane == 0) *abort_flag = 1;
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t t_acc = lane_base + (uint32_t)(b * kTile);
#pragma unroll 1
      for (int cb = 0; cb < kTile / 16; ++cb) {
        const uint32_t off = (uint32_t)(cb * 16);
        uint32_t a[16], h[16], l[16];
        tmem_ld16_nowait(t_acc + off, a);
        if (c > 0) {
          tmem_ld16_nowait(t_hi + off, h);
          tmem_ld16_nowait(t_lo + off, l);
        }
        tmem_ld_wait();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const float x = __uint_as_float(a[q]);
          if (c == 0) {
            h[q] = a[q];
            l[q] = 0u;
          } else {
            const float hv = __uint_as_float(h[q]);
            const float s = __fadd_rn(hv, x);
            const float bb = __fsub_rn(s, hv);
            const float e = __fadd_rn(__fsub_rn(hv, __fsub_rn(s, bb)), __fsub_rn(x, bb));
            h[q] = __float_as_uint(s);
            l[q] = __float_as_uint(__fadd_rn(__uint_as_float(l[q]), e));
          }
        }
        tmem_st16(t_hi + off, h);
        tmem_st16(t_lo + off, l);
      }
      tmem_st_wait();
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
    }
    if (ok) {
      // diagonal: F_i . F_i = sum_k w_k (cos^2 + sin^2) = sum_k w_k exactly,
      // taken from the FP64 weight sum instead of the FP32 accumulation.
      // With a real-space table the entry (and its mirror) is written once
      // as table value + Fourier value; otherwise it is added to the real
      // and self terms already in the output.
      int rb = 0, rx = 0, ry = 0, rz = 0;
      if (rt.rows && row < n) site_cell(rt, row, rb, rx, ry, rz);
      const double* trow = rt.rows ? rt.rows + (int64_t)rb * n : nullptr;
#pragma unroll 1
      for (int cb = 0; cb < kTile / 16; ++cb) {
        const uint32_t off = (uint32_t)(cb * 16);
        uint32_t h[16], l[16];
        tmem_ld16_nowait(t_hi + off, h);
        tmem_ld16_nowait(t_lo + off, l);
        tmem_ld_wait();
        const int64_t col0 = (int64_t)bj * kTile + cb * 16;
        if (row < n) {
          int cbs = 0, cx = 0, cy = 0, cz = 0;
          if (trow) site_cell(rt, col0, cbs, cx, cy, cz);
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int64_t col = col0 + q;
            if (col < n) {
              double v = (double)__uint_as_float(h[q]) + (double)__uint_as_float(l[q]);
              if (col == row) v = diag_value;
              if (trow) {
                int dx = cx - rx, dy = cy - ry, dz = cz - rz;
                if (dx < 0) dx += rt.s0;
                if (dy < 0) dy += rt.s1;
                if (dz < 0) dz += rt.s2;
                const int64_t o = (((int64_t)dx * rt.s1 + dy) * rt.s2 + dz) * rt.nb + cbs;
                const double a = __dadd_rn(__ldg(trow + o), v);
                out[row * n + col] = a;
                if (bi != bj) out[col * n + row] = a;
              } else {
                out[row * n + col] += v;
                if (bi != bj) out[col * n + row] += v;
              }
            }
            // next column's site in the layout
            if (trow && ++cbs == rt.nb) {
              cbs = 0;
              if (++cz == rt.s2) {
                cz = 0;
                if (++cy == rt.s1) { cy = 0; ++cx; }
              }
            }
          }
        }
      }
    }
  }  // tiles of this CTA
  }

  // ---------------- teardown ----------------
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err.flag, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 4) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
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

// Feature rows F_i = [sqrt(w_k) cos(k.r_i), sqrt(w_k) sin(k.r_i)]_k,
// w_k = 2 c_k / (k^2 eps), written directly as the hi + lo operands of the
// split contraction (no FP64 copy of F), zero-padded to `ld` columns.
// As in the FP64 feature kernel, every k is m0 b0 + m1 b1 + m2 b2, so
// e^{i k.r} is the product of per-site tables e^{i m phi_d}, phi_d = b_d . r,
// built with FP64 sincos.  The BF16 split keeps ~16 bits of each feature,
// so its two complex products run in FP32 (accurate to ~2e-7, far inside
// the split); the TF32 split keeps ~22 bits and takes them in FP64.  A block
// whose tables would not fit evaluates sincos(k . r) in FP64.
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
  extern __shared__ double2 tab[];  // [kSfSites][T], float2 pairs for BF16
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
  const int64_t esz = TF32 ? sizeof(double2) : sizeof(float2);
  const bool use_tab = (int64_t)T * kSfSites * esz <= kSfSmem;
  float2* tabf = (float2*)tab;
  if (use_tab) {
    for (int e = tid; e < kSfSites * T; e += kSfThreads) {
      const int si = e / T, j = e - si * T;
      const int d = j < off1 ? 0 : (j < off2 ? 1 : 2);
      const int m = j - (d == 0 ? M0 : (d == 1 ? off1 + M1 : off2 + M2));
      double sv, cv;
      sincos(__dmul_rn((double)m, phi[si][d]), &sv, &cv);
      if (TF32) tab[e] = make_double2(cv, sv);
      else tabf[e] = make_float2((float)cv, (float)sv);
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
        double2 z = make_double2(0.0, 0.0);
        if (live) {
          if (use_tab) {
            const double2* t = tab + si * T;
            z = cmul2(cmul2(t[M0 + m0], t[off1 + M1 + m1]), t[off2 + M2 + m2]);
          } else {
            const double* r = cart + (site0 + si) * 3;
            sincos(kc[k * 3] * r[0] + kc[k * 3 + 1] * r[1] + kc[k * 3 + 2] * r[2], &z.y, &z.x);
          }
        }
        const double f0 = w * z.x, f1 = w * z.y;
        uint32_t h0, h1, l0, l1;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h0) : "f"((float)f0));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h1) : "f"((float)f1));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l0) : "f"((float)(f0 - (double)__uint_as_float(h0))));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l1) : "f"((float)(f1 - (double)__uint_as_float(h1))));
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
  const int64_t per = tf32 ? kRowBytes / 4 : kRowBytes / 2;  // elements per K block
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
                      const double* real_rows, void* ws, size_t ws_bytes, cudaStream_t s) {
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
  int* flag = (int*)p;
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
  PYCD_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
  RealTable rt{};
  if (real_rows) {
    rt.rows = real_rows;
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
  const cuuint32_t box[2] = {(cuuint32_t)(kRowBytes / es), (cuuint32_t)kTile};
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
  const int k_blocks = (int)(ld / (kRowBytes / es));
  const int chunk_blocks = (int)(kChunkCols / (kRowBytes / es));
  const size_t smem = (size_t)kStages * kStageBytes + 1024 + 256;
  const int nb = (int)((n + kTile - 1) / kTile);
  const int nbb = (nb + kRaster - 1) / kRaster;
  // tile slots of the blocked raster order; one persistent CTA per SM walks
  // slots blockIdx.x, blockIdx.x + gridDim.x, ... (some slots hold no tile)
  const int n_slots = nbb * (nbb + 1) / 2 * kRaster * kRaster;
  int dev = 0, sms = 0;
  PYCD_CUDA(cudaGetDevice(&dev));
  PYCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned ctas = (unsigned)(n_slots < sms ? n_slots : sms);
  SplitErr err{flag};
  if (tf32) {
    PYCD_CUDA(cudaFuncSetAttribute(ewald_split_kernel<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ewald_split_kernel<true><<<ctas, 192, smem, s>>>(
        mh, ml, n, k_blocks, chunk_blocks, nb, n_slots, out, diag_sum, rt, err);
  } else {
    PYCD_CUDA(cudaFuncSetAttribute(ewald_split_kernel<false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ewald_split_kernel<false><<<ctas, 192, smem, s>>>(
        mh, ml, n, k_blocks, chunk_blocks, nb, n_slots, out, diag_sum, rt, err);
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
