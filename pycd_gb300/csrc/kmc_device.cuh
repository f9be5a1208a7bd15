// Device side of the lattice KMC step: the Run.do_kmc_steps loop
// (PyCD/core.py:2787-2861) as a persistent kernel template, shared by the
// translation units that instantiate its launch shapes.
//
// Mapping.  A trajectory is owned by a group of G lanes of one warp
// (G = 1..32, a power of two); a warp holds 32/G trajectories.  Process p of
// a trajectory is (carrier c = p / S, slot s = p % S), the reference's order
// (core.py:1946-1987).  Lane g owns the contiguous processes
// p = g*MAXP + j (j < MAXP) and carrier g's site; G*MAXP >= n_carriers * S.
// The carriers' displacement and path-row values and the energy are spread
// over the lanes by slot (component k of carrier c is slot 3c + k).
//
// Arithmetic.  GB300 issues ~2 DFMA/clk/SM: one FP64 unit per SM
// sub-partition, which a warp's FP64 instruction holds for 64 cycles
// whatever its active lanes.  FP64 is the bound of this kernel, so the step
// is written to spend few FP64 instructions while keeping every rate within
// ~1e-15 relative of the reference's expression:
//   dE0   = 2q (term01 + term02) + (E_rel[n] - E_rel[o])      core.py:2004-2026
//           term01 = (phi_bg[n] - phi_bg[o]) + q (sum_c' A[n,occ_c'] - sum_c' A[o,occ_c'])
//           term02 = q (A[o,o] - A[o,n])
//   rate  = exp(c1 (lam + dE0)^2 + c0),  c1 = -1/(4 lam kT),
//           c0 = (V_ab + shift)/kT + ln vn   (= vn exp(-dG/kT), core.py:2045-2047)
//   associated as term = q (P - Q) + cq and sqrt(-c1) (lam + dE0) =
//   xa term + xb, with per-slot constants cq = (phi_bg[n] - phi_bg[o]) +
//   term02, xa = 2q sqrt(-c1) and xb = ((E_rel[n] - E_rel[o]) + lam) sqrt(-c1)
//   computed once per system: four FP64 instructions per process before the
//   exponential (the rates move by ~1e-15 relative, as any association of
//   the reference's np.dot does).
//   The carrier sums in term01 are balanced binary trees over the carrier
//   index, kept incrementally between exact refreshes.
//   k_tot and every cumulative rate are sums over a fixed balanced binary
//   tree over the process index (zero-padded to a power of two), so the
//   event stream does not depend on G or MAXP: a trajectory advanced alone
//   (the plain form) and inside a batch of thousands give identical events.
//   The event is the first process whose cumulative rate exceeds u1 k_tot
//   (core.py:2796-2800); t -= log(u2) / k_tot (core.py:2802-2803).
// exp() is a table-driven method after Tang (ACM TOMS 15(2), 1989):
// x = n ln2/4096 + r, exp(x) = 2^(n/4096) (1 + expm1(r)).  For |x| < 704 it
// runs on the integer pipe (kmc_exp, below): GB300 issues one FP64 warp
// instruction per 64 cycles per SM sub-partition, and the rates' exp() was
// the largest share of the step's FP64 instructions.  Outside that range
// the FP64 form of the same method is used.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "exp_seed.h"
#include "kmc_internal.cuh"

namespace pycd {

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// ---------------------------------------------------------------------------
// exp(x), Tang's method with a table of 2^(j/4096)
// ---------------------------------------------------------------------------
// g_exp2_tab[j] = (hi, lo) with hi + lo = 2^(j/4096) to ~2^-100 relative,
// hi = RN(2^(j/4096)) and |lo| < ulp(hi)/2.  Every translation unit that
// includes this header has its own copy; the library fills each once per
// device (exp_table_upload) before any kernel of the unit runs.
static __device__ double2 g_exp2_tab[4096];
// g_exp2_fix[j] = 2^(j/4096) 2^62 rounded to an integer (exp_fix_host)
static __device__ uint64_t g_exp2_fix[4096];

static inline cudaError_t exp_table_upload(const double2* h_tab, const uint64_t* h_fix) {
  cudaError_t e = cudaMemcpyToSymbol(g_exp2_tab, h_tab, sizeof(double2) * 4096);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_exp2_fix, h_fix, sizeof(uint64_t) * 4096);
  return e;
}

// v = 2^(j/4096) (1 + expm1(r)) in [2^-1/8192, 2^(1+1/8192)) for
// x = (4096m + j) ln2/4096 + r
__device__ __forceinline__ double exp_tang_core(double x, int& m) {
  const double kShift = 6755399441055744.0;      // 1.5 * 2^52
  // N = round(x * 4096/ln2) in the low word of t
  const double t = fma(x, PYCD_EXP_INVL, kShift);
  const int n = __double2loint(t);
  const double nd = dsub(t, kShift);
  const double r = fma(-nd, PYCD_EXP_L2, fma(-nd, PYCD_EXP_L1, x));
  const int j = n & 4095;
  m = (n - j) >> 12;
  // p = expm1(r) on |r| <= ln2/8192 to degree 3 (r^4/24 < 2.2e-18)
  const double p = fma(fma(r, 1.0 / 6.0, 0.5), dmul(r, r), r);
  const double2 e = g_exp2_tab[j];
  // 2^(j/4096) (1 + p) = hi + (lo + (hi + lo) p), where hi + lo rounds to hi
  return dadd(e.x, fma(e.x, p, e.y));
}

static __device__ __noinline__ double exp_tang_wide(double x) {
  if (!(x < 709.782712893384)) return (x != x) ? x : INFINITY;
  if (x < -745.1332191019412) return 0.0;
  int m;
  const double v = exp_tang_core(x, m);
  // scale by 2^m through the exponent field (two steps below the normal range)
  if (m >= -1021) {
    return __hiloint2double(__double2hiint(v) + (m << 20), __double2loint(v));
  }
  const double v2 = __hiloint2double(__double2hiint(v) + ((m + 64) << 20),
                                     __double2loint(v));
  return dmul(v2, 5.421010862427522e-20);  // 2^-64
}

// exp(x) for |x| < 704 with integer instructions only.
//   n:  round(|x| 4096/ln2) from the top 32 bits of x's significand times
//       4096/ln2 in 32 bits (off by at most one from the true rounding, so
//       |r| <= 0.51 ln2/4096);
//   r:  x - n ln2/4096 in 2^-88 units (x is exact there; ln2/4096 to 76
//       bits), kept in 2^-64 units; for |x| < 2^-13, n = 0 and r = x;
//   p:  expm1(r) = r + r^2/2 + r^3/6 + r^4/24 in 2^-64 units (r^5/120 is
//       below one unit);
//   v:  2^(j/4096) (1 + p) from the 62-bit table, j = n mod 4096, rounded
//       once to 53 bits and scaled by 2^floor(n/4096) in the exponent.
// v carries a relative error near 2^-61, so the result is within ~0.502
// ulp of exp(x) (correctly rounded in all but ~0.1 % of arguments).
constexpr uint64_t kExpC19 = 3098164009ull;           // 4096/ln2 2^19
constexpr uint64_t kExpL88Hi = 0xb17ull;              // ln2/4096 2^88 =
constexpr uint64_t kExpL88Lo = 0x217f7d1cf79abc9eull;  //   Hi 2^64 + Lo

__device__ __forceinline__ double exp_int(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const bool neg = (b >> 63) != 0;
  const int eb = (int)((b >> 52) & 0x7ff);
  const uint64_t mx = (b & 0xFFFFFFFFFFFFFull) | (eb ? (1ull << 52) : 0ull);
  const int ex = eb - 1023;  // |x| = mx 2^(ex - 52)
  int64_t nm = 0, rm;        // |n| and the reduced magnitude
  if (ex >= -13) {
    const int sh = 50 - ex;  // 41 ... 63 for ex in [-13, 9]
    const uint64_t pr = (mx >> 21) * kExpC19;
    nm = (int64_t)((pr + (1ull << (sh - 1))) >> sh);
    const unsigned __int128 xf = (unsigned __int128)mx << (ex + 36);
    const unsigned __int128 lf = ((unsigned __int128)kExpL88Hi << 64) | kExpL88Lo;
    const __int128 d = (__int128)(xf - (unsigned __int128)(uint64_t)nm * lf);
    rm = (int64_t)(d >> 24);
  } else {
    const int s = -ex - 12;  // >= 2
    rm = s < 64 ? (int64_t)(mx >> s) : 0;
  }
  const int64_t n = neg ? -nm : nm;
  const int64_t r = neg ? -rm : rm;
  const int64_t r2 = __mul64hi(r, r);
  const int64_t r3 = __mul64hi(r2, r);
  const int64_t r4 = __mul64hi(r2, r2);
  const int64_t p = r + (r2 >> 1) + r3 / 6 + r4 / 24;
  const uint64_t t = __ldg(reinterpret_cast<const unsigned long long*>(g_exp2_fix) +
                           (n & 4095));
  // 2^(j/4096) (1 + p) in 2^-62 units: the top bit is bit 61 or 62
  const uint64_t v = t + (uint64_t)__mul64hi((int64_t)t, p);
  const int lead = 63 - __clzll((long long)v);
  const int sh = lead - 52;
  uint64_t m53 = v >> sh;
  const uint64_t rem = v & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (m53 & 1))) ++m53;
  int e = lead - 62 + (int)(n >> 12) + 1023;
  if (m53 >> 53) {
    m53 >>= 1;
    ++e;
  }
  return __longlong_as_double((long long)(((uint64_t)e << 52) | (m53 & 0xFFFFFFFFFFFFFull)));
}

// The KMC kernels' exp: the integer form for |x| < 704 (high word below
// 0x40860000, a test on the integer pipe), the FP64 form outside.
__device__ __forceinline__ double kmc_exp(double x) {
  if ((__double2hiint(x) & 0x7fffffff) >= 0x40860000) return exp_tang_wide(x);
  return exp_int(x);
}

// a > b for doubles known to be >= +0 and not NaN: their bit patterns order
// as integers, which keeps the comparison on the integer pipe
__device__ __forceinline__ bool nonneg_gt(double a, double b) {
  return __double_as_longlong(a) > __double_as_longlong(b);
}

template <int G>
__device__ __forceinline__ double gshfl(unsigned mask, double v, int src) {
  return __shfl_sync(mask, v, src, G);
}
template <int G>
__device__ __forceinline__ int gshfl(unsigned mask, int v, int src) {
  return __shfl_sync(mask, v, src, G);
}

// Balanced-tree sums over the MAXP register values: node sums of the
// subtree rooted at each internal node, in heap order (1 = root).
template <int MAXP>
struct LocalTree {
  double node[2 * MAXP];  // node[MAXP + j] = leaf j
  __device__ __forceinline__ void build(const double* leaf) {
#pragma unroll
    for (int j = 0; j < MAXP; ++j) node[MAXP + j] = leaf[j];
#pragma unroll
    for (int i = MAXP - 1; i >= 1; --i) node[i] = dadd(node[2 * i], node[2 * i + 1]);
  }
  __device__ __forceinline__ double total() const { return node[1]; }
};

// Per-process cache of one lane: geometry, constants that change only when
// the process' own carrier moves (the slot constants cq, xa, xb, de, c0),
// and the two carrier-potential sums.  firstq marks the first of the lane's
// processes of a carrier (the one that evaluates the carrier's Q).
template <int MAXP>
struct ProcCache {
  int oldsite[MAXP], newsite[MAXP], carrier[MAXP];
  double cq[MAXP], xa[MAXP], xb[MAXP], de[MAXP], c0[MAXP];
  double P[MAXP], Q[MAXP];
  bool valid[MAXP], firstq[MAXP];
};

// Build geometry and constants of this lane's processes.  Every lane runs
// the shuffles.  Returns true when an index is out of range (no gather was
// issued with it).
template <int G, int MAXP>
__device__ __forceinline__ bool setup_processes(const PycdKmcSystem& sy,
                                                const double2* __restrict__ coef,
                                                const double2* __restrict__ slotc,
                                                int g, unsigned gmask, int occ,
                                                ProcCache<MAXP>& pc) {
  const int64_t N = sy.n_sites;
  const int S = sy.n_slots;
  const int NP = sy.n_carriers * S;
  bool bad = false;
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const int p = g * MAXP + j;
    const bool v = p < NP;
    const int c = v ? p / S : 0;
    const int o = gshfl<G>(gmask, occ, c);
    pc.valid[j] = v;
    pc.firstq[j] = v && (j == 0 || (p - 1) / S != c);
    if (v) {
      pc.carrier[j] = c;
      const int s = p - c * S;
      const int n = sy.d_nbr[(int64_t)o * S + s];
      pc.oldsite[j] = o;
      pc.newsite[j] = n;
      if (n < 0 || n >= N || o < 0 || o >= N) {
        bad = true;
        continue;
      }
      const int64_t slot = (int64_t)o * S + s;
      const double2 sa = __ldg(slotc + 2 * slot), sb = __ldg(slotc + 2 * slot + 1);
      pc.cq[j] = sa.x;
      pc.xb[j] = sa.y;
      pc.de[j] = sb.x;
      pc.xa[j] = sb.y;
      pc.c0[j] = __ldg(coef + slot).y;
    } else {
      pc.carrier[j] = -1;
      pc.oldsite[j] = 0;
      pc.newsite[j] = 0;
    }
  }
  return bad;
}

// Every carrier sum of this kernel, P = sum_c' A[n, occ_c'] and
// Q = sum_c' A[o, occ_c'], is the balanced binary tree over carrier index
// 0..31 with +0 leaves for missing carriers (which leave every node
// unchanged).  A lane forms it from 8-carrier blocks; the rebuild of a moved
// carrier forms it across lanes; both give the same doubles, and the tree
// has log2 depth instead of one dependent addition per carrier.
template <int U>
__device__ __forceinline__ double tree_reduce(double (&v)[U]) {
#pragma unroll
  for (int w = U / 2; w >= 1; w /= 2) {
#pragma unroll
    for (int i = 0; i < w; ++i) v[i] = dadd(v[2 * i], v[2 * i + 1]);
  }
  return v[0];
}

// Exact carrier sums for this lane's processes in the tree order; U = 4 for
// at most 4 carriers (one block), else 8 (up to 4 blocks, combined as
// (b0 + b1) + (b2 + b3)).  Q is evaluated once per carrier and shared by its
// processes.  Every lane runs the shuffles.
template <int G, int MAXP, int U>
__device__ __forceinline__ void fresh_sums_tree(const double* __restrict__ A, int64_t N,
                                                int NC, unsigned gmask, int occ,
                                                ProcCache<MAXP>& pc) {
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const bool doit = pc.valid[j], ownq = doit && pc.firstq[j];
    const double* rn = A + (int64_t)(doit ? pc.newsite[j] : 0) * N;
    const double* ro = A + (int64_t)(doit ? pc.oldsite[j] : 0) * N;
    double p_lo = 0.0, p_hi = 0.0, q_lo = 0.0, q_hi = 0.0;
#pragma unroll
    for (int b = 0; b < (U == 4 ? 1 : 4); ++b) {
      if (b * U < NC) {
        double vn[U], vo[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int c = b * U + u;
          const int sc = gshfl<G>(gmask, occ, min(c, NC - 1));
          vn[u] = (doit && c < NC) ? __ldg(rn + sc) : 0.0;
          vo[u] = (ownq && c < NC) ? __ldg(ro + sc) : 0.0;
        }
        const double bp = tree_reduce<U>(vn);
        const double bq = tree_reduce<U>(vo);
        if (b == 0) { p_lo = bp; q_lo = bq; }
        if (b == 1) { p_lo = dadd(p_lo, bp); q_lo = dadd(q_lo, bq); }
        if (b == 2) { p_hi = bp; q_hi = bq; }
        if (b == 3) { p_hi = dadd(p_hi, bp); q_hi = dadd(q_hi, bq); }
      }
    }
    if (doit) {
      pc.P[j] = (NC > 16) ? dadd(p_lo, p_hi) : p_lo;
      if (ownq) pc.Q[j] = (NC > 16) ? dadd(q_lo, q_hi) : q_lo;
      else if (j > 0) pc.Q[j] = pc.Q[j - 1];
    }
  }
}

template <int G, int MAXP>
__device__ __forceinline__ void fresh_sums(const PycdKmcSystem& sy, int g,
                                           unsigned gmask, int occ,
                                           ProcCache<MAXP>& pc) {
  if (sy.n_carriers <= 4)
    fresh_sums_tree<G, MAXP, 4>(sy.d_A, sy.n_sites, sy.n_carriers, gmask, occ, pc);
  else
    fresh_sums_tree<G, MAXP, 8>(sy.d_A, sy.n_sites, sy.n_carriers, gmask, occ, pc);
}

// Lane holding the sum of job u after job_sums<G, J>: the log2(J)-bit
// reversal of u (and every lane J k + that).
template <int J>
__device__ __forceinline__ int job_lane(int u) {
  int r = 0;
#pragma unroll
  for (int b = 1; b < J; b *= 2) {
    r = (r << 1) | (u & 1);
    u >>= 1;
  }
  return r;
}

// Reduce-scatter of J jobs (J = 1, 2, 4 or 8) over G lanes: v[u] is lane
// g's leaf (carrier g) of job u; lane g returns the sum of the job whose
// job_lane<J> is g mod J.  Level l adds the partial sums of lanes g and
// g ^ 2^l, i.e. the subtrees of 2^(l+1) carriers: the balanced tree over
// carriers 0..G-1, with J - 1 + log2(G/J) additions and as many shuffles
// for all J jobs.
template <int G, int J>
__device__ __forceinline__ double job_sums(unsigned gmask, int g, double (&v)[J]) {
#pragma unroll
  for (int l = 0, n = J / 2; n >= 1; ++l, n /= 2) {
    const bool up = (g >> l) & 1;
#pragma unroll
    for (int i = 0; i < n; ++i) {
      const double keep = up ? v[n + i] : v[i];
      const double send = up ? v[i] : v[n + i];
      v[i] = dadd(keep, __shfl_xor_sync(gmask, send, 1 << l, G));
    }
  }
  double y = v[0];
#pragma unroll
  for (int m = J; m < G; m *= 2) y = dadd(y, __shfl_xor_sync(gmask, y, m, G));
  return y;
}

// After carrier c_sel moved to n_sel: rebuild its S processes (slot s:
// o = n_sel, n = nbr[n_sel, s]) and their sums, as setup_processes and
// fresh_sums would give them.  Jobs i = 0..S (slot i for i < S; the carrier's
// Q, row n_sel, for i = S) are done 8 per round:
//   * lane c holds carrier c's site, so it loads A[row_i, occ_c] of every job
//     of the round at once: one memory round trip for all the rows;
//   * job_sums adds them across lanes in the tree order;
//   * lane u builds the constants of slot job u.
// Owner lanes pull the results.  Returns true on a bad index (no load is
// issued with one).  For more than 8 carriers (G = 16 or 32).
template <int G, int MAXP>
__device__ __forceinline__ bool rebuild_moved_jb(const PycdKmcSystem& sy,
                                                 const double2* __restrict__ coef,
                                                 const double2* __restrict__ slotc,
                                                 int g, unsigned gmask, int occ,
                                                 int c_sel, int n_sel,
                                                 ProcCache<MAXP>& pc) {
  constexpr int JB = 8;
  const int64_t N = sy.n_sites;
  const int S = sy.n_slots;
  const int NC = sy.n_carriers;
  const double* __restrict__ A = sy.d_A;
  bool bad = false;
  for (int i0 = 0; i0 <= S; i0 += JB) {
    int row[JB];
#pragma unroll
    for (int u = 0; u < JB; ++u) {
      int r = n_sel;
      if (i0 + u < S) {
        r = sy.d_nbr[(int64_t)n_sel * S + i0 + u];
        if (r < 0 || r >= N) { bad = true; r = n_sel; }
      }
      row[u] = r;
    }
    double v[JB];
#pragma unroll
    for (int u = 0; u < JB; ++u)
      v[u] = (g < NC && i0 + u <= S) ? __ldg(A + (int64_t)row[u] * N + occ) : 0.0;
    const double sum = job_sums<G, JB>(gmask, g, v);
    int n = n_sel;
#pragma unroll
    for (int u = 0; u < JB; ++u)
      if (g == u) n = row[u];
    double cq = 0.0, xb = 0.0, de = 0.0, xa = 0.0, c0 = 0.0;
    if (g < JB && i0 + g < S) {
      const int64_t slot = (int64_t)n_sel * S + i0 + g;
      const double2 sa = __ldg(slotc + 2 * slot), sb = __ldg(slotc + 2 * slot + 1);
      cq = sa.x;
      xb = sa.y;
      de = sb.x;
      xa = sb.y;
      c0 = __ldg(coef + slot).y;
    }
    // the carrier's Q is summed in the round that holds job S
    const int qsrc = S - i0;
    double qv = 0.0;
    if (qsrc < JB) qv = gshfl<G>(gmask, sum, job_lane<JB>(qsrc));
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const bool mine = pc.valid[j] && pc.carrier[j] == c_sel;
      const int src = g * MAXP + j - c_sel * S - i0;
      const bool take = mine && src >= 0 && src < JB;
      const int sl = take ? src : 0;
      const int nn = gshfl<G>(gmask, n, sl);
      const double v_cq = gshfl<G>(gmask, cq, sl);
      const double v_xb = gshfl<G>(gmask, xb, sl);
      const double v_de = gshfl<G>(gmask, de, sl);
      const double v_xa = gshfl<G>(gmask, xa, sl);
      const double v_c0 = gshfl<G>(gmask, c0, sl);
      const double v_p = gshfl<G>(gmask, sum, job_lane<JB>(sl));
      if (take) {
        pc.oldsite[j] = n_sel;
        pc.newsite[j] = nn;
        pc.cq[j] = v_cq;
        pc.xb[j] = v_xb;
        pc.de[j] = v_de;
        pc.xa[j] = v_xa;
        pc.c0[j] = v_c0;
        pc.P[j] = v_p;
      }
      if (mine && qsrc < JB) pc.Q[j] = qv;
    }
  }
  return bad;
}

// A row's carrier sum for at most U carriers (one block of the tree order;
// every lane runs the shuffles; lanes with act == false load nothing)
template <int G, int U>
__device__ __forceinline__ double carrier_row_tree(const double* __restrict__ rp, bool act,
                                                   int NC, unsigned gmask, int occ) {
  double v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int sc = gshfl<G>(gmask, occ, min(u, NC - 1));
    v[u] = (act && u < NC) ? __ldg(rp + sc) : 0.0;
  }
  return tree_reduce<U>(v);
}

// The moved carrier's rebuild for at most 8 carriers: job i = i0 + g on lane
// g (slot i for i < S, the carrier's Q for i = S), each job lane loading its
// own row entries; owner lanes pull the results.
template <int G, int MAXP>
__device__ __forceinline__ bool rebuild_moved_direct(const PycdKmcSystem& sy,
                                              const double2* __restrict__ coef,
                                              const double2* __restrict__ slotc,
                                              int g, unsigned gmask, int occ,
                                              int c_sel, int n_sel,
                                              ProcCache<MAXP>& pc) {
  const int64_t N = sy.n_sites;
  const int S = sy.n_slots;
  const int NC = sy.n_carriers;
  const double* __restrict__ A = sy.d_A;
  bool bad = false;
  for (int i0 = 0; i0 <= S; i0 += G) {
    const int i = i0 + g;
    const bool is_slot = i < S;
    int n = n_sel;
    double cq = 0.0, xb = 0.0, de = 0.0, xa = 0.0, c0 = 0.0;
    bool act = i <= S;
    if (is_slot) {
      const int64_t slot = (int64_t)n_sel * S + i;
      n = sy.d_nbr[slot];
      if (n < 0 || n >= N) {
        bad = true;
        act = false;
      } else {
        const double2 sa = __ldg(slotc + 2 * slot), sb = __ldg(slotc + 2 * slot + 1);
        cq = sa.x;
        xb = sa.y;
        de = sb.x;
        xa = sb.y;
        c0 = __ldg(coef + slot).y;
      }
    }
    const double* rp = A + (int64_t)(act ? n : 0) * N;
    const double sum = (NC <= 4) ? carrier_row_tree<G, 4>(rp, act, NC, gmask, occ)
                                 : carrier_row_tree<G, 8>(rp, act, NC, gmask, occ);
    // the carrier's Q is computed in the round that holds job S
    const int qsrc = S - i0;
    double qv = 0.0;
    if (qsrc < G) qv = gshfl<G>(gmask, sum, qsrc);
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const bool mine = pc.valid[j] && pc.carrier[j] == c_sel;
      const int src = g * MAXP + j - c_sel * S - i0;
      const bool take = mine && src >= 0 && src < G;
      const int sl = take ? src : 0;
      const int nn = gshfl<G>(gmask, n, sl);
      const double v_cq = gshfl<G>(gmask, cq, sl);
      const double v_xb = gshfl<G>(gmask, xb, sl);
      const double v_de = gshfl<G>(gmask, de, sl);
      const double v_xa = gshfl<G>(gmask, xa, sl);
      const double v_c0 = gshfl<G>(gmask, c0, sl);
      const double v_p = gshfl<G>(gmask, sum, sl);
      if (take) {
        pc.oldsite[j] = n_sel;
        pc.newsite[j] = nn;
        pc.cq[j] = v_cq;
        pc.xb[j] = v_xb;
        pc.de[j] = v_de;
        pc.xa[j] = v_xa;
        pc.c0[j] = v_c0;
        pc.P[j] = v_p;
      }
      if (mine && qsrc < G) pc.Q[j] = qv;
    }
  }
  return bad;
}

// At most 8 carriers: the job lanes load their rows directly (no value
// shuffles).  More: lane-parallel row loads (one round trip) and a
// reduce-scatter of the sums (G >= 16 then, since G >= n_carriers).
template <int G, int MAXP>
__device__ __forceinline__ bool rebuild_moved(const PycdKmcSystem& sy,
                                              const double2* __restrict__ coef,
                                              const double2* __restrict__ slotc,
                                              int g, unsigned gmask, int occ,
                                              int c_sel, int n_sel,
                                              ProcCache<MAXP>& pc) {
  if constexpr (G < 16) {
    return rebuild_moved_direct<G, MAXP>(sy, coef, slotc, g, gmask, occ, c_sel, n_sel, pc);
  } else {
    if (sy.n_carriers <= 8)
      return rebuild_moved_direct<G, MAXP>(sy, coef, slotc, g, gmask, occ, c_sel, n_sel, pc);
    return rebuild_moved_jb<G, MAXP>(sy, coef, slotc, g, gmask, occ, c_sel, n_sel, pc);
  }
}

// Rates of this lane's processes (core.py:1989-2050):
//   term = q (P - Q) + cq,   x' = sqrt(-c1) (lam + dE0) = xa term + xb,
//   k = exp(c0 - x'^2),      dE0 = 2q term + de (for the selected process).
template <int MAXP>
__device__ __forceinline__ void process_rates(const ProcCache<MAXP>& pc, double q,
                                              double two_q, double (&kp)[MAXP],
                                              double (&term)[MAXP]) {
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    kp[j] = 0.0;
    term[j] = 0.0;
    if (pc.valid[j]) {
      term[j] = fma(q, dsub(pc.P[j], pc.Q[j]), pc.cq[j]);
      const double xs = fma(pc.xa[j], term[j], pc.xb[j]);
      kp[j] = kmc_exp(fma(-xs, xs, pc.c0[j]));
    }
  }
}

// ---------------------------------------------------------------------------
// Residence times t -= log(u2) / k_tot (core.py:2802-2803), deferred.
//
// The exact FP64 chain is what the reference computes; only its timing
// changes.  Lane j keeps step j of a window of up to G steps; an upper bound
// of the elapsed time is accumulated in FP32 with upward rounding (integer
// bit operations and the FP32 pipe only).  While the bound stays below
// `slack` (the gap to t_guard minus the rounding of G chained subtractions),
// no grid boundary can have been reached and the exact time is not needed.
// A flush divides the pending steps in parallel, one per lane, and applies
// the G subtractions in step order: the same doubles as one division and one
// subtraction per step, at about a G-th of the FP64 divisions.
// ---------------------------------------------------------------------------
// float <= x for a double x >= 0 (integer operations only)
__device__ __forceinline__ float f32_below(double x) {
  const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
  const int e = (int)(hi >> 20) - 1023 + 127;
  if (e >= 255) return 3.4028234663852886e38f;
  if (e <= 0) return 0.0f;
  return __uint_as_float(((unsigned)e << 23) | ((hi & 0xfffffu) << 3));
}

template <int G>
struct TimeChain {
  double kt = 1.0, nlu2 = 0.0;  // this lane's pending step: k_tot, log(u2)
  int64_t col = -1;             // and its column in a per-step time log
  int npend = 0;
  float bound = 0.0f, slack = -1.0f;

  // slack = (t_guard - t) - 2^(e(t_guard) - 46) >= the rounding of up to 32
  // chained subtractions below t_guard, as a float rounded down
  // (a t_guard below 2^-975 keeps the chain exact at every step)
  __device__ __forceinline__ void reset(double t_guard, double t) {
    bound = 0.0f;
    slack = -1.0f;
    const int ef = (__double2hiint(t_guard) >> 20) & 0x7ff;
    if (ef <= 47 || ef == 0x7ff) return;
    const double m = __hiloint2double((ef - 46) << 20, 0);  // 64 ulp(t_guard)
    const double gap = dsub(dsub(t_guard, t), m);
    if (__double_as_longlong(gap) > 0) slack = f32_below(gap);
  }
  // record this step (c: its column in a per-step time log); true when the
  // exact time is needed now
  __device__ __forceinline__ bool push(int g, double ktot, double lu2, bool force,
                                       int64_t c) {
    if (g == npend) { kt = ktot; nlu2 = lu2; col = c; }
    ++npend;
    // From the exponent fields alone: -lu2 < 2^(a - 1022) (a = its biased
    // exponent; also for +0 and subnormals, a = 0) and ktot >= 2^(b - 1023)
    // for a normal ktot (b >= 1), so the double quotient RN(-lu2 / ktot) <=
    // 2^(a - b + 1); +inf for a subnormal ktot or beyond the float range,
    // 2^-126 below it.  The bound is loose by at most 4, which only brings
    // an exact flush nearer a grid boundary sooner (same values).
    const int a_exp = (__double2hiint(lu2) >> 20) & 0x7ff;  // lu2 <= 0
    const int b_exp = (__double2hiint(ktot) >> 20) & 0x7ff;
    const int k2 = a_exp - b_exp + 1;
    const float inc = (b_exp == 0 || k2 > 127)
                          ? INFINITY
                          : __int_as_float(((k2 < -126 ? -126 : k2) + 127) << 23);
    bound = __fadd_ru(bound, inc);
    return force || npend == G || !(bound < slack);
  }
  // apply the pending steps in step order; with a log row, lane j stores
  // the time after its step (the reference's value at that step) in its
  // column, when the column is inside [0, cap)
  __device__ __forceinline__ void flush(int g, unsigned gmask, double& t,
                                        double* log_row = nullptr, int64_t cap = 0) {
    const double q = (g < npend) ? ddiv(nlu2, kt) : 0.0;
    double mine = 0.0;
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const double qj = gshfl<G>(gmask, q, j);
      if (j < npend) {
        t = dsub(t, qj);
        if (g == j) mine = t;
      }
    }
    if (log_row && g < npend && col >= 0 && col < cap) log_row[col] = mine;
    npend = 0;
  }
};

// One group of G lanes advances one trajectory by up to max_steps steps.
// The trajectory's state is read through the L2 (__ldcg): in the queue
// form its previous round may have run on another SM.  t_launch: the global
// timer when the launch began for this warp (the time limit's origin), or 0
// to take it when the trajectory starts.
template <int G, int MAXP>
__device__ void advance_trajectory(const KmcArgs& a, int64_t t, int g,
                                   unsigned gmask, int64_t max_steps,
                                   uint64_t t_launch) {
  const PycdKmcState& st = a.st;
  int32_t status = __ldcg(st.d_status + t);
  if (status != PYCD_TRAJ_RUNNING) return;
  const int sys_id = st.d_sys_index ? st.d_sys_index[t] : 0;
  if (sys_id < 0 || sys_id >= a.n_systems) {
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  const KmcSysDev& sd = a.systems[sys_id];
  const PycdKmcSystem& sy = sd.pub;
  const int64_t N = sy.n_sites;
  const int S = sy.n_slots;
  const int NC = sy.n_carriers;
  const int NP = NC * S;
  const int MC = st.max_carriers;
  const double q = sy.carrier_charge;
  const double two_q = dmul(2.0, q);
  const double* __restrict__ A = sy.d_A;
  const double2* __restrict__ coef = sd.coef;
  const double2* __restrict__ slotc = sd.slotc;
  const double dt_grid = sy.time_interval;
  if (NP > G * MAXP || NC > G || (st.d_csum && 2 * NP > st.csum_stride)) {
    // launch shape or carrier-sum storage too small for this system
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  // refresh period of the carrier sums (every step without storage)
  const int64_t R = (st.d_csum && st.csum_refresh > 0) ? st.csum_refresh : 1;
  double* csum = st.d_csum ? st.d_csum + t * (int64_t)st.csum_stride : nullptr;
  const int half = st.csum_stride / 2;

  // The carriers' displacements since the last path row (slot 3c + k:
  // component k of carrier c), their path-row values and the energy (slot
  // 3 NC) are spread over the lanes: lane g holds slots g + G r, r < 4
  // (3 NC + 1 <= 4 G).  A step's additions (the moved carrier's three
  // components and the energy) then take ceil((3 NC + 1) / G) FP64
  // instructions instead of four.  Every value gets the same additions in
  // the same order; a slot a step does not touch adds +0, which is exact
  // (none of these sums is -0).
  constexpr int kSlotRegs = 4;
  const int n_disp = 3 * NC;
  const int n_regs = (n_disp + 1 + G - 1) / G;
  const int64_t sbase = t * 3 * (int64_t)MC;
  int occ = (g < NC) ? __ldcg(st.d_occ + t * MC + g) : 0;
  double dacc[kSlotRegs], racc[kSlotRegs];
  {
    const double e0 = st.d_energy ? __ldcg(st.d_energy + t) : 0.0;
#pragma unroll
    for (int r = 0; r < kSlotRegs; ++r) {
      const int j = g + G * r;
      dacc[r] = (j < n_disp) ? __ldcg(st.d_disp + sbase + j) : (j == n_disp ? e0 : 0.0);
      racc[r] = (j < n_disp) ? __ldcg(st.d_last_row + sbase + j) : 0.0;
    }
  }
  double sim_time = __ldcg(st.d_time + t);
  int64_t step = (int64_t)__ldcg((const long long*)st.d_step + t);
  const int64_t step_at_entry = step;
  int64_t start_path = (int64_t)__ldcg((const long long*)st.d_path_index + t);
  int64_t ucur = st.d_u_cursor ? (int64_t)__ldcg((const long long*)st.d_u_cursor + t) : 0;
  const int64_t step_limit = st.d_step_limit ? st.d_step_limit[t] : INT64_MAX;
  const double* ubase = a.rng.d_uniforms
                            ? a.rng.d_uniforms + (int64_t)t * a.rng.u_stride
                            : nullptr;
  const uint64_t stream_id = a.rng.d_traj_ids ? a.rng.d_traj_ids[t]
                                              : a.rng.traj_offset + (uint64_t)t;
  const int64_t n_path = sy.n_path_steps;
  const int64_t row_len = 3 * (int64_t)MC;
  double* unw = a.out.d_unwrapped
                    ? a.out.d_unwrapped +
                          (int64_t)t * (a.out.unwrapped_stride
                                            ? a.out.unwrapped_stride
                                            : n_path * row_len)
                    : nullptr;
  // below t_guard the quotient sim_time / dt cannot reach start_path + 1
  double t_guard = dmul(dmul((double)(start_path + 1), dt_grid), 1.0 - 0x1p-40);
  TimeChain<G> tc;
  tc.reset(t_guard, sim_time);
  // per-step log: the event is stored at its step, its time when the chain
  // is next made exact (the flush stores each pending step's time)
  double* tlog = a.out.d_step_time
                     ? a.out.d_step_time + (int64_t)t * a.out.step_capacity : nullptr;

  // uniforms of steps pre_base + g, prepared G at a time
  double pre_u1 = 0.0, pre_lu2 = 0.0;
  int64_t pre_base = -(int64_t)G - 1;
  // cooperative stop: lane 0 of the group checks every `poll` steps
  const bool polling = st.d_cancel != nullptr || st.time_limit_ns > 0;
  const int64_t poll = st.poll_interval > 0 ? st.poll_interval : 256;
  const uint64_t t_start = polling ? (t_launch ? t_launch : global_timer_ns()) : 0;

  // ---- process cache: geometry, constants, carrier sums ----------------
  ProcCache<MAXP> pc;
  bool bad = setup_processes<G, MAXP>(sy, coef, slotc, g, gmask, occ, pc);
  if (__ballot_sync(gmask, bad) & gmask) {
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  if (csum && (step & (R - 1)) != 0) {
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = g * MAXP + j;
      if (pc.valid[j]) { pc.P[j] = __ldcg(csum + p); pc.Q[j] = __ldcg(csum + half + p); }
    }
  } else {
    fresh_sums<G, MAXP>(sy, g, gmask, occ, pc);
  }

  for (int64_t it = 0; it < max_steps; ++it) {
    if (step >= step_limit) { status = PYCD_TRAJ_STEP_LIMIT; break; }
    if (polling && (it & (poll - 1)) == 0) {
      int32_t stop = (g == 0) ? kmc_stop_request(st, t, t_start) : 0;
      stop = gshfl<G>(gmask, stop, 0);
      if (stop) { status = stop; break; }
    }
    // ---- uniforms (core.py:2799, 2802) --------------------------------
    if (ubase && ucur + 2 > a.rng.u_count) { status = PYCD_TRAJ_NEED_UNIFORMS; break; }
    const int64_t since = step - pre_base;
    int k = (int)since;
    if (since < 0 || since >= G) {
      pre_base = step;
      k = 0;
      double u1, u2;
      if (ubase) {
        const int64_t idx = ucur + 2 * (int64_t)g;
        const bool ok = idx + 2 <= a.rng.u_count;
        u1 = ok ? ubase[idx] : 0.5;
        u2 = ok ? ubase[idx + 1] : 0.5;
      } else {
        philox_step_uniforms(a.rng.seed, stream_id, (uint64_t)(step + g), u1, u2);
      }
      pre_u1 = u1;
      pre_lu2 = log(u2);
    }
    const double u1 = gshfl<G>(gmask, pre_u1, k);
    const double lu2 = gshfl<G>(gmask, pre_lu2, k);

    // periodic exact refresh of every carrier sum (global step index)
    if (it > 0 && (step & (R - 1)) == 0) fresh_sums<G, MAXP>(sy, g, gmask, occ, pc);

    // ---- rates (core.py:1989-2050) ------------------------------------
    double kp[MAXP], term[MAXP];
    process_rates<MAXP>(pc, q, two_q, kp, term);

    // ---- selection (core.py:2796-2800) on the balanced tree ------------
    LocalTree<MAXP> lt;
    lt.build(kp);
    double lvl[6];
    lvl[0] = lt.total();
#pragma unroll
    for (int l = 0; (1 << l) < G; ++l) {
      const double other = __shfl_xor_sync(gmask, lvl[l], 1 << l, G);
      lvl[l + 1] = dadd(lvl[l], other);
    }
    int lg = 0;
    while ((1 << lg) < G) ++lg;
    const double ktot = lvl[lg];
    // ktot is a sum of exp() values: +0 <= ktot, or NaN; stall unless 0 < ktot < inf
    {
      const long long kb = __double_as_longlong(ktot);
      if (kb <= 0 || kb >= 0x7ff0000000000000LL) { status = PYCD_TRAJ_STALLED; break; }
    }
    const double thr = dmul(u1, ktot);
    double acc = 0.0;
    int base = 0;
#pragma unroll
    for (int l = 5; l >= 0; --l) {
      if (l < lg) {
        const double left = gshfl<G>(gmask, lvl[l], base);
        const double s = dadd(acc, left);
        if (!nonneg_gt(s, thr)) { acc = s; base += 1 << l; }
      }
    }
    int node = 1;
#pragma unroll
    for (int l = 0; (MAXP >> (l + 1)) > 0; ++l) {
      double left = 0.0;
#pragma unroll
      for (int i = 1; i < MAXP; ++i) {
        const double v = gshfl<G>(gmask, lt.node[2 * i], base);
        if (i == node) left = v;
      }
      const double s = dadd(acc, left);
      if (!nonneg_gt(s, thr)) { acc = s; node = 2 * node + 1; } else { node = 2 * node; }
    }
    const int jsel = node - MAXP;
    const int sel = base * MAXP + jsel;
    // only a u1 within rounding of 1 can walk into the zero padding
    if (sel >= NP) { status = PYCD_TRAJ_NO_EVENT; break; }

    // ---- residence time (core.py:2802-2804) ---------------------------
    const bool exact = tc.push(g, ktot, lu2, false, step - a.out.step_offset);
    if (exact) tc.flush(g, gmask, sim_time, tlog, a.out.step_capacity);
    int64_t end_path = start_path - 1;
    // without a flush sim_time < t_guard is guaranteed by the bound
    if (exact && !nonneg_gt(t_guard, sim_time)) {  // sim_time >= t_guard, both >= +0
      const double tq = ddiv(sim_time, dt_grid);
      end_path = (tq < 9.0e18) ? (int64_t)tq : INT64_MAX;
    }

    // broadcast the selected process' data from its owner lane
    double term_sel = 0.0, de_slot = 0.0, k_sel = 0.0;
    int n_sel = 0, o_sel = 0, c_sel = 0;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const double d = gshfl<G>(gmask, term[j], base);
      const double e = gshfl<G>(gmask, pc.de[j], base);
      const double kk = gshfl<G>(gmask, kp[j], base);
      const int ns = gshfl<G>(gmask, pc.newsite[j], base);
      const int os = gshfl<G>(gmask, pc.oldsite[j], base);
      const int cs = gshfl<G>(gmask, pc.carrier[j], base);  // sel / S, without a division
      if (j == jsel) {
        term_sel = d; de_slot = e; k_sel = kk; n_sel = ns; o_sel = os; c_sel = cs;
      }
    }
    const double de_sel = fma(two_q, term_sel, de_slot);  // dE0 of the event
    const int s_sel = sel - c_sel * S;

    // delG0 grid rows [start, end) (core.py:2807-2809)
    if (a.out.d_delg0_grid) {
      const int64_t e = end_path < n_path ? end_path : n_path;
      double* dgr = a.out.d_delg0_grid + (int64_t)t * n_path;
      for (int64_t r = start_path + g; r < e; r += G) dgr[r] = de_sel;
    }

    // ---- state update (core.py:2810-2830) -----------------------------
    {
      const double* hv = sy.d_hop + ((int64_t)o_sel * S + s_sel) * 3;
      const double h0 = __ldg(hv), h1 = __ldg(hv + 1), h2 = __ldg(hv + 2);
      if (g == c_sel) {
        occ = n_sel;
        if (a.out.d_drift) {
          double* dr = a.out.d_drift + ((int64_t)t * MC + g) * 3;
          dr[0] = dadd(__ldcg(dr), dmul(h0, k_sel));
          dr[1] = dadd(__ldcg(dr + 1), dmul(h1, k_sel));
          dr[2] = dadd(__ldcg(dr + 2), dmul(h2, k_sel));
        }
      }
      const int j0 = 3 * c_sel;
#pragma unroll
      for (int r = 0; r < kSlotRegs; ++r) {
        if (r < n_regs) {
          const int j = g + G * r;
          const double v = (j == j0) ? h0 : (j == j0 + 1) ? h1 : (j == j0 + 2) ? h2
                         : (j == n_disp) ? de_sel : 0.0;
          dacc[r] = dadd(dacc[r], v);
        }
      }
    }
    if (g == 0 && a.out.d_step_proc) {
      const int64_t col = step - a.out.step_offset;
      if (col >= 0 && col < a.out.step_capacity)
        a.out.d_step_proc[(int64_t)t * a.out.step_capacity + col] = sel;
    }
    ++step;
    if (ubase) ucur += 2;

    // ---- carrier sums after the move o_sel -> n_sel --------------------
    // other carriers' processes: add the moving charge's change; the moved
    // carrier's processes: new geometry and exact sums.  Q belongs to the
    // carrier: its first process on this lane updates it, the others copy.
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      if (pc.valid[j] && pc.carrier[j] != c_sel) {
        const int64_t rn = (int64_t)pc.newsite[j] * N, ro = (int64_t)pc.oldsite[j] * N;
        pc.P[j] = dadd(pc.P[j], dsub(__ldg(A + rn + n_sel), __ldg(A + rn + o_sel)));
        if (pc.firstq[j] || j == 0)
          pc.Q[j] = dadd(pc.Q[j], dsub(__ldg(A + ro + n_sel), __ldg(A + ro + o_sel)));
        else
          pc.Q[j] = pc.Q[j > 0 ? j - 1 : 0];
      }
    }
    bad = rebuild_moved<G, MAXP>(sy, coef, slotc, g, gmask, occ, c_sel, n_sel, pc);
    if (__ballot_sync(gmask, bad) & gmask) { status = PYCD_TRAJ_BAD_INDEX; break; }

    // ---- path-grid rows (core.py:2847-2861) ---------------------------
    if (end_path >= start_path + 1) {
      if (end_path >= n_path) end_path = n_path;
#pragma unroll
      for (int q = 0; q < kSlotRegs; ++q) {
        const int j = g + G * q;
        if (q < n_regs && j < n_disp) {
          racc[q] = dadd(racc[q], dacc[q]);
          dacc[q] = 0.0;
          if (unw)
            for (int64_t r = start_path; r < end_path; ++r) unw[r * row_len + j] = racc[q];
        }
      }
      if (a.out.d_energy_grid) {
        double en = 0.0;
#pragma unroll
        for (int q = 0; q < kSlotRegs; ++q)
          if (q == n_disp / G) en = dacc[q];
        en = gshfl<G>(gmask, en, n_disp % G);
        double* eg = a.out.d_energy_grid + (int64_t)t * n_path;
        for (int64_t r = start_path + g; r < end_path; r += G) eg[r] = en;
      }
      start_path = end_path;
      t_guard = dmul(dmul((double)(start_path + 1), dt_grid), 1.0 - 0x1p-40);
    }
    if (end_path >= n_path) { status = PYCD_TRAJ_DONE; break; }
    if (exact) tc.reset(t_guard, sim_time);
  }
  if (tc.npend > 0) tc.flush(g, gmask, sim_time, tlog, a.out.step_capacity);

  // ---- write the state back ---------------------------------------------
  // a call that took no step keeps the stored sums: an exact refresh made
  // at entry is made again at the next entry, and the stored values stay
  // the ones an uninterrupted run holds
  if (csum && step != step_at_entry) {
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = g * MAXP + j;
      if (pc.valid[j]) { csum[p] = pc.P[j]; csum[half + p] = pc.Q[j]; }
    }
  }
  if (g < NC) st.d_occ[t * MC + g] = occ;
#pragma unroll
  for (int q = 0; q < kSlotRegs; ++q) {
    const int j = g + G * q;
    if (j < n_disp) {
      st.d_disp[sbase + j] = dacc[q];
      st.d_last_row[sbase + j] = racc[q];
    } else if (j == n_disp && st.d_energy) {
      st.d_energy[t] = dacc[q];
    }
  }
  if (g == 0) {
    st.d_time[t] = sim_time;
    st.d_step[t] = step;
    st.d_path_index[t] = start_path;
    if (st.d_u_cursor) st.d_u_cursor[t] = ucur;
    st.d_status[t] = status;
  }
}

__device__ __forceinline__ int32_t ld_acquire_gpu(const int32_t* p) {
  int32_t v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(int32_t* p, int32_t v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// bounded waits of the queue form (each ~0.25 us or more)
constexpr uint32_t kQueueWaitLimit = 1u << 23;

// Queue form (PycdKmcLaunch.sched_steps > 0).  A set is the 32/G
// trajectories one warp advances together.  Items are (round, set): items
// 0 .. sets-1 are round 0 of every set; a warp that finishes round r of a
// set (its state written and fenced) queues round r + 1, so the queue holds
// only rounds whose previous round is complete, in the order they became
// ready.  Warps take items in queue order; a warp whose item is not queued
// yet waits for it (bounded; every earlier item is held by a running warp,
// so the wait ends).  Each round advances min(sched_steps, steps left).
template <int G, int MAXP>
__device__ void kmc_queue_loop(const KmcArgs& a, int lane, int sub, int g,
                               unsigned gmask) {
  constexpr int64_t gpw = 32 / G;
  const int64_t sets = a.sched_sets, total = sets * a.sched_rounds;
  int32_t* head = a.sched;
  int32_t* tail = a.sched + 1;
  int32_t* fail = a.sched + 2;
  int32_t* items = a.sched + 4;
  const bool polling = a.st.d_cancel != nullptr || a.st.time_limit_ns > 0;
  const uint64_t t_launch = polling ? global_timer_ns() : 0;
  while (true) {
    int32_t idx = 0;
    if (lane == 0) idx = atomicAdd(head, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= total) break;
    int64_t item = idx;
    if (idx >= sets) {
      // lane 0 waits and the warp takes its answer, so that every lane
      // makes the same choice
      int32_t v = 0;
      if (lane == 0) {
        for (uint32_t w = 0; w < kQueueWaitLimit; ++w) {
          v = ld_acquire_gpu(items + (idx - sets));
          if (v != 0) break;
          __nanosleep(256);
        }
        if (v == 0) atomicExch(fail, 1);  // cannot happen while every
                                          // taken item is in progress
      }
      v = __shfl_sync(0xffffffffu, v, 0);
      if (v == 0) break;
      __threadfence();
      item = (int64_t)v - 1;
    }
    const int64_t r = item / sets, set = item - r * sets;
    const int64_t left = a.max_steps - r * a.sched_steps;
    const int64_t steps = left < a.sched_steps ? left : a.sched_steps;
    const int64_t t = set * gpw + sub;
    if (t < a.st.n_traj) advance_trajectory<G, MAXP>(a, t, g, gmask, steps, t_launch);
    if (r + 1 < a.sched_rounds) {
      __threadfence();  // this lane's state writes before the round is queued
      __syncwarp();
      if (lane == 0) {
        const int32_t j = atomicAdd(tail, 1);
        st_release_gpu(items + j, (int32_t)((r + 1) * sets + set + 1));
      }
    }
  }
}

// MINB > 1 caps the registers so that MINB blocks of 256 threads fit on an
// SM: more resident warps to hide the latency of the row loads, at the price
// of spills.  The launch shape picks the variant (it does not change results).
template <int G, int MAXP, int MINB>
__global__ void __launch_bounds__(256, MINB) kmc_advance_kernel(KmcArgs a) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / G;
  const int g = lane - sub * G;
  const unsigned gmask =
      (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
  if (a.sched) {
    kmc_queue_loop<G, MAXP>(a, lane, sub, g, gmask);
    return;
  }
  const int64_t groups_per_warp = 32 / G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp * groups_per_warp + sub; t < a.st.n_traj;
       t += n_warps * groups_per_warp) {
    advance_trajectory<G, MAXP>(a, t, g, gmask, a.max_steps, 0);
  }
}

template <int G, int MAXP, int MINB>
static cudaError_t launch_g(const KmcArgs& a, int warps_per_block, int blocks,
                            cudaStream_t s) {
  kmc_advance_kernel<G, MAXP, MINB><<<blocks, warps_per_block * 32, 0, s>>>(a);
  return cudaGetLastError();
}

// (lanes per trajectory, processes per lane) instances; the register-capped
// variant exists for at most 2 processes per lane
#define PYCD_KMC_SHAPES(X)                                                   \
  X(1, 1) X(2, 1) X(4, 1) X(8, 1) X(16, 1) X(32, 1) X(2, 2) X(4, 2) X(8, 2)  \
  X(16, 2) X(32, 2) X(4, 4) X(8, 4) X(16, 4) X(32, 4) X(4, 8) X(8, 8)        \
  X(16, 8) X(32, 8)
#define PYCD_KMC_CAPPED_SHAPES(X)                                            \
  X(1, 1) X(2, 1) X(4, 1) X(8, 1) X(16, 1) X(32, 1) X(2, 2) X(4, 2) X(8, 2)  \
  X(16, 2) X(32, 2)

}  // namespace pycd
