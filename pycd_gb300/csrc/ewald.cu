// Ewald pairwise-energy array on sm_103a (System.get_precomputed_array,
// PyCD/core.py:1611-1679).
//
//   A = A_real + A_fourier + A_self
//   A_real[i,j]    = erfc(sqrt(alpha) r_ij) / (2 r_ij) / eps, r_ij < r_cut,
//                    diagonal keeps erfc(0)/2 (no division)   core.py:799-814
//   A_fourier[i,j] = 2/eps sum_k c_k cos(k . d_ij) / k^2,
//                    c_k = (2 pi / V) exp(-k^2 / (4 alpha))    core.py:853-878
//   A_self         = -sqrt(alpha/pi)/eps on the diagonal       core.py:1659
//
// FP64_DIRECT evaluates the Fourier sum per pair from the caller's
// minimum-image vectors (any pmiv, the reference's exact semantics).
// FP64_GEMM factorises cos(k.(r_j - r_i)) = cos_i cos_j + sin_i sin_j and
// contracts N x 2K feature rows with themselves (symmetric, upper tiles
// computed, lower tiles mirrored).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "common.cuh"

namespace pycd {


__device__ __forceinline__ void min_image(const Mat3& cell, const Mat3& inv,
                                          const int32_t pbc[3], double d[3]) {
  // fractional displacement, nearest image, then the 26 neighbours of that
  // image; first strictly shorter candidate wins (core.py:304-361)
  double f[3], base[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    f[c] = __dadd_rn(__dadd_rn(__dmul_rn(d[0], inv.m[0 * 3 + c]),
                               __dmul_rn(d[1], inv.m[1 * 3 + c])),
                     __dmul_rn(d[2], inv.m[2 * 3 + c]));
#pragma unroll
  for (int c = 0; c < 3; ++c) base[c] = pbc[c] ? -rint(f[c]) : 0.0;
  double best[3], bestd;
  {
    double w[3] = {f[0] + base[0], f[1] + base[1], f[2] + base[2]};
#pragma unroll
    for (int c = 0; c < 3; ++c)
      best[c] = __dadd_rn(__dadd_rn(__dmul_rn(w[0], cell.m[0 * 3 + c]),
                                    __dmul_rn(w[1], cell.m[1 * 3 + c])),
                          __dmul_rn(w[2], cell.m[2 * 3 + c]));
    bestd = __dadd_rn(__dadd_rn(__dmul_rn(best[0], best[0]),
                                __dmul_rn(best[1], best[1])),
                      __dmul_rn(best[2], best[2]));
  }
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        if (dx == 0 && dy == 0 && dz == 0) continue;
        const int ox = pbc[0] ? dx : 0, oy = pbc[1] ? dy : 0, oz = pbc[2] ? dz : 0;
        if (ox == 0 && oy == 0 && oz == 0) continue;
        double w[3] = {f[0] + (base[0] + ox), f[1] + (base[1] + oy),
                       f[2] + (base[2] + oz)};
        double cnd[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
          cnd[c] = __dadd_rn(__dadd_rn(__dmul_rn(w[0], cell.m[0 * 3 + c]),
                                       __dmul_rn(w[1], cell.m[1 * 3 + c])),
                             __dmul_rn(w[2], cell.m[2 * 3 + c]));
        const double cd = __dadd_rn(__dadd_rn(__dmul_rn(cnd[0], cnd[0]),
                                              __dmul_rn(cnd[1], cnd[1])),
                                    __dmul_rn(cnd[2], cnd[2]));
        if (cd < bestd) {
          bestd = cd;
          best[0] = cnd[0]; best[1] = cnd[1]; best[2] = cnd[2];
        }
      }
  d[0] = best[0]; d[1] = best[1]; d[2] = best[2];
}

struct EwaldGeom {
  const double* cart;
  const double* pmiv;
  Mat3 cell, inv;
  float cell_f[9], inv_f[9];  // FP32 copies for the screen (no per-pair conversions)
  int32_t pbc[3];
  int64_t n;
};

// Squared minimum-image distance in FP32 (screening only: pairs whose FP32
// distance is not clearly beyond r_cut are recomputed in FP64).
__device__ __forceinline__ float min_image_r2_f32(const EwaldGeom& g, int64_t i,
                                                  int64_t j) {
  float d[3], f[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) d[c] = (float)(g.cart[j * 3 + c] - g.cart[i * 3 + c]);
#pragma unroll
  for (int c = 0; c < 3; ++c)
    f[c] = d[0] * g.inv_f[c] + d[1] * g.inv_f[3 + c] + d[2] * g.inv_f[6 + c];
#pragma unroll
  for (int c = 0; c < 3; ++c) f[c] = g.pbc[c] ? f[c] - rintf(f[c]) : f[c];
  float best = 3.0e38f;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        const float w0 = f[0] + (g.pbc[0] ? dx : 0), w1 = f[1] + (g.pbc[1] ? dy : 0),
                    w2 = f[2] + (g.pbc[2] ? dz : 0);
        float r2 = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float v = w0 * g.cell_f[c] + w1 * g.cell_f[3 + c] + w2 * g.cell_f[6 + c];
          r2 += v * v;
        }
        best = fminf(best, r2);
      }
  return best;
}

__device__ __forceinline__ void pair_vector(const EwaldGeom& g, int64_t i,
                                            int64_t j, double d[3]) {
  if (g.pmiv) {
    const double* p = g.pmiv + (i * g.n + j) * 3;
    d[0] = p[0]; d[1] = p[1]; d[2] = p[2];
  } else {
    d[0] = __dsub_rn(g.cart[j * 3 + 0], g.cart[i * 3 + 0]);
    d[1] = __dsub_rn(g.cart[j * 3 + 1], g.cart[i * 3 + 1]);
    d[2] = __dsub_rn(g.cart[j * 3 + 2], g.cart[i * 3 + 2]);
    min_image(g.cell, g.inv, g.pbc, d);
  }
}

// Per-k constants: Cartesian k, k^2 and c_k = (2 pi / V) exp(-k^2 / 4 alpha).
__global__ void kvec_prepare_kernel(const int32_t* __restrict__ kv, int64_t K,
                                    Mat3 recip, double coeff, double alpha4,
                                    double* __restrict__ kc,
                                    double* __restrict__ k2,
                                    double* __restrict__ ck) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const double m0 = kv[k * 3], m1 = kv[k * 3 + 1], m2 = kv[k * 3 + 2];
  double v[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    v[c] = __dadd_rn(__dadd_rn(__dmul_rn(m0, recip.m[0 * 3 + c]),
                               __dmul_rn(m1, recip.m[1 * 3 + c])),
                     __dmul_rn(m2, recip.m[2 * 3 + c]));
  const double kk = fma(v[2], v[2], fma(v[1], v[1], __dmul_rn(v[0], v[0])));
  kc[k * 3] = v[0]; kc[k * 3 + 1] = v[1]; kc[k * 3 + 2] = v[2];
  k2[k] = kk;
  ck[k] = __dmul_rn(coeff, exp(__ddiv_rn(-kk, alpha4)));
}

// A_real + A_self, and (direct mode) A_fourier, one thread per pair.
template <bool DIRECT>
__global__ void __launch_bounds__(256)
    ewald_pair_kernel(EwaldGeom g, double sqrt_alpha, double r_cut,
                      double eps, double self_term,
                      const double* __restrict__ kc,
                      const double* __restrict__ k2,
                      const double* __restrict__ ck, int64_t K,
                      double* __restrict__ out) {
  extern __shared__ double sk[];  // DIRECT: staged k data, 5 doubles per k
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = blockIdx.y;
  double d[3] = {0.0, 0.0, 0.0};
  const bool valid = j < g.n;
  if (!DIRECT && valid && !g.pmiv && i != j) {
    // beyond r_cut by a margin far above FP32 error: no real-space term
    const float rc = (float)r_cut * 1.0001f;
    if (min_image_r2_f32(g, i, j) > rc * rc) {
      out[i * g.n + j] = 0.0;
      return;
    }
  }
  if (valid) pair_vector(g, i, j, d);
  double four = 0.0;
  if (DIRECT) {
    const int64_t TILE = 512;
    for (int64_t k0 = 0; k0 < K; k0 += TILE) {
      const int64_t nk = (K - k0) < TILE ? (K - k0) : TILE;
      __syncthreads();
      for (int64_t t = threadIdx.x; t < nk; t += blockDim.x) {
        sk[t * 5 + 0] = kc[(k0 + t) * 3 + 0];
        sk[t * 5 + 1] = kc[(k0 + t) * 3 + 1];
        sk[t * 5 + 2] = kc[(k0 + t) * 3 + 2];
        sk[t * 5 + 3] = ck[k0 + t];
        sk[t * 5 + 4] = k2[k0 + t];
      }
      __syncthreads();
      if (valid) {
        for (int64_t t = 0; t < nk; ++t) {
          const double th = fma(d[2], sk[t * 5 + 2],
                                fma(d[1], sk[t * 5 + 1], __dmul_rn(d[0], sk[t * 5 + 0])));
          four = __dadd_rn(four,
                           __ddiv_rn(__dmul_rn(sk[t * 5 + 3], cos(th)), sk[t * 5 + 4]));
        }
      }
    }
    four = __ddiv_rn(__dmul_rn(four, 2.0), eps);
  }
  if (!valid) return;
  const double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]),
                                            __dmul_rn(d[1], d[1])),
                                  __dmul_rn(d[2], d[2])));
  double real = 0.0;
  if (r < r_cut) {
    real = __ddiv_rn(erfc(__dmul_rn(sqrt_alpha, r)), 2.0);
    if (i != j) real = __ddiv_rn(real, r);
  }
  real = __ddiv_rn(real, eps);
  double v = __dadd_rn(real, four);
  if (i == j) v = __dadd_rn(v, self_term);
  out[i * g.n + j] = v;
}

// Feature rows F[i] = [sqrt(w_k) cos(k.r_i), sqrt(w_k) sin(k.r_i)]_k with
// w_k = 2 c_k / (k^2 eps); rows padded with zeros to `ld` columns.
//
// Every k is m0 b0 + m1 b1 + m2 b2 (integers m, reciprocal basis rows b), so
// e^{i k.r} = e^{i m0 phi0} e^{i m1 phi1} e^{i m2 phi2} with phi_d = b_d . r.
// A block owns kFeatSites sites: it finds max |m_d| over the k list, tabulates
// e^{i m phi_d} for |m| <= max |m_d| in shared memory (a few hundred sincos
// per site instead of K), and forms each feature with two complex products
// (8 FP64 instructions instead of a sincos).  When the tables would not fit
// in the block's shared memory the block evaluates sincos(k . r) directly.
constexpr int kFeatSites = 16;
constexpr int kFeatThreads = 256;
constexpr int kFeatSmem = 96 * 1024;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -__dmul_rn(a.y, b.y)), fma(a.x, b.y, __dmul_rn(a.y, b.x)));
}

__global__ void __launch_bounds__(kFeatThreads)
ewald_features_kernel(const double* __restrict__ cart, int64_t n,
                      const int32_t* __restrict__ kv, Mat3 recip,
                      const double* __restrict__ kc, const double* __restrict__ k2,
                      const double* __restrict__ ck, int64_t K, double eps, int64_t ld,
                      double* __restrict__ F) {
  extern __shared__ double2 tab[];  // [kFeatSites][T]
  __shared__ int mmax[3];
  __shared__ double phi[kFeatSites][3];
  const int tid = threadIdx.x;
  const int64_t site0 = (int64_t)blockIdx.x * kFeatSites;
  const int ns = (int)min((int64_t)kFeatSites, n - site0);
  if (tid < 3) mmax[tid] = 0;
  if (tid < kFeatSites * 3) {
    const int si = tid / 3, d = tid % 3;
    double v = 0.0;
    if (si < ns) {
      const double* r = cart + (site0 + si) * 3;
      v = fma(recip.m[d * 3 + 2], r[2], fma(recip.m[d * 3 + 1], r[1], __dmul_rn(recip.m[d * 3], r[0])));
    }
    phi[si][d] = v;
  }
  __syncthreads();
  for (int64_t k = tid; k < K; k += kFeatThreads) {
    atomicMax(&mmax[0], abs(kv[k * 3]));
    atomicMax(&mmax[1], abs(kv[k * 3 + 1]));
    atomicMax(&mmax[2], abs(kv[k * 3 + 2]));
  }
  __syncthreads();
  const int M0 = mmax[0], M1 = mmax[1], M2 = mmax[2];
  const int off1 = 2 * M0 + 1, off2 = off1 + 2 * M1 + 1, T = off2 + 2 * M2 + 1;
  const bool use_tab = (int64_t)T * kFeatSites * (int64_t)sizeof(double2) <= kFeatSmem;
  if (use_tab) {
    for (int e = tid; e < kFeatSites * T; e += kFeatThreads) {
      const int si = e / T, j = e - si * T;
      const int d = j < off1 ? 0 : (j < off2 ? 1 : 2);
      const int m = j - (d == 0 ? M0 : (d == 1 ? off1 + M1 : off2 + M2));
      double sv, cv;
      sincos(__dmul_rn((double)m, phi[si][d]), &sv, &cv);
      tab[e] = make_double2(cv, sv);
    }
  }
  __syncthreads();
  for (int64_t k = tid; 2 * k < ld; k += kFeatThreads) {
    const int64_t c = 2 * k;
    if (k >= K) {
      for (int si = 0; si < ns; ++si) {
        double* row = F + (site0 + si) * ld;
        row[c] = 0.0;
        if (c + 1 < ld) row[c + 1] = 0.0;
      }
      continue;
    }
    const double w = sqrt(2.0 * ck[k] / (k2[k] * eps));
    const int m0 = kv[k * 3], m1 = kv[k * 3 + 1], m2 = kv[k * 3 + 2];
    for (int si = 0; si < ns; ++si) {
      double2 z;
      if (use_tab) {
        const double2* t = tab + si * T;
        z = cmul(cmul(t[M0 + m0], t[off1 + M1 + m1]), t[off2 + M2 + m2]);
      } else {
        const double* r = cart + (site0 + si) * 3;
        const double th = kc[k * 3] * r[0] + kc[k * 3 + 1] * r[1] + kc[k * 3 + 2] * r[2];
        sincos(th, &z.y, &z.x);
      }
      double* row = F + (site0 + si) * ld;
      row[c] = w * z.x;
      row[c + 1] = w * z.y;
    }
  }
}

int ewald_features_launch(const double* cart, int64_t n, const int32_t* kv, Mat3 recip,
                          const double* kc, const double* k2, const double* ck, int64_t K,
                          double eps, int64_t ld, double* F, cudaStream_t s) {
  // per device and cheap: set on every launch
  PYCD_CUDA(cudaFuncSetAttribute(ewald_features_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, kFeatSmem));
  const unsigned blocks = (unsigned)((n + kFeatSites - 1) / kFeatSites);
  ewald_features_kernel<<<blocks, kFeatThreads, kFeatSmem, s>>>(cart, n, kv, recip, kc, k2,
                                                                ck, K, eps, ld, F);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "ewald_features_kernel", __FILE__, __LINE__);
  return PYCD_OK;
}

// out += F F^T for the upper block tiles; each off-diagonal tile is also
// written transposed.  BM = BN = 64, BK = 16, 256 threads, 4 x 4 per thread.
constexpr int GB = 64, GK = 16;
__global__ void __launch_bounds__(256)
    syrk_fp64_kernel(const double* __restrict__ F, int64_t n, int64_t ld,
                     int64_t kdim, double* __restrict__ out) {
  __shared__ double As[GK][GB + 1];
  __shared__ double Bs[GK][GB + 1];
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bi > bj) return;  // lower tiles are written by their mirror
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4] = {};
  const int64_t row0 = (int64_t)bi * GB, col0 = (int64_t)bj * GB;
  for (int64_t k0 = 0; k0 < kdim; k0 += GK) {
    // 64 rows x 16 cols per operand: 1024 values, 4 per thread
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const int idx = threadIdx.x + l * 256;
      const int r = idx >> 4, c = idx & 15;
      const int64_t ga = row0 + r, gb = col0 + r, gk = k0 + c;
      As[c][r] = (ga < n && gk < kdim) ? F[ga * ld + gk] : 0.0;
      Bs[c][r] = (gb < n && gk < kdim) ? F[gb * ld + gk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty * 4 + u];
        b[u] = Bs[kk][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int64_t r = row0 + ty * 4 + u, c = col0 + tx * 4 + v;
      if (r < n && c < n) {
        out[r * n + c] += acc[u][v];
        if (bi != bj) out[c * n + r] += acc[u][v];
      }
    }
}

// phi = A q (one warp per row) and, optionally, E = q . phi.
__global__ void gemv_rows_kernel(const double* __restrict__ A, int64_t n,
                                 const double* __restrict__ q,
                                 double* __restrict__ phi) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double s = 0.0;
  for (int64_t c = lane; c < n; c += 32) s = fma(A[row * n + c], q[c], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) phi[row] = s;
}

// phi[i] = sum_j q_j A[idx_j][i] for a few charged sites idx_j: the array is
// symmetric, so the columns A[:, idx_j] are read as rows (coalesced);
// charges are added in the given order.
__global__ void sparse_potential_kernel(const double* __restrict__ A, int64_t n,
                                        const int32_t* __restrict__ idx,
                                        const double* __restrict__ q, int32_t m,
                                        double* __restrict__ phi) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int32_t j = 0; j < m; ++j) s = fma(q[j], A[(int64_t)idx[j] * n + i], s);
  phi[i] = s;
}

int potential_sparse(const double* A, int64_t n, const int32_t* idx,
                     const double* q, int32_t m, double* phi, cudaStream_t s) {
  PYCD_REQUIRE(A && phi && n > 0 && m >= 0 && (m == 0 || (idx && q)),
               "potential_sparse: bad arguments");
  sparse_potential_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A, n, idx, q, m, phi);
  PYCD_CUDA(cudaGetLastError());
  return PYCD_OK;
}

__global__ void dot_kernel(const double* __restrict__ a,
                           const double* __restrict__ b, int64_t n,
                           double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(a[i], b[i], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *out = s;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct EwaldWs {
  double* kc;
  double* k2;
  double* ck;
  double* F;
  int64_t ld;
  double* real_rows;  // split modes on a translation-invariant supercell
};

static int64_t feature_ld(int64_t K) { return ((2 * K + GK - 1) / GK) * GK; }

// Split modes of a whole array on a described supercell take the real-space
// and self terms from the first basis_sites rows (RealTable in
// ewald_split.cu) instead of a pass over all N^2 pairs.
static bool use_real_table(const PycdEwaldDesc* d, int mode) {
  const int parts = d->parts ? d->parts : PYCD_EWALD_PART_ALL;
  return (mode == PYCD_EWALD_BF16X3 || mode == PYCD_EWALD_TF32X3) &&
         parts == PYCD_EWALD_PART_ALL && d->basis_sites > 0 && d->n_kvec > 0;
}

static size_t ewald_ws_layout(const PycdEwaldDesc* d, int mode, EwaldWs* ws,
                              char* base) {
  const int64_t K = d->n_kvec, n = d->n_sites;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  EwaldWs w{};
  w.kc = (double*)take(sizeof(double) * 3 * (K > 0 ? K : 1));
  w.k2 = (double*)take(sizeof(double) * (K > 0 ? K : 1));
  w.ck = (double*)take(sizeof(double) * (K > 0 ? K : 1));
  if (mode == PYCD_EWALD_FP64_GEMM) {
    w.ld = feature_ld(K);
    w.F = (double*)take(sizeof(double) * (size_t)n * (size_t)w.ld);
  }
  if (use_real_table(d, mode))
    w.real_rows = (double*)take(sizeof(double) * (size_t)d->basis_sites * (size_t)n);
  if (ws) *ws = w;
  return off;
}

int ewald_validate(const PycdEwaldDesc* d, int mode) {
  PYCD_REQUIRE(d != nullptr, "desc is NULL");
  PYCD_REQUIRE(d->n_sites > 0, "n_sites must be positive");
  PYCD_REQUIRE(d->n_kvec >= 0, "n_kvec must be >= 0");
  PYCD_REQUIRE(d->n_kvec == 0 || d->d_kvec != nullptr, "d_kvec is NULL");
  PYCD_REQUIRE(d->d_cart != nullptr || d->d_pmiv != nullptr,
               "need d_cart or d_pmiv");
  PYCD_REQUIRE(d->parts >= 0 && d->parts <= PYCD_EWALD_PART_ALL,
               "parts must be a mask of PYCD_EWALD_PART_* (got %d)", d->parts);
  PYCD_REQUIRE(d->alpha > 0.0 && d->volume > 0.0 && d->dielectric != 0.0,
               "alpha, volume must be > 0 and dielectric != 0");
  PYCD_REQUIRE(mode >= PYCD_EWALD_FP64_DIRECT && mode <= PYCD_EWALD_TF32X3,
               "unknown Ewald mode %d", mode);
  if (mode != PYCD_EWALD_FP64_DIRECT)
    PYCD_REQUIRE(d->d_cart != nullptr, "feature modes need d_cart");
  PYCD_REQUIRE(d->n_sites <= 65535, "n_sites above 65535 is not supported");
  PYCD_REQUIRE(d->basis_sites >= 0, "basis_sites must be >= 0");
  PYCD_REQUIRE(d->split_form >= 0 && d->split_form <= 2,
               "split_form must be 0 (default), 1 (CTA pairs) or 2 (single CTAs)");
  PYCD_REQUIRE(d->split_raster >= 0 && d->split_raster <= 64,
               "split_raster must be 0 (default) or 1-64");
  if (d->basis_sites > 0) {
    PYCD_REQUIRE(d->supercell[0] > 0 && d->supercell[1] > 0 && d->supercell[2] > 0 &&
                     (int64_t)d->basis_sites * d->supercell[0] * d->supercell[1] *
                             d->supercell[2] == d->n_sites,
                 "basis_sites x supercell cells must equal n_sites");
  }
  return PYCD_OK;
}

size_t ewald_workspace_bytes(const PycdEwaldDesc* d, int mode) {
  return ewald_ws_layout(d, mode, nullptr, nullptr);
}

// real_rows (or nullptr): the first basis_sites rows of the real-space and
// self terms; the split build rewrites them in place as FP32 pairs
int ewald_build_split(const PycdEwaldDesc* d, int mode, double* out,
                      const double* kc, const double* k2, const double* ck,
                      double* real_rows, void* ws, size_t ws_bytes, cudaStream_t s);
size_t ewald_split_workspace_bytes(const PycdEwaldDesc* d, int mode);

int ewald_build(const PycdEwaldDesc* d, int mode, double* out, void* ws,
                size_t ws_bytes, cudaStream_t s, float* real_ms,
                float* fourier_ms) {
  int rc = ewald_validate(d, mode);
  if (rc) return rc;
  const size_t need = ewald_workspace_bytes(d, mode) +
                      ((mode == PYCD_EWALD_BF16X3 || mode == PYCD_EWALD_TF32X3)
                           ? ewald_split_workspace_bytes(d, mode)
                           : 0);
  if (ws_bytes < need) {
    set_error("workspace too small: %zu < %zu bytes", ws_bytes, need);
    return PYCD_ERR_WORKSPACE;
  }
  EwaldWs w;
  ewald_ws_layout(d, mode, &w, (char*)ws);
  const int parts = d->parts ? d->parts : PYCD_EWALD_PART_ALL;
  const int64_t n = d->n_sites;
  // a part left out contributes exactly zero: no k-vectors, no pair passes
  // the cutoff (the diagonal's r = 0 included), a zero self term
  const int64_t K = (parts & PYCD_EWALD_PART_FOURIER) ? d->n_kvec : 0;
  const double r_cut = (parts & PYCD_EWALD_PART_REAL) ? d->r_cut : -1.0;
  Mat3 recip, cell, inv;
  for (int c = 0; c < 9; ++c) {
    recip.m[c] = d->recip[c];
    cell.m[c] = d->sim_cell[c];
    inv.m[c] = d->sim_cell_inv[c];
  }
  const double coeff = 2.0 * M_PI / d->volume;
  // timing events, released on every return path
  struct Events {
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    ~Events() {
      for (cudaEvent_t ev : e)
        if (ev) cudaEventDestroy(ev);
    }
  } ev;
  cudaEvent_t &e0 = ev.e[0], &e1 = ev.e[1], &e2 = ev.e[2];
  const bool timing = real_ms || fourier_ms;
  if (timing) {
    PYCD_CUDA(cudaEventCreate(&e0));
    PYCD_CUDA(cudaEventCreate(&e1));
    PYCD_CUDA(cudaEventCreate(&e2));
    PYCD_CUDA(cudaEventRecord(e0, s));
  }
  if (K > 0) {
    kvec_prepare_kernel<<<(unsigned)((K + 255) / 256), 256, 0, s>>>(
        d->d_kvec, K, recip, coeff, 4.0 * d->alpha, w.kc, w.k2, w.ck);
    PYCD_CUDA(cudaGetLastError());
  }
  EwaldGeom g{};
  g.cart = d->d_cart;
  g.pmiv = d->d_pmiv;
  g.cell = cell;
  g.inv = inv;
  for (int c = 0; c < 9; ++c) {
    g.cell_f[c] = (float)cell.m[c];
    g.inv_f[c] = (float)inv.m[c];
  }
  g.pbc[0] = d->pbc[0]; g.pbc[1] = d->pbc[1]; g.pbc[2] = d->pbc[2];
  g.n = n;
  const double sqrt_alpha = sqrt(d->alpha);
  const double self_term =
      (parts & PYCD_EWALD_PART_SELF) ? -(sqrt(d->alpha / M_PI)) / d->dielectric : 0.0;
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)n);
  if (mode == PYCD_EWALD_FP64_DIRECT) {
    ewald_pair_kernel<true><<<grid, 256, 512 * 5 * sizeof(double), s>>>(
        g, sqrt_alpha, r_cut, d->dielectric, self_term, w.kc, w.k2,
        w.ck, K, out);
    PYCD_CUDA(cudaGetLastError());
    if (timing) {
      PYCD_CUDA(cudaEventRecord(e1, s));
      PYCD_CUDA(cudaEventRecord(e2, s));
    }
  } else {
    if (w.real_rows) {
      // the first basis_sites rows of the real-space and self terms only;
      // the split kernel writes every entry from them
      dim3 tgrid((unsigned)((n + 255) / 256), (unsigned)d->basis_sites);
      ewald_pair_kernel<false><<<tgrid, 256, 0, s>>>(
          g, sqrt_alpha, r_cut, d->dielectric, self_term, w.kc, w.k2,
          w.ck, 0, w.real_rows);
    } else {
      ewald_pair_kernel<false><<<grid, 256, 0, s>>>(
          g, sqrt_alpha, r_cut, d->dielectric, self_term, w.kc, w.k2,
          w.ck, 0, out);
    }
    PYCD_CUDA(cudaGetLastError());
    if (timing) PYCD_CUDA(cudaEventRecord(e1, s));
    if (K > 0) {
      if (mode == PYCD_EWALD_FP64_GEMM) {
        rc = ewald_features_launch(d->d_cart, n, d->d_kvec, recip, w.kc, w.k2, w.ck, K,
                                   d->dielectric, w.ld, w.F, s);
        if (rc) return rc;
        const unsigned nb = (unsigned)((n + GB - 1) / GB);
        syrk_fp64_kernel<<<dim3(nb, nb), 256, 0, s>>>(w.F, n, w.ld, w.ld, out);
        PYCD_CUDA(cudaGetLastError());
      } else {
        const size_t base = ewald_workspace_bytes(d, mode);
        rc = ewald_build_split(d, mode, out, w.kc, w.k2, w.ck, w.real_rows,
                               (char*)ws + base, ws_bytes - base, s);
        if (rc) return rc;
      }
    }
    if (timing) PYCD_CUDA(cudaEventRecord(e2, s));
  }
  if (timing) {
    PYCD_CUDA(cudaEventSynchronize(e2));
    float a = 0.f, b = 0.f;
    PYCD_CUDA(cudaEventElapsedTime(&a, e0, e1));
    PYCD_CUDA(cudaEventElapsedTime(&b, e1, e2));
    if (real_ms) *real_ms = a;
    if (fourier_ms) *fourier_ms = b;
  }
  return PYCD_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the FP64 feature-contraction build.
//
// Some callers cannot allocate device memory: a host program that is handed
// only the input and output device buffers by another runtime whose caching
// allocator owns the GPU's memory (a C or Fortran code coupled to a larger
// framework, for instance) must not create allocations of its own.  For them
// the scratch (per-k constants and the N x 2K feature rows) lives in this
// fixed file-scope array instead of a caller workspace.  Every GPU that loads
// the library keeps these 32 MiB reserved until the process exits.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host code cannot use &g_noalloc_scratch as a device address (it names a
// host-side stand-in), so the address is resolved once per device with that
// device current and cached here.  A cudaDeviceReset reloads the module and
// may move the array, leaving the cached address stale: the library is not
// usable across a device reset.
static void* g_noalloc_ptr[kMaxDevices] = {nullptr};
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(void** out) {
  int dev = 0;
  PYCD_CUDA(cudaGetDevice(&dev));
  PYCD_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return PYCD_OK;
}

// One block per k-vector: sum over all pairs of q_i q_j cos(k . d_ij) in a
// fixed order (thread-strided, then a tree over the block), times the k
// prefactor (2 pi / V) exp(-k^2 / 4 alpha) / k^2.
constexpr int kKvecThreads = 256;
__global__ void __launch_bounds__(kKvecThreads)
kvector_energy_kernel(EwaldGeom g, const int32_t* __restrict__ kv, Mat3 recip,
                      double coeff, double alpha4, const double* __restrict__ q,
                      double* __restrict__ out) {
  __shared__ double red[kKvecThreads];
  const int64_t k = blockIdx.x;
  const double m0 = kv[k * 3], m1 = kv[k * 3 + 1], m2 = kv[k * 3 + 2];
  double kc[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    kc[c] = __dadd_rn(__dadd_rn(__dmul_rn(m0, recip.m[0 * 3 + c]),
                                __dmul_rn(m1, recip.m[1 * 3 + c])),
                      __dmul_rn(m2, recip.m[2 * 3 + c]));
  const double k2 = fma(kc[2], kc[2], fma(kc[1], kc[1], __dmul_rn(kc[0], kc[0])));
  double acc = 0.0;
  const int64_t n = g.n, pairs = n * n;
  for (int64_t p = threadIdx.x; p < pairs; p += kKvecThreads) {
    const int64_t i = p / n, j = p - i * n;
    double d[3];
    pair_vector(g, i, j, d);
    const double th = fma(d[2], kc[2], fma(d[1], kc[1], __dmul_rn(d[0], kc[0])));
    acc = fma(__dmul_rn(q[i], q[j]), cos(th), acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kKvecThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    out[k] = __ddiv_rn(__dmul_rn(__dmul_rn(coeff, exp(__ddiv_rn(-k2, alpha4))), red[0]), k2);
}

int kvector_energies(const PycdEwaldDesc* d, const double* q, double* out, cudaStream_t s) {
  PYCD_REQUIRE(d != nullptr && q != nullptr && out != nullptr, "NULL argument");
  PYCD_REQUIRE(d->n_sites > 0 && d->n_kvec >= 0 && (d->n_kvec == 0 || d->d_kvec),
               "bad n_sites / k list");
  PYCD_REQUIRE(d->d_cart != nullptr || d->d_pmiv != nullptr, "need d_cart or d_pmiv");
  PYCD_REQUIRE(d->alpha > 0.0 && d->volume > 0.0, "alpha and volume must be > 0");
  PYCD_REQUIRE(d->n_kvec <= 0x7fffffff, "too many k-vectors");
  if (d->n_kvec == 0) return PYCD_OK;
  EwaldGeom g{};
  g.cart = d->d_cart;
  g.pmiv = d->d_pmiv;
  Mat3 recip;
  for (int c = 0; c < 9; ++c) {
    g.cell.m[c] = d->sim_cell[c];
    g.inv.m[c] = d->sim_cell_inv[c];
    g.cell_f[c] = (float)d->sim_cell[c];
    g.inv_f[c] = (float)d->sim_cell_inv[c];
    recip.m[c] = d->recip[c];
  }
  g.pbc[0] = d->pbc[0]; g.pbc[1] = d->pbc[1]; g.pbc[2] = d->pbc[2];
  g.n = d->n_sites;
  kvector_energy_kernel<<<(unsigned)d->n_kvec, kKvecThreads, 0, s>>>(
      g, d->d_kvec, recip, 2.0 * M_PI / d->volume, 4.0 * d->alpha, q, out);
  PYCD_CUDA(cudaGetLastError());
  return PYCD_OK;
}

int potential_gemv(const double* A, int64_t n, const double* q, double* phi,
                   double* energy, cudaStream_t s) {
  PYCD_REQUIRE(A && q && phi && n > 0, "potential_gemv: bad arguments");
  const int64_t threads = n * 32;
  gemv_rows_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(A, n, q, phi);
  PYCD_CUDA(cudaGetLastError());
  if (energy) {
    dot_kernel<<<1, 1024, 0, s>>>(q, phi, n, energy);
    PYCD_CUDA(cudaGetLastError());
  }
  return PYCD_OK;
}

}  // namespace pycd

extern "C" int pycd_ewald_kvector_energies(const PycdEwaldDesc* desc, const double* d_q,
                                           double* d_out, void* stream) {
  pycd::clear_error();
  return pycd::kvector_energies(desc, d_q, d_out, (cudaStream_t)stream);
}

extern "C" int pycd_ewald_build_noalloc(const PycdEwaldDesc* desc, double* d_out,
                                        void* stream) {
  using namespace pycd;
  clear_error();
  PYCD_REQUIRE(d_out != nullptr, "d_out is NULL");
  int rc = ewald_validate(desc, PYCD_EWALD_FP64_GEMM);
  if (rc) return rc;
  // a build without the Fourier part uses no k-vectors and needs scratch
  // for none of them
  PycdEwaldDesc eff = *desc;
  const int parts = eff.parts ? eff.parts : PYCD_EWALD_PART_ALL;
  if (!(parts & PYCD_EWALD_PART_FOURIER)) eff.n_kvec = 0;
  const size_t need = ewald_workspace_bytes(&eff, PYCD_EWALD_FP64_GEMM);
  if (need > kNoAllocScratchBytes) {
    set_error("pycd_ewald_build_noalloc: N=%lld with K=%lld needs %zu bytes of "
              "scratch; the fixed scratch holds %zu bytes (use pycd_ewald_build "
              "with a workspace)",
              (long long)eff.n_sites, (long long)eff.n_kvec, need,
              kNoAllocScratchBytes);
    return PYCD_ERR_WORKSPACE;
  }
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  // Nothing in the scratch needs clearing: each call writes every byte it
  // later reads (per-k constants, then all feature rows including padding)
  // before reading it.
  return ewald_build(&eff, PYCD_EWALD_FP64_GEMM, d_out, scratch,
                     kNoAllocScratchBytes, (cudaStream_t)stream, nullptr, nullptr);
}
