// Lattice KMC on sm_103a: launch dispatch of the persistent kernel
// (kmc_device.cuh) and the small helper kernels.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "kmc_device.cuh"

namespace pycd {

static double seed_bits(unsigned long long b) {
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
}

// 2^(j/4096) for j = 16 a + b as the double-double product of the seeds
// 2^(a/256) and 2^(b/4096): ph + pl = h1 h2 exactly (FMA), plus the cross
// terms; hi = RN(ph + c), lo = (ph - hi) + c (exact).  IEEE operations
// only (host code is built without contraction), so every host gets the
// same table; hi + lo is within ~2^-100 of 2^(j/4096).
void exp_table_host(double2* out) {
  for (int j = 0; j < 4096; ++j) {
    const int a = j >> 4, b = j & 15;
    const double h1 = seed_bits(kExpSeedHi256[a]), l1 = seed_bits(kExpSeedLo256[a]);
    const double h2 = seed_bits(kExpSeedHi16[b]), l2 = seed_bits(kExpSeedLo16[b]);
    const double ph = h1 * h2;
    const double pl = std::fma(h1, h2, -ph);
    const double c = std::fma(h1, l2, std::fma(l1, h2, pl));
    const double hi = ph + c;
    const double lo = (ph - hi) + c;
    out[j] = make_double2(hi, lo);
  }
}

// T_j = round(2^(j/4096) 2^62) from the (hi, lo) pairs, with integer
// operations only: hi in [1, 2) is its 53-bit significand times 2^10, and
// lo (|lo| < 2^-53) adds its value in 2^-62 units rounded to nearest.
void exp_fix_host(const double2* pairs, uint64_t* out) {
  const uint64_t mask52 = (1ull << 52) - 1;
  for (int j = 0; j < 4096; ++j) {
    uint64_t hb, lb;
    std::memcpy(&hb, &pairs[j].x, sizeof hb);
    std::memcpy(&lb, &pairs[j].y, sizeof lb);
    int64_t t = (int64_t)(((hb & mask52) | (1ull << 52)) << 10);
    const int el = (int)((lb >> 52) & 0x7ff);
    if (el != 0) {
      // lo = ml 2^(el - 1075): ml 2^(el - 1013) in 2^-62 units
      const uint64_t ml = (lb & mask52) | (1ull << 52);
      const int sh = 1013 - el;  // >= 44
      const int64_t q = sh < 64 ? (int64_t)((ml + (1ull << (sh - 1))) >> sh) : 0;
      t += (lb >> 63) ? -q : q;
    }
    out[j] = (uint64_t)t;
  }
}

// Fill the exp tables of every KMC translation unit on the current device
// (once per device; device ordinals >= kMaxDevices are rejected).  A
// cudaDeviceReset zeroes the tables without clearing this record: the
// library is not usable across a device reset.
int kmc_exp_init() {
  static std::mutex mu;
  static bool done[kMaxDevices] = {false};
  static double2 host[4096];
  static uint64_t host_fix[4096];
  static bool built = false;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__);
  PYCD_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return PYCD_OK;
  if (!built) {
    exp_table_host(host);
    exp_fix_host(host, host_fix);
    built = true;
  }
  e = exp_table_upload(host, host_fix);
  if (e == cudaSuccess) e = kmc_exp_upload_capped(host, host_fix);
  if (e == cudaSuccess) e = kmc_exp_upload_cta(host, host_fix);
  if (e != cudaSuccess) return cuda_fail(e, "exp table upload", __FILE__, __LINE__);
  done[dev] = true;
  return PYCD_OK;
}

// Per-slot exponent coefficients: c1 = -1/(4 lam kT), c0 = (V + shift)/kT + ln vn.
__device__ __forceinline__ double2 rate_coef(const double* __restrict__ lam,
                                             const double* __restrict__ vab,
                                             const double* __restrict__ shift, int64_t i,
                                             double kT, double vn) {
  const double l = lam[i];
  const double v = vab[i] + (shift ? shift[i] : 0.0);
  return make_double2(-1.0 / (4.0 * l * kT), v / kT + log(vn));
}

__global__ void kmc_coef_kernel(const double* __restrict__ lam,
                                const double* __restrict__ vab,
                                const double* __restrict__ shift, int64_t n,
                                double kT, double vn, double2* __restrict__ coef) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  coef[i] = rate_coef(lam, vab, shift, i, kT, vn);
}

// Per-slot tables of every system of a workspace, in one launch
// (blockIdx.y = system).  The rate coefficients (c1, c0) (core.py:2041-2047)
// are written for the systems that do not bring their own.  The slot
// constants change only with the slot's own site (core.py:2004-2026), with
// n = nbr[o, s]:
//   cq = (phi_bg[n] - phi_bg[o]) + q (A[o,o] - A[o,n]),
//   de = e_rel[n] - e_rel[o],   w = sqrt(-c1),
//   xa = 2q w,   xb = (de + lam) w,
// stored as {cq, xb}, {de, xa}.  The step then forms x' = w (lam + dE0) =
// xa term + xb and c1 (lam + dE0)^2 + c0 = c0 - x'^2.  A slot with an
// out-of-range neighbour gets zeros; the step stops on that index before it
// uses them.
__global__ void kmc_derive_kernel(const KmcSysDev* __restrict__ systems, int sys0) {
  const KmcSysDev& sd = systems[sys0 + blockIdx.y];
  const PycdKmcSystem& s = sd.pub;
  const int64_t N = s.n_sites;
  const int64_t total = N * s.n_slots;
  double2* out = (double2*)sd.slotc;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 cf;
    if (s.d_rate_coef) {
      cf = sd.coef[i];
    } else {
      cf = rate_coef(s.d_lam, s.d_vab, s.d_field_shift, i, s.kT, s.vn);
      ((double2*)sd.coef)[i] = cf;
    }
    const int64_t o = i / s.n_slots;
    const int n = s.d_nbr[i];
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    if (n >= 0 && n < N) {
      const double w = __dsqrt_rn(-cf.x);
      const double dphi = dsub(s.d_phi_bg[n], s.d_phi_bg[o]);
      const double t02q = dmul(s.carrier_charge, dsub(s.d_A[o * N + o], s.d_A[o * N + n]));
      const double de = dsub(s.d_e_rel[n], s.d_e_rel[o]);
      a = make_double2(dadd(dphi, t02q), dmul(dadd(de, s.d_lam[i]), w));
      b = make_double2(de, dmul(dmul(2.0, s.carrier_charge), w));
    }
    out[2 * i] = a;
    out[2 * i + 1] = b;
  }
}

__global__ void exp_probe_kernel(const double* __restrict__ x, int64_t n,
                                 double* __restrict__ ours,
                                 double* __restrict__ ref) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ours[i] = kmc_exp(x[i]);
  ref[i] = exp(x[i]);
}

__global__ void philox_uniforms_kernel(uint64_t seed, uint64_t traj,
                                       int64_t step0, int64_t n, double* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double u1, u2;
    philox_step_uniforms(seed, traj, (uint64_t)(step0 + i), u1, u2);
    out[2 * i] = u1;
    out[2 * i + 1] = u2;
  }
}

// ---------------------------------------------------------------------------
// host launch
// ---------------------------------------------------------------------------
static int pow2_at_least(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

static int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      n = v;
    else
      return 1;
  }
  return n;
}

// One block of W = G / 32 warps per trajectory (G = 64 or 128).
static int kmc_launch_blocks(const KmcArgs& a, int G, int max_np,
                             const PycdKmcLaunch* launch, cudaStream_t s) {
  PYCD_REQUIRE(G == 64 || G == 128,
               "lanes_per_traj above 32 must be 64 or 128 (got %d)", G);
  const int W = G / 32;
  const int need = (max_np + G - 1) / G;
  const int MAXP = need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : 8;
  PYCD_REQUIRE(MAXP <= 4, "processes per trajectory (%d) exceed 4 per lane at "
               "%d lanes", max_np, G);
  int64_t blocks = launch && launch->blocks ? launch->blocks : a.st.n_traj;
  if (blocks < 1) blocks = 1;
  if (blocks > 0x7fffffff) blocks = 0x7fffffff;
  bool found = false;
  const cudaError_t e = kmc_launch_cta(a, W, MAXP, (int)blocks, s, &found);
  PYCD_REQUIRE(found, "no block-per-trajectory instance for %d warps x %d "
               "processes per lane", W, MAXP);
  if (e != cudaSuccess) return cuda_fail(e, "kmc_cta_kernel launch", __FILE__, __LINE__);
  return PYCD_OK;
}

// Lanes per trajectory when the launch leaves them open.  The fewest lanes
// (about two processes per lane, at least one lane per carrier) spend the
// fewest FP64 instructions per step; more lanes, up to one block of 4 warps,
// shorten a step by spreading its FP64 instructions over more SM
// sub-partitions.  Measured on GB300 (8 to 32 carriers, 38 to 4,864
// trajectories): widening pays while the launch keeps at most 2 warps per
// sub-partition, i.e. 8 warps per SM.
int kmc_default_lanes(int max_np, int max_nc, int64_t n_traj) {
  const int half = (max_np + 1) / 2;
  int G = pow2_at_least(half < 32 ? half : 32);
  if (G < 2 && max_np > 1) G = 2;  // one lane runs only a single process
  if (G < max_nc) G = pow2_at_least(max_nc);
  const int wide = 2 * pow2_at_least(max_np > 1 ? max_np : 1);
  const int cap = wide < 32 ? 32 : wide > 128 ? 128 : wide;
  const int64_t warp_budget = 8 * (int64_t)sm_count();
  const int64_t T = n_traj > 0 ? n_traj : 1;
  while (2 * G <= cap && T * 2 * G <= 32 * warp_budget) G *= 2;
  return G;
}

int kmc_launch(const KmcArgs& a, int max_np, int max_nc,
               const PycdKmcLaunch* launch, cudaStream_t s) {
  int G = launch && launch->lanes_per_traj ? launch->lanes_per_traj
                                           : kmc_default_lanes(max_np, max_nc, a.st.n_traj);
  if (G > 32) return kmc_launch_blocks(a, G, max_np, launch, s);
  if (G < max_nc) G = pow2_at_least(max_nc);
  PYCD_REQUIRE(G >= 1 && G <= 32 && (G & (G - 1)) == 0,
               "lanes_per_traj must be a power of two in [1, 32] (got %d)", G);
  PYCD_REQUIRE(max_nc <= G, "carriers per trajectory (%d) exceed lanes (%d)",
               max_nc, G);
  const int need = (max_np + G - 1) / G;
  const int MAXP = need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : need <= 8 ? 8 : 16;
  PYCD_REQUIRE(MAXP <= 8, "processes per trajectory (%d) exceed 8 per lane at "
               "%d lanes", max_np, G);
  // default one-warp blocks: the finest split of the trajectories over SMs
  int wpb = launch && launch->warps_per_block ? launch->warps_per_block : 1;
  PYCD_REQUIRE(wpb >= 1 && wpb <= 8, "warps_per_block must be in [1, 8]");
  const int minb = launch && launch->min_blocks_per_sm ? launch->min_blocks_per_sm : 1;
  PYCD_REQUIRE(minb == 1 || (minb == 2 && MAXP <= 2),
               "min_blocks_per_sm must be 0, 1, or 2 with at most 2 processes "
               "per lane (got %d with %d)", minb, MAXP);
  const int64_t tpw = 32 / G;
  const int64_t warps_needed = (a.st.n_traj + tpw - 1) / tpw;
  int blocks = launch && launch->blocks ? launch->blocks
                                        : (int)((warps_needed + wpb - 1) / wpb);
  KmcArgs b = a;
  if (launch && launch->sched_steps > 0) {
    // queue form: rounds of sched_steps steps handed to free warps
    PYCD_REQUIRE(launch->d_sched != nullptr, "sched_steps > 0 needs d_sched");
    const int64_t sets = warps_needed;
    const int64_t rounds = (a.max_steps + launch->sched_steps - 1) / launch->sched_steps;
    const int64_t need = 4 + sets * rounds;
    PYCD_REQUIRE(need < ((int64_t)1 << 30), "too many scheduling rounds (%lld)",
                 (long long)need);
    PYCD_REQUIRE(need <= launch->sched_capacity,
                 "d_sched holds %lld values; this launch needs %lld",
                 (long long)launch->sched_capacity, (long long)need);
    PYCD_CUDA(cudaMemsetAsync(launch->d_sched, 0, sizeof(int32_t) * (size_t)need, s));
    b.sched = launch->d_sched;
    b.sched_steps = launch->sched_steps;
    b.sched_rounds = rounds;
    b.sched_sets = sets;
    if (!launch->blocks) {
      // two warps per SM sub-partition, or one per set when fewer
      int dev = 0, sms = 0;
      PYCD_CUDA(cudaGetDevice(&dev));
      PYCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      const int64_t warps = sets < 8LL * sms ? sets : 8LL * sms;
      blocks = (int)((warps + wpb - 1) / wpb);
    }
  }
  if (blocks < 1) blocks = 1;
  cudaError_t e = cudaErrorInvalidConfiguration;
  bool found = false;
  if (minb == 2) {
    e = kmc_launch_capped(b, G, MAXP, wpb, blocks, s, &found);
  } else {
#define PYCD_KMC_CASE(g_, m_)                                                \
  if (!found && G == g_ && MAXP == m_) {                                     \
    e = launch_g<g_, m_, 1>(b, wpb, blocks, s);                              \
    found = true;                                                            \
  }
    PYCD_KMC_SHAPES(PYCD_KMC_CASE)
#undef PYCD_KMC_CASE
  }
  PYCD_REQUIRE(found, "no kernel instance for %d lanes x %d processes per lane",
               G, MAXP);
  if (e != cudaSuccess) return cuda_fail(e, "kmc_advance_kernel launch", __FILE__, __LINE__);
  return PYCD_OK;
}

int kmc_preload() {
  const int rc = kmc_exp_init();
  if (rc) return rc;
  cudaFuncAttributes fa;
  cudaError_t e = cudaSuccess;
#define PYCD_KMC_LOAD(g_, m_)                                                \
  if (e == cudaSuccess)                                                      \
    e = cudaFuncGetAttributes(&fa, (const void*)kmc_advance_kernel<g_, m_, 1>);
  PYCD_KMC_SHAPES(PYCD_KMC_LOAD)
#undef PYCD_KMC_LOAD
  if (e == cudaSuccess) e = kmc_preload_capped();
  if (e == cudaSuccess) e = kmc_preload_cta();
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes", __FILE__, __LINE__);
  return PYCD_OK;
}

int kmc_coef_launch(const PycdKmcSystem& s, double2* coef, cudaStream_t st) {
  const int64_t n = s.n_sites * (int64_t)s.n_slots;
  kmc_coef_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      s.d_lam, s.d_vab, s.d_field_shift, n, s.kT, s.vn, coef);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kmc_coef_kernel", __FILE__, __LINE__);
  return PYCD_OK;
}

int kmc_derive_launch(const KmcSysDev* d_systems, int n_systems, int64_t max_slots,
                      cudaStream_t st) {
  int64_t bx = (max_slots + 255) / 256;
  if (bx > 128) bx = 128;
  if (bx < 1) bx = 1;
  for (int s0 = 0; s0 < n_systems; s0 += 65535) {
    const int ny = n_systems - s0 < 65535 ? n_systems - s0 : 65535;
    kmc_derive_kernel<<<dim3((unsigned)bx, (unsigned)ny), 256, 0, st>>>(d_systems, s0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kmc_derive_kernel", __FILE__, __LINE__);
  }
  return PYCD_OK;
}

int exp_probe_launch(const double* x, int64_t n, double* ours, double* ref,
                     cudaStream_t s) {
  if (n <= 0) return PYCD_OK;
  const int rc = kmc_exp_init();
  if (rc) return rc;
  exp_probe_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, n, ours, ref);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "exp_probe_kernel", __FILE__, __LINE__);
  return PYCD_OK;
}

int philox_launch(uint64_t seed, uint64_t traj, int64_t step0, int64_t n,
                  double* out, cudaStream_t s) {
  if (n <= 0) return PYCD_OK;
  const int bs = 256;
  philox_uniforms_kernel<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(
      seed, traj, step0, n, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "philox_uniforms_kernel", __FILE__, __LINE__);
  return PYCD_OK;
}

}  // namespace pycd
