// Lattice KMC on sm_103a: the Run.do_kmc_steps loop (PyCD/core.py:2787-2861).
//
// Mapping.  A trajectory is owned by a group of G lanes of one warp
// (G = 1..32, a power of two); a warp holds 32/G trajectories.  Process p of
// a trajectory is (carrier c = p / S, slot s = p % S), the reference's order
// (core.py:1946-1987).  Lane g of the group owns processes p = g + j*G,
// j < MAXP, and carrier g (its site and its displacement accumulator).
// Every trajectory runs the same device step, so a trajectory advanced alone
// (the plain form) and inside a batch of thousands produce identical events.
//
// Arithmetic that decides events follows the reference's expression order
// in FP64 with no contraction (__dmul_rn / __dadd_rn / __ddiv_rn):
//   dE0   = 2 q (term01 + term02) + (E_rel[n] - E_rel[o])      core.py:2004-2026
//   dG    = (((lam + dE0)^2 / (4 lam)) - V_ab) - shift          core.py:2045-2046
//   k     = vn * exp(-dG / kT)                                  core.py:2047
//   k_tot = k_0 + k_1 + ... (left to right)                     core.py:2796
//   cum_i = sum_{j<=i} (k_j / k_tot) (left to right)            core.py:2797
//   idx   = first i with cum_i > u1                             core.py:2800
//   t    -= log(u2) / k_tot                                     core.py:2803
// term01 = np.dot(q, A[n]-A[o]) is evaluated as (phi_bg[n] - phi_bg[o]) plus
// the carriers' part sum_c' q (A[n,occ_c'] - A[o,occ_c']), phi_bg = A q_fixed.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"

namespace pycd {

struct KmcArgs {
  const PycdKmcSystem* systems;  // device table
  int32_t n_systems;
  PycdKmcState st;
  PycdKmcOutputs out;
  PycdKmcRng rng;
  int64_t max_steps;
};

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

template <int G>
__device__ __forceinline__ double gshfl(unsigned mask, double v, int src) {
  return __shfl_sync(mask, v, src, G);
}
template <int G>
__device__ __forceinline__ int gshfl(unsigned mask, int v, int src) {
  return __shfl_sync(mask, v, src, G);
}

// One group of G lanes advances one trajectory by up to max_steps steps.
template <int G, int MAXP>
__device__ void advance_trajectory(const KmcArgs& a, int64_t t, int g,
                                   unsigned gmask) {
  const PycdKmcState& st = a.st;
  int32_t status = st.d_status[t];
  if (status != PYCD_TRAJ_RUNNING) return;
  const int sys_id = st.d_sys_index ? st.d_sys_index[t] : 0;
  if (sys_id < 0 || sys_id >= a.n_systems) {
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  const PycdKmcSystem sy = a.systems[sys_id];
  const int64_t N = sy.n_sites;
  const int S = sy.n_slots;
  const int NC = sy.n_carriers;
  const int NP = NC * S;
  const int MC = st.max_carriers;
  const double q = sy.carrier_charge;
  const double* __restrict__ A = sy.d_A;

  // carrier state owned by lane g (carrier c == g)
  int occ = 0;
  double disp0 = 0.0, disp1 = 0.0, disp2 = 0.0;
  double row0 = 0.0, row1 = 0.0, row2 = 0.0;
  const bool owns_carrier = g < NC;
  if (owns_carrier) {
    occ = st.d_occ[t * MC + g];
    const double* dp = st.d_disp + (t * MC + g) * 3;
    disp0 = dp[0]; disp1 = dp[1]; disp2 = dp[2];
    const double* lr = st.d_last_row + (t * MC + g) * 3;
    row0 = lr[0]; row1 = lr[1]; row2 = lr[2];
  }
  double sim_time = st.d_time[t];
  int64_t step = st.d_step[t];
  int64_t start_path = st.d_path_index[t];
  double energy = st.d_energy ? st.d_energy[t] : 0.0;
  int64_t ucur = st.d_u_cursor ? st.d_u_cursor[t] : 0;
  const double* ubase = a.rng.d_uniforms
                            ? a.rng.d_uniforms + (int64_t)t * a.rng.u_stride
                            : nullptr;
  const int64_t n_path = sy.n_path_steps;
  const int64_t row_len = 3 * (int64_t)MC;
  double* unw = a.out.d_unwrapped
                    ? a.out.d_unwrapped +
                          (int64_t)t * (a.out.unwrapped_stride
                                            ? a.out.unwrapped_stride
                                            : n_path * row_len)
                    : nullptr;

  for (int64_t it = 0; it < a.max_steps; ++it) {
    // ---- uniforms (core.py:2799, 2802) --------------------------------
    double u1, u2;
    if (ubase) {
      if (ucur + 2 > a.rng.u_count) { status = PYCD_TRAJ_NEED_UNIFORMS; break; }
      u1 = ubase[ucur];
      u2 = ubase[ucur + 1];
    } else {
      philox_step_uniforms(a.rng.seed, a.rng.traj_offset + (uint64_t)t,
                           (uint64_t)step, u1, u2);
    }

    // ---- process attributes and rates (core.py:1946-2050) -------------
    double kp[MAXP], dE[MAXP];
    int newsite[MAXP], oldsite[MAXP];
    bool bad = false;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = g + j * G;
      kp[j] = 0.0; dE[j] = 0.0; newsite[j] = 0; oldsite[j] = 0;
      // every lane joins the shuffles; lanes past NP discard the result
      const int c = (p < NP) ? p / S : 0;
      const int o = gshfl<G>(gmask, occ, c);
      if (p < NP) {
        const int s = p - c * S;
        const int n = sy.d_nbr[(int64_t)o * S + s];
        oldsite[j] = o;
        newsite[j] = n;
        if (n < 0 || n >= N || o < 0 || o >= N) bad = true;
      }
    }
    // all lanes of the group agree on `bad` before any gather
    const unsigned any_bad = __ballot_sync(gmask, bad) & gmask;
    if (any_bad) { status = PYCD_TRAJ_BAD_INDEX; break; }

    double t01[MAXP];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) t01[j] = 0.0;
    // carriers' part of term01, carrier order c' = 0..NC-1
    for (int cc = 0; cc < NC; ++cc) {
      const int sc = gshfl<G>(gmask, occ, cc);
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        const int p = g + j * G;
        if (p < NP) {
          const double an = __ldg(A + (int64_t)newsite[j] * N + sc);
          const double ao = __ldg(A + (int64_t)oldsite[j] * N + sc);
          t01[j] = dadd(t01[j], dmul(q, dsub(an, ao)));
        }
      }
    }
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = g + j * G;
      if (p < NP) {
        const int o = oldsite[j], n = newsite[j];
        const int64_t slot = (int64_t)o * S + (p % S);
        const double term01 =
            dadd(dsub(__ldg(sy.d_phi_bg + n), __ldg(sy.d_phi_bg + o)), t01[j]);
        const double term02 =
            dmul(q, dsub(__ldg(A + (int64_t)o * N + o), __ldg(A + (int64_t)o * N + n)));
        const double ewald = dmul(dmul(2.0, q), dadd(term01, term02));
        const double shift = dsub(__ldg(sy.d_e_rel + n), __ldg(sy.d_e_rel + o));
        const double de0 = dadd(ewald, shift);
        const double lam = __ldg(sy.d_lam + slot);
        const double x = dadd(lam, de0);
        double dg = dsub(ddiv(dmul(x, x), dmul(4.0, lam)), __ldg(sy.d_vab + slot));
        if (sy.d_field_shift) dg = dsub(dg, __ldg(sy.d_field_shift + slot));
        dE[j] = de0;
        kp[j] = dmul(sy.vn, exp(ddiv(-dg, sy.kT)));
      }
    }

    // ---- selection (core.py:2796-2800), left-to-right sums -------------
    double ktot = 0.0;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      if (j * G >= NP) break;
      for (int src = 0; src < G; ++src) {
        const double v = gshfl<G>(gmask, kp[j], src);
        if (j * G + src < NP) ktot = dadd(ktot, v);
      }
    }
    if (!(ktot > 0.0) || !isfinite(ktot)) { status = PYCD_TRAJ_STALLED; break; }
    double frac[MAXP];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) frac[j] = ddiv(kp[j], ktot);
    double cum = 0.0;
    int sel = -1;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      if (j * G >= NP) break;
      for (int src = 0; src < G; ++src) {
        const double v = gshfl<G>(gmask, frac[j], src);
        const int p = j * G + src;
        if (p < NP) {
          cum = dadd(cum, v);
          if (sel < 0 && cum > u1) sel = p;
        }
      }
    }
    if (sel < 0) { status = PYCD_TRAJ_NO_EVENT; break; }

    // ---- residence time (core.py:2802-2804) ---------------------------
    sim_time = dsub(sim_time, ddiv(log(u2), ktot));
    const double tq = ddiv(sim_time, sy.time_interval);
    int64_t end_path = (tq < 9.0e18) ? (int64_t)tq : INT64_MAX;

    // broadcast the selected process' data from its owner lane
    const int jsel = sel / G, lsel = sel - jsel * G;
    double de_sel = 0.0, k_sel = 0.0;
    int n_sel = 0, o_sel = 0;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const double d = gshfl<G>(gmask, dE[j], lsel);
      const double kk = gshfl<G>(gmask, kp[j], lsel);
      const int ns = gshfl<G>(gmask, newsite[j], lsel);
      const int os = gshfl<G>(gmask, oldsite[j], lsel);
      if (j == jsel) { de_sel = d; k_sel = kk; n_sel = ns; o_sel = os; }
    }
    const int c_sel = sel / S, s_sel = sel - c_sel * S;

    // delG0 grid rows [start, end) before the clamp (core.py:2807-2809)
    if (a.out.d_delg0_grid) {
      const int64_t e = end_path < n_path ? end_path : n_path;
      double* dg = a.out.d_delg0_grid + (int64_t)t * n_path;
      for (int64_t r = start_path + g; r < e; r += G) dg[r] = de_sel;
    }

    // ---- state update (core.py:2810-2830) -----------------------------
    if (g == c_sel) {
      occ = n_sel;
      const double* hv = sy.d_hop + ((int64_t)o_sel * S + s_sel) * 3;
      const double h0 = __ldg(hv), h1 = __ldg(hv + 1), h2 = __ldg(hv + 2);
      disp0 = dadd(disp0, h0);
      disp1 = dadd(disp1, h1);
      disp2 = dadd(disp2, h2);
      if (a.out.d_drift) {
        double* dr = a.out.d_drift + ((int64_t)t * MC + g) * 3;
        dr[0] = dadd(dr[0], dmul(h0, k_sel));
        dr[1] = dadd(dr[1], dmul(h1, k_sel));
        dr[2] = dadd(dr[2], dmul(h2, k_sel));
      }
    }
    energy = dadd(energy, de_sel);
    if (g == 0 && a.out.d_step_time) {
      const int64_t col = step - a.out.step_offset;
      if (col >= 0 && col < a.out.step_capacity) {
        a.out.d_step_time[(int64_t)t * a.out.step_capacity + col] = sim_time;
        a.out.d_step_proc[(int64_t)t * a.out.step_capacity + col] = sel;
      }
    }
    ++step;
    if (ubase) ucur += 2;

    // ---- path-grid rows (core.py:2847-2861) ---------------------------
    if (end_path >= start_path + 1) {
      if (end_path >= n_path) end_path = n_path;
      if (owns_carrier) {
        row0 = dadd(row0, disp0);
        row1 = dadd(row1, disp1);
        row2 = dadd(row2, disp2);
        if (unw) {
          for (int64_t r = start_path; r < end_path; ++r) {
            double* rp = unw + r * row_len + 3 * g;
            rp[0] = row0; rp[1] = row1; rp[2] = row2;
          }
        }
        disp0 = disp1 = disp2 = 0.0;
      }
      if (a.out.d_energy_grid) {
        double* eg = a.out.d_energy_grid + (int64_t)t * n_path;
        for (int64_t r = start_path + g; r < end_path; r += G) eg[r] = energy;
      }
      start_path = end_path;
    }
    if (end_path >= n_path) { status = PYCD_TRAJ_DONE; break; }
  }

  // ---- write the state back ---------------------------------------------
  if (owns_carrier) {
    st.d_occ[t * MC + g] = occ;
    double* dp = st.d_disp + (t * MC + g) * 3;
    dp[0] = disp0; dp[1] = disp1; dp[2] = disp2;
    double* lr = st.d_last_row + (t * MC + g) * 3;
    lr[0] = row0; lr[1] = row1; lr[2] = row2;
  }
  if (g == 0) {
    st.d_time[t] = sim_time;
    st.d_step[t] = step;
    st.d_path_index[t] = start_path;
    if (st.d_energy) st.d_energy[t] = energy;
    if (st.d_u_cursor) st.d_u_cursor[t] = ucur;
    st.d_status[t] = status;
  }
}

template <int G, int MAXP>
__global__ void __launch_bounds__(256) kmc_advance_kernel(KmcArgs a) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / G;
  const int g = lane - sub * G;
  const unsigned gmask =
      (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
  const int64_t groups_per_warp = 32 / G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // persistent grid-stride loop over trajectories
  for (int64_t t = warp * groups_per_warp + sub; t < a.st.n_traj;
       t += n_warps * groups_per_warp) {
    advance_trajectory<G, MAXP>(a, t, g, gmask);
  }
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

template <int G, int MAXP>
static cudaError_t launch_g(const KmcArgs& a, int warps_per_block, int blocks,
                            cudaStream_t s) {
  kmc_advance_kernel<G, MAXP><<<blocks, warps_per_block * 32, 0, s>>>(a);
  return cudaGetLastError();
}

int kmc_launch(const KmcArgs& a, int max_np, int max_nc,
               const PycdKmcLaunch* launch, cudaStream_t s) {
  int G = launch && launch->lanes_per_traj ? launch->lanes_per_traj : 0;
  if (G == 0) G = pow2_at_least(max_np < 32 ? max_np : 32);
  if (G < max_nc) G = pow2_at_least(max_nc);
  PYCD_REQUIRE(G >= 1 && G <= 32 && (G & (G - 1)) == 0,
               "lanes_per_traj must be a power of two in [1, 32] (got %d)", G);
  PYCD_REQUIRE(max_nc <= G, "carriers per trajectory (%d) exceed lanes (%d)",
               max_nc, G);
  const int maxp_needed = (max_np + G - 1) / G;
  PYCD_REQUIRE(maxp_needed <= 8,
               "processes per trajectory (%d) exceed 8 per lane at G=%d",
               max_np, G);
  const int MAXP = maxp_needed <= 1 ? 1 : maxp_needed <= 2 ? 2
                   : maxp_needed <= 4 ? 4 : 8;
  int wpb = launch && launch->warps_per_block ? launch->warps_per_block : 4;
  PYCD_REQUIRE(wpb >= 1 && wpb <= 8, "warps_per_block must be in [1, 8]");
  const int64_t tpw = 32 / G;
  const int64_t warps_needed = (a.st.n_traj + tpw - 1) / tpw;
  int blocks = launch && launch->blocks ? launch->blocks
                                        : (int)((warps_needed + wpb - 1) / wpb);
  if (blocks < 1) blocks = 1;
  cudaError_t e = cudaSuccess;
  if (MAXP == 1) {
    switch (G) {
      case 1: e = launch_g<1, 1>(a, wpb, blocks, s); break;
      case 2: e = launch_g<2, 1>(a, wpb, blocks, s); break;
      case 4: e = launch_g<4, 1>(a, wpb, blocks, s); break;
      case 8: e = launch_g<8, 1>(a, wpb, blocks, s); break;
      case 16: e = launch_g<16, 1>(a, wpb, blocks, s); break;
      case 32: e = launch_g<32, 1>(a, wpb, blocks, s); break;
    }
  } else {
    PYCD_REQUIRE(G == 32, "more than one process per lane needs 32 lanes");
    switch (MAXP) {
      case 2: e = launch_g<32, 2>(a, wpb, blocks, s); break;
      case 4: e = launch_g<32, 4>(a, wpb, blocks, s); break;
      case 8: e = launch_g<32, 8>(a, wpb, blocks, s); break;
    }
  }
  if (e != cudaSuccess) return cuda_fail(e, "kmc_advance_kernel launch", __FILE__, __LINE__);
  return PYCD_OK;
}

// Load every kernel instance now, so that a later launch inside CUDA-graph
// capture never triggers lazy module loading.
int kmc_preload() {
  cudaFuncAttributes fa;
  const void* fns[] = {
      (const void*)kmc_advance_kernel<1, 1>, (const void*)kmc_advance_kernel<2, 1>,
      (const void*)kmc_advance_kernel<4, 1>, (const void*)kmc_advance_kernel<8, 1>,
      (const void*)kmc_advance_kernel<16, 1>, (const void*)kmc_advance_kernel<32, 1>,
      (const void*)kmc_advance_kernel<32, 2>, (const void*)kmc_advance_kernel<32, 4>,
      (const void*)kmc_advance_kernel<32, 8>};
  for (const void* f : fns) {
    cudaError_t e = cudaFuncGetAttributes(&fa, f);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes", __FILE__, __LINE__);
  }
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
