// Lattice KMC step with one thread block per trajectory (PyCD/core.py:2787-2861).
//
// A warp's FP64 instruction holds its SM sub-partition's FP64 unit for 64
// cycles whatever its active lanes, so a trajectory owned by one warp is
// bound by the FP64 instructions of that warp.  Here W warps (W = 2 or 4,
// one per sub-partition) share a trajectory and divide its rates, sums and
// rebuild between W FP64 units: the latency form for trajectories of many
// carriers when there are too few trajectories to fill the GPU.
//
// Lane g = threadIdx.x owns processes g*MAXP + j, the process order of the
// warp form, and every sum is the same balanced tree (the warp totals are
// its top W-1 nodes), so the events and every double equal the warp form's.
// Each warp keeps the carrier sites in its lanes 0..NC-1 and runs the
// residence-time chain itself (identical values in every warp); warp 0's
// lanes own the carriers' displacements and path rows.  A step has three
// block barriers: warp totals; the selected event; the rebuilt processes of
// the moved carrier.
#pragma once

#include "kmc_device.cuh"

namespace pycd {

constexpr int kCtaMaxJobs = 33;  // n_slots + 1 rebuild jobs, n_slots <= 32

// Neighbour lists of the processes' destination sites are cached per process
// (in registers) for up to this many slots, so that the moved carrier's new
// neighbours are known when the event is: its rebuild then needs no
// dependent load of the neighbour table.
constexpr int kNbrCache = 4;

struct CtaShared {
  double wsum[4];
  double de_sel, k_sel;
  int sel, n_sel, o_sel, c_sel;
  int stop;  // cooperative stop status for this step (0 = go on), from thread 0
  int nb[kNbrCache];  // neighbours of n_sel (from the selected process' cache)
  // rebuilt processes of the moved carrier: job i < S is slot i, job S its Q
  double jp[kCtaMaxJobs], jcq[kCtaMaxJobs], jxb[kCtaMaxJobs], jde[kCtaMaxJobs];
  double jxa[kCtaMaxJobs], jc0[kCtaMaxJobs];
  int jn[kCtaMaxJobs];
};

// The carrier sums after carrier c_sel hopped o_sel -> n_sel.
//   * Other carriers' processes: P += A[n, n_sel] - A[n, o_sel] (and Q).
//   * The moved carrier's jobs (slot i < S: site n = nbr[n_sel, i], its
//     constants and P; job S: the carrier's Q, row n_sel), 8 per round, job
//     i0 + w + W u on warp w: its lane c loads A[row, occ_c], job_sums adds
//     them in the tree order, and the results go to shared memory.
// Every load of the first round (the incremental entries, the job rows and
// the slot constants) is issued before any of them is used, and the rows
// come from the neighbour cache (nbc, S <= kNbrCache): one memory round trip.
// Returns true on a bad index (no load is issued with one).
template <int W, int MAXP>
__device__ __forceinline__ bool cta_update_sums(const PycdKmcSystem& sy,
                                                const double2* __restrict__ coef,
                                                const double2* __restrict__ slotc,
                                                int w, int l, int occ, int c_sel,
                                                int o_sel, int n_sel, const int* nbc,
                                                ProcCache<MAXP>& pc, CtaShared& sh) {
  constexpr int JW = 8 / W;
  const int64_t N = sy.n_sites;
  const int S = sy.n_slots;
  const int NC = sy.n_carriers;
  const double* __restrict__ A = sy.d_A;
  // incremental entries
  double an[MAXP], ao[MAXP], qn[MAXP], qo[MAXP];
  bool upd[MAXP], updq[MAXP];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    upd[j] = pc.valid[j] && pc.carrier[j] != c_sel;
    updq[j] = upd[j] && (pc.firstq[j] || j == 0);
    const int64_t rn = (int64_t)pc.newsite[j] * N, rq = (int64_t)pc.oldsite[j] * N;
    an[j] = upd[j] ? __ldg(A + rn + n_sel) : 0.0;
    ao[j] = upd[j] ? __ldg(A + rn + o_sel) : 0.0;
    qn[j] = updq[j] ? __ldg(A + rq + n_sel) : 0.0;
    qo[j] = updq[j] ? __ldg(A + rq + o_sel) : 0.0;
  }
  bool bad = false;
  for (int i0 = 0; i0 <= S; i0 += 8) {
    int row[JW];
#pragma unroll
    for (int u = 0; u < JW; ++u) {
      const int i = i0 + w + W * u;
      int r = n_sel;
      if (i < S) {
        r = nbc ? nbc[i] : sy.d_nbr[(int64_t)n_sel * S + i];
        if (r < 0 || r >= N) { bad = true; r = n_sel; }
      }
      row[u] = r;
    }
    double v[JW];
#pragma unroll
    for (int u = 0; u < JW; ++u)
      v[u] = (l < NC && i0 + w + W * u <= S) ? __ldg(A + (int64_t)row[u] * N + occ) : 0.0;
    // slot constants of job i0 + w + W l on lane l < JW
    const int ic = i0 + w + W * l;
    const bool cst = l < JW && ic < S;
    int n = n_sel;
#pragma unroll
    for (int u = 0; u < JW; ++u)
      if (u == l) n = row[u];
    const int64_t slot = (int64_t)n_sel * S + (cst ? ic : 0);
    double2 cf = make_double2(0.0, 0.0), sa = cf, sb = cf;
    if (cst) {
      cf = __ldg(coef + slot);
      sa = __ldg(slotc + 2 * slot);
      sb = __ldg(slotc + 2 * slot + 1);
    }
    if (i0 == 0) {
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        if (upd[j]) pc.P[j] = dadd(pc.P[j], dsub(an[j], ao[j]));
        if (updq[j])
          pc.Q[j] = dadd(pc.Q[j], dsub(qn[j], qo[j]));
        else if (upd[j])
          pc.Q[j] = pc.Q[j > 0 ? j - 1 : 0];
      }
    }
    const double sum = job_sums<32, JW>(0xffffffffu, l, v);
#pragma unroll
    for (int u = 0; u < JW; ++u) {
      const int i = i0 + w + W * u;
      if (i <= S && l == job_lane<JW>(u)) sh.jp[i] = sum;
    }
    if (cst) {
      sh.jn[ic] = n;
      sh.jcq[ic] = sa.x;
      sh.jxb[ic] = sa.y;
      sh.jde[ic] = sb.x;
      sh.jxa[ic] = sb.y;
      sh.jc0[ic] = cf.y;
    }
  }
  return bad;
}

template <int W, int MAXP>
__device__ void advance_trajectory_cta(const KmcArgs& a, int64_t t, CtaShared& sh) {
  constexpr int L = 32 * W;
  constexpr unsigned full = 0xffffffffu;
  const int g = threadIdx.x;
  const int w = g >> 5, l = g & 31;
  const PycdKmcState& st = a.st;
  int32_t status = st.d_status[t];
  __syncthreads();  // every thread has read the status before it can change
  if (status != PYCD_TRAJ_RUNNING) return;
  const int sys_id = st.d_sys_index ? st.d_sys_index[t] : 0;
  if (sys_id < 0 || sys_id >= a.n_systems) {
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  const KmcSysDev& sd = a.systems[sys_id];
  const PycdKmcSystem& sy = sd.pub;
  const int S = sy.n_slots;
  const int NC = sy.n_carriers;
  const int NP = NC * S;
  const int MC = st.max_carriers;
  const double q = sy.carrier_charge;
  const double two_q = dmul(2.0, q);
  const double2* __restrict__ coef = sd.coef;
  const double2* __restrict__ slotc = sd.slotc;
  const double dt_grid = sy.time_interval;
  if (NP > L * MAXP || NC > 32 || S + 1 > kCtaMaxJobs ||
      (st.d_csum && 2 * NP > st.csum_stride)) {
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  const int64_t R = (st.d_csum && st.csum_refresh > 0) ? st.csum_refresh : 1;
  double* csum = st.d_csum ? st.d_csum + t * (int64_t)st.csum_stride : nullptr;
  const int half = st.csum_stride / 2;

  // carrier sites in lanes 0..NC-1 of every warp; warp 0 owns the rest
  const bool owner = w == 0 && l < NC;
  int occ = (l < NC) ? st.d_occ[t * MC + l] : 0;
  double disp0 = 0.0, disp1 = 0.0, disp2 = 0.0;
  double row0 = 0.0, row1 = 0.0, row2 = 0.0;
  if (owner) {
    const double* dp = st.d_disp + (t * MC + l) * 3;
    disp0 = dp[0]; disp1 = dp[1]; disp2 = dp[2];
    const double* lr = st.d_last_row + (t * MC + l) * 3;
    row0 = lr[0]; row1 = lr[1]; row2 = lr[2];
  }
  double sim_time = st.d_time[t];
  int64_t step = st.d_step[t];
  const int64_t step_at_entry = step;
  int64_t start_path = st.d_path_index[t];
  double energy = st.d_energy ? st.d_energy[t] : 0.0;
  int64_t ucur = st.d_u_cursor ? st.d_u_cursor[t] : 0;
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
  double t_guard = dmul(dmul((double)(start_path + 1), dt_grid), 1.0 - 0x1p-40);
  TimeChain<32> tc;
  tc.reset(t_guard, sim_time);
  // per-step log: warp 0 stores each step's time when its chain flushes
  double* tlog = (w == 0 && a.out.d_step_time)
                     ? a.out.d_step_time + (int64_t)t * a.out.step_capacity : nullptr;
  double pre_u1 = 0.0, pre_lu2 = 0.0;
  int64_t pre_base = -33;
  // cooperative stop: thread 0 checks every `poll` steps; the block reads
  // its verdict after the step's first barrier
  const bool polling = st.d_cancel != nullptr || st.time_limit_ns > 0;
  const int64_t poll = st.poll_interval > 0 ? st.poll_interval : 256;
  const uint64_t t_start = polling ? global_timer_ns() : 0;

  ProcCache<MAXP> pc;
  bool bad = setup_processes<32, MAXP>(sy, coef, slotc, g, full, occ, pc);
  if (__syncthreads_or(bad)) {
    if (g == 0) st.d_status[t] = PYCD_TRAJ_BAD_INDEX;
    return;
  }
  // neighbours of each process' destination site (checked where used)
  const bool use_nbc = S <= kNbrCache;
  int nbrc[MAXP][kNbrCache];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
#pragma unroll
    for (int s = 0; s < kNbrCache; ++s)
      nbrc[j][s] = (use_nbc && pc.valid[j] && s < S)
                       ? __ldg(sy.d_nbr + (int64_t)pc.newsite[j] * S + s) : 0;
  }
  if (csum && (step & (R - 1)) != 0) {
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = g * MAXP + j;
      if (pc.valid[j]) { pc.P[j] = csum[p]; pc.Q[j] = csum[half + p]; }
    }
  } else {
    fresh_sums<32, MAXP>(sy, g, full, occ, pc);
  }

  for (int64_t it = 0; it < a.max_steps; ++it) {
    if (step >= step_limit) { status = PYCD_TRAJ_STEP_LIMIT; break; }
    if (ubase && ucur + 2 > a.rng.u_count) { status = PYCD_TRAJ_NEED_UNIFORMS; break; }
    const int64_t since = step - pre_base;
    int k = (int)since;
    if (since < 0 || since >= 32) {
      pre_base = step;
      k = 0;
      double u1, u2;
      if (ubase) {
        const int64_t idx = ucur + 2 * (int64_t)l;
        const bool ok = idx + 2 <= a.rng.u_count;
        u1 = ok ? ubase[idx] : 0.5;
        u2 = ok ? ubase[idx + 1] : 0.5;
      } else {
        philox_step_uniforms(a.rng.seed, stream_id, (uint64_t)(step + l), u1, u2);
      }
      pre_u1 = u1;
      pre_lu2 = log(u2);
    }
    const double u1 = __shfl_sync(full, pre_u1, k);
    const double lu2 = __shfl_sync(full, pre_lu2, k);

    if (it > 0 && (step & (R - 1)) == 0) fresh_sums<32, MAXP>(sy, g, full, occ, pc);

    // ---- rates ----------------------------------------------------------
    double kp[MAXP], term[MAXP];
    process_rates<MAXP>(pc, q, two_q, kp, term);

    // ---- tree: lane, warp, then the W warp totals -----------------------
    LocalTree<MAXP> lt;
    lt.build(kp);
    double lvl[6];
    lvl[0] = lt.total();
#pragma unroll
    for (int v = 0; v < 5; ++v)
      lvl[v + 1] = dadd(lvl[v], __shfl_xor_sync(full, lvl[v], 1 << v));
    if (l == 0) sh.wsum[w] = lvl[5];
    if (g == 0)
      sh.stop = (polling && (it & (poll - 1)) == 0) ? kmc_stop_request(st, t, t_start) : 0;
    __syncthreads();
    if (sh.stop) { status = sh.stop; break; }
    double ws[W];
#pragma unroll
    for (int i = 0; i < W; ++i) ws[i] = sh.wsum[i];
    double ktot, top0 = 0.0;
    if constexpr (W == 2) {
      ktot = dadd(ws[0], ws[1]);
    } else {
      top0 = dadd(ws[0], ws[1]);
      ktot = dadd(top0, dadd(ws[2], ws[3]));
    }
    {
      const long long kb = __double_as_longlong(ktot);
      if (kb <= 0 || kb >= 0x7ff0000000000000LL) { status = PYCD_TRAJ_STALLED; break; }
    }
    const double thr = dmul(u1, ktot);
    double acc = 0.0;
    int wsel = 0;
    double left = ws[0];
    if constexpr (W == 4) {
      const double s = dadd(acc, top0);
      if (!nonneg_gt(s, thr)) { acc = s; wsel = 2; left = ws[2]; }
    }
    {
      const double s = dadd(acc, left);
      if (!nonneg_gt(s, thr)) { acc = s; wsel += 1; }
    }
    if (w == wsel) {
      int base = 0;
#pragma unroll
      for (int v = 4; v >= 0; --v) {
        const double lv = __shfl_sync(full, lvl[v], base);
        const double s = dadd(acc, lv);
        if (!nonneg_gt(s, thr)) { acc = s; base += 1 << v; }
      }
      int node = 1;
#pragma unroll
      for (int v = 0; (MAXP >> (v + 1)) > 0; ++v) {
        double ln = 0.0;
#pragma unroll
        for (int i = 1; i < MAXP; ++i) {
          const double x = __shfl_sync(full, lt.node[2 * i], base);
          if (i == node) ln = x;
        }
        const double s = dadd(acc, ln);
        if (!nonneg_gt(s, thr)) { acc = s; node = 2 * node + 1; } else { node = 2 * node; }
      }
      const int jsel = node - MAXP;
      double term_s = 0.0, dslot_s = 0.0, k_s = 0.0;
      int n_s = 0, o_s = 0, c_s = 0;
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        const double d = __shfl_sync(full, term[j], base);
        const double e = __shfl_sync(full, pc.de[j], base);
        const double kk = __shfl_sync(full, kp[j], base);
        const int ns = __shfl_sync(full, pc.newsite[j], base);
        const int os = __shfl_sync(full, pc.oldsite[j], base);
        const int cs = __shfl_sync(full, pc.carrier[j], base);  // sel / S
        if (j == jsel) { term_s = d; dslot_s = e; k_s = kk; n_s = ns; o_s = os; c_s = cs; }
      }
      const double de_s = fma(two_q, term_s, dslot_s);  // dE0 of the event
      int cand[kNbrCache];
#pragma unroll
      for (int s = 0; s < kNbrCache; ++s) {
        cand[s] = 0;
#pragma unroll
        for (int j = 0; j < MAXP; ++j)
          if (j == jsel) cand[s] = nbrc[j][s];
        cand[s] = __shfl_sync(full, cand[s], base);
      }
      if (l == 0) {
#pragma unroll
        for (int s = 0; s < kNbrCache; ++s) sh.nb[s] = cand[s];
        sh.sel = (wsel * 32 + base) * MAXP + jsel;
        sh.de_sel = de_s;
        sh.k_sel = k_s;
        sh.n_sel = n_s;
        sh.o_sel = o_s;
        sh.c_sel = c_s;
      }
    }
    __syncthreads();
    const int sel = sh.sel;
    const double de_sel = sh.de_sel, k_sel = sh.k_sel;
    const int n_sel = sh.n_sel, o_sel = sh.o_sel, c_sel = sh.c_sel;
    if (sel >= NP) { status = PYCD_TRAJ_NO_EVENT; break; }

    // ---- residence time (every warp, identical values) -------------------
    const bool exact = tc.push(l, ktot, lu2, false, step - a.out.step_offset);
    if (exact) tc.flush(l, full, sim_time, tlog, a.out.step_capacity);
    int64_t end_path = start_path - 1;
    if (exact && !nonneg_gt(t_guard, sim_time)) {
      const double tq = ddiv(sim_time, dt_grid);
      end_path = (tq < 9.0e18) ? (int64_t)tq : INT64_MAX;
    }
    const int s_sel = sel - c_sel * S;

    if (a.out.d_delg0_grid) {
      const int64_t e = end_path < n_path ? end_path : n_path;
      double* dgr = a.out.d_delg0_grid + (int64_t)t * n_path;
      for (int64_t r = start_path + g; r < e; r += L) dgr[r] = de_sel;
    }

    // ---- state update ------------------------------------------------------
    if (l == c_sel) occ = n_sel;
    if (owner && l == c_sel) {
      const double* hv = sy.d_hop + ((int64_t)o_sel * S + s_sel) * 3;
      const double h0 = __ldg(hv), h1 = __ldg(hv + 1), h2 = __ldg(hv + 2);
      disp0 = dadd(disp0, h0);
      disp1 = dadd(disp1, h1);
      disp2 = dadd(disp2, h2);
      if (a.out.d_drift) {
        double* dr = a.out.d_drift + ((int64_t)t * MC + l) * 3;
        dr[0] = dadd(dr[0], dmul(h0, k_sel));
        dr[1] = dadd(dr[1], dmul(h1, k_sel));
        dr[2] = dadd(dr[2], dmul(h2, k_sel));
      }
    }
    energy = dadd(energy, de_sel);
    if (g == 0 && a.out.d_step_proc) {
      const int64_t col = step - a.out.step_offset;
      if (col >= 0 && col < a.out.step_capacity)
        a.out.d_step_proc[(int64_t)t * a.out.step_capacity + col] = sel;
    }
    ++step;
    if (ubase) ucur += 2;

    // ---- carrier sums after the move o_sel -> n_sel ----------------------
    bad = cta_update_sums<W, MAXP>(sy, coef, slotc, w, l, occ, c_sel, o_sel, n_sel,
                                   use_nbc ? sh.nb : nullptr, pc, sh);
    if (__syncthreads_or(bad)) { status = PYCD_TRAJ_BAD_INDEX; break; }
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      if (pc.valid[j] && pc.carrier[j] == c_sel) {
        const int s = g * MAXP + j - c_sel * S;
        pc.oldsite[j] = n_sel;
        pc.newsite[j] = sh.jn[s];
        pc.cq[j] = sh.jcq[s];
        pc.xb[j] = sh.jxb[s];
        pc.de[j] = sh.jde[s];
        pc.xa[j] = sh.jxa[s];
        pc.c0[j] = sh.jc0[s];
        pc.P[j] = sh.jp[s];
        pc.Q[j] = sh.jp[S];
        // the new destination's neighbours, used when this process is next selected
#pragma unroll
        for (int u = 0; u < kNbrCache; ++u)
          nbrc[j][u] = (use_nbc && u < S)
                           ? __ldg(sy.d_nbr + (int64_t)pc.newsite[j] * S + u) : 0;
      }
    }

    // ---- path-grid rows ---------------------------------------------------
    if (end_path >= start_path + 1) {
      if (end_path >= n_path) end_path = n_path;
      if (owner) {
        row0 = dadd(row0, disp0);
        row1 = dadd(row1, disp1);
        row2 = dadd(row2, disp2);
        if (unw) {
          for (int64_t r = start_path; r < end_path; ++r) {
            double* rp = unw + r * row_len + 3 * l;
            rp[0] = row0; rp[1] = row1; rp[2] = row2;
          }
        }
        disp0 = disp1 = disp2 = 0.0;
      }
      if (a.out.d_energy_grid) {
        double* eg = a.out.d_energy_grid + (int64_t)t * n_path;
        for (int64_t r = start_path + g; r < end_path; r += L) eg[r] = energy;
      }
      start_path = end_path;
      t_guard = dmul(dmul((double)(start_path + 1), dt_grid), 1.0 - 0x1p-40);
    }
    if (end_path >= n_path) { status = PYCD_TRAJ_DONE; break; }
    if (exact) tc.reset(t_guard, sim_time);
  }
  if (tc.npend > 0) tc.flush(l, full, sim_time, tlog, a.out.step_capacity);

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
  if (owner) {
    st.d_occ[t * MC + l] = occ;
    double* dp = st.d_disp + (t * MC + l) * 3;
    dp[0] = disp0; dp[1] = disp1; dp[2] = disp2;
    double* lr = st.d_last_row + (t * MC + l) * 3;
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

// One block of W warps per trajectory; blocks stride over the trajectories.
// The barrier after each trajectory keeps the shared records of one
// trajectory from being overwritten while a slower warp still reads them.
template <int W, int MAXP>
__global__ void __launch_bounds__(32 * W) kmc_cta_kernel(KmcArgs a) {
  __shared__ CtaShared sh;
  for (int64_t t = blockIdx.x; t < a.st.n_traj; t += gridDim.x) {
    advance_trajectory_cta<W, MAXP>(a, t, sh);
    __syncthreads();
  }
}

// (warps per trajectory, processes per lane) instances
#define PYCD_KMC_CTA_SHAPES(X) X(2, 1) X(2, 2) X(2, 4) X(4, 1) X(4, 2) X(4, 4)

}  // namespace pycd
