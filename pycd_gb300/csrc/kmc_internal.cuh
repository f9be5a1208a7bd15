// Internal KMC types shared by kmc.cu and capi.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pycd_gb300.h"

namespace pycd {

// Device copy of a system descriptor plus the library-derived per-slot
// tables kept in the KMC workspace: the exponent coefficients (c1, c0) and
// the slot constants {cq, xb}, {de, xa} (two double2 per slot).
struct KmcSysDev {
  PycdKmcSystem pub;
  const double2* coef;
  const double2* slotc;
};

struct KmcArgs {
  const KmcSysDev* systems;  // device table
  int32_t n_systems;
  PycdKmcState st;
  PycdKmcOutputs out;
  PycdKmcRng rng;
  int64_t max_steps;
  // queue form of the warp-form launch (PycdKmcLaunch.sched_steps);
  // sched == nullptr for the static form.  sched[0]: items taken,
  // sched[1]: items queued, sched[2]: a wait ran out, sched[4 + j]: the
  // j-th queued item (round * sets + set + 1)
  int32_t* sched;
  int64_t sched_steps, sched_rounds, sched_sets;
};

int kmc_launch(const KmcArgs& a, int max_np, int max_nc,
               const PycdKmcLaunch* launch, cudaStream_t s);
int kmc_preload();
// the exp tables: built on the host (exp_table_host, 4096 (hi, lo) pairs;
// exp_fix_host, the same values as 62-bit integers), copied into each KMC
// translation unit once per device (kmc_exp_init)
void exp_table_host(double2* out);
void exp_fix_host(const double2* pairs, uint64_t* out);
int kmc_exp_init();
cudaError_t kmc_exp_upload_capped(const double2* h_tab, const uint64_t* h_fix);
cudaError_t kmc_exp_upload_cta(const double2* h_tab, const uint64_t* h_fix);
int kmc_default_lanes(int max_np, int max_nc, int64_t n_traj);
// the register-capped instances (kmc_capped.cu); *found = false when
// there is no instance for (G, MAXP)
cudaError_t kmc_launch_capped(const KmcArgs& a, int G, int MAXP, int warps_per_block,
                              int blocks, cudaStream_t s, bool* found);
cudaError_t kmc_preload_capped();
// the block-per-trajectory instances (kmc_cta.cu): W warps per trajectory;
// *found = false when there is no instance for (W, MAXP)
cudaError_t kmc_launch_cta(const KmcArgs& a, int W, int MAXP, int blocks,
                           cudaStream_t s, bool* found);
cudaError_t kmc_preload_cta();
int kmc_coef_launch(const PycdKmcSystem& s, double2* coef, cudaStream_t st);
// the per-slot tables (coefficients where not given, slot constants) of
// every system in a device descriptor table, in one launch per 65,535
// systems; max_slots = the largest n_sites * n_slots
int kmc_derive_launch(const KmcSysDev* d_systems, int n_systems, int64_t max_slots,
                      cudaStream_t st);
int exp_probe_launch(const double* x, int64_t n, double* ours, double* ref,
                     cudaStream_t s);
int philox_launch(uint64_t seed, uint64_t traj, int64_t step0, int64_t n,
                  double* out, cudaStream_t s);

}  // namespace pycd
