// Shared internals of libpycd_gb300: error plumbing and the counter-based RNG.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "pycd_gb300.h"

namespace pycd {

// 3 x 3 matrix passed by value to kernels (row-major)
struct Mat3 {
  double m[9];
};

// Thread-local last-error text behind pycd_last_error().
void set_error(const char* fmt, ...);
void clear_error();

// Map a CUDA error to PYCD_ERR_CUDA with context text.
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

// Per-device state (the exp tables, the fixed no-alloc scratch address) is
// kept for device ordinals below this bound; higher ordinals are rejected
// with PYCD_ERR_INVALID_ARG by every entry point that needs such state.
constexpr int kMaxDevices = 64;

}  // namespace pycd

#define PYCD_CUDA(call)                                                    \
  do {                                                                     \
    cudaError_t _e = (call);                                               \
    if (_e != cudaSuccess)                                                 \
      return ::pycd::cuda_fail(_e, #call, __FILE__, __LINE__);             \
  } while (0)

#define PYCD_REQUIRE(cond, ...)                                            \
  do {                                                                     \
    if (!(cond)) {                                                         \
      ::pycd::set_error(__VA_ARGS__);                                      \
      return PYCD_ERR_INVALID_ARG;                                         \
    }                                                                      \
  } while (0)

namespace pycd {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11).  Round function: two 32x32->64 multiplies by the
// paper's multipliers, xor with the key, Weyl key schedule.
// ---------------------------------------------------------------------------
struct Philox4 {
  uint32_t v[4];
};

// GPU global nanosecond timer
__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Cooperative stop of trajectory t (PycdKmcState.d_cancel / time_limit_ns):
// the status to stop with, or 0 to go on.  t_start: the global timer when
// the trajectory began this launch.
__device__ __forceinline__ int32_t kmc_stop_request(const PycdKmcState& st, int64_t t,
                                                    uint64_t t_start) {
  if (st.d_cancel && st.d_cancel[t] != 0) return PYCD_TRAJ_CANCELLED;
  if (st.time_limit_ns > 0 &&
      (int64_t)(global_timer_ns() - t_start) > st.time_limit_ns)
    return PYCD_TRAJ_TIMEOUT;
  return 0;
}

__host__ __device__ __forceinline__ void philox_mulhilo(uint32_t a, uint32_t b,
                                                        uint32_t& hi,
                                                        uint32_t& lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ Philox4 philox4x32_10(Philox4 ctr,
                                                          uint32_t k0,
                                                          uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(M0, ctr.v[0], hi0, lo0);
    philox_mulhilo(M1, ctr.v[2], hi1, lo1);
    Philox4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// 53-bit uniform in [0, 1) from two 32-bit words: the top 27 bits of `a`
// and the top 26 bits of `b`, the same construction CPython's
// random.random() applies to MT19937 output.
__host__ __device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) *
         (1.0 / 9007199254740992.0);
}

// The two uniforms of KMC step `step` of trajectory `traj`.
__host__ __device__ __forceinline__ void philox_step_uniforms(
    uint64_t seed, uint64_t traj, uint64_t step, double& u1, double& u2) {
  Philox4 c;
  c.v[0] = (uint32_t)step;
  c.v[1] = (uint32_t)(step >> 32);
  c.v[2] = (uint32_t)traj;
  c.v[3] = (uint32_t)(traj >> 32);
  Philox4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u1 = u53(r.v[0], r.v[1]);
  u2 = u53(r.v[2], r.v[3]);
}

}  // namespace pycd
