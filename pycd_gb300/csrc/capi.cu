// extern "C" entry points of libpycd_gb300 (declared in include/pycd_gb300.h).
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "kmc_internal.cuh"

namespace pycd {

static thread_local char g_err[1024] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_error("%s failed at %s:%d: %s (%s)", what, file, line,
            cudaGetErrorName(e), cudaGetErrorString(e));
  return PYCD_ERR_CUDA;
}

// defined in ewald.cu / kmc.cu
int ewald_validate(const PycdEwaldDesc* d, int mode);
size_t ewald_workspace_bytes(const PycdEwaldDesc* d, int mode);
size_t ewald_split_workspace_bytes(const PycdEwaldDesc* d, int mode);
int ewald_build(const PycdEwaldDesc* d, int mode, double* out, void* ws,
                size_t ws_bytes, cudaStream_t s, float* real_ms,
                float* fourier_ms);
int potential_gemv(const double* A, int64_t n, const double* q, double* phi,
                   double* energy, cudaStream_t s);
int msd_compute(const PycdMsdDesc& d, double* sd, double* avg, double* msd, double* sem,
                double* slopes, double* stats, cudaStream_t s);
int potential_sparse(const double* A, int64_t n, const int32_t* idx,
                     const double* q, int32_t m, double* phi, cudaStream_t s);

}  // namespace pycd

using namespace pycd;

// KMC workspace layout: a 256-byte header with the shape maxima, the device
// descriptors (KmcSysDev), one (c1, c0) coefficient array per system that
// does not bring its own, then one slot-constant array per system.
struct KmcTableHeader {
  int32_t n_systems;
  int32_t max_np;
  int32_t max_nc;
  int32_t pad;
};
static_assert(sizeof(KmcTableHeader) == 16, "header layout");

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static size_t kmc_table_bytes(int32_t n_systems) {
  return 256 + align256(sizeof(KmcSysDev) * (size_t)(n_systems > 0 ? n_systems : 1));
}

static size_t kmc_coef_bytes(const PycdKmcSystem& s) {
  return s.d_rate_coef ? 0
                       : align256(sizeof(double2) * (size_t)s.n_sites * (size_t)s.n_slots);
}

static size_t kmc_slotc_bytes(const PycdKmcSystem& s) {
  return align256(2 * sizeof(double2) * (size_t)s.n_sites * (size_t)s.n_slots);
}

static size_t kmc_ws_bytes(const PycdKmcSystem* systems, int32_t n_systems) {
  size_t b = kmc_table_bytes(n_systems);
  for (int i = 0; i < n_systems; ++i) b += kmc_coef_bytes(systems[i]) + kmc_slotc_bytes(systems[i]);
  return b;
}

extern "C" {

const char* pycd_last_error(void) { return g_err; }

int pycd_abi_version(void) { return PYCD_ABI_VERSION; }

int pycd_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor) {
  clear_error();
  int dev = 0, n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device: %s", cudaGetErrorString(e));
    return PYCD_ERR_NO_DEVICE;
  }
  PYCD_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp p;
  PYCD_CUDA(cudaGetDeviceProperties(&p, dev));
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  if (!(p.major == 10 && p.minor == 3)) {
    set_error("device %s is sm_%d%d; this library is built for sm_103a",
              p.name, p.major, p.minor);
    return PYCD_ERR_NO_DEVICE;
  }
  return PYCD_OK;
}

// Half-space k-vector list of PyCD/core.py:816-838 with the k^2 < k_cut^2
// filter of core.py:868: grid points (m0, m1, m2) in C order over
// [-k_max, k_max]^3, excluding 0, keeping the first member of every +-m
// pair, i.e. exactly the points that precede the origin in that order.
int pycd_ewald_kvectors(const double recip[9], const int32_t k_max[3],
                        double k_cut, int32_t* h_kvec, int64_t capacity,
                        int64_t* n_out) {
  clear_error();
  PYCD_REQUIRE(recip && k_max && n_out, "pycd_ewald_kvectors: NULL argument");
  for (int c = 0; c < 3; ++c)
    PYCD_REQUIRE(k_max[c] >= 0 && k_max[c] < 100000, "bad k_max[%d]", c);
  const double kc2 = k_cut * k_cut;
  int64_t n = 0;
  for (int a = -k_max[0]; a <= k_max[0]; ++a)
    for (int b = -k_max[1]; b <= k_max[1]; ++b)
      for (int c = -k_max[2]; c <= k_max[2]; ++c) {
        // first-of-pair: strictly before the origin in C order
        if (a > 0 || (a == 0 && (b > 0 || (b == 0 && c >= 0)))) goto done;
        {
          double v[3];
          for (int j = 0; j < 3; ++j)
            v[j] = (a * recip[0 * 3 + j] + b * recip[1 * 3 + j]) +
                   c * recip[2 * 3 + j];
          const double k2 = fma(v[2], v[2], fma(v[1], v[1], v[0] * v[0]));
          if (k2 < kc2) {
            if (h_kvec) {
              if (n >= capacity) {
                set_error("k-vector capacity %lld exceeded", (long long)capacity);
                return PYCD_ERR_INVALID_ARG;
              }
              h_kvec[3 * n] = a;
              h_kvec[3 * n + 1] = b;
              h_kvec[3 * n + 2] = c;
            }
            ++n;
          }
        }
      }
done:
  *n_out = n;
  return PYCD_OK;
}

int pycd_ewald_workspace_size(const PycdEwaldDesc* desc, int mode,
                              size_t* bytes) {
  clear_error();
  PYCD_REQUIRE(bytes != nullptr, "bytes is NULL");
  int rc = ewald_validate(desc, mode);
  if (rc) return rc;
  size_t b = ewald_workspace_bytes(desc, mode);
  if (mode == PYCD_EWALD_BF16X3 || mode == PYCD_EWALD_TF32X3)
    b += ewald_split_workspace_bytes(desc, mode);
  *bytes = b;
  return PYCD_OK;
}

int pycd_ewald_build(const PycdEwaldDesc* desc, int mode, double* d_out,
                     void* d_workspace, size_t workspace_bytes, void* stream,
                     float* real_ms, float* fourier_ms) {
  clear_error();
  PYCD_REQUIRE(d_out != nullptr, "d_out is NULL");
  return ewald_build(desc, mode, d_out, d_workspace, workspace_bytes,
                     (cudaStream_t)stream, real_ms, fourier_ms);
}

int pycd_potential_gemv(const double* d_A, int64_t n_sites, const double* d_q,
                        double* d_phi, double* d_energy, void* stream) {
  clear_error();
  return potential_gemv(d_A, n_sites, d_q, d_phi, d_energy,
                        (cudaStream_t)stream);
}

int pycd_kmc_workspace_size(const PycdKmcSystem* systems, int32_t n_systems,
                            size_t* bytes) {
  clear_error();
  PYCD_REQUIRE(bytes && systems && n_systems > 0, "bad arguments");
  *bytes = kmc_ws_bytes(systems, n_systems);
  return PYCD_OK;
}

static int validate_systems(const PycdKmcSystem* systems, int32_t n_systems,
                            int32_t max_carriers, int* max_np, int* max_nc) {
  PYCD_REQUIRE(systems && n_systems > 0, "no systems");
  int np = 0, nc = 0;
  for (int i = 0; i < n_systems; ++i) {
    const PycdKmcSystem& s = systems[i];
    PYCD_REQUIRE(s.d_A && s.d_phi_bg && s.d_e_rel && s.d_nbr && s.d_hop &&
                     s.d_lam && s.d_vab,
                 "system %d: a required table pointer is NULL", i);
    PYCD_REQUIRE(s.n_sites > 0 && s.n_sites < (1LL << 31),
                 "system %d: n_sites out of range", i);
    PYCD_REQUIRE(s.n_slots > 0 && s.n_carriers > 0 && s.n_carriers <= 32,
                 "system %d: need 1..32 carriers and >=1 slot", i);
    PYCD_REQUIRE(s.n_carriers <= max_carriers,
                 "system %d: %d carriers exceed state stride %d", i,
                 s.n_carriers, max_carriers);
    PYCD_REQUIRE(s.kT > 0.0 && s.time_interval > 0.0 && s.n_path_steps >= 1,
                 "system %d: kT, time_interval, n_path_steps must be > 0", i);
    const int p = s.n_carriers * s.n_slots;
    if (p > np) np = p;
    if (s.n_carriers > nc) nc = s.n_carriers;
  }
  *max_np = np;
  *max_nc = nc;
  return PYCD_OK;
}

static int validate_state(const PycdKmcState* st, const PycdKmcOutputs* out,
                          const PycdKmcRng* rng) {
  PYCD_REQUIRE(st && out && rng, "NULL state/outputs/rng");
  PYCD_REQUIRE(st->n_traj > 0 && st->max_carriers > 0, "empty state");
  PYCD_REQUIRE(st->d_occ && st->d_time && st->d_step && st->d_path_index &&
                   st->d_disp && st->d_last_row && st->d_status,
               "a required state array is NULL");
  PYCD_REQUIRE(!rng->d_uniforms || st->d_u_cursor,
               "injected uniforms need d_u_cursor");
  PYCD_REQUIRE(!rng->d_uniforms || rng->u_stride >= rng->u_count,
               "u_stride < u_count");
  PYCD_REQUIRE(!out->d_step_time == !out->d_step_proc,
               "d_step_time and d_step_proc go together");
  PYCD_REQUIRE(!st->d_csum || (st->csum_refresh > 0 &&
                               (st->csum_refresh & (st->csum_refresh - 1)) == 0),
               "csum_refresh must be a positive power of two");
  PYCD_REQUIRE(st->poll_interval >= 0 && (st->poll_interval & (st->poll_interval - 1)) == 0,
               "poll_interval must be 0 or a power of two");
  PYCD_REQUIRE(st->time_limit_ns >= 0, "time_limit_ns must be >= 0");
  return PYCD_OK;
}

int pycd_kmc_upload_systems(const PycdKmcSystem* systems, int32_t n_systems,
                            void* d_workspace, size_t workspace_bytes,
                            void* stream, PycdKmcLaunch* launch) {
  clear_error();
  int np = 0, nc = 0;
  int rc = validate_systems(systems, n_systems, 32, &np, &nc);
  if (rc) return rc;
  const size_t need = kmc_ws_bytes(systems, n_systems);
  if (!d_workspace || workspace_bytes < need) {
    set_error("KMC workspace too small (%zu < %zu)", workspace_bytes, need);
    return PYCD_ERR_WORKSPACE;
  }
  const size_t table = kmc_table_bytes(n_systems);
  std::vector<char> host(table, 0);
  KmcTableHeader h{n_systems, np, nc, 0};
  memcpy(host.data(), &h, sizeof(h));
  KmcSysDev* dev = (KmcSysDev*)(host.data() + 256);
  char* coef_base = (char*)d_workspace + table;
  size_t off = 0;
  for (int i = 0; i < n_systems; ++i) {
    dev[i].pub = systems[i];
    PYCD_REQUIRE(((uintptr_t)systems[i].d_rate_coef & 15) == 0,
                 "system %d: d_rate_coef must be 16-byte aligned", i);
    dev[i].coef = systems[i].d_rate_coef
                      ? (const double2*)systems[i].d_rate_coef
                      : (const double2*)(coef_base + off);
    off += kmc_coef_bytes(systems[i]);
  }
  for (int i = 0; i < n_systems; ++i) {
    dev[i].slotc = (const double2*)(coef_base + off);
    off += kmc_slotc_bytes(systems[i]);
  }
  cudaStream_t s = (cudaStream_t)stream;
  PYCD_CUDA(cudaMemcpyAsync(d_workspace, host.data(), host.size(),
                            cudaMemcpyHostToDevice, s));
  int64_t max_slots = 0;
  for (int i = 0; i < n_systems; ++i) {
    const int64_t m = systems[i].n_sites * (int64_t)systems[i].n_slots;
    if (m > max_slots) max_slots = m;
  }
  rc = kmc_derive_launch((const KmcSysDev*)((const char*)d_workspace + 256), n_systems,
                         max_slots, s);
  if (rc) return rc;
  PYCD_CUDA(cudaStreamSynchronize(s));
  rc = kmc_preload();
  if (rc) return rc;
  if (launch) {
    launch->max_processes = np;
    launch->max_carriers = nc;
  }
  return PYCD_OK;
}

int pycd_kmc_default_lanes(int32_t max_processes, int32_t max_carriers,
                           int64_t n_traj, int32_t* lanes) {
  clear_error();
  PYCD_REQUIRE(lanes && max_processes > 0 && max_carriers > 0 && max_carriers <= 32 &&
                   n_traj >= 0,
               "pycd_kmc_default_lanes: bad arguments");
  *lanes = kmc_default_lanes(max_processes, max_carriers, n_traj);
  return PYCD_OK;
}

int pycd_kmc_advance_uploaded(int32_t n_systems, const PycdKmcState* state,
                              const PycdKmcOutputs* out, const PycdKmcRng* rng,
                              int64_t max_steps, const PycdKmcLaunch* launch,
                              void* d_workspace, size_t workspace_bytes,
                              void* stream) {
  clear_error();
  int rc = validate_state(state, out, rng);
  if (rc) return rc;
  PYCD_REQUIRE(max_steps >= 0, "max_steps < 0");
  if (!d_workspace || workspace_bytes < kmc_table_bytes(n_systems)) {
    set_error("KMC workspace too small");
    return PYCD_ERR_WORKSPACE;
  }
  PYCD_REQUIRE(launch && launch->max_processes > 0 && launch->max_carriers > 0,
               "launch shape maxima missing (call pycd_kmc_upload_systems)");
  PYCD_REQUIRE(launch->max_carriers <= state->max_carriers,
               "carriers exceed the state stride");
  PYCD_REQUIRE(!state->d_csum || state->csum_stride >= 2 * launch->max_processes,
               "csum_stride %d below 2 x %d processes", state->csum_stride,
               launch->max_processes);
  KmcArgs a;
  a.systems = (const KmcSysDev*)((const char*)d_workspace + 256);
  a.n_systems = n_systems;
  a.st = *state;
  a.out = *out;
  a.rng = *rng;
  a.max_steps = max_steps;
  a.sched = nullptr;
  a.sched_steps = a.sched_rounds = a.sched_sets = 0;
  if (max_steps == 0) return PYCD_OK;
  return kmc_launch(a, launch->max_processes, launch->max_carriers, launch,
                    (cudaStream_t)stream);
}

int pycd_kmc_advance(const PycdKmcSystem* systems, int32_t n_systems,
                     const PycdKmcState* state, const PycdKmcOutputs* out,
                     const PycdKmcRng* rng, int64_t max_steps,
                     const PycdKmcLaunch* launch, void* d_workspace,
                     size_t workspace_bytes, void* stream) {
  clear_error();
  int rc = validate_state(state, out, rng);
  if (rc) return rc;
  int np = 0, nc = 0;
  rc = validate_systems(systems, n_systems, state->max_carriers, &np, &nc);
  if (rc) return rc;
  PycdKmcLaunch l{};
  if (launch) l = *launch;
  rc = pycd_kmc_upload_systems(systems, n_systems, d_workspace,
                               workspace_bytes, stream, &l);
  if (rc) return rc;
  return pycd_kmc_advance_uploaded(n_systems, state, out, rng, max_steps, &l,
                                   d_workspace, workspace_bytes, stream);
}

int pycd_philox_uniforms(uint64_t seed, uint64_t traj, int64_t step0,
                         int64_t n_steps, double* d_out, void* stream) {
  clear_error();
  PYCD_REQUIRE(d_out && n_steps >= 0 && step0 >= 0, "bad arguments");
  return philox_launch(seed, traj, step0, n_steps, d_out, (cudaStream_t)stream);
}

int pycd_potential_sparse(const double* d_A, int64_t n_sites,
                          const int32_t* d_idx, const double* d_q, int32_t m,
                          double* d_phi, void* stream) {
  clear_error();
  return potential_sparse(d_A, n_sites, d_idx, d_q, m, d_phi, (cudaStream_t)stream);
}

int pycd_kmc_rate_coefficients(const PycdKmcSystem* system, double* d_out,
                               void* stream) {
  clear_error();
  PYCD_REQUIRE(system && d_out && system->d_lam && system->d_vab &&
                   system->n_sites > 0 && system->n_slots > 0 && system->kT > 0.0,
               "pycd_kmc_rate_coefficients: bad arguments");
  PYCD_REQUIRE(((uintptr_t)d_out & 15) == 0, "d_out must be 16-byte aligned");
  return kmc_coef_launch(*system, (double2*)d_out, (cudaStream_t)stream);
}

int pycd_msd_compute(const PycdMsdDesc* desc, double* d_sd, double* d_species_avg,
                     double* d_msd_data, double* d_sem_data, double* d_slopes,
                     double* d_slope_stats, void* stream) {
  clear_error();
  PYCD_REQUIRE(desc && desc->d_rows && d_sd, "pycd_msd_compute: NULL descriptor or output");
  const PycdMsdDesc& d = *desc;
  PYCD_REQUIRE(d.n_traj >= 1 && d.n_rows >= 1 && d.n_lags >= 1,
               "n_traj, n_rows and n_lags must be >= 1");
  PYCD_REQUIRE(d.n_species >= 1 && d.n_species <= PYCD_MSD_MAX_SPECIES,
               "n_species must be in [1, %d] (got %d)", PYCD_MSD_MAX_SPECIES, d.n_species);
  PYCD_REQUIRE(d.row_stride >= 3 * (int64_t)d.n_species,
               "row_stride (%lld) must hold 3 * n_species doubles", (long long)d.row_stride);
  PYCD_REQUIRE(d.n_traj == 1 || d.traj_stride >= d.n_rows * d.row_stride,
               "traj_stride must hold n_rows rows");
  PYCD_REQUIRE(d.n_types >= 1 && d.n_types <= PYCD_MSD_MAX_TYPES,
               "n_types must be in [1, %d]", PYCD_MSD_MAX_TYPES);
  int total = 0;
  for (int k = 0; k < d.n_types; ++k) {
    PYCD_REQUIRE(d.type_count[k] > 0, "type_count[%d] must be > 0", k);
    total += d.type_count[k];
  }
  PYCD_REQUIRE(total == d.n_species, "type counts sum to %d, not n_species %d", total,
               d.n_species);
  PYCD_REQUIRE(!(d_slopes || d_slope_stats) ||
                   (d.trim_length >= 0 && d.n_lags - 2 * d.trim_length >= 2),
               "the slope fit needs at least 2 lags in [trim, n_lags - trim)");
  PYCD_REQUIRE(d_species_avg || !(d_msd_data || d_sem_data || d_slopes || d_slope_stats),
               "later MSD outputs need d_species_avg");
  PYCD_REQUIRE(d_msd_data || !(d_sem_data || d_slopes || d_slope_stats),
               "later MSD outputs need d_msd_data");
  PYCD_REQUIRE(d_slopes || !d_slope_stats, "d_slope_stats needs d_slopes");
  return msd_compute(d, d_sd, d_species_avg, d_msd_data, d_sem_data, d_slopes,
                     d_slope_stats, (cudaStream_t)stream);
}

int pycd_debug_exp(const double* d_x, int64_t n, double* d_ours, double* d_cuda,
                   void* stream) {
  clear_error();
  PYCD_REQUIRE(d_x && d_ours && d_cuda && n >= 0, "bad arguments");
  return exp_probe_launch(d_x, n, d_ours, d_cuda, (cudaStream_t)stream);
}

int pycd_debug_exp_table(double* h_out) {
  clear_error();
  PYCD_REQUIRE(h_out, "bad arguments");
  exp_table_host((double2*)h_out);
  return PYCD_OK;
}

int pycd_debug_exp_table_fixed(uint64_t* h_out) {
  clear_error();
  PYCD_REQUIRE(h_out, "bad arguments");
  double2 pairs[4096];
  exp_table_host(pairs);
  exp_fix_host(pairs, h_out);
  return PYCD_OK;
}

}  // extern "C"
