/*
 * pycd_gb300.h - C ABI of the GB300 (sm_103a) lattice-KMC hot path.
 *
 * Two parts of PyCD are replaced:
 *   1. the Ewald precomputed pairwise-energy array,
 *      System.get_precomputed_array            (PyCD/core.py:1611-1679)
 *      with pot_r_ewald                        (PyCD/core.py:799-814)
 *      get_effective_k_vectors                 (PyCD/core.py:816-838)
 *      pot_k_ewald                             (PyCD/core.py:853-878)
 *      and the self term                       (PyCD/core.py:1659-1661);
 *   2. the KMC loop, Run.do_kmc_steps          (PyCD/core.py:2647-2917)
 *      with get_process_attributes             (PyCD/core.py:1946-1987)
 *      get_process_rates                       (PyCD/core.py:1989-2050)
 *      selection / residence time / update     (PyCD/core.py:2796-2830)
 *      and the path-grid output rows           (PyCD/core.py:2847-2861).
 *
 * Conventions
 *   - Every entry point returns PYCD_OK (0) or a negative PycdStatus.  No C++
 *     exception crosses this boundary.  pycd_last_error() returns a
 *     thread-local message for the most recent failure on the calling thread.
 *   - Pointers named d_* are device pointers owned by the caller; the library
 *     never frees caller memory.  Pointers named h_* are host pointers.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     Launches are asynchronous on that stream unless stated otherwise.
 *   - Units are Hartree atomic units (bohr, Hartree, a.u. time), as in PyCD.
 *   - Thread safety: distinct calls on distinct streams and buffers are
 *     independent.  Global state: the per-thread error string; per device,
 *     the exp tables of the KMC kernels (filled once, then read-only) and
 *     the fixed scratch array of pycd_ewald_build_noalloc, which every call
 *     of that entry point shares (overlapping calls race).  Per-device state
 *     is kept for device ordinals below 64.  The library is not usable
 *     across a cudaDeviceReset: the reset reloads its device arrays while
 *     the host-side records of them stay.
 */
#ifndef PYCD_GB300_H
#define PYCD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYCD_ABI_VERSION 4

#if defined(__GNUC__)
#define PYCD_API __attribute__((visibility("default")))
#else
#define PYCD_API
#endif

typedef enum PycdStatus {
  PYCD_OK = 0,
  PYCD_ERR_INVALID_ARG = -1,   /* bad size, null pointer, unsupported mode  */
  PYCD_ERR_CUDA = -2,          /* a CUDA runtime call failed                */
  PYCD_ERR_STALLED = -3,       /* some trajectory had k_total 0 or not finite */
  PYCD_ERR_BAD_INDEX = -4,     /* a device gather index fell outside its table */
  PYCD_ERR_NO_DEVICE = -5,     /* no CUDA device / wrong architecture       */
  PYCD_ERR_WORKSPACE = -6      /* workspace smaller than the required size   */
} PycdStatus;

/* Per-trajectory status codes written by the KMC kernels (d_status). */
typedef enum PycdTrajStatus {
  PYCD_TRAJ_RUNNING = 0,       /* can be advanced further                    */
  PYCD_TRAJ_DONE = 1,          /* time grid full: end_path_index reached     */
  PYCD_TRAJ_NEED_UNIFORMS = 2, /* injected uniform stream exhausted; refill  */
  PYCD_TRAJ_STALLED = 3,       /* k_total == 0 or not finite (core.py:2800)  */
  PYCD_TRAJ_BAD_INDEX = 4,     /* neighbour / site index out of range        */
  PYCD_TRAJ_NO_EVENT = 5,      /* u1 at or above the last cumulative rate    */
  PYCD_TRAJ_STEP_LIMIT = 6,    /* reached its d_step_limit                   */
  PYCD_TRAJ_CANCELLED = 7,     /* its d_cancel flag was set (see PycdKmcState) */
  PYCD_TRAJ_TIMEOUT = 8        /* ran past time_limit_ns in one launch;
                                * resumable: set the status back to RUNNING  */
} PycdTrajStatus;

/* ------------------------------------------------------------------------ */
/* Library                                                                   */
/* ------------------------------------------------------------------------ */

/* Thread-local text of the last error on this thread ("" if none). */
PYCD_API const char* pycd_last_error(void);

/* ABI version compiled into the library (== PYCD_ABI_VERSION). */
PYCD_API int pycd_abi_version(void);

/* Device properties used by the launch heuristics: SM count, CC major/minor.
 * Fails with PYCD_ERR_NO_DEVICE when no sm_103 device is current. */
PYCD_API int pycd_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);

/* ------------------------------------------------------------------------ */
/* Ewald pairwise-energy array                                               */
/* ------------------------------------------------------------------------ */

/* Precision / algorithm of the reciprocal-space sum. */
typedef enum PycdEwaldMode {
  /* Per-pair sum over k of cos(k . d_ij), d_ij taken from d_pmiv (or the
   * minimum image of the coordinates when d_pmiv is NULL).  Exactly the
   * reference's formula for any pmiv; O(N^2 K) FP64.                      */
  PYCD_EWALD_FP64_DIRECT = 0,
  /* Feature contraction F F^T with F = [sqrt(w) cos(k.r), sqrt(w) sin(k.r)]
   * (N x 2K), FP64 throughout.  Valid when every pmiv_ij is r_j - r_i plus
   * a supercell translation and k . T is a multiple of 2 pi.              */
  PYCD_EWALD_FP64_GEMM = 1,
  /* Same contraction on tcgen05 tensor cores: F split into BF16 hi + lo,
   * three products (hi.hi + hi.lo + lo.hi), FP32 accumulation in TMEM per
   * K-chunk, error-free sum across chunks.  Runs on CTA pairs (2-CTA
   * clusters, 256-row MMAs) where the device can place them, else on
   * single CTAs (PycdEwaldDesc.split_form; same results).                  */
  PYCD_EWALD_BF16X3 = 2,
  /* As BF16X3 with TF32 operands (hi + lo split, three products).         */
  PYCD_EWALD_TF32X3 = 3
} PycdEwaldMode;

typedef struct PycdEwaldDesc {
  int64_t n_sites;              /* N                                         */
  int64_t n_kvec;               /* K: half-space k-vectors kept (k^2<k_cut^2) */
  const double* d_cart;         /* N x 3 site coordinates (bohr)             */
  const double* d_pmiv;         /* N x N x 3 min-image vectors, or NULL      */
  const int32_t* d_kvec;        /* K x 3 integer multiples of the rec. basis */
  double recip[9];              /* reciprocal basis rows (bohr^-1), includes 2 pi/V */
  double sim_cell[9];           /* simulation-cell rows for the min image    */
  double sim_cell_inv[9];       /* inverse of sim_cell                       */
  int32_t pbc[3];               /* periodic flags                            */
  double alpha;                 /* Ewald alpha as used by PyCD (bohr^-2)     */
  double r_cut;                 /* real-space cutoff (bohr), strict <        */
  double volume;                /* cell volume used by the Fourier prefactor */
  double dielectric;            /* relative permittivity                     */
  int32_t parts;                /* PYCD_EWALD_PART_* mask of the terms to
                                 * build; 0 = all.  The real part alone is
                                 * get_precomputed_array_real (core.py:1594-
                                 * 1596), the Fourier part alone
                                 * get_precomputed_array_fourier (1598-1602)  */
  /* Supercell layout, or basis_sites = 0 when unknown.  basis_sites > 0
   * states that site i is basis site i % basis_sites of cell
   * c = i / basis_sites, cells in C order over supercell[0..2] (the last
   * index fastest), and that site positions repeat with the supercell's
   * cells.  Every entry then depends only on (basis_i, basis_j, cell offset
   * modulo the supercell), so the split modes take the real-space and self
   * terms of all rows from the first basis_sites rows.                    */
  int32_t supercell[3];
  int32_t basis_sites;
  /* Launch shape of the split modes; 0 = the library's default.  The array
   * does not depend on it (pycd_gb300/autotune.py picks it by timing).
   * split_form: 1 = CTA pairs (2-CTA clusters, 256-row MMAs; single CTAs
   * where the device cannot place the clusters), 2 = single CTAs.
   * split_raster: super-tiles per side of the blocked tile order, 1-64
   * (default 8).  No counterpart in the reference.                         */
  int32_t split_form;
  int32_t split_raster;
} PycdEwaldDesc;

#define PYCD_EWALD_PART_REAL 1     /* erfc(sqrt(alpha) r)/(2 r eps), r < r_cut */
#define PYCD_EWALD_PART_FOURIER 2  /* the k-space sum / eps                  */
#define PYCD_EWALD_PART_SELF 4     /* -sqrt(alpha/pi)/eps on the diagonal    */
#define PYCD_EWALD_PART_ALL 7

/* Enumerate the half-space k-vector list of PyCD/core.py:816-838 filtered by
 * k^2 < k_cut^2 (PyCD/core.py:868), in the reference's order, on the host.
 * h_kvec may be NULL to query the count only (returned in *n_out).          */
PYCD_API int pycd_ewald_kvectors(const double recip[9], const int32_t k_max[3],
                        double k_cut, int32_t* h_kvec, int64_t capacity,
                        int64_t* n_out);

/* Bytes of device workspace pycd_ewald_build needs for (desc, mode).       */
PYCD_API int pycd_ewald_workspace_size(const PycdEwaldDesc* desc, int mode,
                              size_t* bytes);

/* Build the N x N FP64 array (row-major, Hartree) into d_out:
 *   A = A_real + A_fourier + A_self          (PyCD/core.py:1659-1661)
 * Replaces System.get_precomputed_array (PyCD/core.py:1611-1679).
 * d_workspace must hold pycd_ewald_workspace_size bytes (may be NULL when 0).
 * Timings of the real and Fourier phases are returned in ms when the
 * pointers are non-NULL (this synchronises the stream).                   */
PYCD_API int pycd_ewald_build(const PycdEwaldDesc* desc, int mode, double* d_out,
                     void* d_workspace, size_t workspace_bytes, void* stream,
                     float* real_ms, float* fourier_ms);

/* Allocation-free variant of pycd_ewald_build in PYCD_EWALD_FP64_GEMM mode.
 * No counterpart in the reference: it exists for callers that must not
 * allocate device memory, e.g. a C or Fortran host that receives only the
 * input and output device buffers from another runtime whose allocator owns
 * the GPU's memory.  The scratch (per-k constants and N x 2K feature rows,
 * 8 * (5K + N * 2K) bytes rounded up) lives in a fixed 32 MiB device array
 * inside the library, reserved on every GPU that loads it until the process
 * exits; larger (N, K) are rejected with PYCD_ERR_WORKSPACE.  K counts only
 * when desc->parts includes the Fourier part.  The caller still passes the
 * descriptor's input buffers and d_out.
 *   - The first call on a device resolves the array's device address with
 *     that device current; make that first call before any stream capture.
 *   - Every call uses the same array: calls whose work overlaps on the GPU
 *     (different streams, or different host threads on one device) race and
 *     must be serialised by the caller.  No state carries over between
 *     calls: each call writes the scratch before it reads it.
 *   - Makes no cudaMalloc/cudaFree or allocating library call.            */
PYCD_API int pycd_ewald_build_noalloc(const PycdEwaldDesc* desc, double* d_out,
                                      void* stream);

/* phi = A q for a dense charge vector (lattice charges with dopants
 * overwritten): the background part of np.dot(charge, A[n]-A[o])
 * (PyCD/core.py:2004-2008).  Also returns E = q^T A q in *d_energy when
 * d_energy is non-NULL.                                                    */
PYCD_API int pycd_potential_gemv(const double* d_A, int64_t n_sites,
                        const double* d_q, double* d_phi, double* d_energy,
                        void* stream);

/* Energy contribution of every k-vector of desc->d_kvec (n_kvec of them) for
 * the charges d_q (N), as get_k_vector_energy_contribution
 * (PyCD/core.py:1171-1184) computes one:
 *   d_out[k] = sum_ij q_i q_j (2 pi / V) exp(-k^2 / 4 alpha) cos(k . d_ij) / k^2
 * with d_ij from d_pmiv (or the minimum image of d_cart).  One pass over the
 * N^2 pairs per k; deterministic.                                           */
PYCD_API int pycd_ewald_kvector_energies(const PycdEwaldDesc* desc, const double* d_q,
                                         double* d_out, void* stream);

/* phi[i] = sum_j q[j] A[idx[j]][i] for m charged sites (dopants on an
 * otherwise neutral lattice): the same background potential as
 * pycd_potential_gemv when q is zero elsewhere, reading m rows of the
 * symmetric array instead of all N^2 entries.                              */
PYCD_API int pycd_potential_sparse(const double* d_A, int64_t n_sites,
                                   const int32_t* d_idx, const double* d_q,
                                   int32_t m, double* d_phi, void* stream);

/* ------------------------------------------------------------------------ */
/* KMC                                                                       */
/* ------------------------------------------------------------------------ */

/* One lattice system: tables shared by every trajectory that runs on it.
 * Process p of a trajectory is (carrier c = p / n_slots, slot s = p % n_slots)
 * which is the reference's process order for one carrier species
 * (PyCD/core.py:1946-1987, 1861-1927).                                      */
typedef struct PycdKmcSystem {
  const double* d_A;            /* N x N precomputed array (Hartree)         */
  const double* d_phi_bg;       /* N: A . q_fixed (lattice + dopant charges) */
  const double* d_e_rel;        /* N: relative site energies (Hartree)       */
  const int32_t* d_nbr;         /* N x S: destination site of slot s, -1 none */
  const double* d_hop;          /* N x S x 3: hop vector of slot s (bohr)    */
  const double* d_lam;          /* N x S: reorganisation energy lambda       */
  const double* d_vab;          /* N x S: coupling V_ab                      */
  const double* d_field_shift;  /* N x S: 0.5 E . hop (or NULL for zero)     */
  int64_t n_sites;              /* N                                         */
  int32_t n_slots;              /* S: processes per carrier                  */
  int32_t n_carriers;           /* carriers per trajectory (one species)     */
  double carrier_charge;        /* species charge in e (e.g. -1)             */
  double vn;                    /* attempt frequency (1/a.u. time)           */
  double kT;                    /* k_B T in Hartree                          */
  double time_interval;         /* path-grid spacing (a.u. time)             */
  int64_t n_path_steps;         /* rows of the path grid: int(t_final/dt)+1  */
  /* Optional N x S (c1, c0) rate-coefficient pairs from
   * pycd_kmc_rate_coefficients, shared by systems on the same lattice; NULL
   * makes the library derive them into its workspace at upload.            */
  const double* d_rate_coef;
} PycdKmcSystem;

/* (c1, c0) per (site, slot) for `system`: c1 = -1/(4 lam kT),
 * c0 = (V_ab + shift)/kT + ln vn, so that the hop rate is
 * exp(c1 (lam + dE0)^2 + c0) = vn exp(-dG/kT) (PyCD/core.py:2045-2047).
 * d_out holds 2 * n_sites * n_slots doubles.                               */
PYCD_API int pycd_kmc_rate_coefficients(const PycdKmcSystem* system,
                                        double* d_out, void* stream);

/* Trajectory state, structure-of-arrays over T trajectories.  All device
 * arrays; the kernels read and update them in place so a run can be resumed
 * chunk by chunk (and snapshotted between chunks).                          */
typedef struct PycdKmcState {
  int32_t n_traj;               /* T                                         */
  int32_t max_carriers;         /* row stride of d_occ and d_disp / 3        */
  const int32_t* d_sys_index;   /* T: system of each trajectory (NULL = 0)   */
  int32_t* d_occ;               /* T x max_carriers: current site per carrier */
  double* d_time;               /* T: simulation time (a.u.)                 */
  int64_t* d_step;              /* T: KMC steps done                         */
  int64_t* d_path_index;        /* T: start_path_index of core.py:2781       */
  double* d_disp;               /* T x 3*max_carriers: displacement since the
                                   last path row (core.py:2784)             */
  double* d_last_row;           /* T x 3*max_carriers: path row start-1      */
  double* d_energy;             /* T: current_state_energy (or NULL)         */
  int32_t* d_status;            /* T: PycdTrajStatus                          */
  int64_t* d_u_cursor;          /* T: uniforms consumed (injected mode)      */
  const int64_t* d_step_limit;  /* T: stop after this many steps, or NULL    */
  /* Carrier-potential sums per process p: sum_c' A[n_p, occ_c'] and
   * sum_c' A[o_p, occ_c'] (T x csum_stride doubles, first half / second
   * half).  After each event only the moving carrier's delta is added
   * (2 gathers per process instead of n_carriers); every csum_refresh steps
   * (global step index) all sums are recomputed exactly.  csum_stride must
   * be >= 2 * max processes.  Results are the same for any launch shape or
   * chunking at a given csum_refresh (a power of two).                     */
  double* d_csum;
  int32_t csum_stride;
  int32_t csum_refresh;
  /* Cooperative stop, checked by every running trajectory once every
   * poll_interval of its steps (and before its first step of a launch).
   * The reference's loop has no such control (core.py:2787); it serves
   * callers that must end or bound long launches.
   *   d_cancel: T flags or NULL; d_cancel[t] != 0 stops trajectory t with
   *     PYCD_TRAJ_CANCELLED.  It may point into host-mapped pinned memory,
   *     so that the host can raise a flag while a launch runs.
   *   time_limit_ns: > 0 stops a trajectory that has advanced for longer
   *     than this within one launch (GPU global timer) with
   *     PYCD_TRAJ_TIMEOUT; 0 = no limit.
   *   poll_interval: steps between checks, a power of two; 0 = 256.
   * A stopped trajectory's state is complete up to its last step: a
   * TIMEOUT trajectory set back to PYCD_TRAJ_RUNNING continues with the
   * same events it would have had without the stop.                        */
  const volatile int32_t* d_cancel;
  int64_t time_limit_ns;
  int32_t poll_interval;
} PycdKmcState;

/* Optional per-trajectory outputs.  Each pointer may be NULL.               */
typedef struct PycdKmcOutputs {
  double* d_unwrapped;          /* T x n_path_steps x 3*max_carriers rows     */
  int64_t unwrapped_stride;     /* elements between trajectories (0 = dense) */
  double* d_energy_grid;        /* T x n_path_steps                          */
  double* d_delg0_grid;         /* T x n_path_steps                          */
  double* d_step_time;          /* T x step_capacity: sim_time after step i  */
  int32_t* d_step_proc;         /* T x step_capacity: selected process of step i */
  int64_t step_capacity;        /* columns of d_step_time / d_step_proc      */
  int64_t step_offset;          /* step i is stored in column i - step_offset */
  double* d_drift;              /* T x max_carriers x 3: sum hop * k_sel     */
} PycdKmcOutputs;

/* Source of the two uniforms (u1, u2) each step consumes
 * (PyCD/core.py:2799, 2802).                                                */
typedef struct PycdKmcRng {
  /* Injected stream: T x u_stride doubles, u_count valid per trajectory.
   * Step i of a trajectory uses u[2*i] then u[2*i+1] (counted from the
   * cursor).  When it runs out the trajectory stops with
   * PYCD_TRAJ_NEED_UNIFORMS and resumes after a refill.                     */
  const double* d_uniforms;
  int64_t u_stride;
  int64_t u_count;
  /* Counter-based stream used when d_uniforms is NULL: Philox4x32-10 with
   * key = seed and counter = (step, trajectory id + traj_offset).           */
  uint64_t seed;
  uint64_t traj_offset;
  /* T stream ids (device), or NULL for traj_offset + t: lets a trajectory
   * keep its stream whichever batch or bucket it is advanced in.           */
  const uint64_t* d_traj_ids;
} PycdKmcRng;

/* Launch shape of the persistent kernel (0 fields = heuristic).  The two
 * shape maxima are filled by pycd_kmc_upload_systems and are required by
 * pycd_kmc_advance_uploaded (pycd_kmc_advance computes them itself).       */
typedef struct PycdKmcLaunch {
  int32_t lanes_per_traj;       /* 1..32 (power of two): lanes of one warp;
                                 * 64 or 128: one block of 2 or 4 warps per
                                 * trajectory (its FP64 work spread over 2 or
                                 * 4 SM sub-partitions; same events and
                                 * doubles); 0 = about 2 processes per lane,
                                 * at least one lane per carrier, and the
                                 * block form for more than 32 processes when
                                 * trajectories x warps <= 4 x SMs          */
  int32_t warps_per_block;      /* 1..8; 0 = 1 (ignored by the block form)  */
  int32_t blocks;               /* grid size; 0 = cover all trajectories     */
  int32_t max_processes;        /* max n_carriers * n_slots over the systems */
  int32_t max_carriers;         /* max n_carriers over the systems           */
  /* 0 or 1: kernel as compiled; 2: a variant limited to 128 registers per
   * thread (two 256-thread blocks per SM, more warps to hide load latency,
   * some spills); only for at most 2 processes per lane.  Results do not
   * depend on it.                                                          */
  int32_t min_blocks_per_sm;
  /* Work distribution of the warp form (lanes_per_traj <= 32).  0: static,
   * each warp keeps its trajectories for the whole launch.  > 0: the
   * trajectories of one warp ("a set") advance in rounds of sched_steps
   * steps, and each finished round puts the set's next round on a queue
   * that free warps take from, so every SM sub-partition stays loaded
   * until the launch ends.  Events, times and state do not change.
   * d_sched: caller scratch of sched_capacity int32 values, at least
   * 4 + sets x ceil(max_steps / sched_steps) with sets = ceil(n_traj /
   * (32 / lanes)); the library clears it (stream-ordered) before each
   * launch.  Ignored by the block form.                                    */
  int32_t sched_steps;
  int32_t* d_sched;
  int64_t sched_capacity;
} PycdKmcLaunch;

/* Advance every trajectory by up to max_steps KMC steps, or until its path
 * grid is full (core.py:2787), its injected uniforms run out, or it stalls.
 * `systems` is an array of n_systems host descriptors (copied to a device
 * table in d_workspace); each trajectory runs on systems[d_sys_index[t]].
 * The same device step function serves the one-trajectory (plain) form and
 * the batched form, so their event streams are identical.
 * Workspace: pycd_kmc_workspace_size(systems, n_systems) bytes; it holds the
 * device copy of the descriptors, per-slot rate coefficients derived from
 * lam, V_ab, the field shift, kT and vn, and per-slot constants derived from
 * phi_bg, e_rel, A and the carrier charge (32 bytes per site and slot).    */
PYCD_API int pycd_kmc_workspace_size(const PycdKmcSystem* systems,
                                     int32_t n_systems, size_t* bytes);

PYCD_API int pycd_kmc_advance(const PycdKmcSystem* systems, int32_t n_systems,
                     const PycdKmcState* state, const PycdKmcOutputs* out,
                     const PycdKmcRng* rng, int64_t max_steps,
                     const PycdKmcLaunch* launch, void* d_workspace,
                     size_t workspace_bytes, void* stream);

/* Upload `systems` into d_workspace without launching (for CUDA-graph
 * capture of pycd_kmc_advance_uploaded, which then does no host->device
 * copy).  Synchronous with respect to `stream`.  Fills the shape maxima of
 * *launch (its other fields are left as they are).                          */
PYCD_API int pycd_kmc_upload_systems(const PycdKmcSystem* systems, int32_t n_systems,
                            void* d_workspace, size_t workspace_bytes,
                            void* stream, PycdKmcLaunch* launch);

/* As pycd_kmc_advance, with the system table already in d_workspace.       */
PYCD_API int pycd_kmc_advance_uploaded(int32_t n_systems, const PycdKmcState* state,
                              const PycdKmcOutputs* out, const PycdKmcRng* rng,
                              int64_t max_steps, const PycdKmcLaunch* launch,
                              void* d_workspace, size_t workspace_bytes,
                              void* stream);

/* The lanes per trajectory the launcher picks when PycdKmcLaunch leaves
 * them at 0, for n_traj trajectories of at most max_processes processes
 * and max_carriers carriers on the current device (a caller that launches
 * a batch whose running trajectories are fewer than its slots passes the
 * running count).  No counterpart in the reference (its loop has no launch
 * shape).                                                                  */
PYCD_API int pycd_kmc_default_lanes(int32_t max_processes, int32_t max_carriers,
                           int64_t n_traj, int32_t* lanes);

/* Philox4x32-10 uniforms exactly as the kernels draw them (for tests and
 * for replaying a batched trajectory in another form): fills
 * h_or_d_out[2*i + {0,1}] for steps [step0, step0 + n_steps) of trajectory
 * `traj`.  d_out is a device pointer.                                      */
PYCD_API int pycd_philox_uniforms(uint64_t seed, uint64_t traj, int64_t step0,
                         int64_t n_steps, double* d_out, void* stream);

/* Self-check of the kernels' exp(): d_ours[i] = the KMC kernels' exp(d_x[i]),
 * d_cuda[i] = CUDA's exp(d_x[i]).  No counterpart in the reference.        */
PYCD_API int pycd_debug_exp(const double* d_x, int64_t n, double* d_ours,
                            double* d_cuda, void* stream);

/* The kernels' exp() table, as the library builds it on the host (no device
 * needed): h_out[2 j] + h_out[2 j + 1] = 2^(j/4096), j < 4096 (8192
 * doubles).  No counterpart in the reference.                              */
PYCD_API int pycd_debug_exp_table(double* h_out);

/* The same values as the integer exp's table: h_out[j] = 2^(j/4096) 2^62
 * rounded to an integer, j < 4096, built from the pairs above with integer
 * operations (no device needed).  No counterpart in the reference.          */
PYCD_API int pycd_debug_exp_table_fixed(uint64_t* h_out);

/* ---------------------------------------------------------------------------
 * Mean squared displacement: Analysis.compute_msd (PyCD/core.py:2974-3081)
 * on unwrapped trajectory rows already in device memory.
 * ------------------------------------------------------------------------- */
#define PYCD_MSD_MAX_SPECIES 64
#define PYCD_MSD_MAX_TYPES 32

typedef struct PycdMsdDesc {
  const double* d_rows;     /* row r of trajectory t at d_rows + t*traj_stride
                             * + r*row_stride: 3 coordinates per carrier, in
                             * bohr, carriers grouped by species type        */
  int64_t n_traj;
  int64_t n_rows;           /* rows used per trajectory (core.py:2947-2948)  */
  int64_t traj_stride;      /* doubles                                       */
  int64_t row_stride;       /* doubles, >= 3 * n_species                     */
  int32_t n_species;        /* carriers per row, 1..PYCD_MSD_MAX_SPECIES     */
  int32_t n_types;          /* species types present, 1..PYCD_MSD_MAX_TYPES  */
  int32_t type_count[PYCD_MSD_MAX_TYPES]; /* carriers per present type, > 0,
                             * summing to n_species (core.py:3009-3024)      */
  int64_t n_lags;           /* lags 0..n_lags-1 (core.py:2971-2972)          */
  int64_t trim_length;      /* slope fit on lags [trim, n_lags - trim)       */
  double dist_conversion;   /* bohr -> output length unit                    */
  double time_interval;     /* atomic units                                  */
  double time_conversion;   /* atomic time -> output time unit               */
} PycdMsdDesc;

/* Squared displacements and their averages, replacing the NumPy loops of
 * Analysis.compute_msd (core.py:2983-3034, 3053-3060).  Outputs (device,
 * float64, C order):
 *   d_sd          n_traj x n_lags x n_species: mean over every pair of rows
 *                 `lag` apart of the squared displacement (lag 0 = 0; NaN
 *                 when lag >= n_rows, as the reference's empty mean)
 *   d_species_avg n_traj x n_lags x n_types   (core.py:3006-3024)
 *   d_msd_data    n_lags x (n_types + 1): time column, then the mean over
 *                 trajectories                (core.py:3026-3033)
 *   d_sem_data    n_lags x n_types: population std / sqrt(n_traj) (3034)
 *   d_slopes      n_traj x n_types: least-squares slope of species_avg on
 *                 the time column over the trimmed lags (core.py:3053-3060)
 *   d_slope_stats 2 x n_types: mean and std / sqrt(n_traj) of d_slopes
 * Any output but d_sd may be NULL only if every later one is NULL too
 * (each is computed from the previous).  Asynchronous on `stream`.         */
PYCD_API int pycd_msd_compute(const PycdMsdDesc* desc, double* d_sd,
                              double* d_species_avg, double* d_msd_data,
                              double* d_sem_data, double* d_slopes,
                              double* d_slope_stats, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PYCD_GB300_H */
