// Mean squared displacement of unwrapped KMC trajectories on sm_103a:
// Analysis.compute_msd (PyCD/core.py:2974-3081).
//
// msd_sd_kernel computes, for every trajectory t, lag l and carrier s,
//   sd[t, l, s] = mean_{i < R-l} |c (x[t, i+l, s] - x[t, i, s])|^2
// (positions scaled by the distance conversion c before the difference, as
// core.py:2983-2990 scales the position array).  It is FP64-pipe bound:
// 6 FP64 instructions (3 DSUB, 3 DFMA) per (row pair, carrier).  A block
// owns one trajectory and a tile of LT consecutive lags; thread (s, l) keeps
// one running sum.  Rows are staged through shared memory component-major
// (one array per coordinate), so the lanes of a warp, which hold consecutive
// lags of one carrier, read consecutive doubles of the lagged window and
// one broadcast double of the base window.  Sums run over i in increasing
// order inside one thread: the result is deterministic.
//
// The reductions that follow (species averages, mean and population std over
// trajectories, least-squares slopes, their mean and standard error) are
// small and run as one thread per output element.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"

namespace pycd {

namespace {

constexpr int kMsdThreads = 256;
constexpr int kMsdSmemBytes = 96 * 1024;

struct MsdTile {
  int lt;  // lags per block (power of two), lt * n_species <= 256
  int ch;  // base rows staged per chunk
};

MsdTile msd_tile(int n_species) {
  MsdTile t;
  t.lt = 1;
  while (t.lt * 2 * n_species <= kMsdThreads) t.lt *= 2;
  const int comps = 3 * n_species;
  // base window ch rows + lagged window ch + lt rows, comps doubles each
  const int rows = kMsdSmemBytes / (8 * comps);
  t.ch = (rows - t.lt) / 2;
  return t;
}

__global__ void __launch_bounds__(kMsdThreads)
msd_sd_kernel(PycdMsdDesc d, int lt, int ch, int64_t n_tiles, double* __restrict__ sd) {
  extern __shared__ double smem[];
  const int S = d.n_species;
  const int C = 3 * S;
  const int64_t R = d.n_rows;
  const int64_t L = d.n_lags;
  const int64_t tile = blockIdx.x % n_tiles;
  const int64_t t = blockIdx.x / n_tiles;
  const int64_t lag0 = 1 + tile * lt;  // lag 0 is written by the host side
  const int tid = threadIdx.x;
  const int s = tid / lt;
  const int ll = tid - s * lt;
  const int64_t lag = lag0 + ll;
  const bool active = s < S && lag < L;
  const int w1 = ch + lt;               // lagged window rows
  double* base = smem;                  // [C][ch]
  double* lagged = smem + (int64_t)C * ch;  // [C][w1]
  const double* rows = d.d_rows + t * d.traj_stride;
  const double cv = d.dist_conversion;

  double acc = 0.0;
  // pairs exist for i < R - lag0 (the tile's smallest lag)
  for (int64_t i0 = 0; i0 < R - lag0; i0 += ch) {
    __syncthreads();
    for (int e = tid; e < C * ch; e += kMsdThreads) {
      const int c = e / ch, r = e - c * ch;
      const int64_t i = i0 + r;
      base[e] = i < R ? __dmul_rn(rows[i * d.row_stride + c], cv) : 0.0;
    }
    for (int e = tid; e < C * w1; e += kMsdThreads) {
      const int c = e / w1, r = e - c * w1;
      const int64_t i = i0 + lag0 + r;
      lagged[e] = i < R ? __dmul_rn(rows[i * d.row_stride + c], cv) : 0.0;
    }
    __syncthreads();
    if (active) {
      int64_t rmax = R - lag - i0;
      if (rmax > ch) rmax = ch;
      const double* bx = base + (3 * s) * ch;
      const double* lx = lagged + (3 * s) * w1 + ll;
      for (int r = 0; r < rmax; ++r) {
        const double dx = __dsub_rn(lx[r], bx[r]);
        const double dy = __dsub_rn(lx[w1 + r], bx[ch + r]);
        const double dz = __dsub_rn(lx[2 * w1 + r], bx[2 * ch + r]);
        acc = fma(dx, dx, acc);
        acc = fma(dy, dy, acc);
        acc = fma(dz, dz, acc);
      }
    }
  }
  if (active) {
    const int64_t n = R - lag;
    sd[(t * L + lag) * S + s] = n > 0 ? __ddiv_rn(acc, (double)n) : __longlong_as_double(0x7ff8000000000000LL);
  }
}

__global__ void msd_lag0_kernel(int64_t n_traj, int64_t L, int S, double* __restrict__ sd) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n_traj * S) sd[(e / S) * L * S + (e % S)] = 0.0;
}

// species_avg[t, l, k] = mean of sd[t, l, s] over the carriers s of type k
__global__ void msd_species_kernel(PycdMsdDesc d, const double* __restrict__ sd,
                                   double* __restrict__ avg) {
  const int K = d.n_types, S = d.n_species;
  const int64_t n = d.n_traj * d.n_lags * K;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int k = (int)(e % K);
  const int64_t tl = e / K;
  int s0 = 0;
  for (int j = 0; j < k; ++j) s0 += d.type_count[j];
  const double* row = sd + tl * S + s0;
  double sum = 0.0;
  for (int j = 0; j < d.type_count[k]; ++j) sum = __dadd_rn(sum, row[j]);
  avg[e] = __ddiv_rn(sum, (double)d.type_count[k]);
}

// msd_data[l] = (l * dt * tc, mean_t avg[t, l, :]); sem = std_t / sqrt(T)
__global__ void msd_table_kernel(PycdMsdDesc d, const double* __restrict__ avg,
                                 double* __restrict__ msd, double* __restrict__ sem) {
  const int K = d.n_types;
  const int64_t L = d.n_lags, T = d.n_traj;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= L * K) return;
  const int64_t l = e / K;
  const int k = (int)(e % K);
  double sum = 0.0;
  for (int64_t t = 0; t < T; ++t) sum = __dadd_rn(sum, avg[(t * L + l) * K + k]);
  const double mean = __ddiv_rn(sum, (double)T);
  double ss = 0.0;
  for (int64_t t = 0; t < T; ++t) {
    const double dv = __dsub_rn(avg[(t * L + l) * K + k], mean);
    ss = __dadd_rn(ss, __dmul_rn(dv, dv));  // NumPy's std: square, then sum
  }
  msd[l * (K + 1) + 1 + k] = mean;
  if (k == 0) msd[l * (K + 1)] = __dmul_rn(__dmul_rn((double)l, d.time_interval), d.time_conversion);
  if (sem) sem[l * K + k] = __ddiv_rn(sqrt(__ddiv_rn(ss, (double)T)), sqrt((double)T));
}

// least-squares slope of avg[t, lo:hi, k] on the time column
__global__ void msd_slope_kernel(PycdMsdDesc d, const double* __restrict__ avg,
                                 double* __restrict__ slopes) {
  const int K = d.n_types;
  const int64_t L = d.n_lags;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n_traj * K) return;
  const int64_t t = e / K;
  const int k = (int)(e % K);
  const int64_t lo = d.trim_length, hi = L - d.trim_length;
  const double n = (double)(hi - lo);
  const double* y = avg + t * L * K + k;
  double sx = 0.0, sy = 0.0;
  for (int64_t l = lo; l < hi; ++l) {
    sx = __dadd_rn(sx, __dmul_rn(__dmul_rn((double)l, d.time_interval), d.time_conversion));
    sy = __dadd_rn(sy, y[l * K]);
  }
  const double mx = __ddiv_rn(sx, n), my = __ddiv_rn(sy, n);
  double sxx = 0.0, sxy = 0.0;
  for (int64_t l = lo; l < hi; ++l) {
    const double x = __dmul_rn(__dmul_rn((double)l, d.time_interval), d.time_conversion);
    const double dx = __dsub_rn(x, mx);
    sxx = fma(dx, dx, sxx);
    sxy = fma(dx, __dsub_rn(y[l * K], my), sxy);
  }
  slopes[e] = __ddiv_rn(sxy, sxx);
}

// mean and std / sqrt(T) of the slopes of each type
__global__ void msd_slope_stats_kernel(PycdMsdDesc d, const double* __restrict__ slopes,
                                       double* __restrict__ stats) {
  const int K = d.n_types;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const int64_t T = d.n_traj;
  double sum = 0.0;
  for (int64_t t = 0; t < T; ++t) sum = __dadd_rn(sum, slopes[t * K + k]);
  const double mean = __ddiv_rn(sum, (double)T);
  double ss = 0.0;
  for (int64_t t = 0; t < T; ++t) {
    const double dv = __dsub_rn(slopes[t * K + k], mean);
    ss = __dadd_rn(ss, __dmul_rn(dv, dv));
  }
  stats[k] = mean;
  stats[K + k] = __ddiv_rn(sqrt(__ddiv_rn(ss, (double)T)), sqrt((double)T));
}

unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

int msd_compute(const PycdMsdDesc& d, double* sd, double* avg, double* msd, double* sem,
                double* slopes, double* stats, cudaStream_t s) {
  const MsdTile tile = msd_tile(d.n_species);
  const int64_t lags = d.n_lags - 1;
  const int64_t n_tiles = lags > 0 ? (lags + tile.lt - 1) / tile.lt : 0;
  const int64_t blocks = n_tiles * d.n_traj;
  PYCD_REQUIRE(blocks < (int64_t)INT32_MAX, "too many (trajectory, lag tile) blocks");
  if (d.n_traj * d.n_species > 0)
    msd_lag0_kernel<<<grid_for(d.n_traj * d.n_species, 256), 256, 0, s>>>(
        d.n_traj, d.n_lags, d.n_species, sd);
  if (blocks > 0) {
    const int smem = 8 * 3 * d.n_species * (2 * tile.ch + tile.lt);
    PYCD_CUDA(cudaFuncSetAttribute(msd_sd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   smem));
    msd_sd_kernel<<<(unsigned)blocks, kMsdThreads, smem, s>>>(d, tile.lt, tile.ch, n_tiles, sd);
  }
  PYCD_CUDA(cudaGetLastError());
  if (!avg) return PYCD_OK;
  msd_species_kernel<<<grid_for(d.n_traj * d.n_lags * d.n_types, 256), 256, 0, s>>>(d, sd, avg);
  if (!msd) return PYCD_OK;
  msd_table_kernel<<<grid_for(d.n_lags * d.n_types, 128), 128, 0, s>>>(d, avg, msd, sem);
  if (!slopes) { PYCD_CUDA(cudaGetLastError()); return PYCD_OK; }
  msd_slope_kernel<<<grid_for(d.n_traj * d.n_types, 128), 128, 0, s>>>(d, avg, slopes);
  if (stats) msd_slope_stats_kernel<<<1, 32, 0, s>>>(d, slopes, stats);
  PYCD_CUDA(cudaGetLastError());
  return PYCD_OK;
}

}  // namespace pycd
