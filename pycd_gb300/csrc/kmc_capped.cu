// Register-capped instances of the KMC kernel (two 256-thread blocks per
// SM), compiled in their own translation unit so that the two variants build
// in parallel.
#include "kmc_device.cuh"

namespace pycd {

cudaError_t kmc_launch_capped(const KmcArgs& a, int G, int MAXP, int warps_per_block,
                              int blocks, cudaStream_t s, bool* found) {
  *found = false;
  cudaError_t e = cudaErrorInvalidConfiguration;
#define PYCD_KMC_CASE(g_, m_)                                                \
  if (!*found && G == g_ && MAXP == m_) {                                    \
    e = launch_g<g_, m_, 2>(a, warps_per_block, blocks, s);                  \
    *found = true;                                                           \
  }
  PYCD_KMC_CAPPED_SHAPES(PYCD_KMC_CASE)
#undef PYCD_KMC_CASE
  return e;
}

cudaError_t kmc_preload_capped() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaSuccess;
#define PYCD_KMC_LOAD(g_, m_)                                                \
  if (e == cudaSuccess)                                                      \
    e = cudaFuncGetAttributes(&fa, (const void*)kmc_advance_kernel<g_, m_, 2>);
  PYCD_KMC_CAPPED_SHAPES(PYCD_KMC_LOAD)
#undef PYCD_KMC_LOAD
  return e;
}

// this translation unit's copy of the exp tables
cudaError_t kmc_exp_upload_capped(const double2* h_tab, const uint64_t* h_fix) {
  return exp_table_upload(h_tab, h_fix);
}

}  // namespace pycd
