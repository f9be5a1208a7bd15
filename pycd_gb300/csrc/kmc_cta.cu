// Block-per-trajectory instances of the KMC step (kmc_cta.cuh), compiled in
// their own translation unit so that they build in parallel with the others.
#include "kmc_cta.cuh"

namespace pycd {

cudaError_t kmc_launch_cta(const KmcArgs& a, int W, int MAXP, int blocks,
                           cudaStream_t s, bool* found) {
  *found = false;
  cudaError_t e = cudaErrorInvalidConfiguration;
#define PYCD_KMC_CTA_CASE(w_, m_)                                            \
  if (!*found && W == w_ && MAXP == m_) {                                    \
    kmc_cta_kernel<w_, m_><<<blocks, 32 * w_, 0, s>>>(a);                    \
    e = cudaGetLastError();                                                  \
    *found = true;                                                           \
  }
  PYCD_KMC_CTA_SHAPES(PYCD_KMC_CTA_CASE)
#undef PYCD_KMC_CTA_CASE
  return e;
}

cudaError_t kmc_preload_cta() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaSuccess;
#define PYCD_KMC_CTA_LOAD(w_, m_)                                            \
  if (e == cudaSuccess)                                                      \
    e = cudaFuncGetAttributes(&fa, (const void*)kmc_cta_kernel<w_, m_>);
  PYCD_KMC_CTA_SHAPES(PYCD_KMC_CTA_LOAD)
#undef PYCD_KMC_CTA_LOAD
  return e;
}

// this translation unit's copy of the exp tables
cudaError_t kmc_exp_upload_cta(const double2* h_tab, const uint64_t* h_fix) {
  return exp_table_upload(h_tab, h_fix);
}

}  // namespace pycd
