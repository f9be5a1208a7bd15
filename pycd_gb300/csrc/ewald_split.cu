// Split-precision (BF16x3 / TF32x3) tcgen05 contraction of the Ewald
// feature rows.  Placeholder until the tensor-core kernel lands.
#include <cuda_runtime.h>

#include "common.cuh"

namespace pycd {

size_t ewald_split_workspace_bytes(const PycdEwaldDesc*, int) { return 0; }

int ewald_build_split(const PycdEwaldDesc*, int, double*, const double*,
                      const double*, const double*, void*, size_t,
                      cudaStream_t) {
  set_error("split-precision Ewald modes are not built in this library");
  return PYCD_ERR_INVALID_ARG;
}

}  // namespace pycd
