// kernels_fast.cu -- kernel flavour compiled with nvcc's default FMA contraction.
#define MFLBM_NS fast
#include "launch.cuh"

namespace mflbm {
const KernelTable *kernels_fast() { return &fast::table; }
}  // namespace mflbm
