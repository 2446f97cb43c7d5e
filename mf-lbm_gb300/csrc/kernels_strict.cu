// kernels_strict.cu -- kernel flavour compiled with --fmad=false: every floating-point
// operation rounds separately in the reference's written order.
#define MFLBM_NS strict
#define MFLBM_STRICT 1
#include "launch.cuh"

namespace mflbm {
const KernelTable *kernels_strict() { return &strict::table; }
}  // namespace mflbm
