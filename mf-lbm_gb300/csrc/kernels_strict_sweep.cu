// kernels_strict_sweep.cu -- the collision-sweep launchers of the --fmad=false kernel flavour (see
// launch.cuh: the launchers of one flavour are split over three translation units).
#define MFLBM_NS strict
#define MFLBM_STRICT 1
#define MFLBM_PART 1
#include "launch.cuh"
