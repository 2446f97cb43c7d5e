// kernels_fast_sweep.cu -- the collision-sweep launchers of the FMA-contracting kernel flavour (see
// launch.cuh: the launchers of one flavour are split over three translation units).
#define MFLBM_NS fast
#define MFLBM_PART 1
#include "launch.cuh"
