// kernels_fast_ens.cu -- the ensemble and velocity-initialisation launchers of the FMA-contracting kernel flavour (see
// launch.cuh: the launchers of one flavour are split over three translation units).
#define MFLBM_NS fast
#define MFLBM_PART 2
#include "launch.cuh"
