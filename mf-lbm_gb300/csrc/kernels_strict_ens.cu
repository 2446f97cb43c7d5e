// kernels_strict_ens.cu -- the ensemble and velocity-initialisation launchers of the --fmad=false kernel flavour (see
// launch.cuh: the launchers of one flavour are split over three translation units).
#define MFLBM_NS strict
#define MFLBM_STRICT 1
#define MFLBM_PART 2
#include "launch.cuh"
