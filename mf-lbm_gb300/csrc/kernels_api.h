// kernels_api.h -- launch interface between the C-ABI layer (api.cu) and the kernel
// translation units.  Each floating-point flavour (fast / strict) exports one
// KernelTable; the ordering of one time step lives only in api.cu.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include "common.cuh"

namespace mflbm {

// Everything a launcher needs: device pointers, layout and parameters.
struct DevState {
    Layout L;
    StepParams P;
    int multiphase;
    int prec;              // MFLBM_FP64 / FP32 / FP16 / FP64FF / FF
    float ref, scale;      // FP16 deviation storage: rest density and scale
    double rk_weight2;     // 1/sqrt(2)/36 evaluated on the host
    void *f;               // species 1 PDFs (19 planes)
    void *g;               // species 2 PDFs (19 planes), multiphase only
    // phase field and colour-gradient fields: double, or float in the multiphase
    // FP32 form (element size felt)
    void *phi;             // halo 4
    void *cn;                         // halo 2: Nrm<T> records (cn_x, cn_y, cn_z, c_norm)
    void *curv;            // halo 1
    int felt;
    double *u, *v, *w, *rho;          // halo 1, FP64 in every form
    int8_t *walls;         // halo 2
    double *w_in;          // (nx+2)(ny+2)
    double *fconv, *gconv, *phiconv;
    const SolidBnd *sb;
    const SolidBndC *sbc;     // compact form of sb (nullptr: a neighbour list is not ascending)
    int glist;                // 1: the packed fluid-cell lists below are valid
    int gsplit;               // 1: curvature and wetting in their own kernels (MFLBM_SPLIT_GRADIENT)
    int gtile;                // 1: normals and curvature by the shared-memory plane-marching
                              //    kernels (default build; the double-word form keeps the lists)
    const uint32_t *gcell_n;  // fluid cells of [-1, n+2]^3 (walls != 1), packed: normals
    int n_gcell_n;
    const uint32_t *gcell_c;  // fluid cells of [1, n]^3 (walls == 0), packed: curvature
    int n_gcell_c;
    int gwet;                 // 1: gcell_n starts with the fluid-boundary nodes in record
                              // order (entry t < nf is record t), so the normals kernel applies
                              // the wetting itself; 0: the separate wetting kernel
    int ns;
    const FluidBnd *fb;
    int nf;
    double *mon;           // MON_NQ * nz slice partials
    double *stage;         // one FP64 plane of the halo-1 box (conversion staging)
    const int32_t *cells;  // padded-layout index of every interior fluid node, ascending
    int ncell;
    // fluid-list layout (singlephase samples that are periodic or walled in every
    // direction): f holds 19 arrays of lstride elements, see listlayout.h
    int list;
    int64_t lstride;
    const int32_t *nb;     // [18][nfl]
    const int32_t *cell1;  // halo-1 index of every fluid node
    const int32_t *link;   // [nlink][3]
    int64_t nlink;
    int nfl;
    const int32_t *lseg;   // [nz+1] first fluid index of every z slice
    // tensor map of the list arrays for the TMA even step: a 2-D tensor of 19 rows (one per
    // direction array, row pitch lstride elements) by nfl fluid nodes; tma = 1 when valid
    // multiphase fluid list (mplist = 1; list = 1 as well): the boundary-condition slot map
    // of every halo-1 cell and the spare slot; the exchange of the porous-plate planes'
    // private y ghosts, nwrap x {ghost 0, image ny, ghost ny+1, image 1} (listlayout.h,
    // MpListLayout)
    int mplist;
    const int32_t *pmap;
    int64_t pspare;
    const int32_t *pwrap;
    int64_t nwrap;
    CUtensorMap tmap;
    int tma;
    int32_t *err;          // device word set when a bounded wait of a sweep kernel gave up
    MrtFold<double> fold;    // singlephase MRT coefficients of the default build (FP64 collision)
    MrtFold<float> fold32;   // the same, converted once on the host for FP32 collision
    MrtFold<ff> foldff;      // the same as double words (MFLBM_FP64FF collision)
    MpConstFF mpff;          // multiphase run constants as double words (MFLBM_FP64FF)
    int unit;                // 1: fold_is_unit(fold), the collision skips the zero terms
};

struct KernelTable {
    // every launcher returns the number of kernels it launched
    // one collision+streaming sweep over the interior (kernel_even / kernel_odd)
    int (*collide)(const DevState &, bool odd, cudaStream_t);
    // periodic halo exchange after the sweep: pull after even, push after odd
    int (*wrap)(const DevState &, bool pull, cudaStream_t);
    // inlet/outlet/porous-plate boundary conditions
    int (*boundary)(const DevState &, bool before_odd, int inlet_bc, int outlet_bc, bool open_z, cudaStream_t);
    // color_gradient: extrapolation, normals, wetting, normal extrapolation, curvature
    int (*color_gradient)(const DevState &, cudaStream_t);
    // compute_macro_vars + per-slice reductions into st.mon
    int (*monitor)(const DevState &, cudaStream_t);
    // cal_saturation per-slice partials into st.mon (2*nz)
    int (*saturation)(const DevState &, cudaStream_t);
    // equilibrium at rest over the halo'd box, then the convective-outlet memory
    int (*init_equilibrium)(const DevState &, bool convec, cudaStream_t);
    // FP64 plane <-> storage plane (q of species s) through st.stage
    int (*convert_in)(const DevState &, int species, int q, cudaStream_t);
    int (*convert_out)(const DevState &, int species, int q, cudaStream_t);
    // FP64 image in st.stage <-> field array (phi, gradient fields) of n elements; field_out
    // reads every stride-th element (4: one component of the Nrm records)
    int (*field_in)(const DevState &, void *dst, int64_t n, cudaStream_t);
    int (*field_out)(const DevState &, const void *src, int64_t n, int stride, cudaStream_t);
    // ensembles (fluid-list arena of many singlephase samples), storage by prec:
    // persistent != 0: one cooperative launch of a.nsteps steps on `grid` blocks;
    // else a.nsteps launches of one step each.  Returns kernels launched, -1 on a
    // launch error.
    int (*ens_run)(const EnsArgs &a, int prec, int persistent, int grid, int block, cudaStream_t);
    // per-sample sums into out[m * nseg + b] (m = 0 sum w, 6 sum rho, 7 max |u|^2)
    int (*ens_monitor)(const EnsArgs &a, int prec, const int32_t *seg0, const int32_t *seg1, int nseg, double *out,
                       cudaStream_t);
    // rest equilibrium in every slot
    int (*ens_init)(const EnsArgs &a, int prec, cudaStream_t);
    // largest co-resident grid of the persistent kernel for this block size
    int (*ens_max_grid)(int prec, int block);
    // singlephase state from rho (device halo-1 array, nullable) and st.u, st.v, st.w
    int (*init_velocity)(const DevState &, const double *rho, int rest_base, cudaStream_t);
    // steady-state / breakthrough partials into out[7 * nz] (phi_old nullable)
    int (*steady)(const DevState &, void *phi_old, double *out, int obs_z, int copy_old, cudaStream_t);
    // change_inlet_fluid_phase over the halo-1 planes k = 0..kmax (cmd 1: into f, 2: into g)
    int (*change_inlet_phase)(const DevState &, int cmd, int kmax, cudaStream_t);
    // writes the curv field when the collision computes each node's curvature itself
    // (before get_gradient reads it; the monitor does this on its own); 0 otherwise
    int (*curvature_field)(const DevState &, cudaStream_t);
};

const KernelTable *kernels_fast();
const KernelTable *kernels_strict();

constexpr int kMonNQ = 10;

}  // namespace mflbm
