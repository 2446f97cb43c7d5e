/*
 * mflbm.h -- C ABI of the GB300 lattice-Boltzmann step library (libmflbm.so).
 *
 * The library replaces the per-time-step device work of MF-LBM's two Fortran
 * programs, multiphase_3D and singlephase_3D, on one GPU:
 *
 *   - the OpenACC data region and the per-step kernels it encloses
 *     (multiphase_3D/0.src/Main_multiphase.F90:104-115, 120-122, 167, 325;
 *      singlephase_3D/0.src/Main.F90:98-103, 140, 278),
 *   - main_iteration_kernel (Main_multiphase.F90:341-486; Main.F90:291-422),
 *     including the inlet/outlet/porous-plate boundary conditions and the
 *     single-rank periodic halo exchange that the reference performs through
 *     MPI messages to itself (multiphase_3D/0.src/Mpi.F90:101-867),
 *   - color_gradient (multiphase_3D/0.src/Phase_gradient.F90:5-265),
 *   - compute_macro_vars (multiphase_3D/0.src/Misc.F90:372-430;
 *     singlephase_3D/0.src/Misc.F90:368-423) and the device-side reductions of
 *     monitor / cal_saturation (multiphase_3D/0.src/Monitor.F90:5-85, 512-550;
 *     singlephase_3D/0.src/Monitor.F90:4-59).
 *
 * The Fortran host keeps deck parsing, geometry preprocessing, initialisation,
 * file I/O and the time loop, and calls these entry points through
 * ISO_C_BINDING (the mechanism the reference already uses for gethostid,
 * multiphase_3D/0.src/Misc.F90:442-447).
 *
 * Conventions
 *   - Every array crossing the ABI uses the reference's halo'd Fortran layout
 *     (column-major, i fastest):
 *       PDFs f_q, g_q, curv, u, v, w, rho : (1-1:n+1) in x, y, z  (halo 1)
 *       phi                               : (1-4:n+4)             (halo 4)
 *       cn_x, cn_y, cn_z, c_norm, walls   : (1-2:n+2)             (halo 2)
 *       w_in, phi_convec_bc               : (0:nx+1, 0:ny+1)
 *       f_convec_bc, g_convec_bc          : (0:nx+1, 0:ny+1, 0:18)
 *   - All functions return MFLBM_OK (0) on success or a negative MFLBM_E* code;
 *     mflbm_last_error() then holds a one-line message.
 *   - One host thread per context; calls on one context are not thread-safe.
 *     mflbm_step / mflbm_run are asynchronous on the context's CUDA stream;
 *     every call that returns data to the host synchronises first.
 *   - Host pointers are only read or written during the call.
 *   - ntime keeps the reference's meaning: even = in-place collision, odd =
 *     streaming collision (AA pattern); the state is in natural order only
 *     after even steps (multiphase_3D/0.src/Init_multiphase.F90:155-159).
 */
#ifndef MFLBM_H
#define MFLBM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFLBM_ABI_VERSION 2

/* status codes */
#define MFLBM_OK        0
#define MFLBM_EINVAL   -1   /* invalid argument or parameter combination            */
#define MFLBM_ECUDA    -2   /* CUDA runtime error (message in mflbm_last_error)     */
#define MFLBM_ENOMEM   -3   /* device allocation failed                             */
#define MFLBM_ESTATE   -4   /* call out of order (e.g. step before set_geometry)    */
#define MFLBM_ETIMEOUT -5   /* a bounded device-side wait gave up                   */
#define MFLBM_ENODEV   -6   /* no usable CUDA device                                */
#define MFLBM_ERANGE   -7   /* a size exceeds a documented limit                    */

/* simulation_end_indicator values reported by mflbm_monitor
 * (multiphase_3D/0.src/Monitor.F90:253-259) */
#define MFLBM_RUNNING 0
#define MFLBM_FAILED  3

/* PDF storage precision */
#define MFLBM_FP64 0   /* plain drop-in: FP64 storage, FP64 collision               */
#define MFLBM_FP32 1   /* FP32 storage, FP32 collision                              */
#define MFLBM_FP16 2   /* FP16 storage of scaled deviations from the rest state, FP32 collision */
#define MFLBM_FP64FF 3 /* FP64 storage, collision in double-word (two-FP32, about 48-bit)
                          arithmetic on the FP32 pipe; every other kernel as MFLBM_FP64
                          (singlephase and multiphase) */
#define MFLBM_FF 4     /* double-word storage (hi + lo FP32 pair per population, 8 bytes,
                          about 48 bits) and the double-word collision; multiphase: also the
                          double-word normal and curvature stencils on FP64 fields */

/* PDF storage layout (no counterpart in the reference, which stores every cell).
 * DENSE: one plane per direction over the halo-1 box, as the reference's arrays.
 * LIST:  only the fluid nodes plus one slot per solid bounce-back link, with an
 *        18-entry neighbour table; with an open z direction (inlet / outlet conditions)
 *        or a porous plate, the cells of the planes those conditions address keep their
 *        own slots.  Multiphase runs with any boundary conditions; singlephase runs with
 *        walls in x when z is open.  Same update, same results on every fluid node;
 *        downloads give the other slots, which no update reads, the rest weight w_q.
 * AUTO:  LIST when the geometry allows it, else DENSE (decided by mflbm_set_geometry). */
#define MFLBM_LAYOUT_AUTO  0
#define MFLBM_LAYOUT_DENSE 1
#define MFLBM_LAYOUT_LIST  2

/* Run parameters: the subset of simulation_control.txt that the per-step path
 * reads, after the reference's own host-side derivations
 * (multiphase_3D/0.src/Init_multiphase.F90:116-150, IO_multiphase.F90:467-468;
 *  singlephase_3D/0.src/Initialization.F90:80-129). */
typedef struct mflbm_params {
    int32_t abi_version;      /* must be MFLBM_ABI_VERSION                                 */
    int32_t multiphase;       /* 1: multiphase_3D colour-gradient model, 0: singlephase_3D */
    int32_t nx, ny, nz;       /* lattice_dimensions (one device holds the whole domain)    */
    int32_t iper, jper, kper; /* periodic_indicator; iper=1 is an extension (singlephase)  */
    int32_t wall_x_min, wall_x_max;   /* domain_wall_status_x                             */
    int32_t wall_y_min, wall_y_max;   /* domain_wall_status_y                             */
    int32_t wall_z_min, wall_z_max;   /* domain_wall_status_z                             */
    int32_t inlet_bc;         /* 1 velocity (bounce-back), 2 Zou-He pressure               */
    int32_t outlet_bc;        /* 1 convective, 2 Zou-He pressure                           */
    int32_t mrt;              /* multiphase: the compile-time `mrt` switch (1..4, ref. 2)
                                 singlephase: MRT_collision_parameter_preset               */
    int32_t porous_plate_cmd; /* 0 none, 1 block fluid 1, 2 block fluid 2                  */
    int32_t z_porous_plate;   /* plane index of the porous plate                           */
    int32_t precision;        /* MFLBM_FP64 / FP32 / FP16 / FP64FF / FF                    */
    int32_t strict_fp;        /* 1: no FMA contraction (bit-identical to an IEEE restatement) */
    int32_t device;           /* CUDA device ordinal                                       */
    int32_t layout;           /* PDF storage layout: MFLBM_LAYOUT_AUTO / _DENSE / _LIST        */
    double  la_nu1;           /* fluid1_viscosity (singlephase: fluid_viscosity)           */
    double  la_nu2;           /* fluid2_viscosity                                          */
    double  gamma;            /* surface_tension                                           */
    double  beta;             /* RK_beta                                                   */
    double  sa_inject;        /* saturation_injection (phi_inlet = 2*sa_inject-1)          */
    double  force_z;          /* effective body force along z (force_Z)                    */
    double  uin_avg;          /* average inlet velocity; convective outlet speed           */
    double  rho_in;           /* inlet density for inlet_bc=2                              */
    double  rho_out;          /* outlet density for outlet_bc=2 (reference: 1)             */
    double  relaxation;       /* `relaxation` (reference: 1)                               */
} mflbm_params;

/* One solid-boundary node: the Fortran derived type indirect_solid_boundary_nodes
 * (multiphase_3D/0.src/Module.F90:90-94), 96 bytes, local halo'd coordinates. */
typedef struct mflbm_solid_bnd {
    int32_t ix, iy, iz, i_fluid_num;
    int32_t neighbor_list[18];   /* D3Q19 direction indices 1..18 of fluid neighbours */
    double  la_weight;
} mflbm_solid_bnd;

/* One fluid-boundary node: indirect_fluid_boundary_nodes
 * (multiphase_3D/0.src/Module.F90:98-101), 48 bytes; theta in radians after the
 * reference's (180-theta)*pi/180 transform (IO_multiphase.F90:467-468). */
typedef struct mflbm_fluid_bnd {
    int32_t ix, iy, iz, _pad;
    double  nwx, nwy, nwz, theta;
} mflbm_fluid_bnd;

typedef struct mflbm_ctx mflbm_ctx;

/* Library ABI version (MFLBM_ABI_VERSION). */
int32_t mflbm_version(void);

/* Singlephase state from density and velocity fields (a warm start; no counterpart in
 * the reference): rho, u, v, w are halo-1 FP64 arrays (rho NULL: 1, velocity NULL: 0).
 * Every fluid slot gets rho (base_q + w_q (3 e.u + 4.5 (e.u)^2 - 1.5 u^2)) with base_q the
 * reference's equilibrium weights w_q (rest_base = 0, initialization_new) or the rest
 * state of the reference MRT collision, 4/21, 13/126, 1/63 (rest_base = 1).  A solid slot
 * that a fluid neighbour pushes into (bounce-back link) gets that neighbour's population
 * toward it; other solid slots get base_q.  Requires mflbm_set_geometry.  Synchronises. */
int32_t mflbm_init_velocity(mflbm_ctx *ctx, const double *rho, const double *u, const double *v,
                            const double *w, int32_t rest_base);

/* Storage layout in use: MFLBM_LAYOUT_DENSE or MFLBM_LAYOUT_LIST, or
 * MFLBM_LAYOUT_AUTO while a context has no geometry yet.
 * No counterpart in the reference. */
int32_t mflbm_layout(const mflbm_ctx *ctx);

/* Allocate a context and its device arrays.  Replaces MemAllocate_multi /
 * MemAllocate (Init_multiphase.F90:583-828; singlephase Initialization.F90:380-516)
 * plus the `!$acc data` region entry (Main_multiphase.F90:104-115).
 * Validates the parameter combinations the reference rejects
 * (IO_multiphase.F90:471-541). */
int32_t mflbm_create(const mflbm_params *params, mflbm_ctx **out);

/* Free all device memory (the `!$acc end data` at Main_multiphase.F90:325). */
void mflbm_destroy(mflbm_ctx *ctx);

/* Last error message of ctx, or of the last failed mflbm_create when ctx is NULL. */
const char *mflbm_last_error(const mflbm_ctx *ctx);

/* Upload the geometry: walls (int8, halo 2, after set_walls' halo transport,
 * multiphase_3D/0.src/Misc.F90:6-210), the solid/fluid boundary lists from
 * geometry_preprocessing_new/_load (Geometry_preprocessing.F90:9-685; ignored
 * for singlephase, may be NULL/0) and the inlet profile w_in (nullable when the
 * inlet is not a velocity inlet). */
int32_t mflbm_set_geometry(mflbm_ctx *ctx, const int8_t *walls,
                           const mflbm_solid_bnd *solid, int32_t n_solid,
                           const mflbm_fluid_bnd *fluid, int32_t n_fluid,
                           const double *w_in);

/* Upload the full halo'd state (copyin of the `!$acc data` region).
 * f[19] / g[19] are arrays of 19 pointers; g, phi and the convective arrays are
 * NULL for singlephase; the convective arrays are required when outlet_bc==1. */
int32_t mflbm_upload_state(mflbm_ctx *ctx, const double *const *f, const double *const *g,
                           const double *phi, const double *f_convec,
                           const double *g_convec, const double *phi_convec);

/* Download the full halo'd state (the `!$acc update host` of save_checkpoint,
 * IO_multiphase.F90:568-571).  NULL pointers are skipped. */
int32_t mflbm_download_state(mflbm_ctx *ctx, double *const *f, double *const *g, double *phi,
                             double *f_convec, double *g_convec, double *phi_convec);

/* Device-side initialisation_new_multi_pdf / initialization_new_pdf with
 * u=v=w=0, rho=1 over the halo'd box, plus the convective-outlet memory
 * (Init_multiphase.F90:357-470; singlephase Initialization.F90:240-309).
 * phi (halo 4) is required for multiphase and ignored for singlephase. */
int32_t mflbm_init_equilibrium(mflbm_ctx *ctx, const double *phi);

/* change_inlet_fluid_phase (multiphase_3D/0.src/Misc.F90:507-621), which the reference
 * calls once after initialisation or restart when change_inlet_fluid_phase_cmd /= 0
 * (Main_multiphase.F90:96-99): in every slot of the halo-1 box with z <= interface_z0,
 * cmd 1 moves all of g into f (f <- f + g, g <- 0), cmd 2 all of f into g; cmd 0 does
 * nothing.  phi is left as it is (the next collision recomputes it).  Synchronises. */
int32_t mflbm_change_inlet_fluid_phase(mflbm_ctx *ctx, int32_t cmd, double interface_z0);

/* One main_iteration_kernel for time step ntime (asynchronous). */
int32_t mflbm_step(mflbm_ctx *ctx, int32_t ntime);

/* nsteps consecutive steps ntime0 .. ntime0+nsteps-1, replayed from a captured
 * CUDA graph of one even+odd pair (asynchronous). */
int32_t mflbm_run(mflbm_ctx *ctx, int32_t ntime0, int32_t nsteps);

/* color_gradient (multiphase only): phi extrapolation, normals, wetting,
 * normal extrapolation, curvature.  Called once after upload, as
 * Main_multiphase.F90:120 does. */
int32_t mflbm_color_gradient(mflbm_ctx *ctx);

/* Download cn_x, cn_y, cn_z, c_norm (halo 2) and curv (halo 1); NULL skips. */
int32_t mflbm_get_gradient(mflbm_ctx *ctx, double *cn_x, double *cn_y, double *cn_z,
                           double *c_norm, double *curv);

/* compute_macro_vars, then download u, v, w, rho (halo 1, NULL skips) and,
 * for multiphase, phi (halo 4, NULL skips).  Like the reference this zeroes
 * phi at wall nodes.  Valid after even steps only. */
int32_t mflbm_macro(mflbm_ctx *ctx, double *u, double *v, double *w, double *rho,
                    double *phi);

/* compute_macro_vars + the device reductions of monitor.
 * multiphase: profiles[7*nz] = fl1, fl2, vol1, vol2, mass1, mass2, pre (per z slice);
 *             scalars[3]     = umax^2, usq1, usq2.
 * singlephase: profiles[2*nz] = fl, pre;  scalars[3] = umax^2, 0, 0.
 * *status = MFLBM_FAILED when a sum is NaN or sqrt(umax^2) > 0.5, else MFLBM_RUNNING.
 * Sums accumulate in FP64 in every precision mode. */
int32_t mflbm_monitor(mflbm_ctx *ctx, double *profiles, double *scalars, int32_t *status);

/* The other monitors of the multiphase loop (Main_multiphase.F90:184-195):
 * kind 0: phi_old <- phi, the set-up of steady_state_option 2 (Init_multiphase.F90:340-351);
 * kind 1: monitor_multiphase_steady_capillarypressure (Monitor.F90:370-462),
 *         out[6] = pc, pre_w, pre_nw, umax, count_w, count_nw;
 * kind 2: monitor_multiphase_steady_phasefield (:287-365), out[2] = max |phi - phi_old| over
 *         the fluid nodes, umax; then phi_old <- phi;
 * kind 3: monitor_breakthrough (:472-507), out[1] = fluid nodes with phi > 0 at z = nz - 1.
 * Kinds 1 and 2 run compute_macro_vars first.  FP64 sums in every precision. */
int32_t mflbm_steady_monitor(mflbm_ctx *ctx, int32_t kind, double *out);

/* cal_saturation (multiphase_3D/0.src/Monitor.F90:512-550): vol1, vol2 sums. */
int32_t mflbm_saturation(mflbm_ctx *ctx, double *vol1, double *vol2);

/* Wait for all work queued on the context's stream. */
int32_t mflbm_synchronize(mflbm_ctx *ctx);

/* Diagnostics for benchmarking; no counterpart in the reference.
 * Starts a measurement region: records a CUDA event on the context's stream and
 * resets the counters below.  enable=1 also makes mflbm_step / mflbm_run launch step
 * by step (no graph replay) with CUDA events around every collision sweep. */
int32_t mflbm_set_profiling(mflbm_ctx *ctx, int32_t enable);

/* Ends the region: device time (ms) since mflbm_set_profiling on the context's
 * stream, the time and number of the timed collision sweeps (profiling mode), and
 * the number of kernels launched by mflbm_step / mflbm_run (graph replays included).
 * Synchronises. */
int32_t mflbm_get_profile(mflbm_ctx *ctx, double *region_ms, double *collide_ms, int64_t *collide_launches,
                          int64_t *kernel_launches);

/* Largest nz that mflbm_saturation_noalloc accepts: its scratch holds two doubles per
 * z slice (256 KiB per device). */
#define MFLBM_NOALLOC_MAX_NZ 16384

/* cal_saturation without a context and without any allocation.  No counterpart in the
 * reference: it is for callers that must not allocate device memory -- a Fortran host
 * whose OpenACC data region owns every device array and passes `use_device` pointers,
 * or a loop that cannot afford cudaMalloc's implicit device-wide synchronisation.
 *   phi   device pointer, halo 4 layout; walls device pointer, halo 2 layout
 *   vol   device pointer to 2 doubles, receives (vol1, vol2) as mflbm_saturation
 *   stream  cudaStream_t to launch on (NULL: legacy default stream); asynchronous
 * Scratch is a fixed __device__ array shared by every call; overlapping calls race.
 * The first call on a device looks up the scratch address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  The address is kept for the life of
 * the process: after cudaDeviceReset on a device, do not call this on that device again.
 * nz > MFLBM_NOALLOC_MAX_NZ returns MFLBM_ERANGE.  A CUDA error already pending from
 * earlier work is reported (MFLBM_ECUDA) and not cleared.  Errors are reported through
 * mflbm_last_error(NULL). */
int32_t mflbm_saturation_noalloc(const double *phi, const int8_t *walls, int32_t nx, int32_t ny, int32_t nz,
                                 double *vol, void *stream);

/* ---------------------------------------------------------------------------------
 * Ensembles: many singlephase samples of uneven sizes updated together in one
 * fluid-list arena (no counterpart in the reference, which runs one sample per job).
 * The samples share `common` (precision, mrt, la_nu1, force_z, periodic and wall flags,
 * strict_fp, device; nx/ny/nz are ignored) and each has its own dims[3*s..3*s+2] = nx, ny, nz and
 * halo-2 wall array walls[s] (Fortran order, 1 = solid).  Every direction must be
 * periodic or walled (no inlet/outlet).  Errors: mflbm_ensemble_last_error.
 * --------------------------------------------------------------------------------- */
typedef struct mflbm_ensemble mflbm_ensemble;

int32_t mflbm_ensemble_create(const mflbm_params *common, int32_t nsamples, const int32_t *dims,
                              const int8_t *const *walls, mflbm_ensemble **out);
void mflbm_ensemble_destroy(mflbm_ensemble *ens);
/* Last error of ens, or of the last failed mflbm_ensemble_create when ens is NULL. */
const char *mflbm_ensemble_last_error(const mflbm_ensemble *ens);
/* Rest state (equilibrium at rho = 1, u = 0) in every sample. */
int32_t mflbm_ensemble_init(mflbm_ensemble *ens);
/* active[s] = 0 drops sample s from the sweep (e.g. once converged); 1 keeps it. */
int32_t mflbm_ensemble_set_active(mflbm_ensemble *ens, const int32_t *active);
/* nsteps time steps of every active sample, starting with ntime0 (odd: stream+collide).
 * Replayed from a CUDA graph captured on first use; asynchronous. */
int32_t mflbm_ensemble_run(mflbm_ensemble *ens, int32_t ntime0, int32_t nsteps);
/* Per-sample sum of w over the fluid nodes and max |u|^2 (valid after even steps);
 * *status = MFLBM_FAILED on NaN or |u| > 0.5 in an active sample.  Returns
 * MFLBM_ETIMEOUT when a grid barrier of the persistent kernel gave up; the PDF state is
 * then undefined, and mflbm_ensemble_init (or mflbm_ensemble_configure) clears the
 * barrier's error word before the next run.  Synchronises. */
int32_t mflbm_ensemble_flux(mflbm_ensemble *ens, double *w_sum, double *umax2, int32_t *status);
/* Launch shape: threads per block (64..1024, multiple of 32) and persistent = 1 for one
 * cooperative launch per run (grid barrier between steps) or 0 for one launch per step. */
int32_t mflbm_ensemble_configure(mflbm_ensemble *ens, int32_t block, int32_t persistent);
/* Times every launch shape over `steps` steps on the ensemble itself and applies the
 * fastest; `report` (may be NULL) receives the timings as JSON.  Changes the PDF
 * state: call mflbm_ensemble_init afterwards. */
int32_t mflbm_ensemble_tune(mflbm_ensemble *ens, int32_t steps, char *report, int32_t report_len);
/* Diagnostics of the persistent kernel's failure path (no counterpart in the reference):
 * spin_limit = polls per grid-barrier wait (<= 0: the default, several seconds), and
 * unreachable = 1 makes every barrier wait for one block more than the grid holds, so
 * each wait runs out and the kernel returns early (mflbm_ensemble_flux then reports
 * MFLBM_ETIMEOUT).  Clears the barrier state and drops captured graphs.  Synchronises. */
int32_t mflbm_ensemble_set_wait(mflbm_ensemble *ens, int64_t spin_limit, int32_t unreachable);
/* Fluid nodes of the active samples and the launch shape in use. */
int32_t mflbm_ensemble_info(const mflbm_ensemble *ens, int64_t *active_nodes, int32_t *block,
                            int32_t *persistent, int32_t *grid);

/* ---------------------------------------------------------------------------------
 * Warm-start network building blocks (no counterpart in the reference).  Device
 * pointers; `stream` is a cudaStream_t (NULL: the legacy default stream); `err` is a
 * device int32 set to nonzero when a bounded device-side wait gave up.
 * --------------------------------------------------------------------------------- */
/* C[M][N] (fp32, row stride ldc) = (accumulate ? C : 0) + A[M][K] * B[N][K]^T with A, B
 * bf16 (row strides lda, ldb), FP32 accumulation on the tcgen05 tensor cores.
 * N % 16 == 0, K % 8 == 0, lda, ldb % 8 == 0, A and B 16-byte aligned. */
int32_t mflbm_nn_gemm_bf16(const void *A, int32_t lda, const void *B, int32_t ldb, float *C, int32_t ldc,
                           int32_t M, int32_t N, int32_t K, int32_t accumulate, int32_t *err, void *stream);
/* The same with the K range split over ksplit CTAs per output tile (long reductions);
 * work holds ksplit * M * N floats. */
int32_t mflbm_nn_gemm_bf16_splitk(const void *A, int32_t lda, const void *B, int32_t ldb, float *C, int32_t ldc,
                                  int32_t M, int32_t N, int32_t K, int32_t accumulate, int32_t ksplit, float *work,
                                  int32_t *err, void *stream);

/* Diagnostics of the GEMM's failure path (no counterpart in the reference): wait_limit =
 * probes per mbarrier wait of later GEMMs (<= 0: the default), skip_commit = 1 makes the
 * MMA thread issue no tensor-core work and no commit, so every wait runs out: the GEMM
 * returns MFLBM_OK, sets *err and leaves its output tiles undefined.  Process-wide. */
int32_t mflbm_nn_set_wait(int64_t wait_limit, int32_t skip_commit);

/* Channels-last activations [D][H][W][C] (bf16 unless stated), 3x3x3 periodic stencil.
 * col[v][tap*Cin + c] = X[v + d_tap][c], zero for k in [27*Cin, Kp). */
int32_t mflbm_nn_im2col(const void *X, int32_t D, int32_t H, int32_t W, int32_t Cin, int32_t Kp, void *col,
                        void *stream);
/* adjoint of im2col: dX[v][c] = sum over taps of dcol[v - d_tap][tap*Cin + c] (fp32) */
int32_t mflbm_nn_col2im(const float *dcol, int32_t D, int32_t H, int32_t W, int32_t Cin, int32_t Kp, float *dX,
                        void *stream);
/* out[r][c] (bf16, ld_out) = in[c][r] (fp32 when in_f32, else bf16), zero-padded to Rp x Cp */
int32_t mflbm_nn_transpose_bf16(const void *in, int32_t in_f32, int64_t ld_in, int64_t R, int64_t C, void *out,
                                int64_t ld_out, int64_t Rp, int64_t Cp, void *stream);
/* y = act(acc + bias): pre (fp32, nullable), Y (bf16, nullable), Yf (fp32, nullable); relu 0/1 */
int32_t mflbm_nn_bias_act(const float *acc, const float *bias, float *pre, void *Y, float *Yf, int64_t nvox,
                          int32_t N, int32_t ld_acc, int32_t relu, void *stream);
int32_t mflbm_nn_relu_back(float *g, const float *pre, int64_t n, void *stream);
int32_t mflbm_nn_bias_grad(const float *g, float *db, int64_t nvox, int32_t N, void *stream);
int32_t mflbm_nn_avgpool2(const void *X, void *Y, int32_t D, int32_t H, int32_t W, int32_t C, void *stream);
int32_t mflbm_nn_avgpool2_back(const float *dY, float *dX, int32_t D, int32_t H, int32_t W, int32_t C, void *stream);
/* Y (C1 + C2 channels, fine grid D x H x W) = [nearest x2 upsampling of Xc, S] */
int32_t mflbm_nn_up2_concat(const void *Xc, int32_t C1, const void *S, int32_t C2, void *Y, int32_t D, int32_t H,
                            int32_t W, void *stream);
int32_t mflbm_nn_up2_concat_back(const float *dY, float *dXc, int32_t C1, float *dS, int32_t C2, int32_t D,
                                 int32_t H, int32_t W, void *stream);
int32_t mflbm_nn_add(float *a, const float *b, int64_t n, void *stream);
int32_t mflbm_nn_to_bf16(const float *a, void *b, int64_t n, void *stream);
/* masked MSE: g = 2 mask (pred - target) * inv_count for the first C channels of pred/g
 * (row stride ldp); partial[ceil(nvox*C/256)] receives sums of squares */
int32_t mflbm_nn_mse(const float *pred, int32_t ldp, const float *target, const float *mask, float *g,
                     double *partial, int64_t nvox, int32_t C, float inv_count, void *stream);
/* one Adam step on fp32 weights w (and their bf16 copy wb, nullable); step counts from 1 */
int32_t mflbm_nn_adam(float *w, const float *g, float *m, float *v, void *wb, int64_t n, float lr, float b1, float b2,
                      float eps, int32_t step, void *stream);

/* ---------------------------------------------------------------------------------
 * geometry_preprocessing_new on the GPU (multiphase_3D/0.src/Geometry_preprocessing.F90:
 * 9-512 for one rank): from the global wall array after channel walls (nx*ny*nz int8,
 * Fortran order, 1 = solid) to the solid- and fluid-boundary lists of mflbm_set_geometry,
 * in the reference's order, theta (radians, after the reference's transform) on every
 * fluid-boundary node.  Pass NULL lists (or too small capacities) to learn the counts
 * in *n_solid / *n_fluid (MFLBM_ERANGE when a list did not fit).  Periodic dimensions
 * must be at least 10 cells.  Errors: mflbm_preprocess_last_error().
 * --------------------------------------------------------------------------------- */
int32_t mflbm_preprocess_geometry(const mflbm_params *params, const int8_t *walls, double theta,
                                  mflbm_solid_bnd *solid, int32_t solid_cap, int32_t *n_solid,
                                  mflbm_fluid_bnd *fluid, int32_t fluid_cap, int32_t *n_fluid);
const char *mflbm_preprocess_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* MFLBM_H */
