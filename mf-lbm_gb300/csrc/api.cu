// api.cu -- the C ABI of libmflbm.so (declared in include/mflbm.h).
//
// One mflbm_ctx owns one CUDA stream and every device array of one simulation.  The
// ordering of a time step follows main_iteration_kernel
// (multiphase_3D/0.src/Main_multiphase.F90:341-486; singlephase_3D/0.src/Main.F90:291-422):
//   collision sweep (even: in place, odd: AA streaming)
//   -> periodic halo exchange (pull after even, push after odd; phi after both)
//   -> inlet/outlet BCs (_before_odd after even, _after_odd after odd) and porous plate
//   -> color_gradient (multiphase)
// mflbm_run replays the same launches from CUDA graphs captured once per context.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/mflbm.h"
#include "kernels_api.h"
#include "listlayout.h"

using namespace mflbm;

struct mflbm_ctx {
    mflbm_params p{};
    int dev = 0;
    cudaStream_t stream = nullptr;
    const KernelTable *kt = nullptr;
    DevState st{};
    size_t elt = 8;
    std::vector<void *> allocs;
    bool have_geometry = false;
    bool open_z = false;
    int64_t cells_cap = 0;
    int64_t gn_cap = 0, gc_cap = 0, sbc_cap = 0;  // capacities of the colour-gradient lists
    int64_t stage_len = 0;                         // FP64 elements of st.stage
    SolidBndC *sbc_buf = nullptr;
    void *pdf = nullptr;          // PDF storage (dense planes or fluid-list arrays)
    size_t pdf_bytes = 0;
    std::vector<void *> list_bufs;  // neighbour table, cell map, link table, slice starts
    void *phi_old = nullptr;        // steady_state_option 2 (allocated on first use)
    double *steady_part = nullptr;  // 7 * nz partials
    // graphs of whole even+odd step pairs
    cudaGraphExec_t g_pair = nullptr, g_block = nullptr;
    int block_pairs = 8;
    std::vector<double> h_mon;
    std::string err;
    // diagnostics: kernel launch count; optional CUDA-event timing of collision sweeps
    int64_t launches = 0;
    int64_t pair_launches = 0, block_launches = 0;  // kernels per captured graph
    bool profiling = false;
    cudaEvent_t region0 = nullptr, region1 = nullptr;  // bracket the region since set_profiling
    std::vector<cudaEvent_t> ev;   // 2 * kEventRing, pairs around each collision sweep
    int ev_used = 0;
    double collide_ms = 0.0;
    int64_t collide_count = 0;
};

static const int kEventRing = 512;
// fluid fraction above which the colour-gradient stencils run as shared-memory tiles
// (measured: lists faster on the C1 tube, 63 % fluid, 4,378 against 3,717 MLUPS in FP32,
// and on the porous packings; tiles for nearly open domains such as free drops)
static const double kGradientTileFraction = 0.9;

static thread_local std::string g_last_create_error;

namespace mflbm {
// errors of calls that have no context land in the same slot as mflbm_create's
void set_global_error(const std::string &msg) { g_last_create_error = msg; }
}  // namespace mflbm

namespace {

int fail(mflbm_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg; else g_last_create_error = msg;
    return code;
}

int cuda_fail(mflbm_ctx *c, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(c, e == cudaErrorMemoryAllocation ? MFLBM_ENOMEM : MFLBM_ECUDA, m);
}

#define CK(ctx, expr)                                             \
    do {                                                          \
        cudaError_t e_ = (expr);                                  \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #expr); \
    } while (0)

int64_t n1(const mflbm_params &p) { return (int64_t)(p.nx + 2) * (p.ny + 2) * (p.nz + 2); }
// the PDFs are stored as FP64 (the plain form and the double-word collision form)
bool f64_storage(const mflbm_params &p) { return p.precision == MFLBM_FP64 || p.precision == MFLBM_FP64FF; }
int64_t n2(const mflbm_params &p) { return (int64_t)(p.nx + 4) * (p.ny + 4) * (p.nz + 4); }
int64_t n4(const mflbm_params &p) { return (int64_t)(p.nx + 8) * (p.ny + 8) * (p.nz + 8); }
int64_t nplane(const mflbm_params &p) { return (int64_t)(p.nx + 2) * (p.ny + 2); }

// parameter checks of read_parameter_multi / read_parameter
// (multiphase_3D/0.src/IO_multiphase.F90:471-541; singlephase_3D/0.src/IO.F90:393-451)
int validate(const mflbm_params *p, std::string &err) {
    if (!p) { err = "params is NULL"; return MFLBM_EINVAL; }
    if (p->abi_version != MFLBM_ABI_VERSION) { err = "abi_version mismatch"; return MFLBM_EINVAL; }
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) { err = "lattice dimensions must be >= 3"; return MFLBM_EINVAL; }
    if ((int64_t)p->nx * p->ny > ((int64_t)1 << 30) || p->nz > 65000 || p->ny > 65000) {
        err = "lattice dimensions exceed the launch-grid limits"; return MFLBM_ERANGE;
    }
    if (p->multiphase) {
        if (p->iper == 1 || p->wall_x_max == 0 || p->wall_x_min == 0) {
            err = "X direction periodic BC enabled or non-slip BC not applied at x = xmin or x = xmax";
            return MFLBM_EINVAL;
        }
        if (p->mrt < 1 || p->mrt > 4) { err = "mrt must be 1..4"; return MFLBM_EINVAL; }
        if (p->precision == MFLBM_FP16) {
            err = "multiphase supports MFLBM_FP64 and MFLBM_FP32 storage (FP16 deviations cannot hold a vanishing species)";
            return MFLBM_EINVAL;
        }
        if (p->la_nu2 <= 0.0) { err = "la_nu2 must be positive"; return MFLBM_EINVAL; }
    } else {
        if (p->iper == 1 && (p->wall_x_max == 1 || p->wall_x_min == 1)) {
            err = "non-slip BC applied at x = xmin or x = xmax while x direction periodic BC enabled";
            return MFLBM_EINVAL;
        }
        if (p->iper == 0 && (p->wall_x_max == 0 || p->wall_x_min == 0)) {
            err = "non-slip BC not applied at x = xmin or x = xmax while x direction periodic BC not enabled";
            return MFLBM_EINVAL;
        }
    }
    if (p->jper == 0 && (p->wall_y_max == 0 || p->wall_y_min == 0)) {
        err = "non-slip BC not applied at y = ymin or y = ymax while y direction periodic BC not enabled";
        return MFLBM_EINVAL;
    }
    if (p->jper == 1 && (p->wall_y_max == 1 || p->wall_y_min == 1)) {
        err = "non-slip BC applied at y = ymin or y = ymax while y direction periodic BC enabled";
        return MFLBM_EINVAL;
    }
    if (p->kper == 1 && (p->wall_z_max == 1 || p->wall_z_min == 1)) {
        err = "non-slip BC applied at z = zmin or z = zmax while z direction periodic BC enabled";
        return MFLBM_EINVAL;
    }
    if (p->outlet_bc == 1 && p->inlet_bc == 2) {
        err = "Inlet pressure + outlet convective BC is not supported";
        return MFLBM_EINVAL;
    }
    if (p->precision < MFLBM_FP64 || p->precision > MFLBM_FF) { err = "unknown precision"; return MFLBM_EINVAL; }
    if (p->layout < MFLBM_LAYOUT_AUTO || p->layout > MFLBM_LAYOUT_LIST) { err = "unknown layout"; return MFLBM_EINVAL; }
    if (p->layout == MFLBM_LAYOUT_LIST && !p->multiphase && p->iper && p->kper == 0 && p->wall_z_min == 0 &&
        p->wall_z_max == 0) {
        err = "the singlephase fluid-list layout with an open z direction needs walls in x";
        return MFLBM_EINVAL;
    }
    if (p->la_nu1 <= 0.0) { err = "la_nu1 must be positive"; return MFLBM_EINVAL; }
    return MFLBM_OK;
}

// A new device buffer, zero-filled.  The fill completes before the call returns: the
// context's stream is non-blocking, so a zero fill still queued on it is not ordered
// against the plain cudaMemcpy that set_geometry then uses to fill the same buffer (a table
// zeroed after its upload sent every thread of the gradient kernels to one cell outside the
// box).  Allocation is not on the time-stepping path.
int dalloc_bytes(mflbm_ctx *c, void **ptr, size_t bytes) {
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
    c->allocs.push_back(p);
    e = cudaMemsetAsync(p, 0, bytes, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync");
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamSynchronize");
    *ptr = p;
    return MFLBM_OK;
}

template <class T> int dalloc(mflbm_ctx *c, T **ptr, int64_t count) {
    void *p = nullptr;
    const int r = dalloc_bytes(c, &p, (size_t)count * sizeof(T));
    if (r) return r;
    *ptr = reinterpret_cast<T *>(p);
    return MFLBM_OK;
}

// cudaFree one tracked allocation
void dfree(mflbm_ctx *c, void *ptr) {
    if (!ptr) return;
    for (size_t t = 0; t < c->allocs.size(); ++t)
        if (c->allocs[t] == ptr) {
            cudaFree(ptr);
            c->allocs.erase(c->allocs.begin() + (long)t);
            return;
        }
}

// (re)allocate the PDF storage; zero-filled
int alloc_pdf(mflbm_ctx *c, size_t bytes) {
    if (c->pdf && c->pdf_bytes == bytes) return MFLBM_OK;
    dfree(c, c->pdf);
    c->pdf = nullptr;
    c->pdf_bytes = 0;
    int r = dalloc_bytes(c, &c->pdf, bytes);
    if (r) return r;
    c->pdf_bytes = bytes;
    return MFLBM_OK;
}

// the dense planes of one or two species
int alloc_dense(mflbm_ctx *c) {
    const int nsp = c->p.multiphase ? 2 : 1;
    const size_t plane = (size_t)19 * c->st.L.qs * c->elt;
    int r = alloc_pdf(c, nsp * plane);
    if (r) return r;
    c->st.f = c->pdf;
    c->st.g = c->p.multiphase ? (void *)((char *)c->pdf + plane) : nullptr;
    c->st.list = 0;
    c->st.mplist = 0;
    c->st.pmap = nullptr;
    c->st.pwrap = nullptr;
    c->st.nwrap = 0;
    c->st.tma = 0;
    return MFLBM_OK;
}

void drop_graphs(mflbm_ctx *c) {
    if (c->g_pair) cudaGraphExecDestroy(c->g_pair);
    if (c->g_block) cudaGraphExecDestroy(c->g_block);
    c->g_pair = c->g_block = nullptr;
}

// fold the recorded event pairs into the running totals
int drain_events(mflbm_ctx *c) {
    if (c->ev_used == 0) return MFLBM_OK;
    CK(c, cudaStreamSynchronize(c->stream));
    for (int t = 0; t < c->ev_used; ++t) {
        float ms = 0.f;
        CK(c, cudaEventElapsedTime(&ms, c->ev[2 * t], c->ev[2 * t + 1]));
        c->collide_ms += ms;
    }
    c->collide_count += c->ev_used;
    c->ev_used = 0;
    return MFLBM_OK;
}

// launches of one main_iteration_kernel; no synchronisation, capturable unless
// profiling (which brackets the collision sweep with events); returns kernels launched
int enqueue_step(mflbm_ctx *c, int32_t ntime) {
    const bool even = (ntime % 2) == 0;
    int n = 0;
    const bool timed = c->profiling;
    if (timed) {
        if (c->ev_used == kEventRing && drain_events(c)) return -1;
        cudaEventRecord(c->ev[2 * c->ev_used], c->stream);
    }
    n += c->kt->collide(c->st, !even, c->stream);
    if (timed) {
        cudaEventRecord(c->ev[2 * c->ev_used + 1], c->stream);
        ++c->ev_used;
    }
    n += c->kt->wrap(c->st, even, c->stream);
    n += c->kt->boundary(c->st, even, c->p.inlet_bc, c->p.outlet_bc, c->open_z, c->stream);
    if (c->p.multiphase) n += c->kt->color_gradient(c->st, c->stream);
    return n;
}

int capture(mflbm_ctx *c, int pairs, cudaGraphExec_t *out, int64_t *nkernels) {
    cudaGraph_t graph = nullptr;
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int64_t n = 0;
    for (int t = 0; t < pairs; ++t) {
        n += enqueue_step(c, 0);
        n += enqueue_step(c, 1);
    }
    *nkernels = n;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
    return MFLBM_OK;
}

int ready(mflbm_ctx *c) {
    if (!c) return MFLBM_EINVAL;
    if (!c->have_geometry) return fail(c, MFLBM_ESTATE, "mflbm_set_geometry must be called first");
    return MFLBM_OK;
}

// The error word of the sweep kernels (set when a bounded wait gave up); read and cleared
// at the calls that synchronise.  Synchronises the context stream.
int check_device_err(mflbm_ctx *c) {
    int32_t e = 0;
    CK(c, cudaMemcpyAsync(&e, c->st.err, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (e) {
        CK(c, cudaMemsetAsync(c->st.err, 0, sizeof(int32_t), c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        return fail(c, MFLBM_ETIMEOUT, "a bounded wait of the TMA list sweep gave up; the PDF state is undefined");
    }
    return MFLBM_OK;
}

// Tensor map of the fluid-list arrays for the TMA even step: dimension 0 the nfl fluid
// nodes (contiguous), dimension 1 the 19 direction arrays (pitch lstride elements), box
// 128 nodes x 19 directions, no swizzle, zero fill outside.  The driver's encoder is
// reached through the runtime's entry-point query (no link against libcuda).  Returns
// false when the encoder is unavailable or rejects the map (the plain sweep then runs).
bool encode_list_map(mflbm_ctx *c) {
    using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static Encode encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return false;
        }
        encode = reinterpret_cast<Encode>(fn);
    }
    const DevState &st = c->st;
    if (st.nfl <= 0) return false;
    const CUtensorMapDataType dt = c->elt == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64
                                 : (c->elt == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16);
    const cuuint64_t dims[2] = {(cuuint64_t)st.nfl, 19};
    const cuuint64_t strides[1] = {(cuuint64_t)st.lstride * c->elt};
    const cuuint32_t box[2] = {128, 19};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(&c->st.tmap, dt, 2, c->pdf, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

extern "C" {

int32_t mflbm_version(void) { return MFLBM_ABI_VERSION; }

int32_t mflbm_layout(const mflbm_ctx *c) {
    if (!c || !c->pdf) return MFLBM_LAYOUT_AUTO;
    return c->st.list ? MFLBM_LAYOUT_LIST : MFLBM_LAYOUT_DENSE;
}

const char *mflbm_last_error(const mflbm_ctx *ctx) {
    return ctx ? ctx->err.c_str() : g_last_create_error.c_str();
}

int32_t mflbm_create(const mflbm_params *params, mflbm_ctx **out) {
    if (!out) return fail(nullptr, MFLBM_EINVAL, "out is NULL");
    *out = nullptr;
    std::string err;
    int rc = validate(params, err);
    if (rc) return fail(nullptr, rc, err);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= 0)
        return fail(nullptr, MFLBM_ENODEV, std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
    if (params->device < 0 || params->device >= ndev) return fail(nullptr, MFLBM_ENODEV, "device ordinal out of range");
    e = cudaSetDevice(params->device);
    if (e != cudaSuccess) return fail(nullptr, MFLBM_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));

    mflbm_ctx *c = new mflbm_ctx();
    c->p = *params;
    c->dev = params->device;
    const mflbm_params &p = c->p;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        g_last_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        delete c;
        return MFLBM_ECUDA;
    }
    c->kt = p.strict_fp ? kernels_strict() : kernels_fast();
    c->open_z = p.kper == 0 && p.wall_z_min == 0 && p.wall_z_max == 0;
    c->elt = p.precision == MFLBM_FP32 ? 4 : (p.precision == MFLBM_FP16 ? 2 : 8);

    // padded PDF layout: i=1 on a 32-byte boundary, rows multiple of 32 bytes
    Layout &L = c->st.L;
    const int A = (int)(32 / c->elt);
    L.nx = p.nx; L.ny = p.ny; L.nz = p.nz;
    L.xo = A - 1;
    L.pitch = ((int64_t)L.xo + p.nx + 2 + A - 1) / A * A;
    L.pz = L.pitch * (p.ny + 2);
    L.qs = L.pz * (p.nz + 2);
    if (L.qs >= ((int64_t)1 << 31)) {
        g_last_create_error = "lattice too large: one PDF plane exceeds 2^31 elements";
        cudaStreamDestroy(c->stream);
        delete c;
        return MFLBM_ERANGE;
    }
    L.h1x = p.nx + 2; L.h1xy = (int64_t)(p.nx + 2) * (p.ny + 2);
    L.h2x = p.nx + 4; L.h2xy = (int64_t)(p.nx + 4) * (p.ny + 4);
    L.h4x = p.nx + 8; L.h4xy = (int64_t)(p.nx + 8) * (p.ny + 8);

    // derived parameters (Init_multiphase.F90:116-128; singlephase Initialization.F90:80-112)
    StepParams &P = c->st.P;
    P.force_z = p.force_z;
    P.gamma = p.gamma;
    P.beta = p.beta;
    P.la_nui1 = 1.0 / p.la_nu1;
    P.la_nui2 = p.multiphase ? 1.0 / p.la_nu2 : 0.0;
    P.sa_inject = p.sa_inject;
    P.phi_inlet = 2.0 * p.sa_inject - 1.0;
    P.uin_avg = p.uin_avg;
    P.rho_in = p.rho_in;
    P.rho_out = p.rho_out;
    P.relaxation = p.relaxation;
    P.mrt = p.mrt;
    P.porous_plate_cmd = p.porous_plate_cmd;
    P.z_porous_plate = p.z_porous_plate;
    P.iper = p.iper; P.jper = p.jper; P.kper = p.kper;
    {
        const double omega = 1.0 / (3.0 * p.la_nu1 + 0.5);
        P.s_nu = omega;
        if (p.mrt == 1) {
            P.s_e = omega; P.s_e2 = omega; P.s_pi = omega;
            P.s_q = 8.0 * (2.0 - omega) / (8.0 - omega);
            P.s_t = P.s_q;
        } else {
            // the reference tests `== 1` twice (Initialization.F90:91-98): other presets are SRT
            P.s_e = omega; P.s_e2 = omega; P.s_pi = omega; P.s_q = omega; P.s_t = omega;
        }
    }
    c->st.fold = fold_rates<double>(P.s_e, P.s_e2, P.s_q, P.s_nu, P.s_pi, P.s_t);
    c->st.fold.fz = P.force_z;
    c->st.fold32 = fold_rates<float>(P.s_e, P.s_e2, P.s_q, P.s_nu, P.s_pi, P.s_t);
    c->st.fold32.fz = (float)P.force_z;
    c->st.foldff = fold_to_ff(c->st.fold);
    c->st.unit = fold_is_unit(c->st.fold) ? 1 : 0;
    c->st.multiphase = p.multiphase;
    c->st.prec = p.precision;
    c->st.felt = (p.multiphase && p.precision == MFLBM_FP32) ? 4 : 8;
    c->st.ref = 1.0f;
    c->st.scale = 4096.0f;
    c->st.rk_weight2 = 1.0 / std::sqrt(2.0) / 36.0;
    c->st.mpff = MpConstFF{ff(0.5 * p.gamma), ff(p.force_z), ff(P.la_nui1), ff(P.la_nui2), ff(p.beta),
                           ff(1.0 / 18.0), ff(c->st.rk_weight2)};

    // device arrays (MemAllocate_multi, Init_multiphase.F90:583-828)
    const int nsp = p.multiphase ? 2 : 1;
    int r = MFLBM_OK;
    (void)nsp;
    // the storage layout is settled by mflbm_set_geometry unless dense is requested
    if (p.layout == MFLBM_LAYOUT_DENSE) {
        if ((r = alloc_dense(c))) goto fail_create;
    }
    if ((r = dalloc(c, &c->st.walls, n2(p)))) goto fail_create;
    if ((r = dalloc(c, &c->st.w_in, nplane(p)))) goto fail_create;
    if ((r = dalloc(c, &c->st.fconv, nplane(p) * 19))) goto fail_create;
    if ((r = dalloc(c, &c->st.u, n1(p)))) goto fail_create;
    if ((r = dalloc(c, &c->st.v, n1(p)))) goto fail_create;
    if ((r = dalloc(c, &c->st.w, n1(p)))) goto fail_create;
    if ((r = dalloc(c, &c->st.rho, n1(p)))) goto fail_create;
    if ((r = dalloc(c, &c->st.mon, (int64_t)kMonNQ * p.nz))) goto fail_create;
    if ((r = dalloc(c, &c->st.err, 1))) goto fail_create;
    // FP64 staging for the converted uploads/downloads (every context: the normal records
    // are downloaded one component at a time through it): one PDF plane, or the halo-4
    // phase field when that is larger
    c->stage_len = p.multiphase ? std::max(n1(p), n4(p)) : n1(p);
    if ((r = dalloc(c, &c->st.stage, c->stage_len))) goto fail_create;
    if (p.multiphase) {
        const size_t fe = (size_t)c->st.felt;
        if ((r = dalloc_bytes(c, &c->st.phi, fe * n4(p)))) goto fail_create;
        if ((r = dalloc_bytes(c, &c->st.cn, 4 * fe * n2(p)))) goto fail_create;
        if ((r = dalloc_bytes(c, &c->st.curv, fe * n1(p)))) goto fail_create;
        if ((r = dalloc(c, &c->st.gconv, nplane(p) * 19))) goto fail_create;
        if ((r = dalloc(c, &c->st.phiconv, nplane(p)))) goto fail_create;
    }
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { r = cuda_fail(c, e, "cudaStreamSynchronize"); goto fail_create; }
    c->h_mon.assign((size_t)kMonNQ * p.nz, 0.0);
    *out = c;
    return MFLBM_OK;

fail_create:
    g_last_create_error = c->err;
    mflbm_destroy(c);
    return r;
}

void mflbm_destroy(mflbm_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->dev);
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
    if (c->region0) cudaEventDestroy(c->region0);
    if (c->region1) cudaEventDestroy(c->region1);
    for (void *p : c->allocs) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

static int gradient_lists(mflbm_ctx *c, const int8_t *walls, const mflbm_solid_bnd *solid, int32_t n_solid,
                          const mflbm_fluid_bnd *fluid, int32_t n_fluid);

int32_t mflbm_set_geometry(mflbm_ctx *c, const int8_t *walls, const mflbm_solid_bnd *solid, int32_t n_solid,
                           const mflbm_fluid_bnd *fluid, int32_t n_fluid, const double *w_in) {
    if (!c) return MFLBM_EINVAL;
    if (!walls) return fail(c, MFLBM_EINVAL, "walls is NULL");
    if (n_solid < 0 || n_fluid < 0) return fail(c, MFLBM_EINVAL, "negative list length");
    if ((n_solid > 0 && !solid) || (n_fluid > 0 && !fluid)) return fail(c, MFLBM_EINVAL, "list pointer is NULL");
    const mflbm_params &p = c->p;
    CK(c, cudaSetDevice(c->dev));
    if (!p.multiphase) { n_solid = 0; n_fluid = 0; }
    // every list entry must stay inside the arrays it touches: solid nodes inside
    // [-2, n+3] (their neighbours reach the phi halo [-3, n+4]); fluid nodes inside
    // [-1, n+2] (Geometry_preprocessing.F90:429-507)
    for (int32_t t = 0; t < n_solid; ++t) {
        const mflbm_solid_bnd &s = solid[t];
        if (s.ix < -2 || s.ix > p.nx + 3 || s.iy < -2 || s.iy > p.ny + 3 || s.iz < -2 || s.iz > p.nz + 3)
            return fail(c, MFLBM_EINVAL, "solid boundary node " + std::to_string(t) + " outside [-2, n+3]");
        if (s.i_fluid_num < 0 || s.i_fluid_num > 18)
            return fail(c, MFLBM_EINVAL, "solid boundary node " + std::to_string(t) + ": i_fluid_num outside 0..18");
        for (int n = 0; n < s.i_fluid_num; ++n)
            if (s.neighbor_list[n] < 1 || s.neighbor_list[n] > 18)
                return fail(c, MFLBM_EINVAL, "solid boundary node " + std::to_string(t) + ": neighbour outside 1..18");
    }
    std::vector<FluidBnd> fb((size_t)n_fluid);
    for (int32_t t = 0; t < n_fluid; ++t) {
        const mflbm_fluid_bnd &f = fluid[t];
        if (f.ix < -1 || f.ix > p.nx + 2 || f.iy < -1 || f.iy > p.ny + 2 || f.iz < -1 || f.iz > p.nz + 2)
            return fail(c, MFLBM_EINVAL, "fluid boundary node " + std::to_string(t) + " outside [-1, n+2]");
        fb[t] = FluidBnd{f.ix, f.iy, f.iz, 0, f.nwx, f.nwy, f.nwz, std::cos(f.theta), std::sin(f.theta)};
    }
    CK(c, cudaStreamSynchronize(c->stream));
    drop_graphs(c);
    CK(c, cudaMemcpy(c->st.walls, walls, (size_t)n2(p), cudaMemcpyHostToDevice));
    if (w_in) CK(c, cudaMemcpy(c->st.w_in, w_in, sizeof(double) * nplane(p), cudaMemcpyHostToDevice));
    else CK(c, cudaMemset(c->st.w_in, 0, sizeof(double) * nplane(p)));
    // lists: reallocate when they grow
    static_assert(sizeof(SolidBnd) == sizeof(mflbm_solid_bnd), "solid boundary ABI");
    if (n_solid > c->st.ns || (n_solid > 0 && !c->st.sb)) {
        SolidBnd *sb = nullptr;
        int r = dalloc(c, &sb, n_solid);
        if (r) return r;
        c->st.sb = sb;
    }
    if (n_fluid > c->st.nf || (n_fluid > 0 && !c->st.fb)) {
        FluidBnd *fbd = nullptr;
        int r = dalloc(c, &fbd, n_fluid);
        if (r) return r;
        c->st.fb = fbd;
    }
    // storage layout of a singlephase run: the fluid list when the geometry allows it.  With
    // an open z direction (inlet / outlet conditions) the list keeps private slots for the
    // cells of the planes the conditions address (the multiphase builder's planes), found
    // through a slot map; otherwise every non-fluid slot is a bounce-back link.
    if (!p.multiphase && p.layout != MFLBM_LAYOUT_DENSE) {
        ListLayout ll;
        MpListLayout ml;
        std::string why;
        const bool planes = c->open_z;
        bool ok;
        if (planes && p.iper) {
            ok = false;
            why = "an open z direction needs walls in x";
        } else if (planes) {
            ok = build_mp_list_layout(walls, p.nx, p.ny, p.nz, p.jper, p.kper, {0, 1, 2, p.nz - 1, p.nz, p.nz + 1}, {},
                                      ml, why);
        } else {
            ok = build_list_layout(walls, p.nx, p.ny, p.nz, p.iper, p.jper, p.kper, ll, why);
        }
        const ListLayout &lay = planes ? static_cast<const ListLayout &>(ml) : ll;
        for (void *b : c->list_bufs) dfree(c, b);
        c->list_bufs.clear();
        if (ok) {
            int r = alloc_pdf(c, (size_t)19 * lay.stride * c->elt);
            if (r) return r;
            int32_t *nb = nullptr, *cell1 = nullptr, *link = nullptr, *seg = nullptr, *map = nullptr;
            if ((r = dalloc(c, &nb, 18 * lay.nf))) return r;
            c->list_bufs.push_back(nb);
            if ((r = dalloc(c, &cell1, lay.nf))) return r;
            c->list_bufs.push_back(cell1);
            if ((r = dalloc(c, &link, std::max<int64_t>(3, 3 * lay.nlink)))) return r;
            c->list_bufs.push_back(link);
            if ((r = dalloc(c, &seg, p.nz + 1))) return r;
            c->list_bufs.push_back(seg);
            if (planes) {
                if ((r = dalloc(c, &map, (int64_t)ml.map.size()))) return r;
                c->list_bufs.push_back(map);
                CK(c, cudaMemcpy(map, ml.map.data(), sizeof(int32_t) * ml.map.size(), cudaMemcpyHostToDevice));
            }
            CK(c, cudaMemcpy(nb, lay.nb.data(), sizeof(int32_t) * lay.nb.size(), cudaMemcpyHostToDevice));
            CK(c, cudaMemcpy(cell1, lay.cell1.data(), sizeof(int32_t) * lay.cell1.size(), cudaMemcpyHostToDevice));
            if (lay.nlink)
                CK(c, cudaMemcpy(link, lay.link.data(), sizeof(int32_t) * lay.link.size(), cudaMemcpyHostToDevice));
            CK(c, cudaMemcpy(seg, lay.slice.data(), sizeof(int32_t) * lay.slice.size(), cudaMemcpyHostToDevice));
            DevState &st = c->st;
            st.list = 1;
            st.mplist = 0;
            st.f = c->pdf;
            st.g = nullptr;
            st.lstride = lay.stride;
            st.nb = nb;
            st.cell1 = cell1;
            st.link = link;
            st.nlink = lay.nlink;
            st.nfl = (int)lay.nf;
            st.lseg = seg;
            st.pmap = map;
            st.pspare = planes ? ml.spare : 0;
            st.pwrap = nullptr;
            st.nwrap = 0;
            st.ncell = 0;
            // the TMA even step, unless MFLBM_NO_TMA is set (a diagnostic switch that selects
            // the plain even step, for comparisons)
            const char *no_tma = std::getenv("MFLBM_NO_TMA");
            st.tma = (!no_tma || !*no_tma || std::strcmp(no_tma, "0") == 0) && encode_list_map(c) ? 1 : 0;
            c->st.ns = 0;
            c->st.nf = 0;
            CK(c, cudaDeviceSynchronize());
            c->have_geometry = true;
            return MFLBM_OK;
        }
        if (p.layout == MFLBM_LAYOUT_LIST) return fail(c, MFLBM_EINVAL, "fluid-list layout: " + why);
        int r = alloc_dense(c);
        if (r) return r;
    }
    // multiphase fluid list (MpListLayout in listlayout.h): f and g hold the fluid nodes, the
    // boundary planes' private slots and the link slots; phi and the gradient fields stay dense
    bool mp_list = false;
    if (p.multiphase && p.layout != MFLBM_LAYOUT_DENSE) {
        std::vector<int> planes, ghost_planes;
        if (c->open_z)
            for (int k : {0, 1, 2, p.nz - 1, p.nz, p.nz + 1}) planes.push_back(k);
        if (p.porous_plate_cmd != 0 && p.z_porous_plate >= 1 && p.z_porous_plate <= p.nz)
            for (int dz = -1; dz <= 1; ++dz) {
                planes.push_back(p.z_porous_plate + dz);
                ghost_planes.push_back(p.z_porous_plate + dz);
            }
        MpListLayout ml;
        std::string why;
        mp_list = build_mp_list_layout(walls, p.nx, p.ny, p.nz, p.jper, p.kper, planes, ghost_planes, ml, why);
        if (!mp_list && p.layout == MFLBM_LAYOUT_LIST)
            return fail(c, MFLBM_EINVAL, "multiphase fluid-list layout: " + why);
        if (mp_list) {
            for (void *b : c->list_bufs) dfree(c, b);
            c->list_bufs.clear();
            int r = alloc_pdf(c, (size_t)2 * 19 * ml.stride * c->elt);
            if (r) return r;
            int32_t *nb = nullptr, *cell1 = nullptr, *link = nullptr, *map = nullptr;
            if ((r = dalloc(c, &nb, 18 * ml.nf))) return r;
            c->list_bufs.push_back(nb);
            if ((r = dalloc(c, &cell1, ml.nf))) return r;
            c->list_bufs.push_back(cell1);
            if ((r = dalloc(c, &link, std::max<int64_t>(3, 3 * ml.nlink)))) return r;
            c->list_bufs.push_back(link);
            if ((r = dalloc(c, &map, (int64_t)ml.map.size()))) return r;
            c->list_bufs.push_back(map);
            int32_t *wrap = nullptr;
            if (ml.nwrap > 0) {
                if ((r = dalloc(c, &wrap, 4 * ml.nwrap))) return r;
                c->list_bufs.push_back(wrap);
                CK(c, cudaMemcpy(wrap, ml.wrap.data(), sizeof(int32_t) * ml.wrap.size(), cudaMemcpyHostToDevice));
            }
            CK(c, cudaMemcpy(nb, ml.nb.data(), sizeof(int32_t) * ml.nb.size(), cudaMemcpyHostToDevice));
            CK(c, cudaMemcpy(cell1, ml.cell1.data(), sizeof(int32_t) * ml.cell1.size(), cudaMemcpyHostToDevice));
            if (ml.nlink) CK(c, cudaMemcpy(link, ml.link.data(), sizeof(int32_t) * ml.link.size(), cudaMemcpyHostToDevice));
            CK(c, cudaMemcpy(map, ml.map.data(), sizeof(int32_t) * ml.map.size(), cudaMemcpyHostToDevice));
            DevState &st = c->st;
            st.list = 1;
            st.mplist = 1;
            st.tma = 0;
            st.f = c->pdf;
            st.g = (void *)((char *)c->pdf + (size_t)19 * ml.stride * c->elt);
            st.lstride = ml.stride;
            st.nb = nb;
            st.cell1 = cell1;
            st.link = link;
            st.nlink = ml.nlink;
            st.nfl = (int)ml.nf;
            st.lseg = nullptr;
            st.pmap = map;
            st.pspare = ml.spare;
            st.pwrap = wrap;
            st.nwrap = ml.nwrap;
        }
    }
    if (p.multiphase && !mp_list && (!c->pdf || c->st.list)) {
        int r = alloc_dense(c);
        if (r) return r;
    }
    // sorted list of interior fluid nodes (walls == 0): the collision sweep runs one
    // thread per entry, so no lane idles on a solid node
    {
        const Layout &L = c->st.L;
        std::vector<int32_t> cells;
        cells.reserve((size_t)p.nx * p.ny * p.nz / 4 + 1);
        for (int k = 1; k <= p.nz; ++k)
            for (int j = 1; j <= p.ny; ++j)
                for (int i = 1; i <= p.nx; ++i)
                    if (walls[L.i2(i, j, k)] == 0) cells.push_back((int32_t)L.cell(i, j, k));
        if ((int64_t)cells.size() > c->cells_cap) {
            int32_t *d = nullptr;
            int r = dalloc(c, &d, (int64_t)cells.size());
            if (r) return r;
            c->st.cells = d;
            c->cells_cap = (int64_t)cells.size();
        }
        if (!cells.empty())
            CK(c, cudaMemcpy((void *)c->st.cells, cells.data(), sizeof(int32_t) * cells.size(), cudaMemcpyHostToDevice));
        c->st.ncell = (int)cells.size();
    }
    if (n_solid) CK(c, cudaMemcpy((void *)c->st.sb, solid, sizeof(SolidBnd) * n_solid, cudaMemcpyHostToDevice));
    if (n_fluid) CK(c, cudaMemcpy((void *)c->st.fb, fb.data(), sizeof(FluidBnd) * n_fluid, cudaMemcpyHostToDevice));
    c->st.ns = n_solid;
    c->st.nf = n_fluid;
    if (p.multiphase) {
        int r = gradient_lists(c, walls, solid, n_solid, fluid, n_fluid);
        if (r) return r;
    }
    CK(c, cudaDeviceSynchronize());
    c->have_geometry = true;
    return MFLBM_OK;
}

// Device lists of the colour-gradient step (multiphase): the fluid cells that need normals
// ([-1, n+2]^3, walls != 1) and curvature ([1, n]^3, walls == 0), packed, for the
// fluid-cell kernels of the default build; and the compact solid-boundary records when every
// neighbour list is ascending (the order of the sums is then the set-bit order).  The
// gradient fields are zeroed: cells the lists skip keep those zeros, as the full-box
// kernels would write them.
static int gradient_lists(mflbm_ctx *c, const int8_t *walls, const mflbm_solid_bnd *solid, int32_t n_solid,
                          const mflbm_fluid_bnd *fluid, int32_t n_fluid) {
    const mflbm_params &p = c->p;
    const Layout &L = c->st.L;
    const size_t fe = (size_t)c->st.felt;
    CK(c, cudaMemsetAsync(c->st.cn, 0, 4 * fe * n2(p), c->stream));
    CK(c, cudaMemsetAsync(c->st.curv, 0, fe * n1(p), c->stream));
    c->st.glist = 0;
    c->st.gwet = 0;
    // MFLBM_SPLIT_GRADIENT=1 (a diagnostic switch, for comparisons): curvature and wetting in
    // their own kernels instead of inside the collision and the normals kernel
    {
        const char *sp = std::getenv("MFLBM_SPLIT_GRADIENT");
        c->st.gsplit = (sp && *sp && std::strcmp(sp, "0") != 0) ? 1 : 0;
    }
    c->st.n_gcell_n = 0;
    c->st.n_gcell_c = 0;
    c->st.sbc = nullptr;
    // Normals and curvature: the shared-memory plane-marching kernels visit every cell of the
    // box, the fluid-cell list kernels only the cells that need a value.  The tiles pay when
    // most cells are fluid; on a porous medium (a third fluid) the lists are faster.  The
    // choice follows the fluid fraction of the interior; MFLBM_GRADIENT=tile|list (a
    // diagnostic switch) overrides it.
    {
        int64_t nfluid = 0;
        for (int k = 1; k <= p.nz; ++k)
            for (int j = 1; j <= p.ny; ++j)
                for (int i = 1; i <= p.nx; ++i) nfluid += walls[L.i2(i, j, k)] == 0;
        const double frac = (double)nfluid / ((double)p.nx * p.ny * p.nz);
        const char *gsel = std::getenv("MFLBM_GRADIENT");
        if (gsel && std::strcmp(gsel, "tile") == 0) c->st.gtile = 1;
        else if (gsel && std::strcmp(gsel, "list") == 0) c->st.gtile = 0;
        else c->st.gtile = frac > kGradientTileFraction ? 1 : 0;
    }
    if (!cell_packable(p.nx, p.ny, p.nz)) return MFLBM_OK;  // the full-box kernels serve
    // The normals list starts with the fluid-boundary nodes in record order when their cells
    // are distinct fluid cells (the normals kernel then applies the wetting of record t at
    // entry t); the other cells follow in cell order.
    std::vector<uint32_t> gn, gc, fbs;
    bool wet = n_fluid > 0 && !c->st.gsplit;
    for (int32_t t = 0; t < n_fluid && wet; ++t) {
        const mflbm_fluid_bnd &f = fluid[t];
        if (walls[L.i2(f.ix, f.iy, f.iz)] == 1) wet = false;
        fbs.push_back(pack_cell(f.ix, f.iy, f.iz));
    }
    if (wet) {
        gn = fbs;
        std::sort(fbs.begin(), fbs.end());
        wet = std::adjacent_find(fbs.begin(), fbs.end()) == fbs.end();
        if (!wet) gn.clear();
    }
    if (!wet) fbs.clear();
    size_t pos = 0;
    for (int k = -1; k <= p.nz + 2; ++k)
        for (int j = -1; j <= p.ny + 2; ++j)
            for (int i = -1; i <= p.nx + 2; ++i) {
                const int8_t w = walls[L.i2(i, j, k)];
                const uint32_t pc = pack_cell(i, j, k);   // ascending in this loop order
                if (w != 1) {
                    while (pos < fbs.size() && fbs[pos] < pc) ++pos;
                    if (!(pos < fbs.size() && fbs[pos] == pc)) gn.push_back(pc);
                }
                if (w == 0 && i >= 1 && i <= p.nx && j >= 1 && j <= p.ny && k >= 1 && k <= p.nz)
                    gc.push_back(pc);
            }
    auto put = [&](const std::vector<uint32_t> &v, const uint32_t **dst, int64_t &cap) -> int {
        if (v.empty()) return MFLBM_OK;
        if ((int64_t)v.size() > cap) {
            uint32_t *d = nullptr;
            int r = dalloc(c, &d, (int64_t)v.size());
            if (r) return r;
            *dst = d;
            cap = (int64_t)v.size();
        }
        CK(c, cudaMemcpy((void *)*dst, v.data(), sizeof(uint32_t) * v.size(), cudaMemcpyHostToDevice));
        return MFLBM_OK;
    };
    int r;
    if ((r = put(gn, &c->st.gcell_n, c->gn_cap))) return r;
    if ((r = put(gc, &c->st.gcell_c, c->gc_cap))) return r;
    c->st.n_gcell_n = (int)gn.size();
    c->st.n_gcell_c = (int)gc.size();
    c->st.glist = 1;
    c->st.gwet = wet ? 1 : 0;
    std::vector<SolidBndC> sc((size_t)n_solid);
    for (int32_t t = 0; t < n_solid; ++t) {
        const mflbm_solid_bnd &s = solid[t];
        uint32_t m = 0;
        int prev = 0;
        for (int n = 0; n < s.i_fluid_num; ++n) {
            const int d = s.neighbor_list[n];
            if (d <= prev) return MFLBM_OK;  // not ascending: keep the record kernels
            prev = d;
            m |= 1u << (d - 1);
        }
        sc[t] = SolidBndC{pack_cell(s.ix, s.iy, s.iz), m, s.la_weight};
    }
    if (n_solid > 0) {
        if (n_solid > c->sbc_cap) {
            if ((r = dalloc(c, &c->sbc_buf, n_solid))) return r;
            c->sbc_cap = n_solid;
        }
        CK(c, cudaMemcpy(c->sbc_buf, sc.data(), sizeof(SolidBndC) * n_solid, cudaMemcpyHostToDevice));
        c->st.sbc = c->sbc_buf;
    }
    return MFLBM_OK;
}

// FP64 host array -> device field (phi or a gradient field) of the context's field type
static int field_put(mflbm_ctx *c, void *dev, const double *host, int64_t n) {
    if (c->st.felt == 8) {
        CK(c, cudaMemcpyAsync(dev, host, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    } else {
        CK(c, cudaMemcpyAsync(c->st.stage, host, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        c->kt->field_in(c->st, dev, n, c->stream);
        CK(c, cudaPeekAtLastError());
    }
    return MFLBM_OK;
}

// device field -> FP64 host array; synchronises the context stream.  stride > 1: every
// stride-th element (one component of the normal records)
static int field_get(mflbm_ctx *c, double *host, const void *dev, int64_t n, int stride = 1) {
    if (!c->st.stage || n > c->stage_len)
        return fail(c, MFLBM_ESTATE, "field download: staging buffer missing or too small");
    if (c->st.felt == 8 && stride == 1) {
        CK(c, cudaMemcpyAsync(host, dev, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    } else {
        c->kt->field_out(c->st, dev, n, stride, c->stream);
        CK(c, cudaPeekAtLastError());
        CK(c, cudaMemcpyAsync(host, c->st.stage, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

int32_t mflbm_upload_state(mflbm_ctx *c, const double *const *f, const double *const *g, const double *phi,
                           const double *f_convec, const double *g_convec, const double *phi_convec) {
    if (!c) return MFLBM_EINVAL;
    if (!c->pdf) return fail(c, MFLBM_ESTATE, "the PDF storage is laid out by mflbm_set_geometry; call it first");
    const mflbm_params &p = c->p;
    if (!f) return fail(c, MFLBM_EINVAL, "f is NULL");
    for (int q = 0; q < 19; ++q) if (!f[q]) return fail(c, MFLBM_EINVAL, "f[q] is NULL");
    if (p.multiphase) {
        if (!g || !phi) return fail(c, MFLBM_EINVAL, "g and phi are required for multiphase");
        for (int q = 0; q < 19; ++q) if (!g[q]) return fail(c, MFLBM_EINVAL, "g[q] is NULL");
    }
    if (p.outlet_bc == 1 && c->open_z && (!f_convec || (p.multiphase && (!g_convec || !phi_convec))))
        return fail(c, MFLBM_EINVAL, "convective outlet memory arrays are required when outlet_bc == 1");
    CK(c, cudaSetDevice(c->dev));
    const Layout &L = c->st.L;
    const int nsp = p.multiphase ? 2 : 1;
    for (int s = 0; s < nsp; ++s) {
        const double *const *src = s == 0 ? f : g;
        char *base = (char *)(s == 0 ? c->st.f : c->st.g);
        for (int q = 0; q < 19; ++q) {
            if (f64_storage(p) && !c->st.list) {
                char *dst = base + ((size_t)q * L.qs + L.xo) * c->elt;
                CK(c, cudaMemcpy2DAsync(dst, (size_t)L.pitch * 8, src[q], (size_t)(p.nx + 2) * 8, (size_t)(p.nx + 2) * 8,
                                        (size_t)(p.ny + 2) * (p.nz + 2), cudaMemcpyHostToDevice, c->stream));
            } else {
                CK(c, cudaMemcpyAsync(c->st.stage, src[q], sizeof(double) * n1(p), cudaMemcpyHostToDevice, c->stream));
                c->kt->convert_in(c->st, s, q, c->stream);
                CK(c, cudaPeekAtLastError());
            }
        }
    }
    if (p.multiphase) {
        int r = field_put(c, c->st.phi, phi, n4(p));
        if (r) return r;
    }
    if (f_convec) CK(c, cudaMemcpyAsync(c->st.fconv, f_convec, sizeof(double) * nplane(p) * 19, cudaMemcpyHostToDevice, c->stream));
    if (p.multiphase && g_convec)
        CK(c, cudaMemcpyAsync(c->st.gconv, g_convec, sizeof(double) * nplane(p) * 19, cudaMemcpyHostToDevice, c->stream));
    if (p.multiphase && phi_convec)
        CK(c, cudaMemcpyAsync(c->st.phiconv, phi_convec, sizeof(double) * nplane(p), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

int32_t mflbm_download_state(mflbm_ctx *c, double *const *f, double *const *g, double *phi, double *f_convec,
                             double *g_convec, double *phi_convec) {
    if (!c) return MFLBM_EINVAL;
    if (!c->pdf) return fail(c, MFLBM_ESTATE, "the PDF storage is laid out by mflbm_set_geometry; call it first");
    const mflbm_params &p = c->p;
    CK(c, cudaSetDevice(c->dev));
    const Layout &L = c->st.L;
    const int nsp = p.multiphase ? 2 : 1;
    for (int s = 0; s < nsp; ++s) {
        double *const *dstv = s == 0 ? f : g;
        if (!dstv) continue;
        const char *base = (const char *)(s == 0 ? c->st.f : c->st.g);
        for (int q = 0; q < 19; ++q) {
            if (!dstv[q]) continue;
            if (f64_storage(p) && !c->st.list) {
                const char *src = base + ((size_t)q * L.qs + L.xo) * c->elt;
                CK(c, cudaMemcpy2DAsync(dstv[q], (size_t)(p.nx + 2) * 8, src, (size_t)L.pitch * 8, (size_t)(p.nx + 2) * 8,
                                        (size_t)(p.ny + 2) * (p.nz + 2), cudaMemcpyDeviceToHost, c->stream));
            } else {
                c->kt->convert_out(c->st, s, q, c->stream);
                CK(c, cudaPeekAtLastError());
                CK(c, cudaMemcpyAsync(dstv[q], c->st.stage, sizeof(double) * n1(p), cudaMemcpyDeviceToHost, c->stream));
            }
        }
    }
    if (p.multiphase && phi) {
        int r = field_get(c, phi, c->st.phi, n4(p));
        if (r) return r;
    }
    if (f_convec) CK(c, cudaMemcpyAsync(f_convec, c->st.fconv, sizeof(double) * nplane(p) * 19, cudaMemcpyDeviceToHost, c->stream));
    if (p.multiphase && g_convec)
        CK(c, cudaMemcpyAsync(g_convec, c->st.gconv, sizeof(double) * nplane(p) * 19, cudaMemcpyDeviceToHost, c->stream));
    if (p.multiphase && phi_convec)
        CK(c, cudaMemcpyAsync(phi_convec, c->st.phiconv, sizeof(double) * nplane(p), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return check_device_err(c);
}

int32_t mflbm_init_equilibrium(mflbm_ctx *c, const double *phi) {
    if (!c) return MFLBM_EINVAL;
    if (!c->pdf) return fail(c, MFLBM_ESTATE, "the PDF storage is laid out by mflbm_set_geometry; call it first");
    const mflbm_params &p = c->p;
    if (p.multiphase && !phi) return fail(c, MFLBM_EINVAL, "phi is required for multiphase");
    CK(c, cudaSetDevice(c->dev));
    if (p.multiphase) {
        int r = field_put(c, c->st.phi, phi, n4(p));
        if (r) return r;
    }
    c->kt->init_equilibrium(c->st, p.outlet_bc == 1, c->stream);
    CK(c, cudaPeekAtLastError());
    CK(c, cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

int32_t mflbm_init_velocity(mflbm_ctx *c, const double *rho, const double *u, const double *v, const double *w,
                            int32_t rest_base) {
    int r = ready(c);
    if (r) return r;
    const mflbm_params &p = c->p;
    if (p.multiphase) return fail(c, MFLBM_EINVAL, "mflbm_init_velocity is singlephase only");
    CK(c, cudaSetDevice(c->dev));
    const size_t b1 = sizeof(double) * n1(p);
    double *dst[4] = {c->st.u, c->st.v, c->st.w, c->st.rho};
    const double *src[4] = {u, v, w, rho};
    for (int a = 0; a < 4; ++a) {
        if (src[a]) CK(c, cudaMemcpyAsync(dst[a], src[a], b1, cudaMemcpyHostToDevice, c->stream));
        else if (a < 3) CK(c, cudaMemsetAsync(dst[a], 0, b1, c->stream));
    }
    c->kt->init_velocity(c->st, rho ? c->st.rho : nullptr, rest_base ? 1 : 0, c->stream);
    CK(c, cudaPeekAtLastError());
    CK(c, cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

int32_t mflbm_steady_monitor(mflbm_ctx *c, int32_t kind, double *out) {
    int r = ready(c);
    if (r) return r;
    const mflbm_params &p = c->p;
    if (!p.multiphase) return fail(c, MFLBM_EINVAL, "steady-state monitors are multiphase");
    if (kind < 0 || kind > 3 || (kind > 0 && !out)) return fail(c, MFLBM_EINVAL, "kind must be 0..3 and out non-NULL");
    CK(c, cudaSetDevice(c->dev));
    if (!c->steady_part && (r = dalloc(c, &c->steady_part, 7 * (int64_t)p.nz))) return r;
    if ((kind == 0 || kind == 2) && !c->phi_old) {
        if ((r = dalloc_bytes(c, &c->phi_old, (size_t)c->st.felt * n4(p)))) return r;
        CK(c, cudaMemcpyAsync(c->phi_old, c->st.phi, (size_t)c->st.felt * n4(p), cudaMemcpyDeviceToDevice, c->stream));
        if (kind == 0) return MFLBM_OK;
    }
    if (kind == 0) {
        CK(c, cudaMemcpyAsync(c->phi_old, c->st.phi, (size_t)c->st.felt * n4(p), cudaMemcpyDeviceToDevice, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        return MFLBM_OK;
    }
    c->kt->monitor(c->st, c->stream);   // compute_macro_vars
    c->kt->steady(c->st, kind == 2 ? c->phi_old : nullptr, c->steady_part, p.nz - 1, kind == 2 ? 1 : 0, c->stream);
    CK(c, cudaPeekAtLastError());
    std::vector<double> h((size_t)7 * p.nz);
    CK(c, cudaMemcpyAsync(h.data(), c->steady_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    double dphi = 0.0, umax2 = 0.0, pw = 0.0, iw = 0.0, pnw = 0.0, inw = 0.0, brk = 0.0;
    for (int k = 0; k < p.nz; ++k) {
        dphi = std::max(dphi, h[k]);
        umax2 = std::max(umax2, h[(size_t)p.nz + k]);
        pw += h[(size_t)2 * p.nz + k];
        iw += h[(size_t)3 * p.nz + k];
        pnw += h[(size_t)4 * p.nz + k];
        inw += h[(size_t)5 * p.nz + k];
        brk += h[(size_t)6 * p.nz + k];
    }
    const double eps = 1.110223025e-16;   // Module.F90:8
    if (kind == 1) {
        const double pre_w = pw / (iw + eps), pre_nw = pnw / (inw + eps);
        out[0] = (pre_nw - pre_w) / 3.0;
        out[1] = pre_w;
        out[2] = pre_nw;
        out[3] = std::sqrt(umax2);
        out[4] = iw;
        out[5] = inw;
    } else if (kind == 2) {
        out[0] = dphi;
        out[1] = std::sqrt(umax2);
    } else {
        out[0] = brk;
    }
    return MFLBM_OK;
}

int32_t mflbm_change_inlet_fluid_phase(mflbm_ctx *c, int32_t cmd, double interface_z0) {
    int r = ready(c);
    if (r) return r;
    const mflbm_params &p = c->p;
    if (!p.multiphase) return fail(c, MFLBM_EINVAL, "change_inlet_fluid_phase is multiphase only");
    if (cmd < 0 || cmd > 2) return fail(c, MFLBM_EINVAL, "change_inlet_fluid_phase_cmd must be 0, 1 or 2");
    if (cmd == 0 || !(interface_z0 >= 0.0)) return MFLBM_OK;
    CK(c, cudaSetDevice(c->dev));
    // k runs over the halo-1 box 0..nz+1; z = k on one rank, and z <= interface_z0
    const int kmax = (int)std::min<double>(std::floor(interface_z0), (double)(p.nz + 1));
    c->kt->change_inlet_phase(c->st, cmd, kmax, c->stream);
    CK(c, cudaPeekAtLastError());
    CK(c, cudaStreamSynchronize(c->stream));
    return MFLBM_OK;
}

int32_t mflbm_step(mflbm_ctx *c, int32_t ntime) {
    int r = ready(c);
    if (r) return r;
    if (ntime < 0) return fail(c, MFLBM_EINVAL, "ntime must be >= 0");
    CK(c, cudaSetDevice(c->dev));
    const int n = enqueue_step(c, ntime);
    if (n < 0) return MFLBM_ECUDA;
    c->launches += n;
    CK(c, cudaPeekAtLastError());
    return MFLBM_OK;
}

int32_t mflbm_run(mflbm_ctx *c, int32_t ntime0, int32_t nsteps) {
    int r = ready(c);
    if (r) return r;
    if (ntime0 < 0 || nsteps < 0) return fail(c, MFLBM_EINVAL, "ntime0 and nsteps must be >= 0");
    CK(c, cudaSetDevice(c->dev));
    int32_t t = ntime0, left = nsteps;
    if (c->profiling) {  // step by step, so every collision sweep is bracketed by events
        for (; left > 0; ++t, --left) {
            const int n = enqueue_step(c, t);
            if (n < 0) return MFLBM_ECUDA;
            c->launches += n;
        }
        CK(c, cudaPeekAtLastError());
        return MFLBM_OK;
    }
    if (left > 0 && (t % 2) != 0) {  // graphs start on an even step
        c->launches += enqueue_step(c, t);
        ++t; --left;
    }
    if (left >= 2 && !c->g_pair) {
        if ((r = capture(c, 1, &c->g_pair, &c->pair_launches))) return r;
    }
    if (left >= 2 * c->block_pairs && !c->g_block) {
        if ((r = capture(c, c->block_pairs, &c->g_block, &c->block_launches))) return r;
    }
    while (left >= 2 * c->block_pairs) {
        CK(c, cudaGraphLaunch(c->g_block, c->stream));
        c->launches += c->block_launches;
        t += 2 * c->block_pairs; left -= 2 * c->block_pairs;
    }
    while (left >= 2) {
        CK(c, cudaGraphLaunch(c->g_pair, c->stream));
        c->launches += c->pair_launches;
        t += 2; left -= 2;
    }
    if (left == 1) c->launches += enqueue_step(c, t);
    CK(c, cudaPeekAtLastError());
    return MFLBM_OK;
}

int32_t mflbm_set_profiling(mflbm_ctx *c, int32_t enable) {
    if (!c) return MFLBM_EINVAL;
    CK(c, cudaSetDevice(c->dev));
    CK(c, cudaStreamSynchronize(c->stream));
    if (enable && c->ev.empty()) {
        c->ev.resize(2 * kEventRing);
        for (auto &e : c->ev) CK(c, cudaEventCreate(&e));
    }
    if (!c->region0) {
        CK(c, cudaEventCreate(&c->region0));
        CK(c, cudaEventCreate(&c->region1));
    }
    c->profiling = enable != 0;
    c->ev_used = 0;
    c->collide_ms = 0.0;
    c->collide_count = 0;
    c->launches = 0;
    CK(c, cudaEventRecord(c->region0, c->stream));
    return MFLBM_OK;
}

int32_t mflbm_get_profile(mflbm_ctx *c, double *region_ms, double *collide_ms, int64_t *collide_launches,
                          int64_t *kernel_launches) {
    if (!c) return MFLBM_EINVAL;
    if (!c->region0) return fail(c, MFLBM_ESTATE, "mflbm_set_profiling was not called");
    CK(c, cudaSetDevice(c->dev));
    CK(c, cudaEventRecord(c->region1, c->stream));
    int r = drain_events(c);
    if (r) return r;
    if ((r = check_device_err(c))) return r;
    CK(c, cudaEventSynchronize(c->region1));
    float rms = 0.f;
    CK(c, cudaEventElapsedTime(&rms, c->region0, c->region1));
    if (region_ms) *region_ms = rms;
    if (collide_ms) *collide_ms = c->collide_ms;
    if (collide_launches) *collide_launches = c->collide_count;
    if (kernel_launches) *kernel_launches = c->launches;
    return MFLBM_OK;
}

int32_t mflbm_color_gradient(mflbm_ctx *c) {
    int r = ready(c);
    if (r) return r;
    if (!c->p.multiphase) return fail(c, MFLBM_EINVAL, "color_gradient is multiphase only");
    CK(c, cudaSetDevice(c->dev));
    c->kt->color_gradient(c->st, c->stream);
    CK(c, cudaPeekAtLastError());
    return MFLBM_OK;
}

int32_t mflbm_get_gradient(mflbm_ctx *c, double *cn_x, double *cn_y, double *cn_z, double *c_norm, double *curv) {
    if (!c) return MFLBM_EINVAL;
    if (!c->p.multiphase) return fail(c, MFLBM_EINVAL, "multiphase only");
    const mflbm_params &p = c->p;
    CK(c, cudaSetDevice(c->dev));
    if (curv) {
        c->kt->curvature_field(c->st, c->stream);
        CK(c, cudaPeekAtLastError());
    }
    CK(c, cudaStreamSynchronize(c->stream));
    double *const dst[5] = {cn_x, cn_y, cn_z, c_norm, curv};
    for (int a = 0; a < 5; ++a) {
        if (!dst[a]) continue;
        // components 0..3 of the normal records (x, y, z, |grad phi|), then curvature
        const void *src = a < 4 ? (const void *)((const char *)c->st.cn + (size_t)a * c->st.felt) : c->st.curv;
        int r = field_get(c, dst[a], src, a < 4 ? n2(p) : n1(p), a < 4 ? 4 : 1);
        if (r) return r;
    }
    return MFLBM_OK;
}

int32_t mflbm_macro(mflbm_ctx *c, double *u, double *v, double *w, double *rho, double *phi) {
    int r = ready(c);
    if (r) return r;
    const mflbm_params &p = c->p;
    CK(c, cudaSetDevice(c->dev));
    c->kt->monitor(c->st, c->stream);
    CK(c, cudaPeekAtLastError());
    CK(c, cudaStreamSynchronize(c->stream));
    const size_t b1 = sizeof(double) * n1(p);
    if (u) CK(c, cudaMemcpy(u, c->st.u, b1, cudaMemcpyDeviceToHost));
    if (v) CK(c, cudaMemcpy(v, c->st.v, b1, cudaMemcpyDeviceToHost));
    if (w) CK(c, cudaMemcpy(w, c->st.w, b1, cudaMemcpyDeviceToHost));
    if (rho) CK(c, cudaMemcpy(rho, c->st.rho, b1, cudaMemcpyDeviceToHost));
    if (phi && p.multiphase) {
        int r2 = field_get(c, phi, c->st.phi, n4(p));
        if (r2) return r2;
    }
    return MFLBM_OK;
}

int32_t mflbm_monitor(mflbm_ctx *c, double *profiles, double *scalars, int32_t *status) {
    int r = ready(c);
    if (r) return r;
    const mflbm_params &p = c->p;
    CK(c, cudaSetDevice(c->dev));
    c->kt->monitor(c->st, c->stream);
    CK(c, cudaPeekAtLastError());
    CK(c, cudaMemcpyAsync(c->h_mon.data(), c->st.mon, sizeof(double) * kMonNQ * p.nz, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if ((r = check_device_err(c))) return r;
    const int nz = p.nz;
    const double *m = c->h_mon.data();
    bool bad = false;
    if (profiles) {
        if (p.multiphase) {
            for (int q = 0; q < 7; ++q)
                for (int k = 0; k < nz; ++k) profiles[q * nz + k] = m[q * nz + k];
        } else {
            for (int k = 0; k < nz; ++k) { profiles[k] = m[k]; profiles[nz + k] = m[6 * nz + k]; }
        }
    }
    const int nq = 7;
    for (int q = 0; q < nq; ++q)
        for (int k = 0; k < nz; ++k)
            if (std::isnan(m[q * nz + k])) bad = true;
    double umax = 0.0, usq1 = 0.0, usq2 = 0.0;
    for (int k = 0; k < nz; ++k) {
        const double t = m[7 * nz + k];
        if (umax < t) umax = t;
        usq1 += m[8 * nz + k];
        usq2 += m[9 * nz + k];
    }
    if (scalars) { scalars[0] = umax; scalars[1] = usq1; scalars[2] = usq2; }
    if (std::isnan(umax) || std::sqrt(umax) > 0.5) bad = true;
    if (status) *status = bad ? MFLBM_FAILED : MFLBM_RUNNING;
    return MFLBM_OK;
}

int32_t mflbm_saturation(mflbm_ctx *c, double *vol1, double *vol2) {
    int r = ready(c);
    if (r) return r;
    if (!c->p.multiphase) return fail(c, MFLBM_EINVAL, "multiphase only");
    const int nz = c->p.nz;
    CK(c, cudaSetDevice(c->dev));
    c->kt->saturation(c->st, c->stream);
    CK(c, cudaPeekAtLastError());
    CK(c, cudaMemcpyAsync(c->h_mon.data(), c->st.mon, sizeof(double) * 2 * nz, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nz; ++k) { a += c->h_mon[k]; b += c->h_mon[nz + k]; }
    if (vol1) *vol1 = a;
    if (vol2) *vol2 = b;
    return MFLBM_OK;
}

int32_t mflbm_synchronize(mflbm_ctx *c) {
    if (!c) return MFLBM_EINVAL;
    CK(c, cudaSetDevice(c->dev));
    CK(c, cudaStreamSynchronize(c->stream));
    return check_device_err(c);
}

}  // extern "C"
