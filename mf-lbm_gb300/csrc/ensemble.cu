// ensemble.cu -- batched singlephase samples of uneven sizes in one fluid-list arena.
//
// No counterpart in the reference, which runs one sample per job.  Every sample is laid
// out as in listlayout.h; the arena stores the fluid nodes of all samples first (sample
// s owns [fbase_s, fbase_s + nf_s)) and then all bounce-back link slots, so one sweep
// kernel with one neighbour table updates every sample at once.  Samples share the
// run parameters (precision, MRT preset, viscosity, body force, periodic flags); each
// has its own dimensions and wall array.  Converged samples leave the tile table and
// cost nothing afterwards.  Launch shape (block size, persistent cooperative kernel or
// one launch per step) is chosen by mflbm_ensemble_tune, which times the candidates on
// the ensemble itself.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/mflbm.h"
#include "kernels_api.h"
#include "listlayout.h"

using namespace mflbm;

struct mflbm_ensemble {
    mflbm_params p{};
    int dev = 0;
    cudaStream_t stream = nullptr;
    const KernelTable *kt = nullptr;
    int n = 0;
    std::vector<int32_t> dims;            // 3 per sample
    std::vector<int64_t> fbase, nf;       // fluid range per sample
    std::vector<int32_t> active;
    int64_t NF = 0, stride = 0, nlink = 0;
    size_t elt = 8;
    std::vector<void *> allocs;
    EnsArgs a{};
    EnsTile *d_tiles = nullptr;
    int32_t *d_ntiles = nullptr;
    int32_t *d_seg0 = nullptr, *d_seg1 = nullptr;
    double *d_mon = nullptr;
    int64_t tiles_cap = 0;
    int block = 128, persistent = 0, grid = 0;
    int64_t active_nodes = 0;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;   // (ntime0 parity, nsteps)
    std::string err;
};

namespace {

thread_local std::string g_ens_create_error;

int efail(mflbm_ensemble *e, int code, const std::string &msg) {
    if (e) e->err = msg;
    else g_ens_create_error = msg;
    return code;
}

int ecuda(mflbm_ensemble *e, cudaError_t c, const char *what) {
    cudaGetLastError();
    return efail(e, c == cudaErrorMemoryAllocation ? MFLBM_ENOMEM : MFLBM_ECUDA,
                 std::string(what) + ": " + cudaGetErrorString(c));
}

#define EK(ens, expr)                                         \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return ecuda((ens), e_, #expr); \
    } while (0)

int ealloc(mflbm_ensemble *e, void **ptr, size_t bytes) {
    void *p = nullptr;
    cudaError_t c = cudaMalloc(&p, bytes);
    if (c != cudaSuccess) return ecuda(e, c, "cudaMalloc");
    e->allocs.push_back(p);
    *ptr = p;
    return MFLBM_OK;
}

void drop_graphs(mflbm_ensemble *e) {
    for (auto &kv : e->graphs) cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
}

// tile table of the active samples for the current block size
int rebuild_tiles(mflbm_ensemble *e) {
    std::vector<EnsTile> tiles;
    e->active_nodes = 0;
    for (int s = 0; s < e->n; ++s) {
        if (!e->active[s]) continue;
        e->active_nodes += e->nf[s];
        for (int64_t x = 0; x < e->nf[s]; x += e->block) {
            EnsTile t;
            t.start = (int32_t)(e->fbase[s] + x);
            t.count = (int32_t)std::min<int64_t>(e->block, e->nf[s] - x);
            tiles.push_back(t);
        }
    }
    if ((int64_t)tiles.size() > e->tiles_cap) return efail(e, MFLBM_ERANGE, "tile table overflow");
    if (!tiles.empty())
        EK(e, cudaMemcpyAsync(e->d_tiles, tiles.data(), sizeof(EnsTile) * tiles.size(), cudaMemcpyHostToDevice, e->stream));
    const int32_t nt = (int32_t)tiles.size();
    EK(e, cudaMemcpyAsync(e->d_ntiles, &nt, sizeof(int32_t), cudaMemcpyHostToDevice, e->stream));
    EK(e, cudaStreamSynchronize(e->stream));
    return MFLBM_OK;
}

int grid_for(mflbm_ensemble *e, int block, int persistent) {
    const int maxg = e->kt->ens_max_grid(e->p.precision, block);
    if (persistent) return maxg;
    // one launch per step: a grid-stride loop over at most every tile of the arena
    const int64_t all = (e->NF + block - 1) / block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(all, std::max(maxg, 1) * 4));
}

// Arrival count, generation and error word of the grid barrier back to zero.  A barrier
// that timed out leaves a partial count and a set error word, which would make every
// later persistent run leave at its first barrier.
int clear_barrier(mflbm_ensemble *e) {
    EK(e, cudaMemsetAsync(e->a.bar, 0, 2 * sizeof(unsigned int), e->stream));
    EK(e, cudaMemsetAsync(e->a.err, 0, sizeof(int32_t), e->stream));
    return MFLBM_OK;
}

int launch(mflbm_ensemble *e, int32_t ntime0, int32_t nsteps) {
    e->a.ntime0 = ntime0;
    e->a.nsteps = nsteps;
    const int r = e->kt->ens_run(e->a, e->p.precision, e->persistent, e->grid, e->block, e->stream);
    if (r < 0) return ecuda(e, cudaGetLastError(), "ensemble launch");
    return MFLBM_OK;
}

}  // namespace

extern "C" {

const char *mflbm_ensemble_last_error(const mflbm_ensemble *e) {
    return e ? e->err.c_str() : g_ens_create_error.c_str();
}

void mflbm_ensemble_destroy(mflbm_ensemble *e) {
    if (!e) return;
    cudaSetDevice(e->dev);
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    for (void *p : e->allocs) cudaFree(p);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

int32_t mflbm_ensemble_create(const mflbm_params *common, int32_t nsamples, const int32_t *dims,
                              const int8_t *const *walls, mflbm_ensemble **out) {
    if (!common || !dims || !walls || !out || nsamples <= 0) return efail(nullptr, MFLBM_EINVAL, "bad arguments");
    if (common->abi_version != MFLBM_ABI_VERSION) return efail(nullptr, MFLBM_EINVAL, "abi_version mismatch");
    if (common->multiphase) return efail(nullptr, MFLBM_EINVAL, "ensembles are singlephase");
    if (common->inlet_bc != 0 || common->outlet_bc != 0)
        return efail(nullptr, MFLBM_EINVAL, "ensembles have no inlet/outlet boundary conditions");
    if (common->precision < MFLBM_FP64 || common->precision > MFLBM_FF)
        return efail(nullptr, MFLBM_EINVAL, "unknown precision");
    if (!(common->la_nu1 > 0.0)) return efail(nullptr, MFLBM_EINVAL, "la_nu1 must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return efail(nullptr, MFLBM_ENODEV, "no CUDA device");
    if (common->device < 0 || common->device >= ndev) return efail(nullptr, MFLBM_ENODEV, "device ordinal out of range");
    // host layouts of every sample
    std::vector<ListLayout> ll((size_t)nsamples);
    for (int s = 0; s < nsamples; ++s) {
        const int nx = dims[3 * s], ny = dims[3 * s + 1], nz = dims[3 * s + 2];
        if (nx < 1 || ny < 1 || nz < 1 || !walls[s])
            return efail(nullptr, MFLBM_EINVAL, "sample " + std::to_string(s) + ": bad dimensions or NULL walls");
        std::string why;
        if (!build_list_layout(walls[s], nx, ny, nz, common->iper, common->jper, common->kper, ll[s], why))
            return efail(nullptr, MFLBM_EINVAL, "sample " + std::to_string(s) + ": " + why);
    }
    mflbm_ensemble *e = new mflbm_ensemble();
    e->p = *common;
    e->dev = common->device;
    e->n = nsamples;
    e->dims.assign(dims, dims + 3 * nsamples);
    e->active.assign((size_t)nsamples, 1);
    e->elt = common->precision == MFLBM_FP32 ? 4 : (common->precision == MFLBM_FP16 ? 2 : 8);
    e->kt = common->strict_fp ? kernels_strict() : kernels_fast();   // strict: no FMA contraction
    int r = MFLBM_OK;
    // arena: fluid nodes of all samples, then the link slots of all samples per direction
    std::vector<int64_t> lbase((size_t)19 * nsamples, 0);
    {
        std::vector<int64_t> lsum(19, 0);
        for (int s = 0; s < nsamples; ++s) {
            e->fbase.push_back(e->NF);
            e->nf.push_back(ll[s].nf);
            e->NF += ll[s].nf;
            std::vector<int64_t> cnt(19, 0);
            for (int64_t l = 0; l < ll[s].nlink; ++l) ++cnt[ll[s].link[3 * l]];
            for (int q = 0; q < 19; ++q) {
                lbase[(size_t)19 * s + q] = lsum[q];
                lsum[q] += cnt[q];
            }
            e->nlink += ll[s].nlink;
        }
        int64_t maxl = 0;
        for (int q = 0; q < 19; ++q) maxl = std::max(maxl, lsum[q]);
        e->stride = (e->NF + maxl + 31) / 32 * 32;
    }
    std::vector<int32_t> nb((size_t)18 * e->NF);
    std::vector<int32_t> seg0((size_t)nsamples), seg1((size_t)nsamples);
    if (e->stride >= ((int64_t)1 << 31)) {
        r = efail(nullptr, MFLBM_ERANGE, "ensemble arena exceeds 2^31 slots per direction");
        goto fail;
    }
    for (int s = 0; s < nsamples; ++s) {
        const int64_t nfs = ll[s].nf, fb = e->fbase[s];
        for (int d = 1; d <= 18; ++d) {
            const int qa = OPP(d);
            const int32_t *src = ll[s].nb.data() + (size_t)(d - 1) * nfs;
            int32_t *dst = nb.data() + (size_t)(d - 1) * e->NF + fb;
            for (int64_t x = 0; x < nfs; ++x) {
                const int64_t v = src[x];
                dst[x] = (int32_t)(v < nfs ? fb + v : e->NF + lbase[(size_t)19 * s + qa] + (v - nfs));
            }
        }
        seg0[s] = (int32_t)fb;
        seg1[s] = (int32_t)(fb + nfs);
        ll[s] = ListLayout();   // release host memory early
    }
    if (cudaSetDevice(e->dev) != cudaSuccess || cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        r = efail(nullptr, MFLBM_ECUDA, "cudaSetDevice/cudaStreamCreate failed");
        goto fail;
    }
    {
        void *pA = nullptr, *pnb = nullptr, *pt = nullptr, *pn = nullptr, *ps0 = nullptr, *ps1 = nullptr, *pm = nullptr,
             *pbar = nullptr, *perr = nullptr;
        // tiles for the smallest block size the tuner tries (64)
        e->tiles_cap = 0;
        for (int s = 0; s < nsamples; ++s) e->tiles_cap += (e->nf[s] + 63) / 64;
        if ((r = ealloc(e, &pA, (size_t)19 * e->stride * e->elt)) || (r = ealloc(e, &pnb, sizeof(int32_t) * nb.size())) ||
            (r = ealloc(e, &pt, sizeof(EnsTile) * std::max<int64_t>(1, e->tiles_cap))) || (r = ealloc(e, &pn, sizeof(int32_t))) ||
            (r = ealloc(e, &ps0, sizeof(int32_t) * nsamples)) || (r = ealloc(e, &ps1, sizeof(int32_t) * nsamples)) ||
            (r = ealloc(e, &pm, sizeof(double) * 8 * nsamples)) || (r = ealloc(e, &pbar, 2 * sizeof(unsigned int))) ||
            (r = ealloc(e, &perr, sizeof(int32_t)))) {
            g_ens_create_error = e->err;
            goto fail;
        }
        if (cudaMemcpy(pnb, nb.data(), sizeof(int32_t) * nb.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(ps0, seg0.data(), sizeof(int32_t) * nsamples, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(ps1, seg1.data(), sizeof(int32_t) * nsamples, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(pbar, 0, 2 * sizeof(unsigned int)) != cudaSuccess || cudaMemset(perr, 0, sizeof(int32_t)) != cudaSuccess) {
            r = efail(nullptr, MFLBM_ECUDA, "ensemble upload failed");
            goto fail;
        }
        e->d_tiles = (EnsTile *)pt;
        e->d_ntiles = (int32_t *)pn;
        e->d_seg0 = (int32_t *)ps0;
        e->d_seg1 = (int32_t *)ps1;
        e->d_mon = (double *)pm;
        EnsArgs &a = e->a;
        a.A = pA;
        a.stride = e->stride;
        a.nb = (const int32_t *)pnb;
        a.nf = e->NF;
        a.tiles = e->d_tiles;
        a.ntiles = e->d_ntiles;
        a.scale = 4096.0f;
        a.bar = (unsigned int *)pbar;
        a.err = (int32_t *)perr;
        StepParams &P = a.P;
        P = StepParams{};
        P.force_z = common->force_z;
        P.la_nui1 = 1.0 / common->la_nu1;
        P.mrt = common->mrt;
        P.iper = common->iper; P.jper = common->jper; P.kper = common->kper;
        // singlephase rates (singlephase_3D/0.src/Initialization.F90:87-112)
        const double omega = 1.0 / (3.0 * common->la_nu1 + 0.5);
        P.s_nu = omega;
        P.s_e = omega; P.s_e2 = omega; P.s_pi = omega;
        P.s_q = common->mrt == 1 ? 8.0 * (2.0 - omega) / (8.0 - omega) : omega;
        P.s_t = P.s_q;
        a.fold = fold_rates<double>(P.s_e, P.s_e2, P.s_q, P.s_nu, P.s_pi, P.s_t);
        a.fold.fz = P.force_z;
        a.fold32 = fold_rates<float>(P.s_e, P.s_e2, P.s_q, P.s_nu, P.s_pi, P.s_t);
        a.fold32.fz = (float)P.force_z;
        a.foldff = fold_to_ff(a.fold);
        a.unit = fold_is_unit(a.fold) ? 1 : 0;
        a.spin_limit = kBarrierSpinsDefault;
        a.bar_extra = 0;
    }
    e->block = 128;
    e->persistent = 0;
    e->grid = grid_for(e, e->block, 0);
    if ((r = rebuild_tiles(e))) {
        g_ens_create_error = e->err;
        goto fail;
    }
    *out = e;
    return MFLBM_OK;
fail:
    mflbm_ensemble_destroy(e);
    return r;
}

int32_t mflbm_ensemble_init(mflbm_ensemble *e) {
    if (!e) return MFLBM_EINVAL;
    EK(e, cudaSetDevice(e->dev));
    int r = clear_barrier(e);
    if (r) return r;
    e->kt->ens_init(e->a, e->p.precision, e->stream);
    EK(e, cudaPeekAtLastError());
    EK(e, cudaStreamSynchronize(e->stream));
    return MFLBM_OK;
}

int32_t mflbm_ensemble_set_active(mflbm_ensemble *e, const int32_t *active) {
    if (!e || !active) return MFLBM_EINVAL;
    EK(e, cudaSetDevice(e->dev));
    for (int s = 0; s < e->n; ++s) e->active[s] = active[s] ? 1 : 0;
    return rebuild_tiles(e);
}

// nsteps AA steps of every active sample, from a CUDA graph captured once per
// (parity of ntime0, nsteps).  Asynchronous.
int32_t mflbm_ensemble_run(mflbm_ensemble *e, int32_t ntime0, int32_t nsteps) {
    if (!e || nsteps < 0) return MFLBM_EINVAL;
    if (nsteps == 0) return MFLBM_OK;
    EK(e, cudaSetDevice(e->dev));
    const std::pair<int, int> key(ntime0 & 1, nsteps);
    auto it = e->graphs.find(key);
    if (it == e->graphs.end()) {
        cudaGraph_t g = nullptr;
        EK(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        int r = launch(e, ntime0, nsteps);
        cudaError_t c = cudaStreamEndCapture(e->stream, &g);
        if (r) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        if (c != cudaSuccess) return ecuda(e, c, "cudaStreamEndCapture");
        cudaGraphExec_t ex = nullptr;
        c = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (c != cudaSuccess) return ecuda(e, c, "cudaGraphInstantiate");
        it = e->graphs.emplace(key, ex).first;
    }
    EK(e, cudaGraphLaunch(it->second, e->stream));
    return MFLBM_OK;
}

// Per-sample sum of w over the fluid nodes (compute_macro_vars, valid after even
// steps), |u|^2 maximum, and the run status: MFLBM_FAILED when a sum is NaN or
// sqrt(umax^2) > 0.5 in an active sample (singlephase Monitor.F90:158-165), or
// MFLBM_ETIMEOUT as the return code when a grid barrier of the persistent kernel gave
// up.  Synchronises.
int32_t mflbm_ensemble_flux(mflbm_ensemble *e, double *w_sum, double *umax2, int32_t *status) {
    if (!e) return MFLBM_EINVAL;
    EK(e, cudaSetDevice(e->dev));
    e->kt->ens_monitor(e->a, e->p.precision, e->d_seg0, e->d_seg1, e->n, e->d_mon, e->stream);
    EK(e, cudaPeekAtLastError());
    std::vector<double> h((size_t)8 * e->n);
    EK(e, cudaMemcpyAsync(h.data(), e->d_mon, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, e->stream));
    int32_t berr = 0;
    EK(e, cudaMemcpyAsync(&berr, e->a.err, sizeof(int32_t), cudaMemcpyDeviceToHost, e->stream));
    EK(e, cudaStreamSynchronize(e->stream));
    if (berr) return efail(e, MFLBM_ETIMEOUT, "a grid barrier of the persistent ensemble kernel timed out");
    int32_t st = MFLBM_RUNNING;
    for (int s = 0; s < e->n; ++s) {
        if (w_sum) w_sum[s] = h[s];
        if (umax2) umax2[s] = h[(size_t)7 * e->n + s];
        if (e->active[s] && (std::isnan(h[s]) || std::isnan(h[(size_t)6 * e->n + s]) || std::sqrt(h[(size_t)7 * e->n + s]) > 0.5))
            st = MFLBM_FAILED;
    }
    if (status) *status = st;
    return MFLBM_OK;
}

// Launch shape in use and the fluid nodes of the active samples.
int32_t mflbm_ensemble_info(const mflbm_ensemble *e, int64_t *active_nodes, int32_t *block, int32_t *persistent,
                            int32_t *grid) {
    if (!e) return MFLBM_EINVAL;
    if (active_nodes) *active_nodes = e->active_nodes;
    if (block) *block = e->block;
    if (persistent) *persistent = e->persistent;
    if (grid) *grid = e->grid;
    return MFLBM_OK;
}

// Apply a launch shape (block 64..1024, multiple of 32; persistent 0/1).
int32_t mflbm_ensemble_configure(mflbm_ensemble *e, int32_t block, int32_t persistent) {
    if (!e || block < 64 || block > 1024 || block % 32) return efail(e, MFLBM_EINVAL, "block must be 64..1024, a multiple of 32");
    EK(e, cudaSetDevice(e->dev));
    const int g = grid_for(e, block, persistent ? 1 : 0);
    if (g <= 0) return efail(e, MFLBM_EINVAL, "block size does not fit the persistent kernel");
    e->block = block;
    e->persistent = persistent ? 1 : 0;
    e->grid = g;
    drop_graphs(e);
    int r = clear_barrier(e);
    if (r) return r;
    return rebuild_tiles(e);
}

// Diagnostics for the failure path of the persistent kernel's grid barrier (no
// counterpart in the reference): spin_limit polls per wait (<= 0: the default), and
// unreachable = 1 makes every barrier wait for one block more than the grid holds, so
// that each wait runs out, the kernel returns early and mflbm_ensemble_flux reports
// MFLBM_ETIMEOUT.  Clears the barrier state; captured graphs are dropped.
int32_t mflbm_ensemble_set_wait(mflbm_ensemble *e, int64_t spin_limit, int32_t unreachable) {
    if (!e) return MFLBM_EINVAL;
    EK(e, cudaSetDevice(e->dev));
    EK(e, cudaStreamSynchronize(e->stream));
    e->a.spin_limit = spin_limit > 0 ? (long long)spin_limit : kBarrierSpinsDefault;
    e->a.bar_extra = unreachable ? 1u : 0u;
    drop_graphs(e);
    int r = clear_barrier(e);
    if (r) return r;
    EK(e, cudaStreamSynchronize(e->stream));
    return MFLBM_OK;
}

// In-project autotuner: times every candidate launch shape over `steps` steps (after
// two warm-up steps) on the ensemble's own arena and applies the fastest.  The PDF
// state changes while tuning; call mflbm_ensemble_init afterwards.  report (may be
// NULL) receives one JSON object with the timings.
int32_t mflbm_ensemble_tune(mflbm_ensemble *e, int32_t steps, char *report, int32_t report_len) {
    if (!e || steps < 2) return MFLBM_EINVAL;
    EK(e, cudaSetDevice(e->dev));
    const int blocks[] = {64, 128, 256, 512};
    cudaEvent_t t0, t1;
    EK(e, cudaEventCreate(&t0));
    EK(e, cudaEventCreate(&t1));
    std::string js = "{\"candidates\": [";
    double best = 1e300;
    int best_b = 128, best_p = 0;
    bool first = true;
    for (int pers = 0; pers < 2; ++pers)
        for (int b : blocks) {
            if (mflbm_ensemble_configure(e, b, pers) != MFLBM_OK) continue;
            if (mflbm_ensemble_run(e, 1, 2) != MFLBM_OK) continue;
            if (mflbm_ensemble_run(e, 3, steps) != MFLBM_OK) continue;   // capture outside the timing
            cudaEventRecord(t0, e->stream);
            mflbm_ensemble_run(e, 3, steps);
            cudaEventRecord(t1, e->stream);
            if (cudaEventSynchronize(t1) != cudaSuccess) break;
            int32_t berr = 0;
            cudaMemcpy(&berr, e->a.err, sizeof(int32_t), cudaMemcpyDeviceToHost);
            if (berr) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            char buf[160];
            std::snprintf(buf, sizeof buf, "%s{\"block\": %d, \"persistent\": %d, \"grid\": %d, \"ms_per_step\": %.5f}",
                          first ? "" : ", ", b, pers, e->grid, ms / steps);
            js += buf;
            first = false;
            if (ms < best) { best = ms; best_b = b; best_p = pers; }
        }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    int32_t berr = 0;
    EK(e, cudaMemcpy(&berr, e->a.err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (berr) return efail(e, MFLBM_ETIMEOUT, "a grid barrier of the persistent ensemble kernel timed out");
    if (first) return efail(e, MFLBM_ECUDA, "no launch shape ran: " + e->err);
    int r = mflbm_ensemble_configure(e, best_b, best_p);
    if (r) return r;
    char buf[128];
    std::snprintf(buf, sizeof buf, "], \"chosen\": {\"block\": %d, \"persistent\": %d, \"grid\": %d}}", e->block,
                  e->persistent, e->grid);
    js += buf;
    if (report && report_len > 0) {
        std::snprintf(report, (size_t)report_len, "%s", js.c_str());
    }
    return MFLBM_OK;
}

}  // extern "C"
