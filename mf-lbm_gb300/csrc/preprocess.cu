// preprocess.cu -- geometry_preprocessing_new on the GPU
// (multiphase_3D/0.src/Geometry_preprocessing.F90:9-512, one rank).
//
// The reference runs this once per job on the host, single-rank and slow for large grids
// (its own comment at :5-7).  Here every stage is a kernel over the extended wall array:
//   1. extension by gl = 10 ghost layers per side: periodic directions wrap, the others
//      repeat the edge plane (:36-119);
//   2. classification (:121-143): solid with a fluid D3Q19 neighbour -> 2 (solid boundary),
//      fluid with a solid neighbour -> -1 (fluid boundary);
//   3. four Jacobi iterations of the 27-point smoothing of the solid indicator with weights
//      8/27, 2/27, 1/54, 1/216 accumulated in the order n = 0..26 (:145-169);
//   4. the two boundary-node lists in the reference's k, j, i order (:171-225, local
//      filters :429-507): la_weight and the fluid-neighbour directions of every solid
//      boundary node, the ISO8 gradient of the smoothed field normalised with + 1e-14 at
//      every fluid boundary node (:234-383), and theta (:505).
// Products and sums use __dmul_rn/__dadd_rn/__dsub_rn (never contracted into FMA) in the
// host restatement's order, so the lists are bit-identical to it.  List order comes from a
// two-level exclusive scan of per-cell flags (block counts scanned on the host).
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/mflbm.h"
#include "common.cuh"

namespace mflbm {
namespace prep {

constexpr int GL = 10;
constexpr int CHUNK = 8;            // cells per thread in the flag scan
constexpr int SCAN_THREADS = 256;

struct Ext {
    int nx, ny, nz;                 // lattice
    int ex, ey, ez;                 // extended extents (n + 2*GL)
    __host__ __device__ int64_t idx(int a, int b, int c) const { return ((int64_t)a * ey + b) * ex + c; }  // [k][j][i]
};

__device__ __forceinline__ int map_axis(int e, int n, int per) {
    int c = e - GL + 1;             // lattice coordinate, 1-based
    if (c >= 1 && c <= n) return c;
    if (per) return c < 1 ? c + n : c - n;
    return c < 1 ? 1 : n;
}

__global__ void k_extend(const int8_t *__restrict__ walls, int8_t *__restrict__ wt, Ext E, int px, int py, int pz) {
    const int64_t n = (int64_t)E.ez * E.ey * E.ex;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t % E.ex), j = (int)((t / E.ex) % E.ey), k = (int)(t / ((int64_t)E.ex * E.ey));
    const int ci = map_axis(i, E.nx, px), cj = map_axis(j, E.ny, py), ck = map_axis(k, E.nz, pz);
    wt[t] = walls[((int64_t)(ck - 1) * E.ny + (cj - 1)) * E.nx + (ci - 1)];
}

// classification and the FP64 copy of the indicator
__global__ void k_classify(const int8_t *__restrict__ wt, int8_t *__restrict__ cls, double *__restrict__ s, Ext E) {
    const int64_t n = (int64_t)E.ez * E.ey * E.ex;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t % E.ex), j = (int)((t / E.ex) % E.ey), k = (int)(t / ((int64_t)E.ex * E.ey));
    const int8_t w = wt[t];
    s[t] = (double)w;
    int8_t c = w;
    if (i >= 1 && i < E.ex - 1 && j >= 1 && j < E.ey - 1 && k >= 1 && k < E.ez - 1) {
        int mn = 127, mx = -128;
#pragma unroll
        for (int q = 1; q < 19; ++q) {
            const int v = wt[E.idx(k + EZ(q), j + EY(q), i + EX(q))];
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
        }
        if (w == 1 && mn <= 0) c = 2;
        else if (w == 0 && mx >= 1) c = -1;
    }
    cls[t] = c;
}

// one smoothing iteration over the inner region (the outer layer keeps its value)
__constant__ int c_iex[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
__constant__ int c_iey[27] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1};
__constant__ int c_iez[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1};

__global__ void k_smooth(const double *__restrict__ src, double *__restrict__ dst, Ext E) {
    const int64_t n = (int64_t)E.ez * E.ey * E.ex;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t % E.ex), j = (int)((t / E.ex) % E.ey), k = (int)(t / ((int64_t)E.ex * E.ey));
    if (!(i >= 1 && i < E.ex - 1 && j >= 1 && j < E.ey - 1 && k >= 1 && k < E.ez - 1)) {
        dst[t] = src[t];
        return;
    }
    const double we[4] = {8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0};
    double acc = 0.0;
    for (int q = 0; q < 27; ++q) {
        const int m = c_iex[q] * c_iex[q] + c_iey[q] * c_iey[q] + c_iez[q] * c_iez[q];
        acc = __dadd_rn(acc, __dmul_rn(src[E.idx(k + c_iez[q], j + c_iey[q], i + c_iex[q])], we[m]));
    }
    dst[t] = acc;
}

// ISO8 gradient terms: (coefficient group, plus offset, minus offset); the order of the
// host restatement (groups in order, pairs in order, acc = (acc + a) - b)
struct Iso8 {
    int ngroup;
    int count[7];
    signed char off[7][12][6];      // dx+, dy+, dz+, dx-, dy-, dz-
};

__constant__ double c_iso8[7];
__constant__ Iso8 c_nw[3];

__device__ double iso8(const double *__restrict__ s, const Ext &E, int k, int j, int i, int comp) {
    const Iso8 &g = c_nw[comp];
    double total = 0.0;
    for (int grp = 0; grp < g.ngroup; ++grp) {
        double acc = 0.0;
        for (int p = 0; p < g.count[grp]; ++p) {
            const signed char *o = g.off[grp][p];
            const double a = s[E.idx(k + o[2], j + o[1], i + o[0])];
            const double b = s[E.idx(k + o[5], j + o[4], i + o[3])];
            acc = p == 0 ? __dsub_rn(a, b) : __dsub_rn(__dadd_rn(acc, a), b);
        }
        const double term = __dmul_rn(c_iso8[grp], acc);
        total = grp == 0 ? term : __dadd_rn(total, term);
    }
    return total;
}

// list region: lattice coordinates [-3, n+4] (the sub-box of the host restatement)
struct Region {
    int lo, nx, ny, nz;             // lo = -3
    int64_t size() const { return (int64_t)(nx + 8) * (ny + 8) * (nz + 8); }
};

__device__ __forceinline__ void region_cell(int64_t r, int nx, int ny, int &i, int &j, int &k) {
    const int rx = nx + 8, ry = ny + 8;
    i = (int)(r % rx) - 3;
    j = (int)((r / rx) % ry) - 3;
    k = (int)(r / ((int64_t)rx * ry)) - 3;
}

__device__ __forceinline__ int8_t cls_at(const int8_t *cls, const Ext &E, int i, int j, int k) {
    // lattice coordinate c sits at extended index c - 1 + GL
    return cls[E.idx(k - 1 + GL, j - 1 + GL, i - 1 + GL)];
}

__device__ __forceinline__ int flag_of(const int8_t *cls, const Ext &E, int i, int j, int k, int which) {
    const int8_t c = cls_at(cls, E, i, j, k);
    if (which == 0)
        return c == 2 && i >= -2 && i <= E.nx + 3 && j >= -2 && j <= E.ny + 3 && k >= -2 && k <= E.nz + 3;
    return c == -1 && i >= -1 && i <= E.nx + 2 && j >= -1 && j <= E.ny + 2 && k >= -1 && k <= E.nz + 2;
}

// per-block flag counts (CHUNK consecutive cells per thread)
__global__ void k_count(const int8_t *__restrict__ cls, Ext E, int64_t nreg, int which, int32_t *__restrict__ counts) {
    const int64_t base = ((int64_t)blockIdx.x * SCAN_THREADS + threadIdx.x) * CHUNK;
    int c = 0;
    for (int u = 0; u < CHUNK; ++u) {
        const int64_t r = base + u;
        if (r < nreg) {
            int i, j, k;
            region_cell(r, E.nx, E.ny, i, j, k);
            c += flag_of(cls, E, i, j, k, which);
        }
    }
    __shared__ int32_t red[SCAN_THREADS];
    red[threadIdx.x] = c;
    __syncthreads();
    for (int s = SCAN_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[blockIdx.x] = red[0];
}

// writes the records of this block at offsets[block] + in-block exclusive scan
__global__ void k_emit(const int8_t *__restrict__ cls, const double *__restrict__ s2, Ext E, int64_t nreg, int which,
                       const int32_t *__restrict__ offsets, mflbm_solid_bnd *solid, mflbm_fluid_bnd *fluid,
                       double theta) {
    const int64_t base = ((int64_t)blockIdx.x * SCAN_THREADS + threadIdx.x) * CHUNK;
    int mine = 0;
    for (int u = 0; u < CHUNK; ++u) {
        const int64_t r = base + u;
        if (r < nreg) {
            int i, j, k;
            region_cell(r, E.nx, E.ny, i, j, k);
            mine += flag_of(cls, E, i, j, k, which);
        }
    }
    __shared__ int32_t sc[SCAN_THREADS];
    sc[threadIdx.x] = mine;
    __syncthreads();
    for (int off = 1; off < SCAN_THREADS; off <<= 1) {      // Hillis-Steele inclusive scan
        const int32_t v = (int)threadIdx.x >= off ? sc[threadIdx.x - off] : 0;
        __syncthreads();
        sc[threadIdx.x] += v;
        __syncthreads();
    }
    int32_t pos = offsets[blockIdx.x] + sc[threadIdx.x] - mine;
    const double w_equ[3] = {1.0 / 3.0, 1.0 / 18.0, 1.0 / 36.0};
    for (int u = 0; u < CHUNK; ++u) {
        const int64_t r = base + u;
        if (r >= nreg) break;
        int i, j, k;
        region_cell(r, E.nx, E.ny, i, j, k);
        if (!flag_of(cls, E, i, j, k, which)) continue;
        if (which == 0) {
            mflbm_solid_bnd b;
            b.ix = i; b.iy = j; b.iz = k;
            int cnt = 0;
            double lw = 0.0;
            for (int q = 0; q < 18; ++q) b.neighbor_list[q] = 0;
            for (int q = 1; q < 19; ++q) {
                if (cls_at(cls, E, i + EX(q), j + EY(q), k + EZ(q)) <= 0) {
                    lw = __dadd_rn(lw, w_equ[q <= 6 ? 1 : 2]);
                    b.neighbor_list[cnt++] = q;
                }
            }
            b.i_fluid_num = cnt;
            b.la_weight = lw;
            solid[pos] = b;
        } else {
            const int ki = k - 1 + GL, ji = j - 1 + GL, ii = i - 1 + GL;
            const double gx = iso8(s2, E, ki, ji, ii, 0);
            const double gy = iso8(s2, E, ki, ji, ii, 1);
            const double gz = iso8(s2, E, ki, ji, ii, 2);
            const double nrm = __dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz));
            const double tmp = __ddiv_rn(1.0, __dadd_rn(__dsqrt_rn(nrm), 1e-14));
            mflbm_fluid_bnd f;
            f.ix = i; f.iy = j; f.iz = k; f._pad = 0;
            f.nwx = __dmul_rn(gx, tmp);
            f.nwy = __dmul_rn(gy, tmp);
            f.nwz = __dmul_rn(gz, tmp);
            f.theta = theta;
            fluid[pos] = f;
        }
        ++pos;
    }
}

}  // namespace prep
}  // namespace mflbm

namespace {

// ISO8 gradient stencils of the x, y, z components: the "+" offsets (dx, dy, dz) of each
// term per coefficient group; every "-" offset is the negation
const int kGroupSize[7] = {1, 4, 4, 1, 8, 12, 4};
const int kNw[3][34][3] = {
    {{1, 0, 0},
     {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1},
     {1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
     {2, 0, 0},
     {2, 1, 0}, {2, -1, 0}, {2, 0, 1}, {2, 0, -1}, {1, 2, 0}, {1, -2, 0}, {1, 0, 2}, {1, 0, -2},
     {2, 1, 1}, {2, 1, -1}, {2, -1, 1}, {2, -1, -1}, {1, 2, 1}, {1, 2, -1}, {1, -2, 1}, {1, -2, -1},
     {1, 1, 2}, {1, 1, -2}, {1, -1, 2}, {1, -1, -2},
     {2, 2, 0}, {2, -2, 0}, {2, 0, 2}, {2, 0, -2}},
    {{0, 1, 0},
     {1, 1, 0}, {-1, 1, 0}, {0, 1, 1}, {0, 1, -1},
     {1, 1, 1}, {1, 1, -1}, {-1, 1, -1}, {-1, 1, 1},
     {0, 2, 0},
     {2, 1, 0}, {-2, 1, 0}, {0, 2, 1}, {0, 2, -1}, {1, 2, 0}, {-1, 2, 0}, {0, 1, 2}, {0, 1, -2},
     {2, 1, 1}, {2, 1, -1}, {-2, 1, 1}, {-2, 1, -1}, {1, 2, 1}, {1, 2, -1}, {-1, 2, 1}, {-1, 2, -1},
     {1, 1, 2}, {1, 1, -2}, {-1, 1, 2}, {-1, 1, -2},
     {2, 2, 0}, {-2, 2, 0}, {0, 2, 2}, {0, 2, -2}},
    {{0, 0, 1},
     {0, 1, 1}, {0, -1, 1}, {1, 0, 1}, {-1, 0, 1},
     {1, 1, 1}, {1, -1, 1}, {-1, 1, 1}, {-1, -1, 1},
     {0, 0, 2},
     {0, 1, 2}, {0, -1, 2}, {2, 0, 1}, {-2, 0, 1}, {0, 2, 1}, {0, -2, 1}, {1, 0, 2}, {-1, 0, 2},
     {2, 1, 1}, {2, -1, 1}, {-2, 1, 1}, {-2, -1, 1}, {1, 2, 1}, {1, -2, 1}, {-1, 2, 1}, {-1, -2, 1},
     {1, 1, 2}, {1, -1, 2}, {-1, 1, 2}, {-1, -1, 2},
     {0, 2, 2}, {0, -2, 2}, {2, 0, 2}, {-2, 0, 2}}};
const double kIso8[7] = {4.0 / 45.0, 1.0 / 21.0, 2.0 / 105.0, 5.0 / 504.0, 1.0 / 315.0, 1.0 / 630.0, 1.0 / 5040.0};

thread_local std::string g_prep_error;

int pfail(int code, const std::string &m) {
    g_prep_error = m;
    return code;
}

struct DevBuf {
    std::vector<void *> p;
    ~DevBuf() {
        for (void *q : p) cudaFree(q);
    }
    template <class T> T *get(size_t n) {
        void *q = nullptr;
        if (cudaMalloc(&q, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (T *)q;
    }
};

}  // namespace

using namespace mflbm;
using namespace mflbm::prep;

extern "C" {

const char *mflbm_preprocess_last_error(void) { return g_prep_error.c_str(); }

int32_t mflbm_preprocess_geometry(const mflbm_params *p, const int8_t *walls, double theta, mflbm_solid_bnd *solid,
                                  int32_t solid_cap, int32_t *n_solid, mflbm_fluid_bnd *fluid, int32_t fluid_cap,
                                  int32_t *n_fluid) {
    if (!p || !walls || !n_solid || !n_fluid) return pfail(MFLBM_EINVAL, "NULL argument");
    const int per[3] = {p->iper, p->jper, p->kper};
    const int n[3] = {p->nx, p->ny, p->nz};
    for (int a = 0; a < 3; ++a) {
        if (n[a] < 1) return pfail(MFLBM_EINVAL, "lattice dimensions must be positive");
        if (per[a] && n[a] < GL) return pfail(MFLBM_EINVAL, "periodic dimensions below 10 cells: use the host preprocessing");
    }
    int dev = p->device;
    if (cudaSetDevice(dev) != cudaSuccess) return pfail(MFLBM_ENODEV, "cudaSetDevice failed");
    Ext E{p->nx, p->ny, p->nz, p->nx + 2 * GL, p->ny + 2 * GL, p->nz + 2 * GL};
    const int64_t next = (int64_t)E.ex * E.ey * E.ez;
    const int64_t nlat = (int64_t)p->nx * p->ny * p->nz;
    const Region R{-3, p->nx, p->ny, p->nz};
    const int64_t nreg = R.size();
    const int64_t per_block = (int64_t)SCAN_THREADS * CHUNK;
    const int64_t nblocks = (nreg + per_block - 1) / per_block;
    if (nblocks > INT32_MAX) return pfail(MFLBM_ERANGE, "lattice too large");
    // stencil tables
    Iso8 tab[3];
    for (int c = 0; c < 3; ++c) {
        tab[c].ngroup = 7;
        int t = 0;
        for (int g = 0; g < 7; ++g) {
            tab[c].count[g] = kGroupSize[g];
            for (int e = 0; e < kGroupSize[g]; ++e, ++t)
                for (int d = 0; d < 3; ++d) {
                    tab[c].off[g][e][d] = (signed char)kNw[c][t][d];
                    tab[c].off[g][e][3 + d] = (signed char)(-kNw[c][t][d]);
                }
        }
    }
    if (cudaMemcpyToSymbol(c_nw, tab, sizeof(tab)) != cudaSuccess ||
        cudaMemcpyToSymbol(c_iso8, kIso8, sizeof(kIso8)) != cudaSuccess)
        return pfail(MFLBM_ECUDA, "stencil tables upload failed");
    DevBuf buf;
    int8_t *dw = buf.get<int8_t>(nlat), *wt = buf.get<int8_t>(next), *cls = buf.get<int8_t>(next);
    double *s1 = buf.get<double>(next), *s2 = buf.get<double>(next);
    int32_t *cnt = buf.get<int32_t>(nblocks), *off = buf.get<int32_t>(nblocks);
    if (!dw || !wt || !cls || !s1 || !s2 || !cnt || !off) return pfail(MFLBM_ENOMEM, "device allocation failed");
    if (cudaMemcpy(dw, walls, nlat, cudaMemcpyHostToDevice) != cudaSuccess) return pfail(MFLBM_ECUDA, "walls upload failed");
    const unsigned g = (unsigned)((next + 255) / 256);
    k_extend<<<g, 256>>>(dw, wt, E, p->iper, p->jper, p->kper);
    k_classify<<<g, 256>>>(wt, cls, s1, E);
    for (int it = 0; it < 4; ++it) {
        k_smooth<<<g, 256>>>(s1, s2, E);
        double *t = s1; s1 = s2; s2 = t;
    }
    double *sm = s1;   // the smoothed field after four iterations
    if (cudaDeviceSynchronize() != cudaSuccess) return pfail(MFLBM_ECUDA, "preprocessing kernels failed");
    std::vector<int32_t> h((size_t)nblocks), o((size_t)nblocks);
    int32_t total[2] = {0, 0};
    for (int which = 0; which < 2; ++which) {
        k_count<<<(unsigned)nblocks, SCAN_THREADS>>>(cls, E, nreg, which, cnt);
        if (cudaMemcpy(h.data(), cnt, sizeof(int32_t) * nblocks, cudaMemcpyDeviceToHost) != cudaSuccess)
            return pfail(MFLBM_ECUDA, "count download failed");
        int64_t acc = 0;
        for (int64_t b = 0; b < nblocks; ++b) {
            o[b] = (int32_t)acc;
            acc += h[b];
        }
        if (acc > INT32_MAX) return pfail(MFLBM_ERANGE, "boundary list exceeds 2^31 entries");
        total[which] = (int32_t)acc;
        const int32_t cap = which == 0 ? solid_cap : fluid_cap;
        void *dst = which == 0 ? (void *)solid : (void *)fluid;
        if (!dst || cap < acc || acc == 0) continue;
        const size_t rec = which == 0 ? sizeof(mflbm_solid_bnd) : sizeof(mflbm_fluid_bnd);
        void *dout = buf.get<uint8_t>((size_t)acc * rec);
        if (!dout) return pfail(MFLBM_ENOMEM, "device allocation failed");
        if (cudaMemcpy(off, o.data(), sizeof(int32_t) * nblocks, cudaMemcpyHostToDevice) != cudaSuccess)
            return pfail(MFLBM_ECUDA, "offset upload failed");
        k_emit<<<(unsigned)nblocks, SCAN_THREADS>>>(cls, sm, E, nreg, which, off, (mflbm_solid_bnd *)dout,
                                                    (mflbm_fluid_bnd *)dout, theta);
        if (cudaMemcpy(dst, dout, (size_t)acc * rec, cudaMemcpyDeviceToHost) != cudaSuccess)
            return pfail(MFLBM_ECUDA, "list download failed");
    }
    *n_solid = total[0];
    *n_fluid = total[1];
    if ((solid && solid_cap < total[0]) || (fluid && fluid_cap < total[1]))
        return pfail(MFLBM_ERANGE, "list capacity too small (counts returned in n_solid, n_fluid)");
    return MFLBM_OK;
}

}  // extern "C"
