// noalloc.cu -- cal_saturation for callers that cannot allocate device memory.
//
// mflbm_saturation_noalloc sums the two phase volumes of a phi field that already lives
// on the device (the same quantity as mflbm_saturation), without a context and without
// allocating anything.  It exists for callers that may not call cudaMalloc themselves
// or have the library do it:
//   - a Fortran/OpenACC host that owns every device array inside its `!$acc data`
//     region and hands the library only `!$acc host_data use_device` pointers -- memory
//     allocated behind the OpenACC runtime's back is outside its present table and pool;
//   - a time loop that shares the GPU with other streams, where cudaMalloc/cudaFree
//     would add an implicit device-wide synchronisation between steps.
//
// The per-slice partial sums go to a fixed scratch array in this file
// (g_noalloc_slices, 2 * MFLBM_NOALLOC_MAX_NZ doubles = 256 KiB per device, held by
// every GPU that loads the library until the process exits).  Every call shares that
// array and it keeps the last call's contents; each call writes all 2*nz slots it later
// reads, so no clearing is needed.  Calls that overlap on the GPU (two streams, or two
// host threads) race on the array and must be serialised by the caller.
//
// The array's device address is looked up once per device (cudaGetSymbolAddress, with
// that device current) and kept for the life of the process.  cudaDeviceReset releases
// the array together with every other allocation of that device, and the kept address
// then points at nothing: a process that resets a device must not call this entry point
// on that device afterwards.
#include <cstdint>
#include <mutex>
#include <string>
#include <cuda_runtime.h>

#include "../../include/mflbm.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_slices[2 * MFLBM_NOALLOC_MAX_NZ];

// per-slice sums of 0.5(1+phi)(1-w) and 0.5(1-phi)(1-w) (Monitor.F90:526-538)
__global__ void __launch_bounds__(kThreads) k_sat_slices(const double *__restrict__ phi, const int8_t *__restrict__ walls,
                                                         int nx, int ny, int nz, double *__restrict__ slices) {
    const int k = blockIdx.x + 1;
    const int64_t n = (int64_t)nx * ny;
    const int64_t h2x = nx + 4, h2xy = (int64_t)(nx + 4) * (ny + 4);
    const int64_t h4x = nx + 8, h4xy = (int64_t)(nx + 8) * (ny + 8);
    double v1 = 0.0, v2 = 0.0;
    for (int64_t t = threadIdx.x; t < n; t += kThreads) {
        const int i = (int)(t % nx) + 1, j = (int)(t / nx) + 1;
        const double m = (double)(1 - walls[(i + 1) + h2x * (j + 1) + h2xy * (k + 1)]);
        const double ph = phi[(i + 3) + h4x * (j + 3) + h4xy * (k + 3)];
        v1 += 0.5 * (1.0 + ph) * m;
        v2 += 0.5 * (1.0 - ph) * m;
    }
    __shared__ double red[2][kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
        v2 += __shfl_down_sync(0xffffffffu, v2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = v1;
        red[1][threadIdx.x >> 5] = v2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) {
            a += red[0][q];
            b += red[1][q];
        }
        slices[k - 1] = a;
        slices[nz + k - 1] = b;
    }
}

// slice order, one thread: the same order as the host loop of mflbm_saturation
__global__ void k_sat_finish(const double *__restrict__ slices, int nz, double *__restrict__ out) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nz; ++k) {
        a += slices[k];
        b += slices[nz + k];
    }
    out[0] = a;
    out[1] = b;
}

std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

}  // namespace

namespace mflbm {
void set_global_error(const std::string &msg);  // api.cu: backs mflbm_last_error(NULL)
}

namespace {
int fail(int code, const std::string &msg) {
    mflbm::set_global_error(msg);
    return code;
}
}  // namespace

extern "C" int32_t mflbm_saturation_noalloc(const double *phi, const int8_t *walls, int32_t nx, int32_t ny, int32_t nz,
                                            double *vol, void *stream) {
    if (!phi || !walls || !vol) return fail(MFLBM_EINVAL, "phi, walls and vol must be device pointers");
    if (nx < 1 || ny < 1 || nz < 1) return fail(MFLBM_EINVAL, "lattice dimensions must be positive");
    if (nz > MFLBM_NOALLOC_MAX_NZ)
        return fail(MFLBM_ERANGE, "nz = " + std::to_string(nz) + " exceeds the scratch limit of " +
                                      std::to_string(MFLBM_NOALLOC_MAX_NZ) + " slices");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MFLBM_ENODEV, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(MFLBM_ENODEV, "device ordinal beyond the supported range");
    void *scratch = nullptr;
    {
        // once per device, with that device current: the host-side name of a
        // __device__ array is not a device address, so look the address up
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_slices);
            if (e != cudaSuccess) return fail(MFLBM_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_addr[dev] = p;
        }
        scratch = g_addr[dev];
    }
    // an error left by earlier work of the caller is reported as such and left in place
    e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return fail(MFLBM_ECUDA, std::string("a CUDA error from earlier work is pending: ") + cudaGetErrorString(e));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    k_sat_slices<<<nz, kThreads, 0, s>>>(phi, walls, nx, ny, nz, static_cast<double *>(scratch));
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        cudaGetLastError();   // this call's own launch error
        return fail(MFLBM_ECUDA, std::string("k_sat_slices launch: ") + cudaGetErrorString(e));
    }
    k_sat_finish<<<1, 1, 0, s>>>(static_cast<const double *>(scratch), nz, vol);
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(MFLBM_ECUDA, std::string("k_sat_finish launch: ") + cudaGetErrorString(e));
    }
    return MFLBM_OK;
}
