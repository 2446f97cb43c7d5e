// nn_gemm.cu -- BF16 GEMM on the fifth-generation tensor cores (tcgen05, TMEM
// accumulators), the contraction under every convolution of the warm-start network.
//
//   C[M][N] (fp32, ldc) = (accumulate ? C : 0) + A[M][K] * B[N][K]^T
//   A, B bf16, K contiguous (row strides lda, ldb: multiples of 8 elements), FP32
//   accumulation in TMEM.  M, N, K arbitrary with N % 16 == 0 and K % 8 == 0: tiles
//   are zero-filled past the edges and the epilogue masks them.
//
// One CTA = 4 warps computes a 128 x BN tile.  K advances in steps of 64 (one 128-byte
// swizzle row) through a 3-stage shared-memory ring filled with cp.async (16-byte
// chunks placed at their 128B-swizzled positions); one thread issues four
// tcgen05.mma (K = 16 each) per stage and commits them to the stage's mbarrier, which
// gates the refill.  The epilogue reads the accumulator rows of each warp's 32 TMEM
// lanes with tcgen05.ld.  Every mbarrier wait is bounded.  A wait that runs out makes
// the whole block give up together (the decision is taken with __syncthreads_and, so no
// warp runs a collective tcgen05 instruction alone): it sets *err, waits (bounded again)
// for the MMAs it issued, frees its TMEM and returns without writing its tile; that
// tile of C is then undefined and the host reports MFLBM_ETIMEOUT from *err.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <mutex>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/mflbm.h"
#include "umma.cuh"

namespace mflbm {
namespace nn {

constexpr int kStages = 3;
constexpr long long kWaitLimit = 1ll << 22;   // probes of one mbarrier wait (default)

// Diagnostics of the timeout path (mflbm_nn_set_wait): the probe limit of every wait,
// and whether the MMA thread skips its tensor-core work and commits, so that no
// mbarrier phase ever completes and every wait runs out.
std::atomic<long long> g_wait_limit{kWaitLimit};
std::atomic<int> g_skip_commit{0};

template <int BN>
struct GemmSmem {
    static constexpr int kA = 128 * 128;   // bytes per stage: 128 rows x 128 B
    static constexpr int kB = BN * 128;
    static constexpr int kStage = kA + kB;
    static constexpr int kBytes = kStages * kStage + 1024;   // + alignment slack
};

template <int BN>
__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16 *__restrict__ A, int lda,
                                                   const __nv_bfloat16 *__restrict__ B, int ldb, float *__restrict__ C,
                                                   int ldc, int M, int N, int K, int accumulate, int *__restrict__ err,
                                                   long long wait_limit, int skip_commit) {
    using namespace umma;
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t bars[kStages];
    __shared__ uint32_t tmem_slot;
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
    // split-K: slice blockIdx.z of gridDim.z covers k-tiles [kt0, kt0 + KT) and writes its
    // partial product to its own C slice (reduced afterwards)
    const int KTall = (K + 63) / 64;
    const int kt0 = (int)((int64_t)KTall * blockIdx.z / gridDim.z);
    const int KT = (int)((int64_t)KTall * (blockIdx.z + 1) / gridDim.z) - kt0;
    C += (int64_t)blockIdx.z * M * ldc;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;

    if (warp == 0) {
        tmem_alloc(&tmem_slot, kCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    auto load_stage = [&](int s, int kt) {
        uint8_t *sa = smem + s * GemmSmem<BN>::kStage;
        uint8_t *sb = sa + GemmSmem<BN>::kA;
        const int k0 = (kt0 + kt) * 64;
        // A: 128 rows x 8 chunks
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = tid + i * 128;
            const int r = idx >> 3, c = idx & 7;
            const int gr = m0 + r, gk = k0 + c * 8;
            const bool ok = gr < M && gk < K;
            const __nv_bfloat16 *src = ok ? A + (int64_t)gr * lda + gk : A;
            cp_async16(sa + r * 128 + ((c ^ (r & 7)) << 4), src, ok);
        }
        // B: BN rows x 8 chunks
#pragma unroll
        for (int i = 0; i < (BN * 8 + 127) / 128; ++i) {
            const int idx = tid + i * 128;
            if (idx < BN * 8) {
                const int r = idx >> 3, c = idx & 7;
                const int gn = n0 + r, gk = k0 + c * 8;
                const bool ok = gn < N && gk < K;
                const __nv_bfloat16 *src = ok ? B + (int64_t)gn * ldb + gk : B;
                cp_async16(sb + r * 128 + ((c ^ (r & 7)) << 4), src, ok);
            }
        }
    };

    bool ok = true;   // block-uniform: every change goes through __syncthreads_and
    int last_commit = -1;   // k-tile of the last commit of thread 0
    for (int s = 0; s < kStages - 1; ++s) {
        if (s < KT) load_stage(s, s);
        cp_async_commit();
    }
    const uint32_t idesc = idesc_bf16_f32(128, BN);
    for (int kt = 0; kt < KT && ok; ++kt) {
        const int s = kt % kStages;
        cp_async_wait<kStages - 2>();
        fence_async_smem();
        __syncthreads();
        if (tid == 0 && !skip_commit) {
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + s * GemmSmem<BN>::kStage);
            const uint32_t sb = sa + GemmSmem<BN>::kA;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                mma_bf16(tmem, desc_sw128(sa + j * 32), desc_sw128(sb + j * 32), idesc, (kt > 0 || j > 0) ? 1u : 0u);
            mma_commit(&bars[s]);
            last_commit = kt;
        }
        // refill the stage that MMA kt-1 read once it has completed (nk < KT is the same
        // for every thread, so all of them reach the vote)
        const int nk = kt + kStages - 1;
        if (nk < KT) {
            bool w = true;
            if (kt >= 1) {
                const int ps = (kt - 1) % kStages;
                w = mbar_wait(&bars[ps], (uint32_t)(((kt - 1) / kStages) & 1), wait_limit);
            }
            ok = __syncthreads_and(w) != 0;
            if (ok) load_stage(nk % kStages, nk);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    // all MMAs issued so far complete when the last commit arrives
    bool fin = ok;
    if (ok && KT > 0) {
        const int ls = (KT - 1) % kStages;
        fin = mbar_wait(&bars[ls], (uint32_t)(((KT - 1) / kStages) & 1), wait_limit);
    }
    ok = __syncthreads_and(fin) != 0;
    if (!ok) {
        if (tid == 0) {
            atomicExch(err, 1);
            // the MMAs this block issued must be done before their TMEM is freed
            if (last_commit >= 0)
                (void)mbar_wait(&bars[last_commit % kStages], (uint32_t)((last_commit / kStages) & 1), wait_limit);
        }
        __syncthreads();
    }
    tc_fence_after();
    if (ok) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if (KT > 0) {
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            if (row < M) {
                float *dst = C + (int64_t)row * ldc + n0 + c0;
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (n0 + c0 + i < N) dst[i] = accumulate ? dst[i] + v[i] : v[i];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kCols);
}

// The dynamic shared-memory opt-in of cudaFuncSetAttribute applies to the current
// device only: it is made once per device and tile width, under a lock.
constexpr int kMaxDevices = 64;
std::mutex g_attr_mu;
bool g_attr_done[kMaxDevices][4] = {};

template <int BN> constexpr int bn_slot() { return BN == 128 ? 0 : (BN == 64 ? 1 : (BN == 32 ? 2 : 3)); }

template <int BN>
int launch_gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, float *C, int ldc, int M, int N, int K,
                int accumulate, int ksplit, int *err, cudaStream_t s) {
    const int bytes = GemmSmem<BN>::kBytes;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MFLBM_ENODEV;
    {
        std::lock_guard<std::mutex> lock(g_attr_mu);
        if (!g_attr_done[dev][bn_slot<BN>()]) {
            if (cudaFuncSetAttribute(k_gemm_bf16<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
                return MFLBM_ECUDA;
            g_attr_done[dev][bn_slot<BN>()] = true;
        }
    }
    dim3 grid((M + 127) / 128, (N + BN - 1) / BN, ksplit);
    k_gemm_bf16<BN><<<grid, 128, bytes, s>>>(A, lda, B, ldb, C, ldc, M, N, K, accumulate, err, g_wait_limit.load(),
                                             g_skip_commit.load());
    return cudaPeekAtLastError() == cudaSuccess ? MFLBM_OK : MFLBM_ECUDA;
}

// C[m][n] (+)= sum over z of P[z][m][n]
__global__ void k_splitk_reduce(const float *__restrict__ P, int ks, float *__restrict__ C, int ldc, int M, int N,
                                int accumulate) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)M * N) return;
    const int64_t m = t / N;
    const int n = (int)(t - m * N);
    float acc = 0.f;
    for (int z = 0; z < ks; ++z) acc += P[((int64_t)z * M + m) * N + n];
    C[m * ldc + n] = accumulate ? C[m * ldc + n] + acc : acc;
}

int gemm_dispatch(const __nv_bfloat16 *a, int lda, const __nv_bfloat16 *b, int ldb, float *C, int ldc, int M, int N,
                  int K, int accumulate, int ks, int *err, cudaStream_t s) {
    if (N % 128 == 0 || N > 64) return launch_gemm<128>(a, lda, b, ldb, C, ldc, M, N, K, accumulate, ks, err, s);
    if (N > 32) return launch_gemm<64>(a, lda, b, ldb, C, ldc, M, N, K, accumulate, ks, err, s);
    if (N > 16) return launch_gemm<32>(a, lda, b, ldb, C, ldc, M, N, K, accumulate, ks, err, s);
    return launch_gemm<16>(a, lda, b, ldb, C, ldc, M, N, K, accumulate, ks, err, s);
}

}  // namespace nn
}  // namespace mflbm

using namespace mflbm;

extern "C" int32_t mflbm_nn_gemm_bf16(const void *A, int32_t lda, const void *B, int32_t ldb, float *C, int32_t ldc,
                                      int32_t M, int32_t N, int32_t K, int32_t accumulate, int32_t *err, void *stream) {
    if (!A || !B || !C || !err || M < 0 || N < 0 || K < 0) return MFLBM_EINVAL;
    if (N % 16 || K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N) return MFLBM_EINVAL;
    if (((uintptr_t)A | (uintptr_t)B) & 15) return MFLBM_EINVAL;
    if (M == 0 || N == 0) return MFLBM_OK;
    return nn::gemm_dispatch((const __nv_bfloat16 *)A, lda, (const __nv_bfloat16 *)B, ldb, C, ldc, M, N, K, accumulate, 1,
                             err, (cudaStream_t)stream);
}

// Diagnostics of the GEMM's timeout path (no counterpart in the reference): the probe
// limit of every mbarrier wait of later GEMMs (<= 0: the default) and skip_commit = 1,
// which makes the MMA thread issue no tensor-core work and no commit, so that every wait
// runs out and *err is set.  Process-wide; not for concurrent use with real GEMMs.
extern "C" int32_t mflbm_nn_set_wait(int64_t wait_limit, int32_t skip_commit) {
    nn::g_wait_limit.store(wait_limit > 0 ? (long long)wait_limit : nn::kWaitLimit);
    nn::g_skip_commit.store(skip_commit ? 1 : 0);
    return MFLBM_OK;
}

// Split-K form for long reductions (weight gradients reduce over every voxel): ksplit
// CTAs share each output tile; work holds ksplit * M * N floats of partial products.
extern "C" int32_t mflbm_nn_gemm_bf16_splitk(const void *A, int32_t lda, const void *B, int32_t ldb, float *C, int32_t ldc,
                                             int32_t M, int32_t N, int32_t K, int32_t accumulate, int32_t ksplit,
                                             float *work, int32_t *err, void *stream) {
    if (!A || !B || !C || !err || !work || M < 0 || N < 0 || K < 0 || ksplit < 1 || ksplit > 4096) return MFLBM_EINVAL;
    if (N % 16 || K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N) return MFLBM_EINVAL;
    if (((uintptr_t)A | (uintptr_t)B) & 15) return MFLBM_EINVAL;
    if (M == 0 || N == 0) return MFLBM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int ks = std::max(1, std::min(ksplit, (K + 63) / 64));
    int r = nn::gemm_dispatch((const __nv_bfloat16 *)A, lda, (const __nv_bfloat16 *)B, ldb, work, N, M, N, K, 0, ks, err, s);
    if (r) return r;
    const int64_t n = (int64_t)M * N;
    nn::k_splitk_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(work, ks, C, ldc, M, N, accumulate);
    return cudaPeekAtLastError() == cudaSuccess ? MFLBM_OK : MFLBM_ECUDA;
}
