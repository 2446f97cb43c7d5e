// nn_ops.cu -- elementwise and data-movement kernels of the warm-start network
// (3-D convolutions on a periodic grid as im2col + tcgen05 GEMM, pooling, upsampling,
// channel concatenation, loss, Adam).  Activations are stored channels-last,
// [D][H][W][C] with voxel index v = (z*H + y)*W + x; the convolutions wrap around the
// grid periodically, like the periodic samples they are trained on.
//
// Every function takes device pointers and a stream and launches its kernels
// asynchronously; sizes are validated on the host.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/mflbm.h"

namespace mflbm {
namespace nn {

__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// col[v][tap*Cin + c] = X[wrap(v + d_tap)][c] for a 3x3x3 stencil, zero in the K padding
// [27*Cin, Kp).  One thread per element of col.
__global__ void k_im2col(const __nv_bfloat16 *__restrict__ X, __nv_bfloat16 *__restrict__ col, int D, int H, int W,
                         int Cin, int Kp) {
    const int64_t nvox = (int64_t)D * H * W;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * Kp) return;
    const int64_t v = t / Kp;
    const int k = (int)(t - v * Kp);
    __nv_bfloat16 val = __float2bfloat16(0.f);
    if (k < 27 * Cin) {
        const int tap = k / Cin, c = k - tap * Cin;
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
        const int64_t u = ((int64_t)wrapi(z + dz, D) * H + wrapi(y + dy, H)) * W + wrapi(x + dx, W);
        val = X[u * Cin + c];
    }
    col[t] = val;
}

// dX[v][c] = sum over taps of dcol[wrap(v - d_tap)][tap*Cin + c]  (adjoint of k_im2col)
__global__ void k_col2im(const float *__restrict__ dcol, float *__restrict__ dX, int D, int H, int W, int Cin, int Kp) {
    const int64_t nvox = (int64_t)D * H * W;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * Cin) return;
    const int64_t v = t / Cin;
    const int c = (int)(t - v * Cin);
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
    float acc = 0.f;
    for (int tap = 0; tap < 27; ++tap) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int64_t u = ((int64_t)wrapi(z - dz, D) * H + wrapi(y - dy, H)) * W + wrapi(x - dx, W);
        acc += dcol[u * Kp + tap * Cin + c];
    }
    dX[t] = acc;
}

// out[r][c] (bf16, ld_out) = in[c][r] (bf16 or fp32 -> bf16) for r < R, c < Cc; zero pad up to
// (Rp, Cp) so the GEMM tiles see zeros.
template <class T>
__global__ void k_transpose_bf16(const T *__restrict__ in, int64_t ld_in, __nv_bfloat16 *__restrict__ out,
                                 int64_t ld_out, int64_t R, int64_t Cc, int64_t Rp, int64_t Cp) {
    __shared__ float tile[32][33];
    // blockIdx.x walks the (long) C dimension, blockIdx.y the R dimension
    const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        tile[i][threadIdx.x] = (c < Cc && r < R) ? (float)in[c * ld_in + r] : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < Rp && c < Cp) out[r * ld_out + c] = __float2bfloat16(tile[threadIdx.x][i]);
    }
}

// Y[v][n] (bf16 activation and fp32 pre-activation copy) = act(acc[v][n] + bias[n])
__global__ void k_bias_act(const float *__restrict__ acc, const float *__restrict__ bias, float *__restrict__ pre,
                           __nv_bfloat16 *__restrict__ Y, float *__restrict__ Yf, int64_t nvox, int N, int ld_acc,
                           int relu) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * N) return;
    const int64_t v = t / N;
    const int n = (int)(t - v * N);
    const float a = acc[v * ld_acc + n] + bias[n];
    if (pre) pre[t] = a;
    const float y = relu ? fmaxf(a, 0.f) : a;
    if (Y) Y[t] = __float2bfloat16(y);
    if (Yf) Yf[t] = y;
}

// gradient through the activation: g[t] *= (pre[t] > 0) for ReLU layers
__global__ void k_relu_back(float *__restrict__ g, const float *__restrict__ pre, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n && pre[t] <= 0.f) g[t] = 0.f;
}

// bias gradient: db[n] = sum_v g[v][n] (one block per channel, fixed-order reduction)
__global__ void k_bias_grad(const float *__restrict__ g, float *__restrict__ db, int64_t nvox, int N) {
    const int n = blockIdx.x;
    float acc = 0.f;
    for (int64_t v = threadIdx.x; v < nvox; v += blockDim.x) acc += g[v * N + n];
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[n] = red[0];
}

// 2x2x2 average pooling, channels-last; out grid (D/2, H/2, W/2)
__global__ void k_avgpool2(const __nv_bfloat16 *__restrict__ X, __nv_bfloat16 *__restrict__ Y, int D, int H, int W,
                           int C) {
    const int D2 = D / 2, H2 = H / 2, W2 = W / 2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)D2 * H2 * W2 * C) return;
    const int c = (int)(t % C);
    const int64_t v = t / C;
    const int x = (int)(v % W2), y = (int)((v / W2) % H2), z = (int)(v / ((int64_t)W2 * H2));
    float s = 0.f;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx)
                s += __bfloat162float(X[(((int64_t)(2 * z + dz) * H + 2 * y + dy) * W + 2 * x + dx) * C + c]);
    Y[t] = __float2bfloat16(0.125f * s);
}

// adjoint of the pooling: dX[fine][c] += dY[coarse][c] / 8   (dX fp32, written, not added)
__global__ void k_avgpool2_back(const float *__restrict__ dY, float *__restrict__ dX, int D, int H, int W, int C) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)D * H * W * C) return;
    const int c = (int)(t % C);
    const int64_t v = t / C;
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
    const int64_t u = ((int64_t)(z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
    dX[t] = 0.125f * dY[u * C + c];
}

// nearest upsampling x2 of Xc (C1 channels) into channels [0, C1) of Y (C1 + C2 channels),
// and the skip tensor S (C2 channels, fine grid) into channels [C1, C1 + C2)
__global__ void k_up2_concat(const __nv_bfloat16 *__restrict__ Xc, int C1, const __nv_bfloat16 *__restrict__ S, int C2,
                             __nv_bfloat16 *__restrict__ Y, int D, int H, int W) {
    const int C = C1 + C2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)D * H * W * C) return;
    const int c = (int)(t % C);
    const int64_t v = t / C;
    if (c < C1) {
        const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((int64_t)W * H));
        const int64_t u = ((int64_t)(z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
        Y[t] = Xc[u * C1 + c];
    } else {
        Y[t] = S[v * C2 + (c - C1)];
    }
}

// adjoint: dXc[coarse][c] = sum of the 8 fine dY[.][c] (c < C1); dS[v][c'] = dY[v][C1 + c']
__global__ void k_up2_concat_back(const float *__restrict__ dY, float *__restrict__ dXc, int C1,
                                  float *__restrict__ dS, int C2, int D, int H, int W) {
    const int C = C1 + C2;
    const int D2 = D / 2, H2 = H / 2, W2 = W / 2;
    const int64_t ncoarse = (int64_t)D2 * H2 * W2 * C1;
    const int64_t nfine = (int64_t)D * H * W * C2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ncoarse) {
        const int c = (int)(t % C1);
        const int64_t u = t / C1;
        const int x = (int)(u % W2), y = (int)((u / W2) % H2), z = (int)(u / ((int64_t)W2 * H2));
        float s = 0.f;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx)
                    s += dY[((((int64_t)(2 * z + dz) * H + 2 * y + dy) * W + 2 * x + dx)) * C + c];
        dXc[t] = s;
    } else if (t - ncoarse < nfine) {
        const int64_t r = t - ncoarse;
        const int c = (int)(r % C2);
        const int64_t v = r / C2;
        dS[r] = dY[v * C + C1 + c];
    }
}

// a += b (fp32)
__global__ void k_add(float *__restrict__ a, const float *__restrict__ b, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] += b[t];
}

// masked mean-squared error over fluid voxels: loss partials and the gradient
// g = 2 m (pred - target) / count.  pred and g have row stride ldp >= C (the extra
// channels of g are left as they are); target is [nvox][C].
__global__ void k_mse(const float *__restrict__ pred, int ldp, const float *__restrict__ target,
                      const float *__restrict__ mask, float *__restrict__ g, double *__restrict__ partial, int64_t nvox,
                      int C, float inv_count) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (t < nvox * C) {
        const int64_t v = t / C;
        const int c = (int)(t - v * C);
        const float m = mask[v];
        const float d = (pred[v * ldp + c] - target[t]) * m;
        g[v * ldp + c] = 2.f * d * inv_count;
        e = (double)d * (double)d;
    }
    __shared__ double red[256];
    red[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Adam (Kingma & Ba 2015) on fp32 master weights, then the bf16 copy used by the GEMM
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ wb, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.f - b1) * gt;
    const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    const float wt = w[t] - lr * (mt * c1) / (sqrtf(vt * c2) + eps);
    w[t] = wt;
    if (wb) wb[t] = __float2bfloat16(wt);
}

// fp32 -> bf16
__global__ void k_to_bf16(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = __float2bfloat16(a[t]);
}

inline unsigned nblk(int64_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

}  // namespace nn
}  // namespace mflbm

using namespace mflbm;
using namespace mflbm::nn;

#define NN_LAUNCH_OK() (cudaPeekAtLastError() == cudaSuccess ? MFLBM_OK : MFLBM_ECUDA)

extern "C" {

int32_t mflbm_nn_im2col(const void *X, int32_t D, int32_t H, int32_t W, int32_t Cin, int32_t Kp, void *col, void *stream) {
    if (!X || !col || D < 1 || H < 1 || W < 1 || Cin < 1 || Kp < 27 * Cin) return MFLBM_EINVAL;
    const int64_t n = (int64_t)D * H * W * Kp;
    k_im2col<<<nblk(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)X, (__nv_bfloat16 *)col, D, H, W, Cin, Kp);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_col2im(const float *dcol, int32_t D, int32_t H, int32_t W, int32_t Cin, int32_t Kp, float *dX,
                        void *stream) {
    if (!dcol || !dX || D < 1 || H < 1 || W < 1 || Cin < 1 || Kp < 27 * Cin) return MFLBM_EINVAL;
    const int64_t n = (int64_t)D * H * W * Cin;
    k_col2im<<<nblk(n), 256, 0, (cudaStream_t)stream>>>(dcol, dX, D, H, W, Cin, Kp);
    return NN_LAUNCH_OK();
}

// out[r][c] = in[c][r] as bf16; in is fp32 (in_f32 = 1) or bf16; zero padding to (Rp, Cp)
int32_t mflbm_nn_transpose_bf16(const void *in, int32_t in_f32, int64_t ld_in, int64_t R, int64_t Cc, void *out,
                                int64_t ld_out, int64_t Rp, int64_t Cp, void *stream) {
    if (!in || !out || R < 0 || Cc < 0 || Rp < R || Cp < Cc || ld_out < Cp || ld_in < R) return MFLBM_EINVAL;
    if ((Rp + 31) / 32 > 65535) return MFLBM_ERANGE;
    dim3 b(32, 8), g((unsigned)((Cp + 31) / 32), (unsigned)((Rp + 31) / 32));
    if (in_f32)
        k_transpose_bf16<float><<<g, b, 0, (cudaStream_t)stream>>>((const float *)in, ld_in, (__nv_bfloat16 *)out, ld_out,
                                                                   R, Cc, Rp, Cp);
    else
        k_transpose_bf16<__nv_bfloat16><<<g, b, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)in, ld_in,
                                                                           (__nv_bfloat16 *)out, ld_out, R, Cc, Rp, Cp);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_bias_act(const float *acc, const float *bias, float *pre, void *Y, float *Yf, int64_t nvox, int32_t N,
                          int32_t ld_acc, int32_t relu, void *stream) {
    if (!acc || !bias || nvox < 0 || N < 1 || ld_acc < N) return MFLBM_EINVAL;
    k_bias_act<<<nblk(nvox * N), 256, 0, (cudaStream_t)stream>>>(acc, bias, pre, (__nv_bfloat16 *)Y, Yf, nvox, N, ld_acc,
                                                                 relu);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_relu_back(float *g, const float *pre, int64_t n, void *stream) {
    if (!g || !pre || n < 0) return MFLBM_EINVAL;
    k_relu_back<<<nblk(n), 256, 0, (cudaStream_t)stream>>>(g, pre, n);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_bias_grad(const float *g, float *db, int64_t nvox, int32_t N, void *stream) {
    if (!g || !db || nvox < 0 || N < 1) return MFLBM_EINVAL;
    k_bias_grad<<<N, 256, 0, (cudaStream_t)stream>>>(g, db, nvox, N);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_avgpool2(const void *X, void *Y, int32_t D, int32_t H, int32_t W, int32_t C, void *stream) {
    if (!X || !Y || D % 2 || H % 2 || W % 2 || C < 1) return MFLBM_EINVAL;
    k_avgpool2<<<nblk((int64_t)D * H * W * C / 8), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)X,
                                                                                  (__nv_bfloat16 *)Y, D, H, W, C);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_avgpool2_back(const float *dY, float *dX, int32_t D, int32_t H, int32_t W, int32_t C, void *stream) {
    if (!dY || !dX || D % 2 || H % 2 || W % 2 || C < 1) return MFLBM_EINVAL;
    k_avgpool2_back<<<nblk((int64_t)D * H * W * C), 256, 0, (cudaStream_t)stream>>>(dY, dX, D, H, W, C);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_up2_concat(const void *Xc, int32_t C1, const void *S, int32_t C2, void *Y, int32_t D, int32_t H,
                            int32_t W, void *stream) {
    if (!Xc || !S || !Y || D % 2 || H % 2 || W % 2 || C1 < 1 || C2 < 1) return MFLBM_EINVAL;
    k_up2_concat<<<nblk((int64_t)D * H * W * (C1 + C2)), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)Xc, C1, (const __nv_bfloat16 *)S, C2, (__nv_bfloat16 *)Y, D, H, W);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_up2_concat_back(const float *dY, float *dXc, int32_t C1, float *dS, int32_t C2, int32_t D, int32_t H,
                                 int32_t W, void *stream) {
    if (!dY || !dXc || !dS || D % 2 || H % 2 || W % 2 || C1 < 1 || C2 < 1) return MFLBM_EINVAL;
    const int64_t n = (int64_t)(D / 2) * (H / 2) * (W / 2) * C1 + (int64_t)D * H * W * C2;
    k_up2_concat_back<<<nblk(n), 256, 0, (cudaStream_t)stream>>>(dY, dXc, C1, dS, C2, D, H, W);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_add(float *a, const float *b, int64_t n, void *stream) {
    if (!a || !b || n < 0) return MFLBM_EINVAL;
    k_add<<<nblk(n), 256, 0, (cudaStream_t)stream>>>(a, b, n);
    return NN_LAUNCH_OK();
}

int32_t mflbm_nn_to_bf16(const float *a, void *b, int64_t n, void *stream) {
    if (!a || !b || n < 0) return MFLBM_EINVAL;
    k_to_bf16<<<nblk(n), 256, 0, (cudaStream_t)stream>>>(a, (__nv_bfloat16 *)b, n);
    return NN_LAUNCH_OK();
}

// partial must hold ceil(nvox*C/256) doubles; the loss is their sum / count
int32_t mflbm_nn_mse(const float *pred, int32_t ldp, const float *target, const float *mask, float *g, double *partial,
                     int64_t nvox, int32_t C, float inv_count, void *stream) {
    if (!pred || !target || !mask || !g || !partial || nvox < 0 || C < 1 || ldp < C) return MFLBM_EINVAL;
    k_mse<<<nblk(nvox * C), 256, 0, (cudaStream_t)stream>>>(pred, ldp, target, mask, g, partial, nvox, C, inv_count);
    return NN_LAUNCH_OK();
}

// one Adam step; `step` counts from 1 (bias corrections 1/(1-b^step))
int32_t mflbm_nn_adam(float *w, const float *g, float *m, float *v, void *wb, int64_t n, float lr, float b1, float b2,
                      float eps, int32_t step, void *stream) {
    if (!w || !g || !m || !v || n < 0 || step < 1) return MFLBM_EINVAL;
    const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
    k_adam<<<nblk(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, (__nv_bfloat16 *)wb, n, lr, b1, b2, eps, c1, c2);
    return NN_LAUNCH_OK();
}

}  // extern "C"
