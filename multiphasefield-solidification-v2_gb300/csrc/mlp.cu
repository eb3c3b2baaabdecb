// mlp.cu -- BF16 tensor-core kernels of the orientation surrogate: a
// strided GEMM with fused bias/activation epilogue, the activation
// derivative, column sums, the MSE loss gradient and a fused Adam update.
//
// No reference counterpart: the reference has no learned component.  The
// network maps (2 quaternions, undercooling, anisotropy strength) to (growth
// velocity ratio, grain-boundary inclination) for the batched bicrystal
// engine; it is small (134,914 parameters), so one generic GEMM kernel with
// arbitrary operand strides serves the forward pass (X W^T), the input
// gradient (dZ W) and the weight gradient (dZ^T X) alike.
//
// The GEMM uses mma.sync.m16n8k16 (BF16 in, FP32 accumulate) from shared
// memory tiles: 64 x 64 output tile per CTA, 4 warps of 32 x 32, k step 32.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mpf3d.h"
#include "mpf3d_internal.h"

namespace mpf3d {
namespace mlp {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

__device__ __forceinline__ float bf16_to_f32(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

// round to nearest even (finite inputs)
__device__ __forceinline__ uint16_t f32_to_bf16(float f) {
    uint32_t u = __float_as_uint(f);
    if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);  // inf / nan
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[m][n] = act(sum_k A(m,k) B(k,n) + bias[n]) with A(m,k) = A[m*sam + k*sak]
// and B(k,n) = B[k*sbk + n*sbn] (BF16); accumulate in FP32.
// act: 0 none, 1 SiLU.  Z (optional) receives the FP32 pre-activation,
// Y the result as BF16 (y_bf16) or FP32; beta = 1 adds the FP32 result to Y.
__global__ void __launch_bounds__(128) gemm_bf16_kernel(int M, int N, int K, const uint16_t *__restrict__ A,
                                                        int64_t sam, int64_t sak, const uint16_t *__restrict__ B,
                                                        int64_t sbk, int64_t sbn, const float *__restrict__ bias,
                                                        int act, float *__restrict__ Z, void *__restrict__ Y,
                                                        int ldy, int y_bf16, int beta) {
    __shared__ __align__(16) uint16_t As[BM][BK + PAD];
    __shared__ __align__(16) uint16_t Bs[BN][BK + PAD];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;

    for (int k0 = 0; k0 < K; k0 += BK) {
        // stage the A tile [BM][BK] and the B tile as [BN][BK]
        for (int e = tid; e < BM * BK; e += 128) {
            const int r = e / BK, kk = e % BK;
            const int m = m0 + r, k = k0 + kk;
            As[r][kk] = (m < M && k < K) ? A[(int64_t)m * sam + (int64_t)k * sak] : (uint16_t)0;
        }
        for (int e = tid; e < BN * BK; e += 128) {
            const int r = e / BK, kk = e % BK;
            const int n = n0 + r, k = k0 + kk;
            Bs[r][kk] = (n < N && k < K) ? B[(int64_t)k * sbk + (int64_t)n * sbn] : (uint16_t)0;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + g;
                const int c = ks + tig * 2;
                a[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][c]);
                a[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][c]);
                a[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][c + 8]);
                a[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][c + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int n = wn + j * 8 + g;
                const int c = ks + tig * 2;
                b[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[n][c]);
                b[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[n][c + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
    // epilogue
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int m = m0 + wm + i * 16 + g + ((r & 2) ? 8 : 0);
                const int n = n0 + wn + j * 8 + tig * 2 + (r & 1);
                if (m >= M || n >= N) continue;
                float z = acc[i][j][r] + (bias ? bias[n] : 0.0f);
                const int64_t o = (int64_t)m * ldy + n;
                if (Z) Z[o] = z;
                const float y = act == 1 ? silu(z) : z;
                if (y_bf16) {
                    static_cast<uint16_t *>(Y)[o] = f32_to_bf16(y);
                } else {
                    float *yf = static_cast<float *>(Y);
                    yf[o] = beta ? yf[o] + y : y;
                }
            }
}

// dZ = dY * silu'(Z) (act = 1) or dZ = dY (act = 0), written as BF16 and,
// optionally, FP32
__global__ void act_backward_kernel(const float *__restrict__ dY, const float *__restrict__ Z, int act, int64_t n,
                                    uint16_t *__restrict__ dZ16, float *__restrict__ dZ32) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = act == 1 ? dY[i] * silu_grad(Z[i]) : dY[i];
        if (dZ16) dZ16[i] = f32_to_bf16(d);
        if (dZ32) dZ32[i] = d;
    }
}

// out[n] = sum_m X[m*ld + n]  (one thread per column; the columns are few)
__global__ void colsum_kernel(const float *__restrict__ X, int M, int N, int ld, float *__restrict__ out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int m = 0; m < M; ++m) s += X[(int64_t)m * ld + n];
    out[n] = s;
}

// MSE over the first n_out columns of pred (ld columns) against target
// [M][n_out] with per-column weights; dpred = 2 w (pred - t) / M, zero in the
// padding columns; loss accumulated into *loss
__global__ void mse_kernel(const float *__restrict__ pred, int ld, const float *__restrict__ target, int M, int n_out,
                           const float *__restrict__ w, float *__restrict__ dpred, float *__restrict__ loss) {
    float part = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M * ld; i += gridDim.x * blockDim.x) {
        const int m = i / ld, c = i % ld;
        float d = 0.0f;
        if (c < n_out) {
            const float e = pred[i] - target[m * n_out + c];
            part += w[c] * e * e / (float)M;
            d = 2.0f * w[c] * e / (float)M;
        }
        dpred[i] = d;
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, part);
}

// Adam on FP32 master weights; writes the BF16 copy used by the GEMMs
__global__ void adam_kernel(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                            const float *__restrict__ g, uint16_t *__restrict__ w16, int64_t n, float lr, float b1,
                            float b2, float eps, float bc1, float bc2, float wd) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i] + wd * w[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        if (w16) w16[i] = f32_to_bf16(wi);
    }
}

__global__ void f32_to_bf16_kernel(const float *__restrict__ x, uint16_t *__restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = f32_to_bf16(x[i]);
}

}  // namespace mlp
}  // namespace mpf3d

using namespace mpf3d::mlp;

namespace {
int grid_for(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)(b < 2048 ? (b > 0 ? b : 1) : 2048);
}
}  // namespace

extern "C" int mpf3d_gemm_bf16(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak, const uint16_t *B,
                               int64_t sbk, int64_t sbn, const float *bias, int act, float *Z, void *Y, int ldy,
                               int y_bf16, int beta, void *stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !Y || ldy < N || (act != 0 && act != 1)) return MPF3D_ERR_ARG;
    if ((M + BM - 1) / BM > 65535) return MPF3D_ERR_TOO_LARGE;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    gemm_bf16_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, act, Z, Y, ldy,
                                                             y_bf16, beta);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_act_backward(const float *dY, const float *Z, int act, int64_t n, uint16_t *dZ16, float *dZ32,
                                  void *stream) {
    if (!dY || (act == 1 && !Z) || n < 0 || (!dZ16 && !dZ32)) return MPF3D_ERR_ARG;
    if (n == 0) return MPF3D_OK;
    act_backward_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dY, Z, act, n, dZ16, dZ32);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_colsum(const float *X, int M, int N, int ld, float *out, void *stream) {
    if (!X || !out || M <= 0 || N <= 0 || ld < N) return MPF3D_ERR_ARG;
    colsum_kernel<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>(X, M, N, ld, out);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_mse(const float *pred, int ld, const float *target, int M, int n_out, const float *w,
                         float *dpred, float *loss, void *stream) {
    if (!pred || !target || !w || !dpred || !loss || M <= 0 || n_out <= 0 || ld < n_out) return MPF3D_ERR_ARG;
    mse_kernel<<<grid_for((int64_t)M * ld), 256, 0, (cudaStream_t)stream>>>(pred, ld, target, M, n_out, w, dpred,
                                                                            loss);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_adam(float *w, float *m, float *v, const float *g, uint16_t *w16, int64_t n, float lr, float b1,
                          float b2, float eps, int step, float weight_decay, void *stream) {
    if (!w || !m || !v || !g || n < 0 || step < 1) return MPF3D_ERR_ARG;
    if (n == 0) return MPF3D_OK;
    const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, m, v, g, w16, n, lr, b1, b2, eps, bc1, bc2,
                                                               weight_decay);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_f32_to_bf16(const float *x, uint16_t *y, int64_t n, void *stream) {
    if (!x || !y || n < 0) return MPF3D_ERR_ARG;
    if (n == 0) return MPF3D_OK;
    f32_to_bf16_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, y, n);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}
