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
// Two GEMM kernels: K-major operands (the forward pass X W^T, K <= 256,
// N <= 256) run on the fifth-generation tensor cores (tcgen05.mma with the
// accumulator in tensor memory); transposed operands (the gradients) use
// mma.sync.m16n8k16 (BF16 in, FP32 accumulate) from shared memory tiles:
// 64 x 64 output tile per CTA, 4 warps of 32 x 32, k step 32.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

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

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
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

// ---------------------------------------------------------------------------
// The K-major GEMM on the fifth-generation tensor cores (tcgen05).  One CTA
// of 128 threads computes a 128 x N tile (N <= 256) with K <= 256:
//   1. the threads stage A [128][K] and B [N][K] (BF16, K contiguous in
//      global memory) in shared memory in the canonical K-major layout
//      without swizzle: 8-row x 16-byte core matrices, the cores of one
//      8-row block adjacent along K (leading byte offset 128), row blocks
//      K/8 cores apart (stride byte offset);
//   2. warp 0 allocates N columns of tensor memory for the FP32
//      accumulator; one thread issues K/16 tcgen05.mma (M = 128, N, K = 16,
//      kind::f16 with BF16 inputs) and commits them to an mbarrier;
//   3. every warp reads its 32 accumulator rows back with tcgen05.ld
//      (32x32b shape, 16 columns at a time) and applies bias, SiLU and the
//      stores of the mma.sync kernel's epilogue, as 16-byte vectors.
// The CTAs are persistent (one or two per SM): B is staged once per CTA,
// the tensor memory allocated once, and the mbarrier phase alternates with
// the tiles.
// The mbarrier poll is bounded: a step that never completes writes NaN
// instead of results, waits once more and still frees its tensor memory.
namespace mpf3d {
namespace mlp {
namespace tc5 {

constexpr int TM = 128;
constexpr int MAX_N = 256;
constexpr int MAX_K = 256;
// bound of every mbarrier wait (nanoseconds of %globaltimer); a wait that
// runs out aborts the CTA's work and reports MPF3D_DEV_GEMM_ABORT
constexpr uint64_t WAIT_LIMIT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all >> 4), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B,
// both K-major, N >> 3 and M >> 4
__host__ __device__ __forceinline__ uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// waits for the phase `parity` of an mbarrier to complete, for at most
// limit_ns; false if it did not
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns = WAIT_LIMIT_NS) {
    const uint64_t t0 = global_ns();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// Stages rows x K of an operand into the K-major core-matrix layout:
// element (r, k) is src[r * s_row + k * s_k]; rows at or past rows_valid
// and columns at or past K_valid are zero.  With s_k == 1 (K contiguous in
// global memory) the chunks of 8 columns are 16-byte loads; otherwise (a
// transposed operand: the gradients' dZ^T, X^T and W^T) they are gathered
// element by element, consecutive threads on consecutive rows.
__device__ __forceinline__ void stage(uint8_t *dst, const uint16_t *__restrict__ src, int64_t s_row, int64_t s_k,
                                      int rows_valid, int rows, int K, int K_valid) {
    // chunk e is row (e % 8) of core (e / 8): 8 consecutive threads fill one
    // 128-byte core matrix; 8 chunks per thread are loaded before any is
    // stored, so the loads overlap
    const int kc = K / 8;
    const uint32_t sbo = (uint32_t)kc * 128u;
    const int total = rows * kc;
    const bool vec = s_k == 1 && K_valid == K && (s_row % 8) == 0 && (((uintptr_t)src & 15u) == 0);
    constexpr int U = 8;
    for (int e0 = threadIdx.x; e0 < total; e0 += U * blockDim.x) {
        uint4 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * blockDim.x;
            v[u] = make_uint4(0u, 0u, 0u, 0u);
            if (e < total) {
                const int core = e >> 3, r8 = e & 7;
                const int rb = core / kc, c = core - rb * kc;
                const int r = rb * 8 + r8;
                if (r < rows_valid) {
                    if (vec) {
                        v[u] = __ldg(reinterpret_cast<const uint4 *>(src + (int64_t)r * s_row + c * 8));
                    } else {
                        uint32_t w[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int k0 = c * 8 + 2 * j;
                            const uint32_t lo = k0 < K_valid ? __ldg(src + (int64_t)r * s_row + (int64_t)k0 * s_k) : 0u;
                            const uint32_t hi =
                                k0 + 1 < K_valid ? __ldg(src + (int64_t)r * s_row + (int64_t)(k0 + 1) * s_k) : 0u;
                            w[j] = lo | (hi << 16);
                        }
                        v[u] = make_uint4(w[0], w[1], w[2], w[3]);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < total) {
                const int core = e >> 3, r8 = e & 7;
                const int rb = core / kc, c = core - rb * kc;
                *reinterpret_cast<uint4 *>(dst + rb * sbo + c * 128u + r8 * 16u) = v[u];
            }
        }
    }
}

// Persistent CTAs: each stages B once, then loops over 128-row tiles of A.
// A(m, k) = A[m * sam + k * sak] and B(n, k) = B[n * sbn + k * sbk] for
// k < K_valid; K (a multiple of 16) >= K_valid is the staged depth.
__global__ void __launch_bounds__(128) gemm_kernel(int M, int N, int K, int K_valid, const uint16_t *__restrict__ A,
                                                   int64_t sam, int64_t sak, const uint16_t *__restrict__ B,
                                                   int64_t sbn, int64_t sbk, const float *__restrict__ bias, int act,
                                                   float *__restrict__ Z, void *__restrict__ Y, int ldy, int y_bf16,
                                                   int beta, int32_t *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int n_mma = (N + 15) & ~15;
    uint8_t *sA = smem;
    uint8_t *sB = smem + TM * K * 2;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sB + n_mma * K * 2);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ncols = n_mma <= 32 ? 32u : (n_mma <= 64 ? 64u : (n_mma <= 128 ? 128u : 256u));
    const int tiles = (M + TM - 1) / TM;

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    stage(sB, B, sbn, sbk, N, n_mma, K, K_valid);
    const uint32_t bar_a = smem_addr(bar);
    const uint32_t idesc = instr_desc(TM, n_mma);
    const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB), sbo = (uint32_t)(K / 8) * 128u;
    const bool vec_ok = (ldy % 8 == 0) && (((uintptr_t)Y & 15u) == 0) && (!Z || ((uintptr_t)Z & 15u) == 0);
    uint32_t tmem = 0;
    bool ok = true;
    int it = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++it) {
        const int m0 = tile * TM;
        stage(sA, A + (int64_t)m0 * sam, sam, sak, min(TM, M - m0), TM, K, K_valid);
        // the tensor core reads shared memory through the async proxy; the
        // previous tile's accumulator reads are complete (barrier below)
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        tmem = *tslot;
        if (threadIdx.x == 0) {
            for (int ks = 0; ks < K / 16; ++ks) {
                const uint64_t ad = smem_desc(a0 + ks * 256u, 128u, sbo);
                const uint64_t bd = smem_desc(b0 + ks * 256u, 128u, sbo);
                const uint32_t accum = ks > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar_a)
                         : "memory");
        }
        // tcgen05.ld is warp-collective: a warp reads the accumulator only
        // if all of its lanes saw the commit; a missed commit ends the loop
        // for the whole CTA
        const bool done = __syncthreads_and(mbar_wait(bar_a, (uint32_t)(it & 1))) != 0;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const int m = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < n_mma; c0 += 16) {
            uint32_t r[16];
            if (done) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
            if (m >= M) continue;
            float z[16], y[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int n = c0 + j;
                const float acc = done ? __uint_as_float(r[j]) : __int_as_float(0x7fc00000);
                z[j] = acc + ((bias && n < N) ? bias[n] : 0.0f);
                y[j] = act == 1 ? silu(z[j]) : z[j];
            }
            const int64_t o = (int64_t)m * ldy + c0;
            if (vec_ok && c0 + 16 <= N) {
                // 16 consecutive columns of one row: whole 16-byte vectors
                if (Z) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        reinterpret_cast<float4 *>(Z + o)[q] =
                            make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
                }
                if (y_bf16) {
                    uint32_t w[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        w[q] = (uint32_t)f32_to_bf16(y[2 * q]) | ((uint32_t)f32_to_bf16(y[2 * q + 1]) << 16);
                    uint4 *yp = reinterpret_cast<uint4 *>(static_cast<uint16_t *>(Y) + o);
                    yp[0] = make_uint4(w[0], w[1], w[2], w[3]);
                    yp[1] = make_uint4(w[4], w[5], w[6], w[7]);
                } else {
                    float4 *yp = reinterpret_cast<float4 *>(static_cast<float *>(Y) + o);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        float4 v = make_float4(y[4 * q], y[4 * q + 1], y[4 * q + 2], y[4 * q + 3]);
                        if (beta) {
                            const float4 prev = yp[q];
                            v.x += prev.x; v.y += prev.y; v.z += prev.z; v.w += prev.w;
                        }
                        yp[q] = v;
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = c0 + j;
                    if (n >= N) break;
                    if (Z) Z[o + j] = z[j];
                    if (y_bf16) {
                        static_cast<uint16_t *>(Y)[o + j] = f32_to_bf16(y[j]);
                    } else {
                        float *yf = static_cast<float *>(Y);
                        yf[o + j] = beta ? yf[o + j] + y[j] : y[j];
                    }
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        if (!done) {
            ok = false;
            break;
        }
    }
    // an overdue MMA must finish before its memory is freed: if its commit
    // never arrives, the tensor memory is left allocated rather than freed
    // under a running MMA
    const bool drained = __syncthreads_and(ok || mbar_wait(bar_a, (uint32_t)(it & 1))) != 0;
    if (!ok && threadIdx.x == 0 && err) atomicOr(err, MPF3D_DEV_GEMM_ABORT);
    if (warp == 0 && drained) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        tmem = *tslot;
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// ---------------------------------------------------------------------------
// The pipelined form for K a multiple of 64: warp-specialised persistent CTAs
// of 320 threads.
//   warp 0 (one lane)  TMA producer: the weights once (K/64 boxes of
//                      64 x N, 128-byte swizzle), then per tile K/64 boxes of
//                      64 x 128 of X into a 4-stage ring (full/empty
//                      mbarriers, transaction-counted);
//   warp 1 (one lane)  MMA issuer: per ring stage 4 tcgen05.mma (K = 16 each,
//                      start address +32 bytes inside the swizzled 128-byte
//                      rows), a commit frees the stage; per tile a commit
//                      hands the accumulator to the epilogue;
//   warps 2-9          epilogue: tcgen05.ld of their 32-lane quarter of the
//                      accumulator (two warps per quarter, alternate 16-column
//                      chunks), bias, SiLU, 16-byte stores, then release the
//                      accumulator buffer.
// Two accumulator buffers in tensor memory let the epilogue of one tile run
// under the MMAs of the next.  Every mbarrier wait is bounded; a wait that
// runs out raises a CTA-wide abort flag, every role leaves its loop, the
// producer waits for the copies it issued and the tensor memory is freed.
namespace tma {

constexpr int STAGES = 4;
constexpr int ATOM_K = 64;                    // bf16 elements per 128-byte swizzled row
constexpr int A_STAGE_BYTES = TM * ATOM_K * 2;  // 16 KB

__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    // K-major, 128-byte swizzle: 8-row groups 1024 bytes apart (stride byte
    // offset); the leading byte offset is unused by this layout
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void arrive_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

__global__ void __launch_bounds__(320, 1) gemm_kernel(const __grid_constant__ CUtensorMap map_x,
                                                      const __grid_constant__ CUtensorMap map_w, int M, int N, int K,
                                                      const float *__restrict__ bias, int act,
                                                      float *__restrict__ Z, void *__restrict__ Y, int ldy,
                                                      int y_bf16, int beta, int32_t *__restrict__ err,
                                                      uint64_t wait_ns, int hold_producer) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte alignment for the swizzled tiles
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int n_mma = (N + 15) & ~15;
    const int KA = K / ATOM_K;
    const uint32_t w_atom_bytes = (uint32_t)n_mma * 128u;
    uint8_t *sW = smem;
    uint8_t *sA = sW + KA * w_atom_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sA + STAGES * A_STAGE_BYTES);
    // bars: full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], w_full, drain
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2 * STAGES + 6);
    int *abort_flag = reinterpret_cast<int *>(tslot + 1);
    int *undrained = abort_flag + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t buf_cols = n_mma <= 32 ? 32u : (n_mma <= 64 ? 64u : (n_mma <= 128 ? 128u : 256u));
    const int tiles = (M + TM - 1) / TM;
    auto bar = [&](int i) { return smem_addr(bars + i); };
    const int FULL = 0, EMPTY = STAGES, ACC_FULL = 2 * STAGES, ACC_EMPTY = 2 * STAGES + 2, W_FULL = 2 * STAGES + 4,
              DRAIN = 2 * STAGES + 5;

    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(FULL + i)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(EMPTY + i)) : "memory");
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(ACC_FULL + b)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;\n" ::"r"(bar(ACC_EMPTY + b)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(W_FULL)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(DRAIN)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        *abort_flag = 0;
        *undrained = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tslot)),
                     "r"(2 * buf_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    volatile int *abort_v = abort_flag;
    auto wait = [&](int i, uint32_t parity) -> bool {
        if (*abort_v) return false;
        if (mbar_wait(bar(i), parity, wait_ns)) return true;
        *abort_v = 1;
        return false;
    };

    if (warp == 0) {
        // hold_producer (a test of the abort path) keeps the producer from
        // issuing anything: every wait of the other roles then runs out
        if (lane == 0 && !hold_producer) {
            // weights once
            arrive_expect(bar(W_FULL), (uint32_t)KA * w_atom_bytes);
            for (int j = 0; j < KA; ++j) tma_load(smem_addr(sW + j * w_atom_bytes), &map_w, j * ATOM_K, 0, bar(W_FULL));
            uint32_t it = 0, issued = 0;
            for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
                for (int j = 0; j < KA; ++j, ++it) {
                    const int s = it % STAGES;
                    if (!wait(EMPTY + s, ((it / STAGES) & 1u) ^ 1u)) break;
                    arrive_expect(bar(FULL + s), A_STAGE_BYTES);
                    tma_load(smem_addr(sA + s * A_STAGE_BYTES), &map_x, j * ATOM_K, tile * TM, bar(FULL + s));
                    issued = it + 1;
                }
                if (*abort_v) break;
            }
            // every copy issued must land before the CTA can go away
            if (*abort_v) {
                bool landed = true;
                for (uint32_t q = issued > STAGES ? issued - STAGES : 0; q < issued; ++q)
                    landed = mbar_wait(bar(FULL + q % STAGES), (q / STAGES) & 1u, wait_ns) && landed;
                landed = mbar_wait(bar(W_FULL), 0, wait_ns) && landed;
                if (!landed) atomicExch(undrained, 1);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = instr_desc(TM, n_mma);
            bool issued = false;
            if (wait(W_FULL, 0)) {
                uint32_t it = 0, t_local = 0;
                for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++t_local) {
                    const uint32_t b = t_local & 1u;
                    if (!wait(ACC_EMPTY + b, ((t_local >> 1) & 1u) ^ 1u)) break;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t d = tmem + b * buf_cols;
                    bool ok = true;
                    for (int j = 0; j < KA; ++j, ++it) {
                        const int s = it % STAGES;
                        if (!wait(FULL + s, (it / STAGES) & 1u)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                        const uint32_t a_base = smem_addr(sA + s * A_STAGE_BYTES);
                        const uint32_t w_base = smem_addr(sW + j * w_atom_bytes);
#pragma unroll
                        for (int ks = 0; ks < ATOM_K / 16; ++ks)
                            umma(d, sw128_desc(a_base + 32u * ks), sw128_desc(w_base + 32u * ks), idesc,
                                 (j > 0 || ks > 0) ? 1u : 0u);
                        issued = true;
                        commit(bar(EMPTY + s));  // the stage is free once these MMAs are done
                    }
                    if (!ok) break;
                    commit(bar(ACC_FULL + b));
                }
            }
            if (*abort_v && issued) {
                // the MMAs issued before the abort must finish before the
                // tensor memory is freed and the CTA leaves: one more commit
                // arrives once all of them are done
                commit(bar(DRAIN));
                if (!mbar_wait(bar(DRAIN), 0, wait_ns)) atomicExch(undrained, 1);
            }
        }
    } else {
        // epilogue warps 2..9: warp w reads lanes 32 * (w % 4) .. + 31 and
        // every other 16-column chunk (the two warps of a lane quarter split
        // the columns)
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const bool vec_ok = (ldy % 8 == 0) && (((uintptr_t)Y & 15u) == 0) && (!Z || ((uintptr_t)Z & 15u) == 0);
        uint32_t t_local = 0;
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++t_local) {
            const uint32_t b = t_local & 1u;
            const bool done = __all_sync(0xffffffffu, wait(ACC_FULL + b, (t_local >> 1) & 1u));
            if (!done) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int m = tile * TM + q * 32 + lane;
            for (int c0 = 16 * half; c0 < n_mma; c0 += 32) {
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + b * buf_cols + (uint32_t)c0, r);
                if (m >= M) continue;
                float z[16], y[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = c0 + j;
                    z[j] = __uint_as_float(r[j]) + ((bias && n < N) ? bias[n] : 0.0f);
                    y[j] = act == 1 ? silu(z[j]) : z[j];
                }
                const int64_t o = (int64_t)m * ldy + c0;
                if (vec_ok && c0 + 16 <= N) {
                    if (Z) {
#pragma unroll
                        for (int v = 0; v < 4; ++v)
                            reinterpret_cast<float4 *>(Z + o)[v] =
                                make_float4(z[4 * v], z[4 * v + 1], z[4 * v + 2], z[4 * v + 3]);
                    }
                    if (y_bf16) {
                        uint32_t w[8];
#pragma unroll
                        for (int v = 0; v < 8; ++v)
                            w[v] = (uint32_t)f32_to_bf16(y[2 * v]) | ((uint32_t)f32_to_bf16(y[2 * v + 1]) << 16);
                        uint4 *yp = reinterpret_cast<uint4 *>(static_cast<uint16_t *>(Y) + o);
                        yp[0] = make_uint4(w[0], w[1], w[2], w[3]);
                        yp[1] = make_uint4(w[4], w[5], w[6], w[7]);
                    } else {
                        float4 *yp = reinterpret_cast<float4 *>(static_cast<float *>(Y) + o);
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            float4 val = make_float4(y[4 * v], y[4 * v + 1], y[4 * v + 2], y[4 * v + 3]);
                            if (beta) {
                                const float4 prev = yp[v];
                                val.x += prev.x; val.y += prev.y; val.z += prev.z; val.w += prev.w;
                            }
                            yp[v] = val;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int n = c0 + j;
                        if (n >= N) break;
                        if (Z) Z[o + j] = z[j];
                        if (y_bf16) {
                            static_cast<uint16_t *>(Y)[o + j] = f32_to_bf16(y[j]);
                        } else {
                            float *yf = static_cast<float *>(Y);
                            yf[o + j] = beta ? yf[o + j] + y[j] : y[j];
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) arrive(bar(ACC_EMPTY + b));
        }
    }
    __syncwarp();  // the single-lane roles rejoin their warps before the block barrier
    __syncthreads();
    if (*abort_v && threadIdx.x == 0) {
        // an aborted run: the outputs of this CTA's tiles are unreliable
        if (err) atomicOr(err, MPF3D_DEV_GEMM_ABORT);
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x)
            for (int r = 0; r < TM && tile * TM + r < M; ++r) {
                const int64_t o = (int64_t)(tile * TM + r) * ldy;
                for (int n = 0; n < N; ++n) {
                    if (y_bf16) static_cast<uint16_t *>(Y)[o + n] = 0x7fc0;
                    else static_cast<float *>(Y)[o + n] = __int_as_float(0x7fc00000);
                }
            }
    }
    // tensor memory that an undrained MMA may still write is left allocated
    if (warp == 0 && !*(volatile int *)undrained) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * buf_cols)
                     : "memory");
    }
}

inline size_t smem_bytes(int N, int K) {
    const int n_mma = (N + 15) & ~15;
    return 1024 + (size_t)(K / ATOM_K) * n_mma * 128 + (size_t)STAGES * A_STAGE_BYTES + 256;
}

}  // namespace tma

inline size_t smem_bytes(int N, int K) {
    const int n_mma = (N + 15) & ~15;
    const size_t need = (size_t)(TM + n_mma) * K * 2 + 16;
    // at least 80 KB keeps two CTAs per SM at most: 2 x 256 tensor-memory
    // columns fit the SM's 512, so an allocation never waits for another CTA
    return need < 80 * 1024 ? 80 * 1024 : need;
}

}  // namespace tc5
}  // namespace mlp
}  // namespace mpf3d

static int sms_of_device() {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

static bool tc5_shape_ok(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb) {
    return M > 0 && N > 0 && N <= mpf3d::mlp::tc5::MAX_N && K >= 16 && K <= mpf3d::mlp::tc5::MAX_K && K % 16 == 0 &&
           lda >= K && ldb >= K && lda % 8 == 0 && ldb % 8 == 0 && ((uintptr_t)A & 15u) == 0 &&
           ((uintptr_t)B & 15u) == 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 2-D map of a row-major BF16 matrix [rows][K] (row pitch ld elements):
// boxes of 64 x box_rows, 128-byte swizzle, rows past the end read as zero
static bool make_map(CUtensorMap *map, const uint16_t *base, int rows, int K, int64_t ld, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1u, 1u};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint16_t *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the pipelined kernel (K a multiple of 64); hold_producer != 0 only in the
// abort-path test.  Returns 1 when no tensor map could be made.
static int launch_tc5_tma(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb,
                          const float *bias, int act, float *Z, void *Y, int ldy, int y_bf16, int beta, int32_t *err,
                          uint64_t wait_ns, int hold_producer, cudaStream_t stream) {
    using namespace mpf3d::mlp;
    CUtensorMap mx, mw;
    const int n_mma = (N + 15) & ~15;
    if (!make_map(&mx, A, M, K, lda, tc5::TM) || !make_map(&mw, B, N, K, ldb, n_mma)) return 1;
    const size_t bytes = tc5::tma::smem_bytes(N, K);
    if (cudaFuncSetAttribute(tc5::tma::gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
        return MPF3D_ERR_CUDA;
    const int tiles = (M + tc5::TM - 1) / tc5::TM;
    const int grid = tiles < sms_of_device() ? tiles : sms_of_device();
    tc5::tma::gemm_kernel<<<grid, 320, bytes, stream>>>(mx, mw, M, N, K, bias, act, Z, Y, ldy, y_bf16, beta, err,
                                                        wait_ns, hold_producer);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_gemm_bf16_tc5(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B,
                                   int64_t ldb, const float *bias, int act, float *Z, void *Y, int ldy, int y_bf16,
                                   int beta, int32_t *err, void *stream) {
    using namespace mpf3d::mlp;
    if (!A || !B || !Y || ldy < N || (act != 0 && act != 1) || !tc5_shape_ok(M, N, K, A, lda, B, ldb))
        return MPF3D_ERR_ARG;
    if (K % tc5::tma::ATOM_K == 0) {
        const int rc = launch_tc5_tma(M, N, K, A, lda, B, ldb, bias, act, Z, Y, ldy, y_bf16, beta, err,
                                      tc5::WAIT_LIMIT_NS, 0, (cudaStream_t)stream);
        if (rc != 1) return rc;  // 1: no tensor map, use the register-staged form
    }
    const size_t bytes = tc5::smem_bytes(N, K);
    if (cudaFuncSetAttribute(tc5::gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
        return MPF3D_ERR_CUDA;
    const int tiles = (M + tc5::TM - 1) / tc5::TM;
    const int per_sm = bytes > 114 * 1024 ? 1 : 2;
    const int grid = tiles < sms_of_device() * per_sm ? tiles : sms_of_device() * per_sm;
    tc5::gemm_kernel<<<grid, 128, bytes, (cudaStream_t)stream>>>(M, N, K, K, A, lda, 1, B, ldb, 1, bias, act, Z, Y,
                                                                 ldy, y_bf16, beta, err);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_gemm_bf16_tc5_strided(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak,
                                           const uint16_t *B, int64_t sbk, int64_t sbn, const float *bias, int act,
                                           float *Z, void *Y, int ldy, int y_bf16, int beta, int32_t *err,
                                           void *stream) {
    using namespace mpf3d::mlp;
    if (M <= 0 || N <= 0 || N > tc5::MAX_N || K <= 0 || !A || !B || !Y || ldy < N || (act != 0 && act != 1))
        return MPF3D_ERR_ARG;
    const int chunks = (K + tc5::MAX_K - 1) / tc5::MAX_K;
    // a reduction deeper than one staged block is accumulated chunk by chunk
    // into an FP32 result: no activation, no pre-activation output
    if (chunks > 1 && (act != 0 || Z || y_bf16)) return MPF3D_ERR_ARG;
    const size_t bytes = tc5::smem_bytes(N, K < tc5::MAX_K ? ((K + 15) & ~15) : tc5::MAX_K);
    if (cudaFuncSetAttribute(tc5::gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
        return MPF3D_ERR_CUDA;
    const int tiles = (M + tc5::TM - 1) / tc5::TM;
    const int per_sm = bytes > 114 * 1024 ? 1 : 2;
    const int grid = tiles < sms_of_device() * per_sm ? tiles : sms_of_device() * per_sm;
    for (int c = 0; c < chunks; ++c) {
        const int k0 = c * tc5::MAX_K;
        const int kv = K - k0 < tc5::MAX_K ? K - k0 : tc5::MAX_K;
        tc5::gemm_kernel<<<grid, 128, bytes, (cudaStream_t)stream>>>(
            M, N, (kv + 15) & ~15, kv, A + (int64_t)k0 * sak, sam, sak, B + (int64_t)k0 * sbk, sbn, sbk,
            c == 0 ? bias : nullptr, act, Z, Y, ldy, y_bf16, c == 0 ? beta : 1, err);
        if (cudaGetLastError() != cudaSuccess) return MPF3D_ERR_CUDA;
    }
    return MPF3D_OK;
}

extern "C" int mpf3d_gemm_bf16_tc5_held(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B,
                                        int64_t ldb, void *Y, int ldy, int32_t *err, uint64_t wait_ns, void *stream) {
    using namespace mpf3d::mlp;
    if (!A || !B || !Y || !err || ldy < N || K % tc5::tma::ATOM_K != 0 || wait_ns == 0 || wait_ns > 100000000ull ||
        !tc5_shape_ok(M, N, K, A, lda, B, ldb))
        return MPF3D_ERR_ARG;
    const int rc = launch_tc5_tma(M, N, K, A, lda, B, ldb, nullptr, 0, nullptr, Y, ldy, 0, 0, err, wait_ns, 1,
                                  (cudaStream_t)stream);
    return rc == 1 ? MPF3D_ERR_CUDA : rc;
}

extern "C" int mpf3d_gemm_bf16_mma(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak,
                                   const uint16_t *B, int64_t sbk, int64_t sbn, const float *bias, int act, float *Z,
                                   void *Y, int ldy, int y_bf16, int beta, void *stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !Y || ldy < N || (act != 0 && act != 1)) return MPF3D_ERR_ARG;
    if ((M + BM - 1) / BM > 65535) return MPF3D_ERR_TOO_LARGE;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    gemm_bf16_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, act, Z, Y, ldy,
                                                             y_bf16, beta);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_gemm_bf16(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak, const uint16_t *B,
                               int64_t sbk, int64_t sbn, const float *bias, int act, float *Z, void *Y, int ldy,
                               int y_bf16, int beta, int32_t *err, void *stream) {
    // K-major operands (the forward pass X W^T) go to the pipelined tcgen05
    // kernel; transposed ones (the gradients dZ W and dZ^T X) to the tcgen05
    // kernel that gathers them into the K-major layout; shapes neither covers
    // to the mma.sync kernel
    if (sak == 1 && sbk == 1 && tc5_shape_ok(M, N, K, A, sam, B, sbn))
        return mpf3d_gemm_bf16_tc5(M, N, K, A, sam, B, sbn, bias, act, Z, Y, ldy, y_bf16, beta, err, stream);
    if (N <= mpf3d::mlp::tc5::MAX_N && (K <= mpf3d::mlp::tc5::MAX_K || (act == 0 && !Z && !y_bf16)))
        return mpf3d_gemm_bf16_tc5_strided(M, N, K, A, sam, sak, B, sbk, sbn, bias, act, Z, Y, ldy, y_bf16, beta, err,
                                           stream);
    return mpf3d_gemm_bf16_mma(M, N, K, A, sam, sak, B, sbk, sbn, bias, act, Z, Y, ldy, y_bf16, beta, stream);
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
