// compact_state.cuh -- accessors of the compact FP32 state shared by the
// step kernels (compact.cu) and the observables/checkpoint kernels
// (observe.cu).
//
// State of one buffer (x fastest: cell = (k*ny + m)*nx + l):
//   head uint32[cells]     bits 0-6 number n of stored phases (phi > 0),
//                          bit 7 "single value stored explicitly",
//                          bits 8-23 id of the first (smallest) stored phase
//   idx  uint16[S][cells]  ids of stored phases 1..n-1 (ascending; slot 0 unused)
//   val  float [S][cells]  fractions of stored phases 0..n-1
// A cell holding one phase at exactly 1 keeps no value: it is implicit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mpf3d {
namespace compact {

constexpr int LIQ = 0;

struct In {
    const uint32_t *__restrict__ head;
    const uint16_t *__restrict__ idx;
    const float *__restrict__ val;
};
struct Out {
    uint32_t *__restrict__ head;
    uint16_t *__restrict__ idx;
    float *__restrict__ val;
};

__device__ __forceinline__ int hcount(uint32_t h) { return (int)(h & 0x7Fu); }
__device__ __forceinline__ bool hexplicit(uint32_t h) { return (h & 0x80u) != 0u; }
__device__ __forceinline__ int hid0(uint32_t h) { return (int)(h >> 8); }
__device__ __forceinline__ uint32_t mkhead(int id0, int n, bool expl) {
    return ((uint32_t)id0 << 8) | (expl ? 0x80u : 0u) | (uint32_t)n;
}
// value of stored entry 0 of a cell with head h
__device__ __forceinline__ float value0(const In &in, uint32_t h, uint32_t q) {
    return (hcount(h) >= 2 || hexplicit(h)) ? __ldg(in.val + q) : 1.0f;
}

__device__ __forceinline__ int wrap_p(int l, int n) { return l < n - 1 ? l + 1 : 0; }
__device__ __forceinline__ int wrap_m(int l, int n) { return l > 0 ? l - 1 : n - 1; }
__device__ __forceinline__ int clamp_p(int k, int n) { return k < n - 1 ? k + 1 : n - 1; }
__device__ __forceinline__ int clamp_m(int k, int n) { return k > 0 ? k - 1 : 0; }

// stored fraction of phase g at cell c (0 if not stored); stride = cells per slot
template <int S>
__device__ __forceinline__ float phase_at(const In &in, uint32_t stride, uint32_t c, int g) {
    const uint32_t h = __ldg(in.head + c);
    const int n = min(hcount(h), S);
    if (n == 0) return 0.0f;
    if (hid0(h) == g) return value0(in, h, c);
    for (int s = 1; s < n; ++s)
        if ((int)__ldg(in.idx + (size_t)s * stride + c) == g) return __ldg(in.val + (size_t)s * stride + c);
    return 0.0f;
}

// Length of the active-phase list of cell (l, m, k) under the APT rule of
// kernel_update_nfmf_3d (src/gpu_kernels_3d.py:462-486) for phi >= 0: the
// number of distinct phases stored in the cell or its 6 face neighbours
// (x, y periodic, z clamped), counted by repeated minimum extraction over
// the 7 ascending lists.
template <int S>
__device__ __forceinline__ int active_count_at(const In &in, int nx, int ny, int nz, int l, int m, int k) {
    const int64_t cells = (int64_t)nx * ny * nz;
    const int lp = wrap_p(l, nx), lm = wrap_m(l, nx), mp = wrap_p(m, ny), mm = wrap_m(m, ny);
    const int kp = clamp_p(k, nz), km = clamp_m(k, nz);
    auto ci = [&](int a, int b, int d) { return ((int64_t)d * ny + b) * nx + a; };
    const int64_t pt[7] = {ci(l, m, k), ci(lp, m, k), ci(lm, m, k), ci(l, mp, k),
                           ci(l, mm, k), ci(l, m, kp), ci(l, m, km)};
    auto id_at = [&](int p, int s) {
        return s == 0 ? hid0(in.head[pt[p]]) : (int)in.idx[s * cells + pt[p]];
    };
    int pos[7];
    for (int p = 0; p < 7; ++p) pos[p] = 0;
    int n = 0, last = -1;
    while (true) {
        int best = 1 << 30;
        for (int p = 0; p < 7; ++p) {
            const int c = min(hcount(in.head[pt[p]]), S);
            while (pos[p] < c && id_at(p, pos[p]) <= last) ++pos[p];
            if (pos[p] < c) best = min(best, id_at(p, pos[p]));
        }
        if (best == (1 << 30)) break;
        last = best;
        ++n;
    }
    return n;
}

}  // namespace compact
}  // namespace mpf3d

// SM count of the current device (grid sizing of persistent launches)
inline int sms_of_current_device() {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// grid dimensions the compact kernels accept
inline bool dims_ok(int nx, int ny, int nz) {
    return nx > 0 && ny > 0 && nz > 0 && nx <= 65535 * 32 && ny <= 65535 * 8 && nz <= 65535 * 8 &&
           (int64_t)nx * ny * nz < ((int64_t)1 << 40);
}
