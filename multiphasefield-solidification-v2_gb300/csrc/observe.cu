// observe.cu -- observables, phase-map slices and checkpoints of the compact
// FP32 state, and the sphere set-up and directional probes of the batched
// orientation scan.  Everything here reads the state where it lives in HBM;
// only reduced numbers, 2D slices or the packed checkpoint leave the GPU.
//
//   metrics      compute_metrics_3d (tests/verification_3d.py:612-654) and
//                interface_positions_3d (:409-416) on the compact state
//   slice        the argmax phase map of save_phase_map_slice_3d
//                (src/plot_utils_3d.py:36-72) and the solid fraction of
//                save_solid_slice (run_orientation_scan_3d.py:199-223)
//   pack/unpack  checkpoint of the occupied entries only (the reference has
//                no checkpoint of its own)
//   sphere/rays  init_singlemode_sphere_3d (src/seed_modes_3d.py:59-113) per
//                batch instance, and the directional radii of
//                measure_observables (run_orientation_scan_3d.py:238-394)
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "compact_state.cuh"
#include "mpf3d.h"
#include "mpf3d_internal.h"

namespace mpf3d {
namespace observe {

using namespace mpf3d::compact;

// ---------------------------------------------------------------------------
// reductions

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_max_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// max / min of non-negative doubles (their bit patterns order like the values)
__device__ __forceinline__ void atomic_max_nonneg(double *a, double v) {
    atomicMax((unsigned long long *)a, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_min_nonneg(double *a, double v) {
    atomicMin((unsigned long long *)a, (unsigned long long)__double_as_longlong(v));
}

// Per-thread cache of running grain sums: a column passes through few
// grains, so most additions stay in registers and the histogram sees one
// atomic per (column, grain run) instead of one per cell.
struct GrainCache {
    int id[4];
    double sum[4];
    int next;
    __device__ void init() {
#pragma unroll
        for (int i = 0; i < 4; ++i) { id[i] = -1; sum[i] = 0.0; }
        next = 0;
    }
    __device__ void flush_one(int i, double *hist) {
        if (id[i] >= 0) atomicAdd(hist + id[i], sum[i]);
    }
    __device__ void add(int g, double v, double *hist) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (id[i] == g) { sum[i] += v; return; }
        flush_one(next, hist);
        id[next] = g;
        sum[next] = v;
        next = (next + 1) & 3;
    }
    __device__ void flush(double *hist) {
#pragma unroll
        for (int i = 0; i < 4; ++i) flush_one(i, hist);
    }
};

// compute_metrics_3d / interface_positions_3d: one thread per (x, y) column
// walking up z (consecutive threads read consecutive cells of every plane).
template <int S, bool SMEM_HIST>
__global__ void __launch_bounds__(256) metrics_kernel(In in, int N, int n_hist, int nx, int ny, int nz,
                                                      float threshold, mpf3d_metrics *__restrict__ res,
                                                      double *__restrict__ grain_sum, float *__restrict__ front) {
    extern __shared__ double hist_s[];
    double *hist = SMEM_HIST ? hist_s : grain_sum;
    if (SMEM_HIST) {
        for (int i = threadIdx.x; i < n_hist; i += blockDim.x) hist_s[i] = 0.0;
        __syncthreads();
    }
    const uint32_t plane = (uint32_t)nx * (uint32_t)ny;
    const uint32_t cells = plane * (uint32_t)nz;
    double solid_sum = 0.0, err_max = 0.0, vmin = INFINITY, vmax = 0.0;
    double fsum = 0.0, fsq = 0.0, fmx = 0.0;
    long long nan = 0, fcols = 0;
    int nfmax = 0;
    GrainCache gc;
    gc.init();
    for (uint32_t col = blockIdx.x * blockDim.x + threadIdx.x; col < plane; col += gridDim.x * blockDim.x) {
        const int l = (int)(col % (uint32_t)nx), m = (int)(col / (uint32_t)nx);
        int top = -1;
        for (int k = 0; k < nz; ++k) {
            const uint32_t c = (uint32_t)k * plane + col;
            const uint32_t h = __ldg(in.head + c);
            const int n = min(hcount(h), S);
            double sum = 0.0;
            float liq = 0.0f;
            for (int s = 0; s < n; ++s) {
                const int id = s == 0 ? hid0(h) : (int)__ldg(in.idx + (size_t)s * cells + c);
                const float v = s == 0 ? value0(in, h, c) : __ldg(in.val + (size_t)s * cells + c);
                sum += (double)v;
                if (id == LIQ) liq = v;
                if (v != v) ++nan;
                vmin = fmin(vmin, (double)v);
                vmax = fmax(vmax, (double)v);
                if (id > 0 && id < n_hist) gc.add(id, (double)v, hist);
            }
            if (n < N) vmin = fmin(vmin, 0.0);  // the dense field's unstored phases are zeros
            err_max = fmax(err_max, fabs(sum - 1.0));
            const float solid = 1.0f - liq;
            solid_sum += (double)solid;
            if (solid > threshold) top = k;
            nfmax = max(nfmax, active_count_at<S>(in, nx, ny, nz, l, m, k));
        }
        if (front) front[col] = top >= 0 ? (float)top : __int_as_float(0x7fc00000);
        if (top >= 0) {
            fsum += top;
            fsq += (double)top * top;
            fmx = fmax(fmx, (double)top);
            ++fcols;
        }
    }
    gc.flush(hist);
    // block reduction: warps, then one atomic per warp leader
    solid_sum = warp_sum(solid_sum);
    fsum = warp_sum(fsum);
    fsq = warp_sum(fsq);
    err_max = warp_max(err_max);
    vmax = warp_max(vmax);
    fmx = warp_max(fmx);
    vmin = warp_min(vmin);
    nan = warp_sum_ll(nan);
    fcols = warp_sum_ll(fcols);
    nfmax = warp_max_i(nfmax);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&res->solid_sum, solid_sum);
        atomicAdd(&res->front_sum, fsum);
        atomicAdd(&res->front_sq_sum, fsq);
        atomic_max_nonneg(&res->sum_err_max, err_max);
        atomic_max_nonneg(&res->phi_max, vmax);
        atomic_max_nonneg(&res->front_max, fmx);
        atomic_min_nonneg(&res->phi_min, vmin);
        atomicAdd((unsigned long long *)&res->nan_count, (unsigned long long)nan);
        atomicAdd((unsigned long long *)&res->front_columns, (unsigned long long)fcols);
        atomicMax(&res->nf_max, nfmax);
    }
    if (SMEM_HIST) {
        __syncthreads();
        for (int i = threadIdx.x; i < n_hist; i += blockDim.x)
            if (hist_s[i] != 0.0) atomicAdd(grain_sum + i, hist_s[i]);
    }
}

__global__ void metrics_init_kernel(mpf3d_metrics *res, double *grain_sum, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        res->solid_sum = 0.0;
        res->sum_err_max = 0.0;
        res->phi_min = INFINITY;
        res->phi_max = 0.0;
        res->front_sum = 0.0;
        res->front_sq_sum = 0.0;
        res->front_max = 0.0;
        res->nan_count = 0;
        res->front_columns = 0;
        res->nf_max = 0;
        res->reserved = 0;
    }
    if (grain_sum)
        for (int g = i; g < N; g += gridDim.x * blockDim.x) grain_sum[g] = 0.0;
}

// ---------------------------------------------------------------------------
// 2D slices: argmax phase id (first maximum, i.e. the smallest id among
// ties, as numpy.argmax over the dense phase axis), its fraction, and the
// solid fraction 1 - phi_liquid.  Output [W][H] row-major with
// (W, H) = (nx, ny) for axis 0 (xy at z = index), (nx, nz) for axis 1
// (xz at y = index), (ny, nz) for axis 2 (yz at x = index).
template <int S>
__global__ void slice_kernel(In in, int nx, int ny, int nz, int axis, int index, int32_t *__restrict__ ids,
                             float *__restrict__ vmax_out, float *__restrict__ solid_out) {
    const int W = axis == 2 ? ny : nx;
    const int H = axis == 0 ? ny : nz;
    const uint32_t cells = (uint32_t)nx * (uint32_t)ny * (uint32_t)nz;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < W * H; p += gridDim.x * blockDim.x) {
        const int a = p / H, b = p % H;
        int l, m, k;
        if (axis == 0) { l = a; m = b; k = index; }
        else if (axis == 1) { l = a; m = index; k = b; }
        else { l = index; m = a; k = b; }
        const uint32_t c = ((uint32_t)k * (uint32_t)ny + (uint32_t)m) * (uint32_t)nx + (uint32_t)l;
        const uint32_t h = __ldg(in.head + c);
        const int n = min(hcount(h), S);
        int best_id = 0;
        float best = -INFINITY, liq = 0.0f;
        for (int s = 0; s < n; ++s) {
            const int id = s == 0 ? hid0(h) : (int)__ldg(in.idx + (size_t)s * cells + c);
            const float v = s == 0 ? value0(in, h, c) : __ldg(in.val + (size_t)s * cells + c);
            if (v > best) { best = v; best_id = id; }
            if (id == LIQ) liq = v;
        }
        // stored ids ascend, so a strict '>' keeps the first maximum; a
        // non-positive best leaves the dense argmax at the smallest unstored id
        if (!(best > 0.0f)) {
            best = 0.0f;
            best_id = 0;
        }
        if (ids) ids[p] = best_id;
        if (vmax_out) vmax_out[p] = best;
        if (solid_out) solid_out[p] = 1.0f - liq;
    }
}

// ---------------------------------------------------------------------------
// Checkpoint packing.  Entries of a cell: its stored (id, value) pairs when
// it keeps values (two or more phases, or one explicit value), none for an
// implicit single phase.  Packed order: cell-major, ascending ids within a
// cell.  Offsets come from a three-kernel exclusive scan over the heads
// (block totals, one-block scan of the totals, per-block scan and copy), so
// the unpacker recomputes them from the heads alone.
constexpr int PK_THREADS = 256;
constexpr int PK_ROUNDS = 8;
constexpr int PK_CELLS = PK_THREADS * PK_ROUNDS;

__device__ __forceinline__ int entries_of(uint32_t h) {
    const int n = hcount(h);
    return (n >= 2 || (n == 1 && hexplicit(h))) ? n : 0;
}

__device__ __forceinline__ long long block_exclusive_scan(long long v, long long *warp_tot, long long &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    long long before = 0, tot = 0;
    for (int i = 0; i < PK_THREADS / 32; ++i) {
        if (i < w) before += warp_tot[i];
        tot += warp_tot[i];
    }
    __syncthreads();
    total = tot;
    return before + x - v;
}

__global__ void __launch_bounds__(PK_THREADS) pack_count_kernel(const uint32_t *__restrict__ head, int64_t cells,
                                                                 long long *__restrict__ block_sum) {
    __shared__ long long warp_tot[PK_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * PK_CELLS;
    long long e = 0;
    for (int j = 0; j < PK_ROUNDS; ++j) {
        const int64_t c = base + (int64_t)j * PK_THREADS + threadIdx.x;
        if (c < cells) e += entries_of(__ldg(head + c));
    }
    long long total;
    block_exclusive_scan(e, warp_tot, total);
    if (threadIdx.x == 0) block_sum[blockIdx.x] = total;
}

// one block: exclusive scan of nb block totals in place, grand total to *total
__global__ void __launch_bounds__(1024) pack_scan_kernel(long long *__restrict__ block_sum, int64_t nb,
                                                         long long *__restrict__ total) {
    __shared__ long long part[1024];
    const int64_t per = (nb + 1023) / 1024;
    const int64_t lo = (int64_t)threadIdx.x * per, hi = min(lo + per, nb);
    long long s = 0;
    for (int64_t i = lo; i < hi; ++i) s += block_sum[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long run = 0;
        for (int i = 0; i < 1024; ++i) {
            const long long t = part[i];
            part[i] = run;
            run += t;
        }
        *total = run;
    }
    __syncthreads();
    long long run = part[threadIdx.x];
    for (int64_t i = lo; i < hi; ++i) {
        const long long t = block_sum[i];
        block_sum[i] = run;
        run += t;
    }
}

template <int S, bool PACK>
__global__ void __launch_bounds__(PK_THREADS) pack_copy_kernel(const uint32_t *__restrict__ head, int64_t cells,
                                                                const long long *__restrict__ block_off,
                                                                uint16_t *__restrict__ idx, float *__restrict__ val,
                                                                uint16_t *__restrict__ pids, float *__restrict__ pvals,
                                                                int64_t capacity, int32_t *__restrict__ err) {
    __shared__ long long warp_tot[PK_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * PK_CELLS;
    long long run = block_off[blockIdx.x];
    bool bad = false, deep = false;
    for (int j = 0; j < PK_ROUNDS; ++j) {
        const int64_t c = base + (int64_t)j * PK_THREADS + threadIdx.x;
        const uint32_t h = c < cells ? __ldg(head + c) : 0u;
        const int e = c < cells ? entries_of(h) : 0;
        long long round_total;
        const long long off = run + block_exclusive_scan(e, warp_tot, round_total);
        run += round_total;
        if (e == 0) continue;
        if (e > S) {  // more stored phases than the slot template holds
            deep = true;
            continue;
        }
        if (off + e > capacity) {
            bad = true;
            continue;
        }
        if (PACK) {
            for (int s = 0; s < e; ++s) {
                pids[off + s] = s == 0 ? (uint16_t)hid0(h) : idx[(size_t)s * cells + c];
                pvals[off + s] = val[(size_t)s * cells + c];
            }
        } else {
            if ((int)pids[off] != hid0(h)) {
                bad = true;
                continue;
            }
            for (int s = 0; s < e; ++s) {
                if (s > 0) idx[(size_t)s * cells + c] = pids[off + s];
                val[(size_t)s * cells + c] = pvals[off + s];
            }
        }
    }
    if (err && bad) atomicOr(err, MPF3D_DEV_BAD_INPUT);
    if (err && deep) atomicOr(err, MPF3D_DEV_SLOT_OVERFLOW);
}

// ---------------------------------------------------------------------------
// Batched spheres and directional probes

__device__ __forceinline__ int instance_of_cell(const mpf3d_instance *__restrict__ inst, int n, uint32_t c) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].offset <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// init_singlemode_sphere_3d: phi_s = 0.5 (1 - tanh(f (|x - c| - R))) in
// float64 with f = float32(2.2/delta), x = cell index * dx, then float32;
// liquid = 1 - phi_s in float32.  Rounded operations keep the float64 steps
// free of fused multiply-adds, as numpy evaluates them.
__global__ void init_sphere_kernel(const mpf3d_instance *__restrict__ inst, int n_inst, uint32_t total, double dx,
                                   float factor, const float *__restrict__ center, const float *__restrict__ radius,
                                   int gid, uint32_t stride, uint32_t *__restrict__ head, uint16_t *__restrict__ idx,
                                   float *__restrict__ val) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
        const int i = instance_of_cell(inst, n_inst, c);
        const mpf3d_instance I = inst[i];
        const uint32_t r = c - I.offset;
        const uint32_t plane = (uint32_t)I.nx * (uint32_t)I.ny;
        const int k = (int)(r / plane);
        const uint32_t q = r - (uint32_t)k * plane;
        const int m = (int)(q / (uint32_t)I.nx);
        const int l = (int)(q - (uint32_t)m * (uint32_t)I.nx);
        const double cx = __dmul_rn((double)center[3 * i], dx), cy = __dmul_rn((double)center[3 * i + 1], dx);
        const double cz = __dmul_rn((double)center[3 * i + 2], dx);
        const double X = __dsub_rn(__dmul_rn((double)l, dx), cx);
        const double Y = __dsub_rn(__dmul_rn((double)m, dx), cy);
        const double Z = __dsub_rn(__dmul_rn((double)k, dx), cz);
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(X, X), __dmul_rn(Y, Y)), __dmul_rn(Z, Z));
        const double sd = __dsub_rn(sqrt(d2), __dmul_rn((double)radius[i], dx));
        const float phs = (float)__dmul_rn(0.5, __dsub_rn(1.0, tanh(__dmul_rn((double)factor, sd))));
        const float liq = 1.0f - phs;
        if (phs > 0.0f && liq > 0.0f) {
            head[c] = mkhead(LIQ, 2, false);
            val[c] = liq;
            idx[(size_t)stride + c] = (uint16_t)gid;
            val[(size_t)stride + c] = phs;
        } else if (phs > 0.0f) {
            head[c] = mkhead(gid, 1, false);
        } else {
            head[c] = mkhead(LIQ, 1, false);
        }
    }
}

// trilinear_sample (run_orientation_scan_3d.py:238-269) of one phase of an
// instance; NaN outside [0, n-1]^3
template <int S>
__device__ double trilinear(const In &in, uint32_t stride, const mpf3d_instance &I, int g, double x, double y,
                            double z) {
    if (x < 0.0 || y < 0.0 || z < 0.0 || x > I.nx - 1 || y > I.ny - 1 || z > I.nz - 1) return NAN;
    const int x0 = (int)floor(x), y0 = (int)floor(y), z0 = (int)floor(z);
    const int x1 = min(x0 + 1, I.nx - 1), y1 = min(y0 + 1, I.ny - 1), z1 = min(z0 + 1, I.nz - 1);
    const double tx = x - x0, ty = y - y0, tz = z - z0;
    auto at = [&](int a, int b, int d) {
        const uint32_t c = I.offset + ((uint32_t)d * (uint32_t)I.ny + (uint32_t)b) * (uint32_t)I.nx + (uint32_t)a;
        return (double)phase_at<S>(in, stride, c, g);
    };
    const double c00 = at(x0, y0, z0) * (1.0 - tx) + at(x1, y0, z0) * tx;
    const double c01 = at(x0, y0, z1) * (1.0 - tx) + at(x1, y0, z1) * tx;
    const double c10 = at(x0, y1, z0) * (1.0 - tx) + at(x1, y1, z0) * tx;
    const double c11 = at(x0, y1, z1) * (1.0 - tx) + at(x1, y1, z1) * tx;
    const double c0 = c00 * (1.0 - ty) + c10 * ty;
    const double c1 = c01 * (1.0 - ty) + c11 * ty;
    return c0 * (1.0 - tz) + c1 * tz;
}

// directional_radius_one_side (run_orientation_scan_3d.py:292-335): march
// from the centre along d in steps of step_cells until the phase drops
// below the threshold, with a linear root between the last two samples.
// One thread per (instance, direction, sign).
template <int S>
__global__ void ray_kernel(In in, uint32_t stride, const mpf3d_instance *__restrict__ inst, int n_inst, int g,
                           const float *__restrict__ center, const float *__restrict__ dirs, int n_dir,
                           double threshold, double step_cells, double *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_inst * n_dir * 2) return;
    const int i = t / (2 * n_dir), rem = t - i * 2 * n_dir, di = rem >> 1, sign = rem & 1;
    const mpf3d_instance I = inst[i];
    double d[3] = {dirs[3 * di], dirs[3 * di + 1], dirs[3 * di + 2]};
    if (sign) { d[0] = -d[0]; d[1] = -d[1]; d[2] = -d[2]; }
    const double c[3] = {center[3 * i], center[3 * i + 1], center[3 * i + 2]};
    double r = NAN;
    const double dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (dn >= 1.0e-12) {
        d[0] /= dn; d[1] /= dn; d[2] /= dn;
        // max_distance_to_boundary (:272-289)
        const double upper[3] = {I.nx - 1.0, I.ny - 1.0, I.nz - 1.0};
        double max_s = INFINITY;
        bool any = false;
        for (int a = 0; a < 3; ++a) {
            if (fabs(d[a]) < 1.0e-12) continue;
            const double lim = d[a] > 0.0 ? (upper[a] - c[a]) / d[a] : (0.0 - c[a]) / d[a];
            if (lim > 0.0) { max_s = fmin(max_s, lim); any = true; }
        }
        if (!any) max_s = 0.0;
        const double v0 = trilinear<S>(in, stride, I, g, c[0], c[1], c[2]);
        if (max_s > 0.0 && isfinite(v0) && !(v0 < threshold)) {
            double prev_s = 0.0, prev_v = v0;
            const int n_steps = max(2, (int)ceil(max_s / step_cells) + 1);
            for (int s_i = 1; s_i <= n_steps; ++s_i) {
                const double s = fmin(s_i * step_cells, max_s);
                const double v = trilinear<S>(in, stride, I, g, c[0] + d[0] * s, c[1] + d[1] * s, c[2] + d[2] * s);
                if (!isfinite(v)) break;
                if (prev_v >= threshold && v < threshold) {
                    const double dv = prev_v - v;
                    if (fabs(dv) < 1.0e-12) { r = s; break; }
                    double frac = (prev_v - threshold) / dv;
                    frac = fmin(fmax(frac, 0.0), 1.0);
                    r = prev_s + frac * (s - prev_s);
                    break;
                }
                prev_s = s;
                prev_v = v;
            }
        }
    }
    out[t] = r;
}

}  // namespace observe
}  // namespace mpf3d

using namespace mpf3d::observe;

#define MPF3D_SLOT_SWITCH(slots, CALL4, CALL8, CALL16) \
    do {                                                \
        if ((slots) == 4) { CALL4; }                    \
        else if ((slots) == 8) { CALL8; }               \
        else if ((slots) == 16) { CALL16; }             \
        else return MPF3D_ERR_ARG;                      \
    } while (0)

extern "C" int mpf3d_compact_metrics(const uint32_t *head, const uint16_t *idx, const float *val, int slots, int N,
                                     int nx, int ny, int nz, float threshold, mpf3d_metrics *result,
                                     double *grain_sum, float *front, void *stream) {
    if (!head || !idx || !val || !result || N <= 0 || N > 65535 || !dims_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    if ((int64_t)nx * ny * nz >= ((int64_t)1 << 32)) return MPF3D_ERR_TOO_LARGE;
    cudaStream_t s = (cudaStream_t)stream;
    In in{head, idx, val};
    metrics_init_kernel<<<grain_sum ? (N + 255) / 256 : 1, 256, 0, s>>>(result, grain_sum, N);
    const int64_t cols = (int64_t)nx * ny;
    int blocks = (int)((cols + 255) / 256);
    const int cap = sms_of_current_device() * 8;
    if (blocks > cap) blocks = cap;
    double *gs = grain_sum;
    // without a grain-sum array no grain id passes the 0 < id < n_hist test
    const int n_hist = gs ? N : 1;
    const bool smem = gs && N <= 4096;
    const size_t shm = smem ? (size_t)N * sizeof(double) : 0;
#define MK(SS)                                                                                             \
    (smem ? metrics_kernel<SS, true><<<blocks, 256, shm, s>>>(in, N, n_hist, nx, ny, nz, threshold, result, gs, \
                                                              front)                                       \
          : metrics_kernel<SS, false><<<blocks, 256, 0, s>>>(in, N, n_hist, nx, ny, nz, threshold, result, gs, \
                                                             front))
    MPF3D_SLOT_SWITCH(slots, MK(4), MK(8), MK(16));
#undef MK
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_compact_slice(const uint32_t *head, const uint16_t *idx, const float *val, int slots, int nx,
                                   int ny, int nz, int axis, int index, int32_t *ids, float *vmax, float *solid,
                                   void *stream) {
    if (!head || !idx || !val || !dims_ok(nx, ny, nz) || axis < 0 || axis > 2) return MPF3D_ERR_ARG;
    if ((int64_t)nx * ny * nz >= ((int64_t)1 << 32)) return MPF3D_ERR_TOO_LARGE;
    const int upper = axis == 0 ? nz : (axis == 1 ? ny : nx);
    if (index < 0 || index >= upper) return MPF3D_ERR_ARG;
    const int64_t pix = axis == 0 ? (int64_t)nx * ny : (axis == 1 ? (int64_t)nx * nz : (int64_t)ny * nz);
    if (pix >= ((int64_t)1 << 31)) return MPF3D_ERR_TOO_LARGE;
    In in{head, idx, val};
    cudaStream_t s = (cudaStream_t)stream;
    int blocks = (int)((pix + 255) / 256);
    if (blocks > 65535) blocks = 65535;
#define SL(SS) slice_kernel<SS><<<blocks, 256, 0, s>>>(in, nx, ny, nz, axis, index, ids, vmax, solid)
    MPF3D_SLOT_SWITCH(slots, SL(4), SL(8), SL(16));
#undef SL
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int64_t mpf3d_compact_pack_scratch_len(int64_t cells) {
    return cells <= 0 ? 1 : (cells + PK_CELLS - 1) / PK_CELLS + 1;
}

static int pack_common(const uint32_t *head, uint16_t *idx, float *val, int slots, int64_t cells,
                       int64_t *scratch, int64_t *total, uint16_t *pids, float *pvals, int64_t capacity,
                       int32_t *err, cudaStream_t s, bool pack) {
    const int64_t nb = (cells + PK_CELLS - 1) / PK_CELLS;
    long long *bsum = (long long *)scratch;
    long long *tot = total ? (long long *)total : bsum + nb;
    pack_count_kernel<<<(unsigned)nb, PK_THREADS, 0, s>>>(head, cells, bsum);
    pack_scan_kernel<<<1, 1024, 0, s>>>(bsum, nb, tot);
    if (!pids || !pvals) return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
#define PC(SS)                                                                                             \
    (pack ? pack_copy_kernel<SS, true><<<(unsigned)nb, PK_THREADS, 0, s>>>(head, cells, bsum, idx, val, pids, pvals, \
                                                                           capacity, err)                  \
          : pack_copy_kernel<SS, false><<<(unsigned)nb, PK_THREADS, 0, s>>>(head, cells, bsum, idx, val, pids,     \
                                                                            pvals, capacity, err))
    MPF3D_SLOT_SWITCH(slots, PC(4), PC(8), PC(16));
#undef PC
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_compact_pack(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                                  int64_t cells, int64_t *scratch, int64_t *total, uint16_t *ids_out,
                                  float *vals_out, int64_t capacity, int32_t *err, void *stream) {
    if (!head || !idx || !val || !scratch || !total || cells <= 0 || cells >= ((int64_t)1 << 32) || capacity < 0)
        return MPF3D_ERR_ARG;
    if ((ids_out == nullptr) != (vals_out == nullptr)) return MPF3D_ERR_ARG;
    if (ids_out && !err) return MPF3D_ERR_ARG;
    return pack_common(head, const_cast<uint16_t *>(idx), const_cast<float *>(val), slots, cells, scratch, total,
                       ids_out, vals_out, capacity, err, (cudaStream_t)stream, true);
}

extern "C" int mpf3d_compact_unpack(const uint32_t *head, const uint16_t *ids_in, const float *vals_in,
                                    int64_t n_entries, int slots, int64_t cells, int64_t *scratch, uint16_t *idx_out,
                                    float *val_out, int32_t *err, void *stream) {
    if (!head || !ids_in || !vals_in || !scratch || !idx_out || !val_out || !err || cells <= 0 ||
        cells >= ((int64_t)1 << 32) || n_entries < 0)
        return MPF3D_ERR_ARG;
    return pack_common(head, idx_out, val_out, slots, cells, scratch, nullptr, const_cast<uint16_t *>(ids_in),
                       const_cast<float *>(vals_in), n_entries, err, (cudaStream_t)stream, false);
}

extern "C" int mpf3d_batched_init_sphere(const mpf3d_instance *inst, int n_inst, uint32_t total_cells, double dx,
                                         double delta, const float *center, const float *radius, int solid_gid,
                                         int slots, uint32_t *head, uint16_t *idx, float *val, void *stream) {
    if (!inst || !center || !radius || !head || !idx || !val || n_inst <= 0 || total_cells == 0 || dx <= 0.0 ||
        delta <= 0.0 || solid_gid <= 0 || solid_gid > 65535 || slots < 2)
        return MPF3D_ERR_ARG;
    const float factor = (float)(2.2 / delta);
    init_sphere_kernel<<<sms_of_current_device() * 16, 256, 0, (cudaStream_t)stream>>>(
        inst, n_inst, total_cells, dx, factor, center, radius, solid_gid, total_cells, head, idx, val);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_batched_ray_radii(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                                       const mpf3d_instance *inst, int n_inst, uint32_t total_cells, int phase,
                                       const float *center, const float *dirs, int n_dir, double threshold,
                                       double step_cells, double *out, void *stream) {
    if (!head || !idx || !val || !inst || !center || !dirs || !out || n_inst <= 0 || n_dir <= 0 || phase < 0 ||
        !(step_cells > 0.0))
        return MPF3D_ERR_ARG;
    In in{head, idx, val};
    const int threads = n_inst * n_dir * 2;
    const int blocks = (threads + 127) / 128;
    cudaStream_t s = (cudaStream_t)stream;
#define RK(SS) ray_kernel<SS><<<blocks, 128, 0, s>>>(in, total_cells, inst, n_inst, phase, center, dirs, n_dir, \
                                                      threshold, step_cells, out)
    MPF3D_SLOT_SWITCH(slots, RK(4), RK(8), RK(16));
#undef RK
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}
