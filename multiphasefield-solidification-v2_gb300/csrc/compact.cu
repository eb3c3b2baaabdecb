// compact.cu -- FP32 compact-slot stepper (throughput tier).
//
// A time step is three kernels that together do what the reference does in
// three dense launches (src/gpu_kernels_3d.py:462-486 APT rebuild, :530-680
// phase update, :833-838 cooling): a sweep writes the cells whose
// neighbourhood holds one phase and queues the rest on work lists; a general
// kernel and an interface kernel then rebuild each queued cell's
// active-phase list from the stored lists of the cell and its 6 face
// neighbours, evaluate the anisotropic interface, torque and kinetic terms
// and the pair sums, clip, renormalise and write only the phases that stay
// positive.
//
// State layout in HBM (x fastest, so a warp of 32 threads along x reads
// 32 consecutive entries of each array and an interface -- normal to z --
// keeps a warp convergent):
//   head uint32[cells]     bits 0-6 number n of stored phases (phi > 0),
//                          bit 7 "single value stored explicitly",
//                          bits 8-23 id of the first (smallest) stored phase
//   idx  uint16[S][cells]  ids of stored phases 1..n-1 (ascending; slot 0 unused)
//   val  float [S][cells]  fractions of stored phases 0..n-1
// A cell holding one phase at exactly 1 -- about nine cells in ten in a
// directional-solidification run -- costs 4 bytes: its value is implicit.
// Temperature is T0[z] - (accumulated cooling) with the accumulator in
// float64 on the host; the per-cell sum-to-one uses a compensated float
// pair (TwoSum), which keeps GB300's slow float64 pipe out of the loop.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string.h>

#include <mutex>
#include <unordered_map>

#include "compact_state.cuh"
#include "mpf3d.h"
#include "mpf3d_internal.h"

namespace mpf3d {
namespace compact {

// the reference's pi approximation in the driving-force prefactor (:651)
constexpr float FORCE_PREF = (float)(8.0 / 3.1415926535);

struct Params {
    int nx, ny, nz, N;
    int64_t cells;
    uint32_t cells32;
    float e2_flat, b_flat;  // eps^2 and b for a liquid gradient below the floor
    float inv_dx2, inv_2dx, half_over_dx, inv_dx, dt;
    float eps0, eps0sq, w0, mu_a, delta_a, mu_da, pp, tan_a0, g2_floor, ksi, theta_c, cos_theta_lo, Sf;
    double Tmc;  // T_melt + accumulated cooling (float64)
    // Device step clock (null: Tmc above).  The sweep reads the step's index
    // s = clock->step[parity], writes clock->tmc[parity] = clock_T_melt +
    // s * clock_rate (rounded operation by operation, like the host's
    // float64 expression) for the work-list kernels and clock->step[parity ^
    // 1] = s + 1 for the next step, so a CUDA graph of steps keeps cooling
    // when it is replayed.
    mpf3d_step_clock *clock;
    double clock_T_melt, clock_rate;
    int parity;
    int use_aniso, use_torque;
    int sym_normals;  // every grain's n111 rows 4..7 are -(rows 3..0)
    // per-domain view (a batch of instances shares the state arrays)
    uint32_t base;    // index of the domain's first cell in the state arrays
    int n111_base;    // first n111 row of the domain's phases
    int t_uniform;    // temperature uniform in the domain ...
    float dT_uniform; // ... with T - T_melt = dT_uniform
};


__device__ __forceinline__ int64_t cell_of(const Params &P, int l, int m, int k) {
    return ((int64_t)k * P.ny + m) * P.nx + l;
}

// max |cos| between a gradient and the grain's 8 rotated {111} normals, with
// the signed cosine and the winning normal (best_cos_from_grad_3d :110-134,
// facet_cos_and_nxyz_from_grad :251-301)
struct Facet {
    bool valid;
    float cabs, cs, nx, ny, nz, q;
};

// When the 8 normals are 4 exact antipodal pairs with one member of each
// pair among the first four (true for the rotated (+-1,+-1,+-1)/sqrt(3) set
// in the reference's order; checked on the host), |cos| ties exactly within
// a pair and the first-maximum search over 8 equals the search over 4.
template <int NT = 8>
__device__ __forceinline__ Facet facet_n(float3 g, const float *__restrict__ u, float g2_floor) {
    Facet f;
    f.q = g.x * g.x + g.y * g.y + g.z * g.z;
    f.valid = !(f.q < g2_floor);
    f.cabs = 0.0f; f.cs = 0.0f; f.nx = 1.0f; f.ny = 0.0f; f.nz = 0.0f;
    if (!f.valid) return f;
    float ig = rsqrtf(f.q);
    float gx = g.x * ig, gy = g.y * ig, gz = g.z * ig;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        float ux = __ldg(u + 3 * t), uy = __ldg(u + 3 * t + 1), uz = __ldg(u + 3 * t + 2);
        float d = gx * ux + gy * uy + gz * uz;
        float a = fabsf(d);
        if (a > f.cabs) {
            f.cabs = a; f.cs = d; f.nx = ux; f.ny = uy; f.nz = uz;
        }
    }
    f.cabs = fminf(f.cabs, 1.0f);
    f.cs = fminf(fmaxf(f.cs, -1.0f), 1.0f);
    return f;
}

// facet_n over normals already held in registers (a grain's normals are
// loaded once per cell and reused at the 7 stencil points)
template <int NT>
__device__ __forceinline__ Facet facet_regs(float3 g, const float (&u)[3 * NT], float g2_floor) {
    Facet f;
    f.q = g.x * g.x + g.y * g.y + g.z * g.z;
    f.valid = !(f.q < g2_floor);
    f.cabs = 0.0f; f.cs = 0.0f; f.nx = 1.0f; f.ny = 0.0f; f.nz = 0.0f;
    if (!f.valid) return f;
    float ig = rsqrtf(f.q);
    float gx = g.x * ig, gy = g.y * ig, gz = g.z * ig;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const float ux = u[3 * t], uy = u[3 * t + 1], uz = u[3 * t + 2];
        float d = gx * ux + gy * uy + gz * uz;
        float a = fabsf(d);
        if (a > f.cabs) {
            f.cabs = a; f.cs = d; f.nx = ux; f.ny = uy; f.nz = uz;
        }
    }
    f.cabs = fminf(f.cabs, 1.0f);
    f.cs = fminf(fmaxf(f.cs, -1.0f), 1.0f);
    return f;
}

// a(theta) (calc_a_from_cos :24-30)
__device__ __forceinline__ float calc_a(const Params &P, float c) {
    float c2 = c * c;
    float C = sqrtf(c2 + P.pp);
    float S = sqrtf(fmaxf(1.0f - c2, 0.0f) + P.pp);
    return P.mu_a * (1.0f + P.delta_a * (C + P.tan_a0 * S));
}

// a * b - c * d with one rounding error at most (Kahan's difference of
// products); the _rn intrinsics keep the compiler from contracting the
// error-free steps into other FMAs
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d) {
    const float w = __fmul_rn(c, d);
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return __fadd_rn(f, e);
}

// theta = acos(c) for the facet's best |cos| c = |g . n| / |g| against the
// float32 normal n, accurate where c is near 1.  There FP32 acos of a
// rounded c loses most of theta (an absolute error of 1e-7 in c is a
// relative error of 1e-7 / theta^2 in 1 - c), and b(theta) is steep.  The
// reference evaluates c in float64 from the same float32 normals, whose
// length differs from 1 by their rounding, so
//   1 - c = (1 - |n|) + |n| (1 - cos t),  t the angle between g and n,
// with 1 - |n|^2 from compensated squares (TwoProduct, TwoSum) and
//   1 - cos t = |g x n|^2 / (|g|^2 |n|^2 (1 + cos t))
// from accurate cross-product components; theta = 2 asin(sqrt((1 - c)/2)).
// |theta - acos(c)| stays within a few 1e-6 rad against float64 (c > 1,
// possible when |n| > 1, gives theta = 0 as the reference's clamp does).
__device__ __forceinline__ float facet_angle(float3 g, const Facet &f) {
    const float nx = f.nx, ny = f.ny, nz = f.nz;
    const float p1 = __fmul_rn(nx, nx), e1 = fmaf(nx, nx, -p1);
    const float p2 = __fmul_rn(ny, ny), e2 = fmaf(ny, ny, -p2);
    const float p3 = __fmul_rn(nz, nz), e3 = fmaf(nz, nz, -p3);
    const float s1 = __fadd_rn(p1, p2);
    const float t1 = __fsub_rn(s1, p1);
    float err = __fadd_rn(__fsub_rn(p1, __fsub_rn(s1, t1)), __fsub_rn(p2, t1));
    const float s2 = __fadd_rn(s1, p3);
    const float t2 = __fsub_rn(s2, s1);
    err = __fadd_rn(err, __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, t2)), __fsub_rn(p3, t2)));
    const float dn2 = __fsub_rn(__fsub_rn(1.0f, s2), __fadd_rn(err, __fadd_rn(e1, __fadd_rn(e2, e3))));  // 1 - |n|^2
    const float cx = diff_of_products(g.y, nz, g.z, ny);
    const float cy = diff_of_products(g.z, nx, g.x, nz);
    const float cz = diff_of_products(g.x, ny, g.y, nx);
    const float sin2 = (cx * cx + cy * cy + cz * cz) / (f.q * (1.0f - dn2));
    const float omc = fmaxf(0.5f * dn2 + sin2 / (1.0f + f.cabs), 0.0f);  // 1 - c
    return 2.0f * asinf(sqrtf(0.5f * omc));
}

// b(theta) (calc_b_from_cos :33-55) for the facet of the liquid gradient g
// at the cell; below the gradient floor the best cos is 0 and b is 1
__device__ __forceinline__ float calc_b(const Params &P, float3 g, const Facet &f) {
    if (!f.valid || f.cabs <= P.cos_theta_lo) return 1.0f;  // theta >= theta_c: outside the cusp
    const float theta = facet_angle(g, f);
    if (theta >= P.theta_c) return 1.0f;
    const float hp = 1.57079632679489662f;
    float y = hp * (theta / P.theta_c);
    y = fminf(fmaxf(y, 1.0e-6f), hp - 1.0e-6f);
    float t = tanf(y);
    return P.ksi + (1.0f - P.ksi) * t * tanhf(1.0f / t);
}

// d a / d(grad phi) (da_dphixyz_A12 :304-341); returns a and the 3 components
__device__ __forceinline__ float4 da_dgrad(const Params &P, float3 g, const Facet &f) {
    if (!f.valid) return make_float4(0.f, 0.f, 0.f, 0.f);
    float a = calc_a(P, f.cabs);
    float ig = rsqrtf(f.q);
    float ig3 = ig * ig * ig;
    float ud = g.x * f.nx + g.y * f.ny + g.z * f.nz;
    float c = f.cs, c2 = c * c;
    float C = sqrtf(c2 + P.pp);
    float S = sqrtf(fmaxf(1.0f - c2, 0.0f) + P.pp);
    float coef = P.mu_da * (c / C - P.tan_a0 * (c / S));
    return make_float4(a, coef * (f.nx * ig - ud * g.x * ig3), coef * (f.ny * ig - ud * g.y * ig3),
                       coef * (f.nz * ig - ud * g.z * ig3));
}

// Work lists of a step (scratch memory owned by the caller): items[cells]
// holds x-fastest cell indices -- cells needing the general update from the
// front, solid-liquid interface cells from the back; count[4] holds the two
// list lengths for even and odd steps (count[2*parity + 0/1]), so the sweep
// of one step can clear the other parity's counters without a memset.
struct Queue {
    uint32_t *__restrict__ items;
    uint32_t *__restrict__ count;
    // With split set, interface cells whose active list holds two or more
    // solids go to a third list at items[cells + ...] (counters count[4 +
    // parity]): their warps loop over the solids, and keeping them apart
    // from the one-solid majority spares those warps the idle iterations.
    int split;
};

struct Mats {
    const double *__restrict__ T0z;
    const float *__restrict__ wij;
    const float *__restrict__ a2ij;
    const float *__restrict__ mij;
    const float *__restrict__ n111;
};

__device__ __forceinline__ uint32_t cidx(const Params &P, int l, int m, int k) {
    return P.base + ((uint32_t)k * (uint32_t)P.ny + (uint32_t)m) * (uint32_t)P.nx + (uint32_t)l;
}

// liquid fraction of cell q; the head and the first value are loaded
// together (the value is ignored where the head says it is not needed), so
// the liquid stencil costs one round of loads rather than two
__device__ __forceinline__ float liquid32(const In &in, uint32_t q) {
    const uint32_t h = __ldg(in.head + q);
    const float v = __ldg(in.val + q);
    if (hcount(h) == 0 || hid0(h) != LIQ) return 0.0f;
    return (hcount(h) >= 2 || hexplicit(h)) ? v : 1.0f;
}

// 7-point Laplacian of one phase, rounded operation by operation
__device__ __forceinline__ float lap7(const Params &P, const float (&v)[7]) {
    float s = __fadd_rn(v[1], v[2]);
    s = __fadd_rn(s, v[3]);
    s = __fadd_rn(s, v[4]);
    s = __fadd_rn(s, v[5]);
    s = __fadd_rn(s, v[6]);
    return __fmul_rn(__fsub_rn(s, __fmul_rn(6.0f, v[0])), P.inv_dx2);
}

// Active list of one cell: the ascending union of the stored lists of the
// cell and its 6 neighbours (the APT rule of kernel_update_nfmf_3d for
// phi >= 0), produced by a 7-way merge of the sorted lists, which also
// yields every active phase's value at the 7 points without any search.
template <int AMAX>
struct Active {
    int n;
    bool ovf;
    int ids[AMAX];
    float vc[AMAX];   // value at the cell
    float lap[AMAX];  // 7-point Laplacian (laplacian_3d :444-459)
    float vL[7];      // liquid at the 7 points
    int ts;           // index of the dominant solid (max value at the cell), -1 if none
    float3 gs;        // its gradient at the cell
};

template <int S, int AMAX>
__device__ __forceinline__ void gather(const In &in, const Params &P, const uint32_t (&pt)[7], Active<AMAX> &A) {
    const uint32_t cells = P.cells32;
    int cnt[7], pos[7], head[7];
    uint32_t hw[7];
#pragma unroll
    for (int p = 0; p < 7; ++p) {
        hw[p] = __ldg(in.head + pt[p]);
        const int c = hcount(hw[p]);
        cnt[p] = c < S ? c : S;
        pos[p] = 0;
        head[p] = cnt[p] > 0 ? hid0(hw[p]) : 0x7fffffff;
        A.vL[p] = 0.0f;
    }
    A.n = 0;
    A.ovf = false;
    A.ts = -1;
    A.gs = make_float3(0.f, 0.f, 0.f);
    float maxv = -1.0f;
    while (true) {
        int id = head[0];
#pragma unroll
        for (int p = 1; p < 7; ++p) id = min(id, head[p]);
        if (id == 0x7fffffff) break;
        float v[7];
#pragma unroll
        for (int p = 0; p < 7; ++p) {
            v[p] = 0.0f;
            if (head[p] == id) {
                v[p] = pos[p] == 0 ? value0(in, hw[p], pt[p]) : __ldg(in.val + (uint32_t)pos[p] * cells + pt[p]);
                ++pos[p];
                head[p] = pos[p] < cnt[p] ? (int)__ldg(in.idx + (uint32_t)pos[p] * cells + pt[p]) : 0x7fffffff;
            }
        }
        if (A.n == AMAX) {
            A.ovf = true;
            break;
        }
        A.ids[A.n] = id;
        A.vc[A.n] = v[0];
        A.lap[A.n] = lap7(P, v);
        if (id == LIQ) {
#pragma unroll
            for (int p = 0; p < 7; ++p) A.vL[p] = v[p];
        } else if (v[0] > maxv) {
            maxv = v[0];
            A.ts = A.n;
            A.gs = make_float3((v[1] - v[2]) * P.inv_2dx, (v[3] - v[4]) * P.inv_2dx, (v[5] - v[6]) * P.inv_2dx);
        }
        ++A.n;
    }
}

// Facet-derived quantities of one grain at one stencil point: the
// anisotropy a(theta) (calc_a_from_cos :24-30), eps^2 = (eps0 a)^2 and
// d a / d(grad phi) (da_dphixyz_A12 :304-341).  C = sqrt(c^2+p^2) and
// S = sqrt(max(1-c^2,0)+p^2) are shared by a and da/dc.
struct PointTerms {
    float e2;        // eps^2 at the point
    float a;         // a(theta)
    float3 da;       // d a / d(phi_x, phi_y, phi_z); zero below the floor
    float coef;      // mu_a delta_a (c/C - tan(a0) c/S)
};

__device__ __forceinline__ PointTerms point_terms(const Params &P, float3 g, const Facet &f, bool want_da) {
    PointTerms t;
    if (!f.valid) {
        t.e2 = P.e2_flat;
        t.a = 0.0f;
        t.da = make_float3(0.f, 0.f, 0.f);
        t.coef = 0.0f;
        return t;
    }
    const float c = f.cs, c2 = c * c;
    const float C = sqrtf(c2 + P.pp);
    const float S = sqrtf(fmaxf(1.0f - c2, 0.0f) + P.pp);
    t.a = P.mu_a * (1.0f + P.delta_a * (C + P.tan_a0 * S));
    const float e = P.eps0 * t.a;
    t.e2 = e * e;
    t.coef = P.mu_da * (__fdividef(c, C) - P.tan_a0 * __fdividef(c, S));
    if (want_da) {
        const float ig = rsqrtf(f.q);
        const float ig3 = ig * ig * ig;
        const float ud = g.x * f.nx + g.y * f.ny + g.z * f.nz;
        t.da = make_float3(t.coef * (f.nx * ig - ud * g.x * ig3), t.coef * (f.ny * ig - ud * g.y * ig3),
                           t.coef * (f.nz * ig - ud * g.z * ig3));
    } else {
        t.da = make_float3(0.f, 0.f, 0.f);
    }
    return t;
}

// eps^2-weighted divergence, torque and kinetic factor of one solid grain at
// a cell from the liquid gradient at the 7 points and the liquid's second
// derivatives at the cell (aniso_term1_solid_3d :149-204, torque_A11_3d
// :386-441, A13_divergence_3d :344-383, calc_b_from_cos :33-55).
template <int NT>
__device__ __forceinline__ void interface_terms(const Params &P, const float3 (&G)[7], const float (&vL)[7],
                                                const float (&h2)[6], const float (&u)[3 * NT], bool torque,
                                                float &lap_sl, float &b_sl) {
    Facet F[7];
    bool any = false;
#pragma unroll
    for (int p = 0; p < 7; ++p) {
        F[p] = facet_regs<NT>(G[p], u, P.g2_floor);
        any = any || F[p].valid;
    }
    const float Lc = vL[0];
    const float h = P.inv_2dx * P.inv_dx;
    if (!any) {
        // flat liquid everywhere: eps^2 = (eps0 a(0))^2 at all 7 points, no torque
        const float e2 = P.e2_flat;
        lap_sl = ((2.0f * e2) * (vL[1] - Lc) - (2.0f * e2) * (Lc - vL[2])) * h +
                 ((2.0f * e2) * (vL[3] - Lc) - (2.0f * e2) * (Lc - vL[4])) * h +
                 ((2.0f * e2) * (vL[5] - Lc) - (2.0f * e2) * (Lc - vL[6])) * h;
        b_sl = P.b_flat;
        return;
    }
    const bool tq = torque && F[0].valid;
    PointTerms T[7];
    T[0] = point_terms(P, G[0], F[0], tq);
#pragma unroll
    for (int p = 1; p < 7; ++p) T[p] = point_terms(P, G[p], F[p], tq);
    float lv = ((T[0].e2 + T[1].e2) * (vL[1] - Lc) - (T[0].e2 + T[2].e2) * (Lc - vL[2])) * h +
               ((T[0].e2 + T[3].e2) * (vL[3] - Lc) - (T[0].e2 + T[4].e2) * (Lc - vL[4])) * h +
               ((T[0].e2 + T[5].e2) * (vL[5] - Lc) - (T[0].e2 + T[6].e2) * (Lc - vL[6])) * h;
    if (tq) {
        const float3 g0 = G[0];
        const float q = F[0].q;
        const float pxx = h2[0], pyy = h2[1], pzz = h2[2], pxy = h2[3], pxz = h2[4], pyz = h2[5];
        const float qx = 2.0f * (g0.x * pxx + g0.y * pxy + g0.z * pxz);
        const float qy = 2.0f * (g0.x * pxy + g0.y * pyy + g0.z * pyz);
        const float qz = 2.0f * (g0.x * pxz + g0.y * pyz + g0.z * pzz);
        const float ig = rsqrtf(q), ig3 = ig * ig * ig;
        const float ud = g0.x * F[0].nx + g0.y * F[0].ny + g0.z * F[0].nz;
        const float dcx = F[0].nx * ig - ud * g0.x * ig3;
        const float dcy = F[0].ny * ig - ud * g0.y * ig3;
        const float dcz = F[0].nz * ig - ud * g0.z * ig3;
        const float cxx = dcx * pxx + dcy * pxy + dcz * pxz;
        const float cyy = dcx * pxy + dcy * pyy + dcz * pyz;
        const float czz = dcx * pxz + dcy * pyz + dcz * pzz;
        const float coef = T[0].coef;
        // A13_divergence_3d: central differences of da/dphi_p at the neighbours
        const float ddx = (T[1].da.x - T[2].da.x) * P.half_over_dx;
        const float ddy = (T[3].da.y - T[4].da.y) * P.half_over_dx;
        const float ddz = (T[5].da.z - T[6].da.z) * P.half_over_dx;
        const float a = T[0].a;
        const float3 d0 = T[0].da;
        const float Ex = coef * cxx * d0.x * q + a * ddx * q + a * d0.x * qx;
        const float Ey = coef * cyy * d0.y * q + a * ddy * q + a * d0.y * qy;
        const float Ez = coef * czz * d0.z * q + a * ddz * q + a * d0.z * qz;
        lv += P.eps0sq * (Ex + Ey + Ez);
    }
    lap_sl = lv;
    b_sl = calc_b(P, G[0], F[0]);
}

// Everything of the update of one cell after its active list is known:
// ids (ascending), values vc and Laplacians lap of the n active phases, the
// liquid at the 7 points, and the dominant solid ts (index, -1 if none) with
// its gradient gs.  HEAVY enables the anisotropic solid-liquid terms (cells
// with liquid and a solid active) with NT normals per grain: 4 where every
// grain's 8 normals are 4 antipodal pairs (checked on the host), else 8.
// The per-phase loops are kept rolled, and each kernel is compiled for one
// NT: unrolled or duplicated copies of this body made the kernels wait on
// instruction fetch.
template <int S, int NA, bool HEAVY, int NT>
__device__ __forceinline__ void update_cell(const In &in, const Out &out, const Mats &M, const Params &P, int l,
                                            int m, int k, uint32_t c, int n, const int (&ids)[NA],
                                            const float (&vc)[NA], const float (&lap)[NA], const float (&vL)[7],
                                            int ts, float3 gs, int32_t *__restrict__ err) {
    const uint32_t cells = P.cells32;
    const int nn = n;
    const bool has_liq = n > 0 && ids[0] == LIQ;
    const bool has_solid = n > (has_liq ? 1 : 0);
    float lap_sl[NA], b_sl[NA];
    float w_sl = P.w0;
    lap_sl[0] = 0.0f;
    b_sl[0] = 1.0f;
    if (has_liq && has_solid) {
        if (HEAVY && P.use_aniso) {
            const int lp = wrap_p(l, P.nx), lm = wrap_m(l, P.nx), mp = wrap_p(m, P.ny), mm = wrap_m(m, P.ny);
            const int kp = clamp_p(k, P.nz), km = clamp_m(k, P.nz);
            // liquid on the 25-point stencil (offsets with |dx|+|dy|+|dz| <= 2)
            const int lpp = wrap_p(lp, P.nx), lmm = wrap_m(lm, P.nx);
            const int mpp = wrap_p(mp, P.ny), mmm = wrap_m(mm, P.ny);
            const int kpp = clamp_p(kp, P.nz), kmm = clamp_m(km, P.nz);
            const float Lxpyp = liquid32(in, cidx(P, lp, mp, k)), Lxpym = liquid32(in, cidx(P, lp, mm, k));
            const float Lxmyp = liquid32(in, cidx(P, lm, mp, k)), Lxmym = liquid32(in, cidx(P, lm, mm, k));
            const float Lxpzp = liquid32(in, cidx(P, lp, m, kp)), Lxpzm = liquid32(in, cidx(P, lp, m, km));
            const float Lxmzp = liquid32(in, cidx(P, lm, m, kp)), Lxmzm = liquid32(in, cidx(P, lm, m, km));
            const float Lypzp = liquid32(in, cidx(P, l, mp, kp)), Lypzm = liquid32(in, cidx(P, l, mp, km));
            const float Lymzp = liquid32(in, cidx(P, l, mm, kp)), Lymzm = liquid32(in, cidx(P, l, mm, km));
            const float Lx2p = liquid32(in, cidx(P, lpp, m, k)), Lx2m = liquid32(in, cidx(P, lmm, m, k));
            const float Ly2p = liquid32(in, cidx(P, l, mpp, k)), Ly2m = liquid32(in, cidx(P, l, mmm, k));
            const float Lz2p = liquid32(in, cidx(P, l, m, kpp)), Lz2m = liquid32(in, cidx(P, l, m, kmm));
            const float g2 = P.inv_2dx;
            float3 G[7];
            G[0] = make_float3((vL[1] - vL[2]) * g2, (vL[3] - vL[4]) * g2, (vL[5] - vL[6]) * g2);
            G[1] = make_float3((Lx2p - vL[0]) * g2, (Lxpyp - Lxpym) * g2, (Lxpzp - Lxpzm) * g2);
            G[2] = make_float3((vL[0] - Lx2m) * g2, (Lxmyp - Lxmym) * g2, (Lxmzp - Lxmzm) * g2);
            G[3] = make_float3((Lxpyp - Lxmyp) * g2, (Ly2p - vL[0]) * g2, (Lypzp - Lypzm) * g2);
            G[4] = make_float3((Lxpym - Lxmym) * g2, (vL[0] - Ly2m) * g2, (Lymzp - Lymzm) * g2);
            // z neighbours sit on the clamped rows: at the top/bottom row the
            // neighbour is the cell itself
            G[5] = (kp == k) ? G[0] : make_float3((Lxpzp - Lxmzp) * g2, (Lypzp - Lymzp) * g2, (Lz2p - vL[0]) * g2);
            G[6] = (km == k) ? G[0] : make_float3((Lxpzm - Lxmzm) * g2, (Lypzm - Lymzm) * g2, (vL[0] - Lz2m) * g2);
            if (kp == k) G[5].z = (vL[5] - vL[6]) * g2;
            if (km == k) G[6].z = (vL[5] - vL[6]) * g2;
            float h2[6];
            const float qq = 0.25f * P.inv_dx2;
            h2[0] = (vL[1] - 2.0f * vL[0] + vL[2]) * P.inv_dx2;
            h2[1] = (vL[3] - 2.0f * vL[0] + vL[4]) * P.inv_dx2;
            h2[2] = (vL[5] - 2.0f * vL[0] + vL[6]) * P.inv_dx2;
            h2[3] = (Lxpyp - Lxpym - Lxmyp + Lxmym) * qq;
            h2[4] = (Lxpzp - Lxpzm - Lxmzp + Lxmzm) * qq;
            h2[5] = (Lypzp - Lypzm - Lymzp + Lymzm) * qq;
#pragma unroll 1
            for (int t = 1; t < nn; ++t) {
                const float *ug = M.n111 + (size_t)(P.n111_base + ids[t]) * 24;
                float un[3 * NT];
#pragma unroll
                for (int q = 0; q < 3 * NT; ++q) un[q] = __ldg(ug + q);
                interface_terms<NT>(P, G, vL, h2, un, P.use_torque != 0, lap_sl[t], b_sl[t]);
            }
            if (ts > 0) {
                const Facet fs = facet_n<NT>(gs, M.n111 + (size_t)(P.n111_base + ids[ts]) * 24, P.g2_floor);
                const float al = calc_a(P, fs.cabs);
                w_sl = P.w0 * (al * al);
            }
        } else {
            // isotropic branch of the switchable kernel (:729-731)
#pragma unroll 1
            for (int t = 1; t < nn; ++t) {
                lap_sl[t] = P.eps0sq * lap[0];
                b_sl[t] = 1.0f;
            }
        }
    } else {
#pragma unroll 1
        for (int t = 1; t < nn; ++t) {
            lap_sl[t] = 0.0f;
            b_sl[t] = 1.0f;
        }
    }

    // Pair sums (:600-661) in O(n^2): for a pair (i, j) the t3 sum of the
    // reference splits into W_i - W_j (potential) plus either the
    // solid-liquid term of lap_sl or (A_i - A_j)/2 (gradient energy).
    const int N = P.N;
    float W[NA], Ag[NA];
#pragma unroll 1
    for (int t1 = 0; t1 < nn; ++t1) {
        const int i = ids[t1];
        float w = 0.0f, a = 0.0f;
#pragma unroll 1
        for (int t3 = 0; t3 < nn; ++t3) {
            const int q = ids[t3];
            const float wik = (q == LIQ && i != LIQ) ? w_sl : __ldg(M.wij + i * N + q);
            w = fmaf(wik, vc[t3], w);
            a = fmaf(__ldg(M.a2ij + i * N + q), lap[t3], a);
        }
        W[t1] = w;
        Ag[t1] = a;
    }
    const double Tmc = P.clock ? P.clock->tmc[P.parity] : P.Tmc;
    const float dT = P.t_uniform ? P.dT_uniform : (float)(M.T0z[k] - Tmc);
    const float inv_n = 1.0f / (float)(n > 0 ? n : 1);
    // the non-heavy build: lap_sl is eps0^2 times the liquid's Laplacian for
    // every solid (the isotropic branch above) and b_sl is 1, so its arrays
    // stay out of local memory
    const float lsl_iso = (has_liq && has_solid) ? P.eps0sq * lap[0] : 0.0f;
    float outv[NA];
#pragma unroll 1
    for (int t1 = 0; t1 < nn; ++t1) {
        const int i = ids[t1];
        float dpi = 0.0f;
#pragma unroll 1
        for (int t2 = 0; t2 < nn; ++t2) {
            if (t2 == t1) continue;
            const int j = ids[t2];
            const bool sl = (i != LIQ && j == LIQ), ls = (i == LIQ && j != LIQ);
            const float L1 = HEAVY ? lap_sl[t1] : lsl_iso, L2 = HEAVY ? lap_sl[t2] : lsl_iso;
            const float T = sl ? 0.5f * L1 : (ls ? -0.5f * L2 : 0.5f * __fsub_rn(Ag[t1], Ag[t2]));
            const float ppp = __fadd_rn(__fsub_rn(W[t1], W[t2]), T);
            const float df = sl ? -P.Sf * dT : (ls ? P.Sf * dT : 0.0f);
            const float tf = __fmul_rn(__fmul_rn(FORCE_PREF, sqrtf(fmaxf(__fmul_rn(vc[t1], vc[t2]), 0.0f))), df);
            float me = __ldg(M.mij + i * N + j);
            if (HEAVY) {
                if (sl) me *= b_sl[t1];
                else if (ls) me *= b_sl[t2];
            }
            dpi = __fsub_rn(dpi, __fmul_rn(__fmul_rn(__fmul_rn(2.0f, me), inv_n), __fsub_rn(ppp, tf)));
        }
        outv[t1] = fminf(fmaxf(fmaf(P.dt, dpi, vc[t1]), 0.0f), 1.0f);
    }

    // renormalise with a compensated (TwoSum) float accumulation (:663-680)
    float sh = 0.0f, sl_ = 0.0f;
#pragma unroll 1
    for (int t = 0; t < nn; ++t) {
        const float a = sh, b = outv[t];
        const float s2 = a + b;
        const float bb = s2 - a;
        sl_ += (a - (s2 - bb)) + (b - bb);
        sh = s2;
    }
    // stored list: the phases that stay positive, ascending
    int cnt_out = 0, id_first = LIQ;
    bool sovf = false;
    const bool normal = sh + sl_ > 1e-20f;
    float inv = 1.0f / sh;
    inv = fmaf(-__fmul_rn(inv, inv), sl_, inv);
    if (!normal) {
        // all clipped to ~0: the liquid takes the cell (:679-680)
        out.val[c] = 1.0f;
        id_first = LIQ;
        cnt_out = 1;
    }
#pragma unroll 1
    for (int t = 0; t < nn; ++t) {
        float v;
        if (normal) {
            v = outv[t] * inv;
        } else {
            if (ids[t] == LIQ) continue;
            v = outv[t];
        }
        if (!(v > 0.0f)) continue;
        if (cnt_out == S) {
            sovf = true;
            continue;
        }
        if (cnt_out == 0) id_first = ids[t];
        else out.idx[(uint32_t)cnt_out * cells + c] = (uint16_t)ids[t];
        out.val[(uint32_t)cnt_out * cells + c] = v;
        ++cnt_out;
    }
    // one stored phase: its renormalised value is 1 and is left implicit
    out.head[c] = mkhead(id_first, cnt_out, false);
    if (sovf) atomicOr(err, MPF3D_DEV_SLOT_OVERFLOW);
}

// Update of one cell whose neighbourhood is not uniform: the 7-way merge of
// the neighbour lists, then update_cell over up to AMAX active phases (NT:
// normals per grain, used by the HEAVY form only).
template <int S, int AMAX, bool HEAVY, int NT = 4>
__device__ __forceinline__ void process_cell(const In &in, const Out &out, const Mats &M, const Params &P,
                                             int32_t *__restrict__ err, int l, int m, int k) {
    const uint32_t cells = P.cells32;
    const int lp = wrap_p(l, P.nx), lm = wrap_m(l, P.nx), mp = wrap_p(m, P.ny), mm = wrap_m(m, P.ny);
    const int kp = clamp_p(k, P.nz), km = clamp_m(k, P.nz);
    const uint32_t pt[7] = {cidx(P, l, m, k), cidx(P, lp, m, k), cidx(P, lm, m, k), cidx(P, l, mp, k),
                            cidx(P, l, mm, k), cidx(P, l, m, kp), cidx(P, l, m, km)};
    const uint32_t c = pt[0];
    Active<AMAX> A;
    gather<S, AMAX>(in, P, pt, A);
    if (A.ovf) {
        // leave the cell as it was and report; the host re-runs the step with
        // a wider template
        atomicOr(err, MPF3D_DEV_SLOT_OVERFLOW);
        const uint32_t h0 = __ldg(in.head + c);
        const int c0 = min(hcount(h0), S);
        out.head[c] = h0;
        for (int s = 0; s < c0; ++s) {
            out.idx[(uint32_t)s * cells + c] = __ldg(in.idx + (uint32_t)s * cells + c);
            out.val[(uint32_t)s * cells + c] = __ldg(in.val + (uint32_t)s * cells + c);
        }
        return;
    }
    update_cell<S, AMAX, HEAVY, NT>(in, out, M, P, l, m, k, c, A.n, A.ids, A.vc, A.lap, A.vL, A.ts, A.gs, err);
}

// Kernel 1 of a step: every cell.  Uniform neighbourhoods (the cell and its
// 6 neighbours hold one and the same phase: active list of one phase, empty
// pair sums, renormalised fraction exactly 1) are written directly; every
// other cell is appended to a work list -- solid-liquid interface cells
// (liquid and a solid in the neighbourhood, anisotropy on) to the back,
// the rest (grain boundaries, junctions without liquid, the isotropic model)
// to the front -- so that the general update runs with converged warps.
constexpr int SWEEP_ZB = 4;  // cells per thread along z (default; batches always use it)

// Where the sweep sends a queued cell: list 0 (general), 1 (interface) or 2
// (interface with several solids).  BlockSink counts a block's cells per
// list in shared memory (one shared atomic per warp, cell and list) and
// keeps each cell's list and offset in registers; the block then reserves
// its segments with one global atomic per list and writes the cell indices
// (flush).  The counters are one address each, and per-warp global atomics
// from every SM queued up at the L2 slice that holds them.  Cells are
// independent, so the order within a list changes no result.

template <int ZB>
struct BlockSink {
    uint32_t *cnt;     // shared: cells of the block per list
    uint32_t off[ZB];  // cell j's position in its list's block segment
    int lst[ZB];       // cell j's list, -1 if it is not queued

    __device__ __forceinline__ explicit BlockSink(uint32_t *c) : cnt(c) {
#pragma unroll
        for (int j = 0; j < ZB; ++j) {
            off[j] = 0;
            lst[j] = -1;
        }
    }
    __device__ __forceinline__ void add(int j, int list, uint32_t) {
        const unsigned am = __activemask();
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int L = 0; L < 3; ++L) {
            const unsigned bm = __ballot_sync(am, list == L);
            if (!bm) continue;
            const int leader = __ffs(bm) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(cnt + L, (uint32_t)__popc(bm));
            base = __shfl_sync(am, base, leader);
            if (list == L) off[j] = base + (uint32_t)__popc(bm & ((1u << lane) - 1u));
        }
        lst[j] = list;
    }
    // after the block's adds and a barrier: base[L] is the block's first
    // position in list L; cell j is (k0 + j) * plane + col
    __device__ __forceinline__ void flush(const Queue &Q, uint32_t cells, const uint32_t *base, uint32_t plane,
                                          uint32_t col, int k0) const {
#pragma unroll
        for (int j = 0; j < ZB; ++j) {
            if (lst[j] < 0) continue;
            const uint32_t pos = base[lst[j]] + off[j];
            const uint32_t c = (uint32_t)(k0 + j) * plane + col;
            Q.items[lst[j] == 0 ? pos : (lst[j] == 1 ? cells - 1u - pos : cells + pos)] = c;
        }
    }
};

// Classification of cell c = (l, m, k0 + j) from its head h0 and its 6
// neighbours' heads hn = {x+, x-, y+, y-, z+, z-} (z clamped: a neighbour
// beyond the domain is the cell itself): a uniform neighbourhood is written
// directly; any other cell goes to a work list.  Returns whether uniform.
template <class Sink>
__device__ __forceinline__ bool sweep_cell(const Out &out, const Params &P, bool split, Sink &sink, int j, uint32_t c,
                                           uint32_t h0, const uint32_t (&hn)[6]) {
    bool uniform = hcount(h0) == 1 && !hexplicit(h0);
#pragma unroll
    for (int p = 0; p < 6; ++p) uniform = uniform && hn[p] == h0;
    if (uniform) {
        // the one phase of the neighbourhood keeps the cell at exactly 1
        out.head[c] = h0;
        return true;
    }
    bool liq = hcount(h0) > 0 && hid0(h0) == LIQ;
    bool sol = hcount(h0) > 1 || (hcount(h0) == 1 && hid0(h0) != LIQ);
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        const uint32_t h = hn[p];
        liq = liq || (hcount(h) > 0 && hid0(h) == LIQ);
        sol = sol || hcount(h) > 1 || (hcount(h) == 1 && hid0(h) != LIQ);
    }
    const bool heavy = liq && sol && P.use_aniso;
    bool multi = false;
    if (heavy && split) {
        // several solids in the active list: a head with 3+ phases or two
        // solids, or two different solid first ids
        int sid = -1;
        const uint32_t hs[7] = {h0, hn[0], hn[1], hn[2], hn[3], hn[4], hn[5]};
#pragma unroll
        for (int p = 0; p < 7; ++p) {
            const int cn = hcount(hs[p]), id = hid0(hs[p]);
            if (cn >= 3 || (cn == 2 && id != LIQ)) multi = true;
            else if (cn >= 1 && id != LIQ) {
                if (sid < 0) sid = id;
                else if (sid != id) multi = true;
            }
        }
    }
    sink.add(j, heavy ? (multi ? 2 : 1) : 0, c);
    return false;
}

// The sweep of one column of ZB cells (l, m, k0..k0+ZB-1) of a domain;
// returns whether every one of them was uniform (cells past the top count
// as uniform).
template <int ZB = SWEEP_ZB, class Sink>
__device__ __forceinline__ bool sweep_column(const In &in, const Out &out, const Params &P, bool split, Sink &sink,
                                             int l, int m, int k0) {
    const uint32_t plane = (uint32_t)P.nx * (uint32_t)P.ny;
    const uint32_t col = P.base + (uint32_t)m * (uint32_t)P.nx + (uint32_t)l;
    const uint32_t dxp = (l < P.nx - 1) ? 1u : (uint32_t)(1 - P.nx);
    const uint32_t dxm = (l > 0) ? (uint32_t)-1 : (uint32_t)(P.nx - 1);
    const uint32_t dyp = (m < P.ny - 1) ? (uint32_t)P.nx : (uint32_t)(-(P.ny - 1) * P.nx);
    const uint32_t dym = (m > 0) ? (uint32_t)(-P.nx) : (uint32_t)((P.ny - 1) * P.nx);
    // heads of the column k0-1 .. k0+ZB (z clamped)
    uint32_t hz[ZB + 2];
    bool all_uniform = true;
#pragma unroll
    for (int j = 0; j < ZB + 2; ++j) {
        const int kk = min(max(k0 - 1 + j, 0), P.nz - 1);
        hz[j] = __ldg(in.head + (uint32_t)kk * plane + col);
    }
#pragma unroll
    for (int j = 0; j < ZB; ++j) {
        const int k = k0 + j;
        if (k >= P.nz) break;
        const uint32_t c = (uint32_t)k * plane + col;
        const uint32_t h0 = hz[j + 1];
        // neighbour indices wrap in 32-bit cell-index arithmetic; the offsets
        // must be added to the index, never to the pointer
        const uint32_t qxp = c + dxp, qxm = c + dxm, qyp = c + dyp, qym = c + dym;
        uint32_t hn[6] = {__ldg(in.head + qxp), __ldg(in.head + qxm), __ldg(in.head + qyp),
                          __ldg(in.head + qym), hz[j + 2], hz[j]};
        // a z neighbour beyond the domain is the cell itself (clamped index)
        if (k == P.nz - 1) hn[4] = h0;
        if (k == 0) hn[5] = h0;
        all_uniform = sweep_cell(out, P, split, sink, j, c, h0, hn) && all_uniform;
    }
    return all_uniform;
}

// The same sweep reading the heads from a shared-memory tile: the block's
// 32 x by x ZB cells plus a one-cell halo, staged by the Tensor Memory
// Accelerator (TMA_X columns from l0 - 4, by + 2 rows from m0 - 1, ZB + 2
// layers from k0 - 1; the periodic x and y halos patched in after the copy).
constexpr int TMA_X = 40;

template <int ZB, class Sink>
__device__ __forceinline__ bool sweep_column_tile(const uint32_t *tile, int rows, const Out &out, const Params &P,
                                                  bool split, Sink &sink, int l, int m, int k0, int l0, int m0) {
    const uint32_t plane = (uint32_t)P.nx * (uint32_t)P.ny;
    const uint32_t col = (uint32_t)m * (uint32_t)P.nx + (uint32_t)l;
    const int xi = l - l0 + 4, yi = m - m0 + 1;
    auto at = [&](int x, int y, int z) { return tile[(z * rows + y) * TMA_X + x]; };
    bool all_uniform = true;
#pragma unroll
    for (int j = 0; j < ZB; ++j) {
        const int k = k0 + j;
        if (k >= P.nz) break;
        const int zi = j + 1;
        const uint32_t c = (uint32_t)k * plane + col;
        const uint32_t h0 = at(xi, yi, zi);
        uint32_t hn[6] = {at(xi + 1, yi, zi), at(xi - 1, yi, zi), at(xi, yi + 1, zi),
                          at(xi, yi - 1, zi), at(xi, yi, zi + 1), at(xi, yi, zi - 1)};
        if (k == P.nz - 1) hn[4] = h0;
        if (k == 0) hn[5] = h0;
        all_uniform = sweep_cell(out, P, split, sink, j, c, h0, hn) && all_uniform;
    }
    return all_uniform;
}

// Quiet tiles.  A tile is the 32 x 1 x ZB cells one warp of the sweep
// covers.  When every cell of a tile is uniform in step n, step n leaves the
// tile unchanged (S(n+1) = S(n) there).  If the tile and its 6 face
// neighbours were all uniform in step n-1, the neighbourhoods of the tile's
// cells are unchanged in step n, so the tile is uniform again, and its
// content in the output buffer -- written by step n-2, i.e. S(n-1) -- already
// equals S(n+1): the warp writes nothing and queues nothing.  flags[2][tiles]
// (one byte per tile, uniform = 1) alternate with the step parity; both
// halves must be zero after the state buffers are written from outside the
// step (the first step then visits every tile).
struct Tiles {
    uint8_t *__restrict__ flags;
    int ntx, nkb;
    uint32_t n;  // tiles per parity half
};

template <int ZB>
__host__ __device__ __forceinline__ uint32_t tiles_of(int nx, int ny, int nz) {
    return (uint32_t)((nz + ZB - 1) / ZB) * (uint32_t)ny * (uint32_t)((nx + 31) / 32);
}

// One thread of the sweep advances the device step clock (Params::clock):
// the step's T_melt + cooling for the work-list kernels, the next index.
__device__ __forceinline__ void advance_clock(const Params &P) {
    if (!P.clock) return;
    const int64_t s = P.clock->step[P.parity];
    P.clock->tmc[P.parity] = __dadd_rn(P.clock_T_melt, __dmul_rn((double)s, P.clock_rate));
    P.clock->step[P.parity ^ 1] = s + 1;
}

// 40 registers (3 blocks of 512 per SM): more resident warps beat keeping
// ZB = 8 columns in registers; the tuner then prefers ZB = 4
template <int S, int AMAX, int ZB = SWEEP_ZB>
__global__ void __launch_bounds__(512, 3) sweep_kernel(In in, Out out, Mats M, Params P, Queue Q, int parity,
                                                    Tiles T, int32_t *__restrict__ err) {
    __shared__ uint32_t s_cnt[3], s_base[3];
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y * blockDim.y + threadIdx.y;
    const int k0 = (blockIdx.z * blockDim.z + threadIdx.z) * ZB;
    const int tlin = threadIdx.x + (int)blockDim.x * threadIdx.y;  // blockDim.z is 1
    if (tlin < 3) s_cnt[tlin] = 0;
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tlin == 3 && threadIdx.z == 0) advance_clock(P);
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x < 2 && threadIdx.y == 0 &&
        threadIdx.z == 0)
        Q.count[2 * (parity ^ 1) + threadIdx.x] = 0;  // the previous step's kernels are done with them
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 2 && threadIdx.y == 0 &&
        threadIdx.z == 0 && Q.split)
        Q.count[4 + (parity ^ 1)] = 0;
    __syncthreads();
    BlockSink<ZB> sink(s_cnt);
    // a warp is one threadIdx.y row: its 32 lanes share m and k0, so every
    // branch below is warp-uniform except l < nx
    if (m < P.ny && k0 < P.nz) {
        if (!T.flags) {
            if (l < P.nx) sweep_column<ZB>(in, out, P, Q.split, sink, l, m, k0);
        } else {
            const int tx = (int)blockIdx.x, kb = k0 / ZB;
            const uint8_t *fin = T.flags + (size_t)(parity ^ 1) * T.n;
            uint8_t *fout = T.flags + (size_t)parity * T.n;
            auto tid = [&](int a, int b, int c) {
                return ((uint32_t)c * (uint32_t)P.ny + (uint32_t)b) * (uint32_t)T.ntx + a;
            };
            const uint32_t t = tid(tx, m, kb);
            // the 7 flags are loaded together (no short-circuit chain of loads)
            const uint32_t f0 = fin[t];
            const uint32_t f1 = fin[tid(tx + 1 < T.ntx ? tx + 1 : 0, m, kb)];
            const uint32_t f2 = fin[tid(tx > 0 ? tx - 1 : T.ntx - 1, m, kb)];
            const uint32_t f3 = fin[tid(tx, m + 1 < P.ny ? m + 1 : 0, kb)];
            const uint32_t f4 = fin[tid(tx, m > 0 ? m - 1 : P.ny - 1, kb)];
            const uint32_t f5 = fin[tid(tx, m, kb + 1 < T.nkb ? kb + 1 : kb)];
            const uint32_t f6 = fin[tid(tx, m, kb > 0 ? kb - 1 : kb)];
            const bool quiet = (f0 & f1 & f2 & f3 & f4 & f5 & f6) != 0u;
            const bool lane0 = (threadIdx.x & 31) == 0;
            if (quiet) {
                if (lane0) fout[t] = 1;
            } else {
                const bool uni = l < P.nx ? sweep_column<ZB>(in, out, P, Q.split, sink, l, m, k0) : true;
                const bool all = __all_sync(0xffffffffu, uni);
                if (lane0) fout[t] = all ? 1 : 0;
            }
        }
    }
    __syncthreads();
    if (tlin < 3) {
        const uint32_t n = s_cnt[tlin];
        uint32_t *ctr = tlin == 2 ? Q.count + 4 + parity : Q.count + 2 * parity + tlin;
        s_base[tlin] = n ? atomicAdd(ctr, n) : 0u;
    }
    __syncthreads();
    if (l < P.nx && m < P.ny && k0 < P.nz)
        sink.flush(Q, P.cells32, s_base, (uint32_t)P.nx * (uint32_t)P.ny,
                   P.base + (uint32_t)m * (uint32_t)P.nx + (uint32_t)l, k0);
}

// Bounded wait on phase `parity` of a shared-memory mbarrier (nanoseconds
// of %globaltimer); false if it did not complete in time.
__device__ __forceinline__ bool mbar_wait_ns(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    uint64_t t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        uint64_t t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit_ns) return false;
    }
}

// Kernel 1 with its heads staged in shared memory by one TMA copy per block
// (cp.async.bulk.tensor.3d of the block's cells plus a one-cell halo from
// the head array, which the tensor map describes as nx x ny x nz uint32).
// Blocks whose warps are all quiet copy nothing.  The x and y halos at the
// domain's periodic edges lie outside the copied box (TMA fills them with
// zeros) and are patched in with plain loads; z halo layers outside the
// domain are never read (the clamped neighbour is the cell itself).  A copy
// that does not land within 1 s sets MPF3D_DEV_STAGING_TIMEOUT and the block
// waits once more before it leaves.  Same results as sweep_kernel.
template <int S, int AMAX, int ZB>
__global__ void __launch_bounds__(512, 3) sweep_kernel_tma(const __grid_constant__ CUtensorMap map, In in, Out out,
                                                         Params P, Queue Q, int parity, Tiles T,
                                                         int32_t *__restrict__ err) {
    constexpr int MAX_ROWS = 16 + 2;
    __shared__ __align__(128) uint32_t tile[TMA_X * MAX_ROWS * (ZB + 2)];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_cnt[3], s_base[3];
    __shared__ int s_need;
    const int by = (int)blockDim.y, rows = by + 2;
    const int l0 = blockIdx.x * 32, m0 = blockIdx.y * by;
    const int l = l0 + threadIdx.x, m = m0 + threadIdx.y;
    const int k0 = blockIdx.z * ZB;
    const int tlin = threadIdx.x + 32 * threadIdx.y;
    const uint32_t bar_a = (uint32_t)__cvta_generic_to_shared(&bar);
    if (tlin < 3) s_cnt[tlin] = 0;
    if (tlin == 0) {
        s_need = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.y == 0 && threadIdx.x < 2)
        Q.count[2 * (parity ^ 1) + threadIdx.x] = 0;  // the previous step's kernels are done with them
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.y == 0 && threadIdx.x == 2 && Q.split)
        Q.count[4 + (parity ^ 1)] = 0;
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.y == 0 && threadIdx.x == 3)
        advance_clock(P);
    // quiet flags of this warp's tile (as sweep_kernel)
    const bool row_ok = m < P.ny && k0 < P.nz;
    bool quiet = false;
    uint32_t t = 0;
    const uint8_t *fin = nullptr;
    uint8_t *fout = nullptr;
    if (row_ok && T.flags) {
        const int tx = (int)blockIdx.x, kb = k0 / ZB;
        fin = T.flags + (size_t)(parity ^ 1) * T.n;
        fout = T.flags + (size_t)parity * T.n;
        auto tid = [&](int a, int b, int c) {
            return ((uint32_t)c * (uint32_t)P.ny + (uint32_t)b) * (uint32_t)T.ntx + a;
        };
        t = tid(tx, m, kb);
        const uint32_t f0 = fin[t];
        const uint32_t f1 = fin[tid(tx + 1 < T.ntx ? tx + 1 : 0, m, kb)];
        const uint32_t f2 = fin[tid(tx > 0 ? tx - 1 : T.ntx - 1, m, kb)];
        const uint32_t f3 = fin[tid(tx, m + 1 < P.ny ? m + 1 : 0, kb)];
        const uint32_t f4 = fin[tid(tx, m > 0 ? m - 1 : P.ny - 1, kb)];
        const uint32_t f5 = fin[tid(tx, m, kb + 1 < T.nkb ? kb + 1 : kb)];
        const uint32_t f6 = fin[tid(tx, m, kb > 0 ? kb - 1 : kb)];
        quiet = (f0 & f1 & f2 & f3 & f4 & f5 & f6) != 0u;
    }
    __syncthreads();
    if (row_ok && !quiet && threadIdx.x == 0) s_need = 1;
    __syncthreads();
    const bool need = s_need != 0;
    bool staged = false;
    if (need) {
        if (tlin == 0) {
            const uint32_t bytes = (uint32_t)(TMA_X * rows * (ZB + 2) * 4);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar_a), "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
                "[%5];\n" ::"r"((uint32_t)__cvta_generic_to_shared(tile)),
                "l"(reinterpret_cast<uint64_t>(&map)), "r"(l0 - 4), "r"(m0 - 1), "r"(k0 - 1), "r"(bar_a)
                : "memory");
        }
        staged = mbar_wait_ns(bar_a, 0, 1000000000ull);
        if (!staged) {
            if (threadIdx.x == 0) atomicOr(err, MPF3D_DEV_STAGING_TIMEOUT);
            mbar_wait_ns(bar_a, 0, 1000000000ull);  // the copy may still land: let it, before leaving
        }
        staged = __syncthreads_and(staged) != 0;
        if (staged) {
            // periodic halos outside the copied box
            const uint32_t plane = (uint32_t)P.nx * (uint32_t)P.ny;
            const int nz_box = ZB + 2;
            if (l0 == 0 || l0 + 32 >= P.nx) {
                for (int e = tlin; e < 2 * rows * nz_box; e += 32 * by) {
                    const int side = e / (rows * nz_box), r = e % (rows * nz_box);
                    const int yi = r % rows, zi = r / rows;
                    const int gy = m0 - 1 + yi, gz = k0 - 1 + zi;
                    if (gy < 0 || gy >= P.ny || gz < 0 || gz >= P.nz) continue;
                    if (side == 0 && l0 == 0)
                        tile[(zi * rows + yi) * TMA_X + 3] = __ldg(in.head + (uint32_t)gz * plane + (uint32_t)gy * P.nx + (P.nx - 1));
                    if (side == 1 && l0 + 32 >= P.nx)
                        tile[(zi * rows + yi) * TMA_X + (P.nx - l0 + 4)] = __ldg(in.head + (uint32_t)gz * plane + (uint32_t)gy * P.nx);
                }
            }
            if (m0 == 0 || m0 + by >= P.ny) {
                for (int e = tlin; e < 2 * 32 * nz_box; e += 32 * by) {
                    const int side = e / (32 * nz_box), r = e % (32 * nz_box);
                    const int xo = r % 32, zi = r / 32;
                    const int gx = l0 + xo, gz = k0 - 1 + zi;
                    if (gx >= P.nx || gz < 0 || gz >= P.nz) continue;
                    if (side == 0 && m0 == 0)
                        tile[(zi * rows + 0) * TMA_X + xo + 4] = __ldg(in.head + (uint32_t)gz * plane + (uint32_t)(P.ny - 1) * P.nx + gx);
                    if (side == 1 && m0 + by >= P.ny)
                        tile[(zi * rows + (P.ny - m0 + 1)) * TMA_X + xo + 4] = __ldg(in.head + (uint32_t)gz * plane + gx);
                }
            }
            __syncthreads();
        }
    }
    BlockSink<ZB> sink(s_cnt);
    if (row_ok && staged) {
        if (!T.flags) {
            if (l < P.nx) sweep_column_tile<ZB>(tile, rows, out, P, Q.split, sink, l, m, k0, l0, m0);
        } else if (quiet) {
            if (threadIdx.x == 0) fout[t] = 1;
        } else {
            const bool uni = l < P.nx ? sweep_column_tile<ZB>(tile, rows, out, P, Q.split, sink, l, m, k0, l0, m0)
                                      : true;
            const bool all = __all_sync(0xffffffffu, uni);
            if (threadIdx.x == 0) fout[t] = all ? 1 : 0;
        }
    } else if (row_ok && quiet && threadIdx.x == 0) {
        fout[t] = 1;
    }
    __syncthreads();
    if (tlin < 3) {
        const uint32_t n = s_cnt[tlin];
        uint32_t *ctr = tlin == 2 ? Q.count + 4 + parity : Q.count + 2 * parity + tlin;
        s_base[tlin] = n ? atomicAdd(ctr, n) : 0u;
    }
    __syncthreads();
    if (l < P.nx && m < P.ny && k0 < P.nz)
        sink.flush(Q, P.cells32, s_base, (uint32_t)P.nx * (uint32_t)P.ny, (uint32_t)m * (uint32_t)P.nx + (uint32_t)l,
                   k0);
}

// Kernel 2 of a step: the cells queued for the general update, one thread
// per cell.  Capped at 48 registers (5 blocks of 256 per SM): it waits on
// memory, and more resident warps beat the few spilled values.
template <int S, int AMAX>
__global__ void __launch_bounds__(256, 5) general_kernel(In in, Out out, Mats M, Params P, Queue Q, int parity,
                                                     int32_t *__restrict__ err) {
    const uint32_t n = *(volatile uint32_t *)(Q.count + 2 * parity);
    const uint32_t plane = (uint32_t)P.nx * (uint32_t)P.ny;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = Q.items[i];
        const int k = (int)(c / plane);
        const uint32_t r = c - (uint32_t)k * plane;
        const int m = (int)(r / (uint32_t)P.nx);
        const int l = (int)(r - (uint32_t)m * (uint32_t)P.nx);
        process_cell<S, AMAX, false>(in, out, M, P, err, l, m, k);
    }
}

// Kernel 3 of a step: the queued solid-liquid interface cells, one thread
// per cell, all lanes of a warp on the same (heavy) path; NT normals per
// grain (4 or 8, from P.sym_normals).
template <int S, int AMAX, int NT>
__global__ void __launch_bounds__(128, 5) interface_kernel(In in, Out out, Mats M, Params P, Queue Q, int parity,
                                                           int32_t *__restrict__ err) {
    const uint32_t na = *(volatile uint32_t *)(Q.count + 2 * parity + 1);
    const uint32_t n = na + (Q.split ? *(volatile uint32_t *)(Q.count + 4 + parity) : 0u);
    const uint32_t plane = (uint32_t)P.nx * (uint32_t)P.ny;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = i < na ? Q.items[P.cells32 - 1u - i] : Q.items[P.cells32 + (i - na)];
        const int k = (int)(c / plane);
        const uint32_t r = c - (uint32_t)k * plane;
        const int m = (int)(r / (uint32_t)P.nx);
        const int l = (int)(r - (uint32_t)m * (uint32_t)P.nx);
        process_cell<S, AMAX, true, NT>(in, out, M, P, err, l, m, k);
    }
}

// ---------------------------------------------------------------------------
// dense [N][nx][ny][nz] (z fastest) -> compact (x fastest)
template <typename T, int S>
__global__ void from_dense_kernel(const T *__restrict__ phi, int N, int nx, int ny, int nz, Out out,
                                  int32_t *__restrict__ err) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y * blockDim.y + threadIdx.y;
    const int l = blockIdx.z * blockDim.z + threadIdx.z;
    if (k >= nz || m >= ny || l >= nx) return;
    const int64_t plane = (int64_t)nx * ny * nz;
    const int64_t src = ((int64_t)l * ny + m) * nz + k;
    const int64_t cells = plane;
    const int64_t dst = ((int64_t)k * ny + m) * nx + l;
    int c = 0, id0 = 0;
    float v0 = 0.0f;
    bool bad = false, ovf = false;
    for (int g = 0; g < N; ++g) {
        const T v = phi[(int64_t)g * plane + src];
        if (!(v >= (T)0)) { bad = true; continue; }
        if (v > (T)0) {
            if (c < S) {
                if (c == 0) { id0 = g; v0 = (float)v; }
                else out.idx[c * cells + dst] = (uint16_t)g;
                out.val[c * cells + dst] = (float)v;
            } else {
                ovf = true;
            }
            ++c;
        }
    }
    const int n = c < S ? c : S;
    out.head[dst] = mkhead(id0, n, n == 1 && v0 != 1.0f);
    if (bad) atomicOr(err, MPF3D_DEV_BAD_INPUT);
    if (ovf) atomicOr(err, MPF3D_DEV_SLOT_OVERFLOW);
}

template <typename T, int S>
__global__ void to_dense_kernel(In in, int N, int nx, int ny, int nz, uint32_t stride, uint32_t base,
                                T *__restrict__ phi) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y * blockDim.y + threadIdx.y;
    const int l = blockIdx.z * blockDim.z + threadIdx.z;
    if (k >= nz || m >= ny || l >= nx) return;
    const int64_t plane = (int64_t)nx * ny * nz;
    const int64_t dstc = ((int64_t)l * ny + m) * nz + k;
    const uint32_t srcc = base + ((uint32_t)k * (uint32_t)ny + (uint32_t)m) * (uint32_t)nx + (uint32_t)l;
    for (int g = 0; g < N; ++g) phi[(int64_t)g * plane + dstc] = (T)0;
    const uint32_t h = in.head[srcc];
    const int c = min(hcount(h), S);
    for (int s = 0; s < c; ++s) {
        const int g = s == 0 ? hid0(h) : (int)in.idx[(size_t)s * stride + srcc];
        const float v = s == 0 ? value0(in, h, srcc) : in.val[(size_t)s * stride + srcc];
        if (g < N) phi[(int64_t)g * plane + dstc] = (T)v;
    }
}

// number of active phases per cell (the APT's nf), dense z-fastest output
template <int S>
__global__ void active_count_kernel(In in, int nx, int ny, int nz, int32_t *__restrict__ nf) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y * blockDim.y + threadIdx.y;
    const int l = blockIdx.z * blockDim.z + threadIdx.z;
    if (k >= nz || m >= ny || l >= nx) return;
    nf[((int64_t)l * ny + m) * nz + k] = active_count_at<S>(in, nx, ny, nz, l, m, k);
}

// ---------------------------------------------------------------------------
// Batches of independent domains ("instances") sharing one set of state
// arrays: instance i owns cells [offset, offset + nx*ny*nz) of every array.
// One launch of each step kernel covers all instances; tiles and queued
// cells find their instance by binary search over the instance table.

__device__ __forceinline__ int find_instance_by_tile(const mpf3d_instance *__restrict__ inst, int n, int tile) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&inst[mid].tile_start) <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int find_instance_by_cell(const mpf3d_instance *__restrict__ inst, int n, uint32_t c) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&inst[mid].offset) <= c) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ Params instance_params(const Params &P0, const mpf3d_instance &I) {
    Params P = P0;
    P.nx = I.nx; P.ny = I.ny; P.nz = I.nz;
    P.base = I.offset;
    P.n111_base = I.n111_base;
    P.delta_a = I.delta_a;
    P.mu_da = I.mu_da;
    P.e2_flat = I.e2_flat;
    P.t_uniform = 1;
    P.dT_uniform = -I.undercooling;
    return P;
}

// The batched sweep.  One block is one 32 x 8 x SWEEP_ZB tile of one
// instance, and each of its 8 warps one 32 x 1 x SWEEP_ZB warp tile, whose
// index is blockIdx.x * 8 + threadIdx.y.  With `flags` (2 x 8 x n_tiles
// bytes, halves alternating with the step parity; NULL: every tile visited)
// a warp tile that was uniform in the previous step together with its 6 face
// neighbours in the same instance (periodic x and y, clamped z) is quiet and
// skipped, by the argument of the single-domain sweep's quiet tiles.
template <int S, int AMAX>
__global__ void __launch_bounds__(256) batched_sweep_kernel(In in, Out out, Params P0,
                                                            const mpf3d_instance *__restrict__ inst, int n_inst,
                                                            Queue Q, int parity, uint8_t *__restrict__ flags) {
    __shared__ uint32_t s_cnt[3], s_base[3];
    const int tlin = threadIdx.x + 32 * threadIdx.y;
    if (tlin < 3) s_cnt[tlin] = 0;
    if (blockIdx.x == 0 && threadIdx.x < 2 && threadIdx.y == 0) Q.count[2 * (parity ^ 1) + threadIdx.x] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 2 && threadIdx.y == 0 && Q.split) Q.count[4 + (parity ^ 1)] = 0;
    __syncthreads();
    // one block is one tile of one instance
    const int i = find_instance_by_tile(inst, n_inst, (int)blockIdx.x);
    const mpf3d_instance I = inst[i];
    const int t = (int)blockIdx.x - I.tile_start;
    const int tx = (I.nx + 31) / 32, ty = (I.ny + 7) / 8, tz = (I.nz + SWEEP_ZB - 1) / SWEEP_ZB;
    const int bx = t % tx, kb = t / (tx * ty);
    const int l = bx * 32 + threadIdx.x;
    const int m = ((t / tx) % ty) * 8 + threadIdx.y;
    const int k0 = kb * SWEEP_ZB;
    const bool row_in = m < I.ny && k0 < I.nz;  // the same for the 32 lanes of a warp
    const bool inside = l < I.nx && row_in;
    const Params P = instance_params(P0, I);
    BlockSink<SWEEP_ZB> sink(s_cnt);
    if (!flags) {
        if (inside) sweep_column(in, out, P, Q.split, sink, l, m, k0);
    } else {
        const uint32_t nw = gridDim.x * 8u;
        const uint8_t *fin = flags + (size_t)(parity ^ 1) * nw;
        uint8_t *fout = flags + (size_t)parity * nw;
        const uint32_t w = blockIdx.x * 8u + threadIdx.y;
        const bool lane0 = threadIdx.x == 0;
        if (!row_in) {
            if (lane0) fout[w] = 1;
        } else {
            // warp tile (x tile a, row mm, z tile c) of this instance
            auto wt = [&](int a, int mm, int c) {
                return (uint32_t)(I.tile_start + (c * ty + mm / 8) * tx + a) * 8u + (uint32_t)(mm % 8);
            };
            // the 7 flags are loaded together (no short-circuit chain of loads)
            const uint32_t f0 = fin[w];
            const uint32_t f1 = fin[wt(bx + 1 < tx ? bx + 1 : 0, m, kb)];
            const uint32_t f2 = fin[wt(bx > 0 ? bx - 1 : tx - 1, m, kb)];
            const uint32_t f3 = fin[wt(bx, m + 1 < I.ny ? m + 1 : 0, kb)];
            const uint32_t f4 = fin[wt(bx, m > 0 ? m - 1 : I.ny - 1, kb)];
            const uint32_t f5 = fin[wt(bx, m, kb + 1 < tz ? kb + 1 : kb)];
            const uint32_t f6 = fin[wt(bx, m, kb > 0 ? kb - 1 : kb)];
            if ((f0 & f1 & f2 & f3 & f4 & f5 & f6) != 0u) {
                if (lane0) fout[w] = 1;
            } else {
                const bool uni = l < I.nx ? sweep_column(in, out, P, Q.split, sink, l, m, k0) : true;
                const bool all = __all_sync(0xffffffffu, uni);
                if (lane0) fout[w] = all ? 1 : 0;
            }
        }
    }
    __syncthreads();
    if (tlin < 3) {
        const uint32_t n = s_cnt[tlin];
        uint32_t *ctr = tlin == 2 ? Q.count + 4 + parity : Q.count + 2 * parity + tlin;
        s_base[tlin] = n ? atomicAdd(ctr, n) : 0u;
    }
    __syncthreads();
    if (inside)
        sink.flush(Q, P.cells32, s_base, (uint32_t)P.nx * (uint32_t)P.ny,
                   P.base + (uint32_t)m * (uint32_t)P.nx + (uint32_t)l, k0);
}

template <int S, int AMAX, bool HEAVY, int NT = 4>
__global__ void __launch_bounds__(HEAVY ? 128 : 256) batched_queue_kernel(In in, Out out, Mats M, Params P0,
                                                                          const mpf3d_instance *__restrict__ inst,
                                                                          int n_inst, Queue Q, int parity,
                                                                          int32_t *__restrict__ err) {
    const uint32_t na = *(volatile uint32_t *)(Q.count + 2 * parity + (HEAVY ? 1 : 0));
    const uint32_t n = na + ((HEAVY && Q.split) ? *(volatile uint32_t *)(Q.count + 4 + parity) : 0u);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = !HEAVY ? Q.items[i] : (i < na ? Q.items[P0.cells32 - 1u - i] : Q.items[P0.cells32 + (i - na)]);
        const mpf3d_instance I = inst[find_instance_by_cell(inst, n_inst, c)];
        const Params P = instance_params(P0, I);
        const uint32_t r0 = c - I.offset;
        const uint32_t plane = (uint32_t)I.nx * (uint32_t)I.ny;
        const int k = (int)(r0 / plane);
        const uint32_t r = r0 - (uint32_t)k * plane;
        const int m = (int)(r / (uint32_t)I.nx);
        const int l = (int)(r - (uint32_t)m * (uint32_t)I.nx);
        process_cell<S, AMAX, HEAVY, NT>(in, out, M, P, err, l, m, k);
    }
}

// Initial bicrystal: a solid base of height base_height (tanh profile
// 0.5*(1 - tanh(2.2/delta*(k - h)*dz)), as src/seed_modes_3d.py:46-56), grain
// 1 for x < split and grain 2 for x >= split, liquid = clip(1 - solid).
__global__ void batched_init_bicrystal_kernel(Out out, const mpf3d_instance *__restrict__ inst, int n_inst,
                                              uint32_t stride, float factor_dz, int32_t *__restrict__ err) {
    const int i = blockIdx.y;
    if (i >= n_inst) return;
    const mpf3d_instance I = inst[i];
    const uint32_t cells = (uint32_t)I.nx * I.ny * I.nz;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < cells; r += gridDim.x * blockDim.x) {
        const uint32_t plane = (uint32_t)I.nx * I.ny;
        const int k = (int)(r / plane);
        const int l = (int)((r - (uint32_t)k * plane) % (uint32_t)I.nx);
        const float s = (float)(0.5 * (1.0 - tanh((double)factor_dz * ((double)k - (double)I.base_height))));
        const float liq = fminf(fmaxf(1.0f - s, 0.0f), 1.0f);
        const int g = l < I.split ? 1 : 2;
        const uint32_t c = I.offset + r;
        int n = 0, id0 = 0;
        float v0 = 0.0f;
        if (liq > 0.0f) { id0 = LIQ; v0 = liq; out.val[c] = liq; n = 1; }
        if (s > 0.0f) {
            if (n == 0) { id0 = g; v0 = s; out.val[c] = s; }
            else { out.idx[(size_t)stride + c] = (uint16_t)g; out.val[(size_t)stride + c] = s; }
            ++n;
        }
        out.head[c] = mkhead(id0, n, n == 1 && v0 != 1.0f);
    }
}

// Per instance: mean front height of each grain half (highest z with solid
// fraction > 0.5 per column, interface_positions_3d of
// tests/verification_3d.py:409-416) and the total fraction of grains 1, 2.
// acc[6*i + ...] = {sum h left, columns left, sum h right, columns right, V1, V2}
template <int S>
__global__ void batched_fronts_kernel(In in, const mpf3d_instance *__restrict__ inst, int n_inst, uint32_t stride,
                                      double *__restrict__ acc) {
    const int i = blockIdx.y;
    const mpf3d_instance I = inst[i];
    const int cols = I.nx * I.ny;
    const uint32_t plane = (uint32_t)cols;
    double hl = 0.0, nl = 0.0, hr = 0.0, nr = 0.0, v1 = 0.0, v2 = 0.0;
    for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < cols; col += gridDim.x * blockDim.x) {
        const int l = col % I.nx;
        int front = -1;
        for (int k = I.nz - 1; k >= 0; --k) {
            const uint32_t c = I.offset + (uint32_t)k * plane + (uint32_t)col;
            const float solid = 1.0f - phase_at<S>(in, stride, c, LIQ);
            if (front < 0 && solid > 0.5f) front = k;
            v1 += phase_at<S>(in, stride, c, 1);
            v2 += phase_at<S>(in, stride, c, 2);
        }
        if (front >= 0) {
            if (l < I.split) { hl += front; nl += 1.0; }
            else { hr += front; nr += 1.0; }
        }
    }
    double vals[6] = {hl, nl, hr, nr, v1, v2};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        double v = vals[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(acc + 6 * i + q, v);
    }
}

// Per instance and z row: the phi1 = phi2 crossing along x nearest the
// initial split, averaged over y, for rows whose solid fraction is >= 0.15
// (the grain-boundary locator of measure_gb_inclination,
// tests/run_paper_verification.py:658-723, with a linear root between the
// two cells of the sign change).  gb[2*(row_base + k) + {0,1}] = {sum x, rows}.
template <int S>
__global__ void batched_gb_rows_kernel(In in, const mpf3d_instance *__restrict__ inst, int n_inst, uint32_t stride,
                                       const int *__restrict__ row_base, double *__restrict__ gb) {
    const int i = blockIdx.y;
    const mpf3d_instance I = inst[i];
    const int rows = I.ny * I.nz;
    const uint32_t plane = (uint32_t)I.nx * I.ny;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const int m = r % I.ny, k = r / I.ny;
        const uint32_t row0 = I.offset + (uint32_t)k * plane + (uint32_t)m * I.nx;
        float solid = 0.0f, best_x = 0.0f, best_d = 1e30f;
        bool found = false;
        float dprev = phase_at<S>(in, stride, row0, 1) - phase_at<S>(in, stride, row0, 2);
        solid += 1.0f - phase_at<S>(in, stride, row0, LIQ);
        for (int l = 1; l < I.nx; ++l) {
            const uint32_t c = row0 + (uint32_t)l;
            const float d = phase_at<S>(in, stride, c, 1) - phase_at<S>(in, stride, c, 2);
            solid += 1.0f - phase_at<S>(in, stride, c, LIQ);
            if ((dprev > 0.0f && d <= 0.0f) || (dprev < 0.0f && d >= 0.0f)) {
                const float x = (float)(l - 1) + dprev / (dprev - d);
                const float dist = fabsf(x - (float)I.split);
                if (dist < best_d) { best_d = dist; best_x = x; found = true; }
            }
            dprev = d;
        }
        if (found && solid >= 0.15f * I.nx) {
            atomicAdd(gb + 2 * (row_base[i] + k), (double)best_x);
            atomicAdd(gb + 2 * (row_base[i] + k) + 1, 1.0);
        }
    }
}


// Initial state from a grain-owner map and a z profile: owner[k][m][l]
// (x fastest) holds the grain of the first `slab` layers; rows above the slab
// repeat the top layer.  The grain holds prof[k], the liquid
// clip(1 - prof[k], 0, 1) (init_phi_from_grain_map_3d,
// src/seed_modes_3d.py:38-57, with a 3-D owner map).
__global__ void init_owner_kernel(Out out, const int32_t *__restrict__ owner, int slab, const float *__restrict__ prof,
                                  int nx, int ny, int nz, uint32_t cells) {
    const uint32_t plane = (uint32_t)nx * (uint32_t)ny;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += gridDim.x * blockDim.x) {
        const int k = (int)(c / plane);
        const uint32_t col = c - (uint32_t)k * plane;
        const int g = owner[(uint32_t)min(k, slab - 1) * plane + col];
        const float s = prof[k];
        const float liq = fminf(fmaxf(1.0f - s, 0.0f), 1.0f);
        int n = 0, id0 = 0;
        float v0 = 0.0f;
        if (liq > 0.0f) { id0 = LIQ; v0 = liq; out.val[c] = liq; n = 1; }
        if (s > 0.0f) {
            if (n == 0) { id0 = g; v0 = s; out.val[c] = s; }
            else { out.idx[(size_t)cells + c] = (uint16_t)g; out.val[(size_t)cells + c] = s; }
            ++n;
        }
        out.head[c] = mkhead(id0, n, n == 1 && v0 != 1.0f);
    }
}

}  // namespace compact
}  // namespace mpf3d

using namespace mpf3d;
using namespace mpf3d::compact;

namespace {

dim3 zfast_grid(int nx, int ny, int nz, dim3 b) {
    return dim3((nz + b.x - 1) / b.x, (ny + b.y - 1) / b.y, (nx + b.z - 1) / b.z);
}


// A second stream of one device, on which the interface kernel runs beside
// the general kernel.  The two read only what the sweep wrote and write
// disjoint cells; both are latency-bound, so running them side by side
// fills each other's idle issue slots.  Created on first use outside a
// stream capture; the fork/join is enqueued under the mutex so that callers
// on other host threads cannot interleave their event records with it.
// The second stream of a step and its fork/join events, one set per
// (device, caller stream): steps that callers issue on independent streams
// stay independent of each other.
struct SideStream {
    bool ready = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

struct SideTable {
    std::mutex mu;
    std::unordered_map<cudaStream_t, SideStream> by_caller;  // element references survive rehashing
};

SideTable &side_table_of(int dev) {
    static SideTable all[64];
    return all[dev & 63];
}

// Creates the side stream and its events once, outside any capture of s.
bool side_ready(SideStream &side, cudaStream_t s) {
    if (!side.ready) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone &&
            cudaStreamCreateWithFlags(&side.stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&side.fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&side.join, cudaEventDisableTiming) == cudaSuccess)
            side.ready = true;
    }
    return side.ready;
}

// general(stream) and interface(stream) launch the two work-list kernels of
// a step; with `both`, the interface kernel goes to the caller stream's side stream,
// forked from s after the sweep and joined back before s continues.
template <class General, class Interface>
void launch_side_by_side(cudaStream_t s, bool both, General &&general, Interface &&interface) {
    if (!both) {
        general(s);
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    SideTable &tab = side_table_of(dev);
    std::lock_guard<std::mutex> lock(tab.mu);
    SideStream &side = tab.by_caller[s];
    if (!side_ready(side, s)) {  // first call inside a capture: both kernels on the caller's stream
        general(s);
        interface(s);
        return;
    }
    cudaEventRecord(side.fork, s);
    cudaStreamWaitEvent(side.stream, side.fork, 0);
    interface(side.stream);
    general(s);
    cudaEventRecord(side.join, side.stream);
    cudaStreamWaitEvent(s, side.join, 0);  // the caller's stream sees the whole step
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
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

// Tensor map of a head array (uint32 nx x ny x nz, x fastest) with boxes of
// TMA_X x (by + 2) x (zb + 2); out-of-range elements read as zero.  Needs
// nx a multiple of 4 (16-byte row pitch) and a 16-byte aligned base.
bool head_map(CUtensorMap *map, const uint32_t *head, int nx, int ny, int nz, int by, int zb) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
    if (!fn || nx % 4 != 0 || ((uintptr_t)head & 15u) != 0) return false;
    cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    cuuint32_t box[3] = {(cuuint32_t)TMA_X, (cuuint32_t)(by + 2), (cuuint32_t)(zb + 2)};
    cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint32_t *>(head), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int S, int AMAX>
void launch_step(const In &in, const Out &out, const Mats &M, const Params &P, const Queue &Q, int parity,
                 uint8_t *tile_flags, int32_t *err, cudaStream_t s, const mpf3d_tuning &T, bool sweep_tma) {
    const int by = T.sweep_by;
    dim3 blk(32, by, 1);
    CUtensorMap map;
    const bool tma = sweep_tma && P.base == 0 && head_map(&map, in.head, P.nx, P.ny, P.nz, by, T.sweep_zb);
#define SWEEP_LAUNCH(ZB)                                                                                           \
    do {                                                                                                           \
        const dim3 grid((P.nx + 31) / 32, (P.ny + by - 1) / by, (P.nz + ZB - 1) / ZB);                             \
        const Tiles tl{tile_flags, (P.nx + 31) / 32, (P.nz + ZB - 1) / ZB, tiles_of<ZB>(P.nx, P.ny, P.nz)};       \
        if (tma) sweep_kernel_tma<S, AMAX, ZB><<<grid, blk, 0, s>>>(map, in, out, P, Q, parity, tl, err);          \
        else sweep_kernel<S, AMAX, ZB><<<grid, blk, 0, s>>>(in, out, M, P, Q, parity, tl, err);                    \
    } while (0)
    if (T.sweep_zb == 2) SWEEP_LAUNCH(2);
    else if (T.sweep_zb == 8) SWEEP_LAUNCH(8);
    else SWEEP_LAUNCH(4);
#undef SWEEP_LAUNCH
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const dim3 g_general(sms * T.general_blocks_per_sm), g_iface(sms * T.iface_blocks_per_sm);
    launch_side_by_side(
        s, P.use_aniso,
        [&](cudaStream_t st) {
            general_kernel<S, AMAX><<<g_general, T.general_threads, 0, st>>>(in, out, M, P, Q, parity, err);
        },
        [&](cudaStream_t st) {
            if (P.sym_normals)
                interface_kernel<S, AMAX, 4><<<g_iface, T.iface_threads, 0, st>>>(in, out, M, P, Q, parity, err);
            else
                interface_kernel<S, AMAX, 8><<<g_iface, T.iface_threads, 0, st>>>(in, out, M, P, Q, parity, err);
        });
}

bool tuning_ok(const mpf3d_tuning &T) {
    return (T.sweep_zb == 2 || T.sweep_zb == 4 || T.sweep_zb == 8) &&
           (T.sweep_by == 4 || T.sweep_by == 8 || T.sweep_by == 16) && T.general_blocks_per_sm >= 1 &&
           T.general_blocks_per_sm <= 64 && (T.general_threads == 128 || T.general_threads == 256) &&
           T.iface_blocks_per_sm >= 1 && T.iface_blocks_per_sm <= 64 &&
           (T.iface_threads == 64 || T.iface_threads == 128);
}

const mpf3d_tuning kDefaultTuning = {4, 8, 8, 256, 8, 128};

}  // namespace

extern "C" int mpf3d_compact_from_dense(const void *phi, int phi_dtype, int N, int nx, int ny, int nz, int slots,
                                        uint32_t *cnt, uint16_t *idx, float *val, int32_t *err, void *stream) {
    if (!phi || !cnt || !idx || !val || !err || N <= 0 || N > 65535 || !dims_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 b(32, 4, 2);
    dim3 g = zfast_grid(nx, ny, nz, b);
    Out o{cnt, idx, val};
#define FD(T, SS) from_dense_kernel<T, SS><<<g, b, 0, s>>>((const T *)phi, N, nx, ny, nz, o, err)
    if (phi_dtype == MPF3D_F32) {
        if (slots == 4) FD(float, 4); else if (slots == 8) FD(float, 8); else if (slots == 16) FD(float, 16);
        else return MPF3D_ERR_ARG;
    } else if (phi_dtype == MPF3D_F64) {
        if (slots == 4) FD(double, 4); else if (slots == 8) FD(double, 8); else if (slots == 16) FD(double, 16);
        else return MPF3D_ERR_ARG;
    } else {
        return MPF3D_ERR_DTYPE;
    }
#undef FD
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_compact_to_dense(const uint32_t *cnt, const uint16_t *idx, const float *val, int slots, int N,
                                      int nx, int ny, int nz, void *phi, int phi_dtype, void *stream) {
    if (!phi || !cnt || !idx || !val || N <= 0 || N > 65535 || !dims_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 b(32, 4, 2);
    dim3 g = zfast_grid(nx, ny, nz, b);
    In in{cnt, idx, val};
#define TD(T, SS) to_dense_kernel<T, SS><<<g, b, 0, s>>>(in, N, nx, ny, nz, (uint32_t)((int64_t)nx * ny * nz), 0u, (T *)phi)
    if (phi_dtype == MPF3D_F32) {
        if (slots == 4) TD(float, 4); else if (slots == 8) TD(float, 8); else if (slots == 16) TD(float, 16);
        else return MPF3D_ERR_ARG;
    } else if (phi_dtype == MPF3D_F64) {
        if (slots == 4) TD(double, 4); else if (slots == 8) TD(double, 8); else if (slots == 16) TD(double, 16);
        else return MPF3D_ERR_ARG;
    } else {
        return MPF3D_ERR_DTYPE;
    }
#undef TD
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_host_device_pointer(const void *host, void **device) {
    if (!host || !device) return MPF3D_ERR_ARG;
    *device = nullptr;
    void *d = nullptr;
    if (cudaHostGetDevicePointer(&d, const_cast<void *>(host), 0) != cudaSuccess) {
        cudaGetLastError();  // not page-locked host memory: clear the error, report it
        return MPF3D_ERR_ARG;
    }
    *device = d;
    return MPF3D_OK;
}

extern "C" int mpf3d_compact_active_count(const uint32_t *cnt, const uint16_t *idx, int slots, int nx, int ny, int nz,
                                          int32_t *nf, void *stream) {
    if (!cnt || !idx || !nf || !dims_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 b(32, 4, 2);
    dim3 g = zfast_grid(nx, ny, nz, b);
    In in{cnt, idx, nullptr};
    if (slots == 4) active_count_kernel<4><<<g, b, 0, s>>>(in, nx, ny, nz, nf);
    else if (slots == 8) active_count_kernel<8><<<g, b, 0, s>>>(in, nx, ny, nz, nf);
    else if (slots == 16) active_count_kernel<16><<<g, b, 0, s>>>(in, nx, ny, nz, nf);
    else return MPF3D_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

namespace {

// physics shared by every cell of a step, from the 13 kernel scalars
Params shared_params(const mpf3d_scalars *sc, int enable_anisotropy, int enable_torque, int symmetric_normals) {
    const double *v = sc->v;
    Params P;
    memset(&P, 0, sizeof P);
    const double dx = v[MPF3D_S_DX];
    P.inv_dx2 = (float)(1.0 / (dx * dx));
    P.inv_2dx = (float)(1.0 / (2.0 * dx));
    P.half_over_dx = (float)(0.5 / dx);
    P.inv_dx = (float)(1.0 / dx);
    P.dt = (float)v[MPF3D_S_DT];
    P.eps0 = (float)v[MPF3D_S_EPS0_SL];
    P.eps0sq = (float)(v[MPF3D_S_EPS0_SL] * v[MPF3D_S_EPS0_SL]);
    P.w0 = (float)v[MPF3D_S_W0_SL];
    P.mu_a = (float)v[MPF3D_S_MU_A];
    P.delta_a = (float)v[MPF3D_S_DELTA_A];
    P.mu_da = (float)(v[MPF3D_S_MU_A] * v[MPF3D_S_DELTA_A]);
    P.pp = (float)(v[MPF3D_S_P_ROUND] * v[MPF3D_S_P_ROUND]);
    P.tan_a0 = (float)tan(v[MPF3D_S_A0]);
    P.g2_floor = (float)v[MPF3D_S_G2_FLOOR];
    P.ksi = (float)v[MPF3D_S_KSI];
    P.theta_c = (float)v[MPF3D_S_THETA_C_RAD];
    // below this best |cos| the facet angle is >= theta_c with a margin far
    // above the FP32 error of c (~1e-7), so b = 1 without computing the angle
    P.cos_theta_lo = (float)(cos(v[MPF3D_S_THETA_C_RAD]) - 1.0e-5);
    P.Sf = (float)v[MPF3D_S_SF];
    P.Tmc = v[MPF3D_S_T_MELT];
    P.use_aniso = enable_anisotropy != 0;
    P.use_torque = enable_anisotropy != 0 && enable_torque != 0;
    P.sym_normals = symmetric_normals != 0;
    const double pp = v[MPF3D_S_P_ROUND] * v[MPF3D_S_P_ROUND];
    const double th = acos(0.0), thc = v[MPF3D_S_THETA_C_RAD];
    double b = 1.0;
    if (th < thc) {
        double y = 0.5 * 3.14159265358979323846 * (th / thc);
        y = fmin(fmax(y, 1e-6), 0.5 * 3.14159265358979323846 - 1e-6);
        const double t = tan(y);
        b = v[MPF3D_S_KSI] + (1.0 - v[MPF3D_S_KSI]) * t * tanh(1.0 / t);
    }
    P.b_flat = (float)b;
    const double a_flat =
        v[MPF3D_S_MU_A] * (1.0 + v[MPF3D_S_DELTA_A] * (sqrt(pp) + tan(v[MPF3D_S_A0]) * sqrt(1.0 + pp)));
    const double e = v[MPF3D_S_EPS0_SL] * a_flat;
    P.e2_flat = (float)(e * e);
    return P;
}


template <int S, int AMAX>
void launch_batched(const In &in, const Out &out, const Mats &M, const Params &P0, const mpf3d_instance *inst,
                    int n_inst, int n_tiles, const Queue &Q, int parity, int32_t *err, cudaStream_t s,
                    const mpf3d_tuning &T, uint8_t *tile_flags) {
    batched_sweep_kernel<S, AMAX><<<n_tiles, dim3(32, 8, 1), 0, s>>>(in, out, P0, inst, n_inst, Q, parity,
                                                                      tile_flags);
    // one stream: the side-by-side launch of the compact step measured no
    // gain here; the work-list grids come from T (the sweep's 32 x 8 x 4
    // tiles are fixed by the instance table)
    const int sms = sms_of_current_device();
    batched_queue_kernel<S, AMAX, false><<<sms * T.general_blocks_per_sm, T.general_threads, 0, s>>>(
        in, out, M, P0, inst, n_inst, Q, parity, err);
    if (P0.use_aniso && P0.sym_normals)
        batched_queue_kernel<S, AMAX, true, 4><<<sms * T.iface_blocks_per_sm, T.iface_threads, 0, s>>>(
            in, out, M, P0, inst, n_inst, Q, parity, err);
    else if (P0.use_aniso)
        batched_queue_kernel<S, AMAX, true, 8><<<sms * T.iface_blocks_per_sm, T.iface_threads, 0, s>>>(
            in, out, M, P0, inst, n_inst, Q, parity, err);
}

// launch shape of the batched step before it was tuned
const mpf3d_tuning kBatchedDefault = {4, 8, 8, 256, 8, 128};

}  // namespace

extern "C" int mpf3d_streams_prepare(void *stream) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MPF3D_ERR_CUDA;
    SideTable &tab = side_table_of(dev);
    std::lock_guard<std::mutex> lock(tab.mu);
    return side_ready(tab.by_caller[(cudaStream_t)stream], (cudaStream_t)stream) ? MPF3D_OK : MPF3D_ERR_CUDA;
}

// The body of mpf3d_compact_step_tuned and mpf3d_compact_step_clocked
// (clock: null, or the device step clock with T_melt and the cooling rate).
static int compact_step_impl(const uint32_t *cnt, const uint16_t *idx, const float *val, uint32_t *cnt_out,
                             uint16_t *idx_out, float *val_out, int slots, int amax, const double *T0z,
                             double Tm_plus_cool, const float *wij, const float *a2ij, const float *mij,
                             const float *n111, int N, int nx, int ny, int nz, const mpf3d_scalars *sc,
                             int enable_anisotropy, int enable_torque, int symmetric_normals, uint32_t *work_items,
                             uint32_t *work_count, int parity, int32_t *err, void *stream,
                             const mpf3d_tuning *tuning, uint8_t *tile_flags, int options, mpf3d_step_clock *clock,
                             double clock_T_melt, double clock_rate) {
    const mpf3d_tuning T = tuning ? *tuning : kDefaultTuning;
    if (!tuning_ok(T)) return MPF3D_ERR_ARG;
    if (!cnt || !idx || !val || !cnt_out || !idx_out || !val_out || !T0z || !wij || !a2ij || !mij || !n111 || !sc ||
        !err || !work_items || !work_count)
        return MPF3D_ERR_ARG;
    if (N <= 0 || N > 65535 || !dims_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    if ((int64_t)nx * ny * nz >= ((int64_t)1 << 31)) return MPF3D_ERR_TOO_LARGE;
    if (cnt == cnt_out || idx == idx_out || val == val_out) return MPF3D_ERR_ARG;
    Params P = shared_params(sc, enable_anisotropy, enable_torque, symmetric_normals);
    P.nx = nx; P.ny = ny; P.nz = nz; P.N = N;
    P.cells = (int64_t)nx * ny * nz;
    P.cells32 = (uint32_t)P.cells;
    P.Tmc = Tm_plus_cool;
    parity &= 1;
    P.clock = clock;
    P.clock_T_melt = clock_T_melt;
    P.clock_rate = clock_rate;
    P.parity = parity;
    In in{cnt, idx, val};
    Out out{cnt_out, idx_out, val_out};
    Mats M{T0z, wij, a2ij, mij, n111};
    Queue Q{work_items, work_count, (options & MPF3D_STEP_MULTI_LIST) ? 1 : 0};
    cudaStream_t s = (cudaStream_t)stream;
    const bool tma = (options & MPF3D_STEP_SWEEP_TMA) != 0;
    if (slots == 4 && amax == 8) launch_step<4, 8>(in, out, M, P, Q, parity, tile_flags, err, s, T, tma);
    else if (slots == 8 && amax == 16) launch_step<8, 16>(in, out, M, P, Q, parity, tile_flags, err, s, T, tma);
    else if (slots == 16 && amax == 32) launch_step<16, 32>(in, out, M, P, Q, parity, tile_flags, err, s, T, tma);
    else return MPF3D_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_compact_step_tuned(const uint32_t *cnt, const uint16_t *idx, const float *val,
                                        uint32_t *cnt_out, uint16_t *idx_out, float *val_out, int slots, int amax,
                                        const double *T0z, double Tm_plus_cool, const float *wij, const float *a2ij,
                                        const float *mij, const float *n111, int N, int nx, int ny, int nz,
                                        const mpf3d_scalars *sc, int enable_anisotropy, int enable_torque,
                                        int symmetric_normals, uint32_t *work_items, uint32_t *work_count,
                                        int parity, int32_t *err, void *stream, const mpf3d_tuning *tuning,
                                        uint8_t *tile_flags, int options) {
    return compact_step_impl(cnt, idx, val, cnt_out, idx_out, val_out, slots, amax, T0z, Tm_plus_cool, wij, a2ij,
                             mij, n111, N, nx, ny, nz, sc, enable_anisotropy, enable_torque, symmetric_normals,
                             work_items, work_count, parity, err, stream, tuning, tile_flags, options, nullptr, 0.0,
                             0.0);
}

extern "C" int mpf3d_compact_step_clocked(const uint32_t *cnt, const uint16_t *idx, const float *val,
                                          uint32_t *cnt_out, uint16_t *idx_out, float *val_out, int slots,
                                          int amax, const double *T0z, mpf3d_step_clock *clock, double T_melt,
                                          double cooling_rate, const float *wij, const float *a2ij,
                                          const float *mij, const float *n111, int N, int nx, int ny, int nz,
                                          const mpf3d_scalars *sc, int enable_anisotropy, int enable_torque,
                                          int symmetric_normals, uint32_t *work_items, uint32_t *work_count,
                                          int parity, int32_t *err, void *stream, const mpf3d_tuning *tuning,
                                          uint8_t *tile_flags, int options) {
    if (!clock) return MPF3D_ERR_ARG;
    return compact_step_impl(cnt, idx, val, cnt_out, idx_out, val_out, slots, amax, T0z, T_melt, wij, a2ij, mij,
                             n111, N, nx, ny, nz, sc, enable_anisotropy, enable_torque, symmetric_normals,
                             work_items, work_count, parity, err, stream, tuning, tile_flags, options, clock, T_melt,
                             cooling_rate);
}

extern "C" int mpf3d_compact_step(const uint32_t *cnt, const uint16_t *idx, const float *val, uint32_t *cnt_out,
                                  uint16_t *idx_out, float *val_out, int slots, int amax, const double *T0z,
                                  double Tm_plus_cool, const float *wij, const float *a2ij, const float *mij,
                                  const float *n111, int N, int nx, int ny, int nz, const mpf3d_scalars *sc,
                                  int enable_anisotropy, int enable_torque, int symmetric_normals,
                                  uint32_t *work_items, uint32_t *work_count, int parity, int32_t *err,
                                  void *stream) {
    return mpf3d_compact_step_tuned(cnt, idx, val, cnt_out, idx_out, val_out, slots, amax, T0z, Tm_plus_cool, wij,
                                    a2ij, mij, n111, N, nx, ny, nz, sc, enable_anisotropy, enable_torque,
                                    symmetric_normals, work_items, work_count, parity, err, stream, nullptr,
                                    nullptr, 0);
}

extern "C" int64_t mpf3d_compact_tile_flags_len(int nx, int ny, int nz) {
    if (!dims_ok(nx, ny, nz)) return 0;
    return 2 * (int64_t)tiles_of<2>(nx, ny, nz);
}

extern "C" int mpf3d_compact_to_dense_view(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                                           uint32_t stride, uint32_t base, int N, int nx, int ny, int nz, void *phi,
                                           int phi_dtype, void *stream) {
    if (!phi || !head || !idx || !val || N <= 0 || N > 65535 || !dims_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    if ((uint64_t)base + (uint64_t)nx * ny * nz > (uint64_t)stride) return MPF3D_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 b(32, 4, 2);
    dim3 g = zfast_grid(nx, ny, nz, b);
    In in{head, idx, val};
#define TDV(T, SS) to_dense_kernel<T, SS><<<g, b, 0, s>>>(in, N, nx, ny, nz, stride, base, (T *)phi)
    if (phi_dtype == MPF3D_F32) {
        if (slots == 4) TDV(float, 4); else if (slots == 8) TDV(float, 8); else if (slots == 16) TDV(float, 16);
        else return MPF3D_ERR_ARG;
    } else if (phi_dtype == MPF3D_F64) {
        if (slots == 4) TDV(double, 4); else if (slots == 8) TDV(double, 8); else if (slots == 16) TDV(double, 16);
        else return MPF3D_ERR_ARG;
    } else {
        return MPF3D_ERR_DTYPE;
    }
#undef TDV
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}


extern "C" int mpf3d_batched_init_bicrystal(const mpf3d_instance *inst, int n_inst, uint32_t total_cells, double dx,
                                            double delta, uint32_t *head, uint16_t *idx, float *val, int32_t *err,
                                            void *stream) {
    if (!inst || n_inst <= 0 || n_inst > 65535 || !head || !idx || !val || !err || total_cells == 0)
        return MPF3D_ERR_ARG;
    const float factor_dz = (float)((double)(float)(2.2 / delta) * dx);
    Out o{head, idx, val};
    batched_init_bicrystal_kernel<<<dim3(64, n_inst), 256, 0, (cudaStream_t)stream>>>(o, inst, n_inst, total_cells,
                                                                                      factor_dz, err);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_batched_step_tuned(const uint32_t *head, const uint16_t *idx, const float *val,
                                        uint32_t *head_out, uint16_t *idx_out, float *val_out, int slots, int amax,
                                        const mpf3d_instance *inst, int n_inst, int n_tiles, uint32_t total_cells,
                                        const float *wij, const float *a2ij, const float *mij, const float *n111, int N,
                                        const mpf3d_scalars *sc, int enable_anisotropy, int enable_torque,
                                        int symmetric_normals, uint32_t *work_items, uint32_t *work_count, int parity,
                                        int32_t *err, void *stream, int options, const mpf3d_tuning *tuning,
                                        uint8_t *tile_flags) {
    const mpf3d_tuning T = tuning ? *tuning : kBatchedDefault;
    if (!tuning_ok(T)) return MPF3D_ERR_ARG;
    if (!head || !idx || !val || !head_out || !idx_out || !val_out || !inst || !wij || !a2ij || !mij || !n111 ||
        !sc || !err || !work_items || !work_count || n_inst <= 0 || n_tiles <= 0 || total_cells == 0 || N <= 0 ||
        N > 65535)
        return MPF3D_ERR_ARG;
    if (total_cells >= (1u << 31)) return MPF3D_ERR_TOO_LARGE;
    if (head == head_out || idx == idx_out || val == val_out) return MPF3D_ERR_ARG;
    Params P0 = shared_params(sc, enable_anisotropy, enable_torque, symmetric_normals);
    P0.cells = total_cells;
    P0.cells32 = total_cells;
    P0.N = N;
    In in{head, idx, val};
    Out out{head_out, idx_out, val_out};
    Mats M{nullptr, wij, a2ij, mij, n111};
    Queue Q{work_items, work_count, (options & MPF3D_STEP_MULTI_LIST) ? 1 : 0};
    cudaStream_t s = (cudaStream_t)stream;
    parity &= 1;
    uint8_t *F = tile_flags;
    if (slots == 4 && amax == 8) launch_batched<4, 8>(in, out, M, P0, inst, n_inst, n_tiles, Q, parity, err, s, T, F);
    else if (slots == 8 && amax == 16) launch_batched<8, 16>(in, out, M, P0, inst, n_inst, n_tiles, Q, parity, err, s, T, F);
    else if (slots == 16 && amax == 32) launch_batched<16, 32>(in, out, M, P0, inst, n_inst, n_tiles, Q, parity, err, s, T, F);
    else return MPF3D_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int64_t mpf3d_batched_tile_flags_len(int n_tiles) {
    return n_tiles > 0 ? 16 * (int64_t)n_tiles : 0;
}

extern "C" int mpf3d_batched_step(const uint32_t *head, const uint16_t *idx, const float *val, uint32_t *head_out,
                                  uint16_t *idx_out, float *val_out, int slots, int amax, const mpf3d_instance *inst,
                                  int n_inst, int n_tiles, uint32_t total_cells, const float *wij, const float *a2ij,
                                  const float *mij, const float *n111, int N, const mpf3d_scalars *sc,
                                  int enable_anisotropy, int enable_torque, int symmetric_normals,
                                  uint32_t *work_items, uint32_t *work_count, int parity, int32_t *err,
                                  void *stream, int options) {
    return mpf3d_batched_step_tuned(head, idx, val, head_out, idx_out, val_out, slots, amax, inst, n_inst, n_tiles,
                                    total_cells, wij, a2ij, mij, n111, N, sc, enable_anisotropy, enable_torque,
                                    symmetric_normals, work_items, work_count, parity, err, stream, options,
                                    nullptr, nullptr);
}

extern "C" int mpf3d_batched_fronts(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                                    const mpf3d_instance *inst, int n_inst, uint32_t total_cells, double *acc,
                                    void *stream) {
    if (!head || !idx || !val || !inst || !acc || n_inst <= 0 || n_inst > 65535) return MPF3D_ERR_ARG;
    In in{head, idx, val};
    dim3 g(16, n_inst);
    cudaStream_t s = (cudaStream_t)stream;
    if (slots == 4) batched_fronts_kernel<4><<<g, 256, 0, s>>>(in, inst, n_inst, total_cells, acc);
    else if (slots == 8) batched_fronts_kernel<8><<<g, 256, 0, s>>>(in, inst, n_inst, total_cells, acc);
    else if (slots == 16) batched_fronts_kernel<16><<<g, 256, 0, s>>>(in, inst, n_inst, total_cells, acc);
    else return MPF3D_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_batched_gb_rows(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                                     const mpf3d_instance *inst, int n_inst, uint32_t total_cells,
                                     const int32_t *row_base, double *gb, void *stream) {
    if (!head || !idx || !val || !inst || !row_base || !gb || n_inst <= 0 || n_inst > 65535) return MPF3D_ERR_ARG;
    In in{head, idx, val};
    dim3 g(16, n_inst);
    cudaStream_t s = (cudaStream_t)stream;
    if (slots == 4) batched_gb_rows_kernel<4><<<g, 128, 0, s>>>(in, inst, n_inst, total_cells, row_base, gb);
    else if (slots == 8) batched_gb_rows_kernel<8><<<g, 128, 0, s>>>(in, inst, n_inst, total_cells, row_base, gb);
    else if (slots == 16) batched_gb_rows_kernel<16><<<g, 128, 0, s>>>(in, inst, n_inst, total_cells, row_base, gb);
    else return MPF3D_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_compact_init_owner(const int32_t *owner, int slab, const float *prof, int nx, int ny, int nz,
                                        int slots, uint32_t *head, uint16_t *idx, float *val, void *stream) {
    if (!owner || !prof || !head || !idx || !val || slab <= 0 || slab > nz || slots < 2 || !dims_ok(nx, ny, nz))
        return MPF3D_ERR_ARG;
    const int64_t cells = (int64_t)nx * ny * nz;
    if (cells >= ((int64_t)1 << 32)) return MPF3D_ERR_TOO_LARGE;
    Out o{head, idx, val};
    init_owner_kernel<<<sms_of_current_device() * 16, 256, 0, (cudaStream_t)stream>>>(o, owner, slab, prof, nx, ny, nz,
                                                                                       (uint32_t)cells);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Step without device allocation.
//
// Some hosts cannot let this library allocate device memory: applications
// that reserve the whole GPU memory budget up front for their own pool and
// give plugins none, or real-time loops where a cudaMalloc -- which may
// synchronise the device -- is not acceptable.  For them the work list of
// the step lives in a file-scope device array instead of caller scratch.
// Every GPU that loads the library holds the array until the process exits.
namespace {

constexpr uint32_t kNoAllocMaxCells = MPF3D_NOALLOC_MAX_CELLS;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) uint32_t g_noalloc_items[kNoAllocMaxCells];
static __device__ __align__(256) uint32_t g_noalloc_count[4];

struct NoAllocScratch {
    uint32_t *items = nullptr;
    uint32_t *count = nullptr;
    bool ready = false;
};
NoAllocScratch g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_mu;

// Device addresses of the array on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up
// once per device, with that device current.
int noalloc_scratch(uint32_t **items, uint32_t **count) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MPF3D_ERR_CUDA;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return MPF3D_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocScratch &s = g_noalloc_dev[dev];
    if (!s.ready) {
        void *pi = nullptr, *pc = nullptr;
        if (cudaGetSymbolAddress(&pi, g_noalloc_items) != cudaSuccess) return MPF3D_ERR_CUDA;
        if (cudaGetSymbolAddress(&pc, g_noalloc_count) != cudaSuccess) return MPF3D_ERR_CUDA;
        s.items = (uint32_t *)pi;
        s.count = (uint32_t *)pc;
        s.ready = true;
    }
    *items = s.items;
    *count = s.count;
    return MPF3D_OK;
}

}  // namespace

extern "C" int mpf3d_compact_step_noalloc(const uint32_t *head, const uint16_t *idx, const float *val,
                                          uint32_t *head_out, uint16_t *idx_out, float *val_out, int slots,
                                          int amax, const double *T0z, double Tm_plus_cool, const float *wij,
                                          const float *a2ij, const float *mij, const float *n111, int N, int nx,
                                          int ny, int nz, const mpf3d_scalars *sc, int enable_anisotropy,
                                          int enable_torque, int symmetric_normals, int32_t *err, void *stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return MPF3D_ERR_ARG;
    if ((int64_t)nx * ny * nz > (int64_t)kNoAllocMaxCells) return MPF3D_ERR_TOO_LARGE;
    uint32_t *items = nullptr, *count = nullptr;
    const int rc = noalloc_scratch(&items, &count);
    if (rc != MPF3D_OK) return rc;
    // the counters must start at zero; the previous call left its totals there
    if (cudaMemsetAsync(count, 0, 4 * sizeof(uint32_t), (cudaStream_t)stream) != cudaSuccess) return MPF3D_ERR_CUDA;
    return mpf3d_compact_step(head, idx, val, head_out, idx_out, val_out, slots, amax, T0z, Tm_plus_cool, wij,
                              a2ij, mij, n111, N, nx, ny, nz, sc, enable_anisotropy, enable_torque,
                              symmetric_normals, items, count, 0, err, stream);
}
