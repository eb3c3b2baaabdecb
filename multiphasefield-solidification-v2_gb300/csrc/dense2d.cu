// dense2d.cu -- the reference's 2D kernels with the reference's numerics, on
// the reference's dense [N][nx][ny] arrays.
//
// Replaces src/gpu_kernels.py:337-525 (kernel_update_nfmf,
// kernel_update_phasefield_active, kernel_update_temp), the 2D module that
// the reference's verification suite compares the 3D step against
// (two_d_limit_consistency, tests/verification_3d.py:1509-1535).
// Boundaries: x periodic, y mirror (clamped index).
//
// Numerics: compiled-Numba arithmetic types, as in dense_ref.cu (float
// literals are float64, float32 op float64 -> float64, float32(...) casts,
// float32 local arrays lap_sl/b_sl); compiled with -fmad=false.
//
// Layout choices (not the reference's): threadIdx.x runs along y, the
// contiguous axis, so warps read whole 128-byte segments; the liquid
// gradient at the 5 stencil points and the facet search per (point, grain)
// are computed once per cell and shared by the anisotropic term, the torque
// term and b(theta); the per-phase Laplacians are computed once per cell
// instead of once per (i, j, k) triple.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mpf3d.h"
#include "mpf3d_internal.h"

namespace mpf3d {
namespace dense2d {

constexpr int KMAX = MPF3D_KMAX;
constexpr int LIQ = 0;

struct Params {
    int N, nx, ny, depth;
    double dx, dt, T_melt, Sf, eps0, w0, a0, delta_a, mu_a, p_round, g2_floor, ksi, theta_c;
    double two_dx, half_over_dx, inv_dx2, pp, mu_da, eps0sq;
    int a0_32, p32, dT32, df32;
};

__device__ __forceinline__ int ixp(int l, int n) { return l < n - 1 ? l + 1 : 0; }
__device__ __forceinline__ int ixm(int l, int n) { return l > 0 ? l - 1 : n - 1; }
__device__ __forceinline__ int iyp(int m, int n) { return m < n - 1 ? m + 1 : n - 1; }
__device__ __forceinline__ int iym(int m, int n) { return m > 0 ? m - 1 : 0; }

template <typename T>
struct Field {
    const T *__restrict__ p;
    int nx, ny;
    size_t plane;
    __device__ __forceinline__ T at(int g, int l, int m) const {
        return __ldg(p + (size_t)g * plane + (size_t)l * ny + m);
    }
};

struct Vec2 {
    double x, y;
};

// grad_phi_xy (:108-115)
template <typename T>
__device__ __forceinline__ Vec2 grad_at(const Field<T> &f, int g, int l, int m, double two_dx) {
    int lp = ixp(l, f.nx), lm = ixm(l, f.nx), mp = iyp(m, f.ny), mm = iym(m, f.ny);
    Vec2 r;
    r.x = (double)(T)(f.at(g, lp, m) - f.at(g, lm, m)) / two_dx;
    r.y = (double)(T)(f.at(g, l, mp) - f.at(g, l, mm)) / two_dx;
    return r;
}

// One search over the x,y components of the 8 rotated {111} normals gives
// best_cos_from_grad (:120-136, float64) and facet_cos_and_nxy_from_grad
// (:207-232, float32 results): both evaluate the same dot products in the
// same order.
struct Facet {
    int valid;
    double best64;
    float cs, ca, nx, ny;
};

__device__ __forceinline__ Facet facet(const Vec2 &g, const float *__restrict__ u, double g2_floor) {
    Facet f;
    double q = g.x * g.x + g.y * g.y;
    if (q < g2_floor) {
        f.valid = 0; f.best64 = 0.0; f.cs = 0.0f; f.ca = 0.0f; f.nx = 1.0f; f.ny = 0.0f;
        return f;
    }
    double inv_g = 1.0 / sqrt(q);
    double gx = g.x * inv_g, gy = g.y * inv_g;
    double best_abs = 0.0, best_signed = 0.0, bx = 1.0, by = 0.0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        double ux = (double)u[3 * t], uy = (double)u[3 * t + 1];
        double dot = gx * ux + gy * uy;
        double ad = fabs(dot);
        if (ad > best_abs) {
            best_abs = ad; best_signed = dot; bx = ux; by = uy;
        }
    }
    if (best_abs > 1.0) best_abs = 1.0;
    if (best_signed > 1.0) best_signed = 1.0;
    if (best_signed < -1.0) best_signed = -1.0;
    f.valid = 1;
    f.best64 = best_abs;
    f.cs = (float)best_signed; f.ca = (float)best_abs; f.nx = (float)bx; f.ny = (float)by;
    return f;
}

// calc_a_from_cos (:25-31), float64 cosine
__device__ __forceinline__ double calc_a64(const Params &P, double tan_a0, double cost) {
    double c2 = cost * cost;
    double C = sqrt(c2 + P.pp);
    double om = 1.0 - c2;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + P.pp);
    return P.mu_a * (1.0 + P.delta_a * (C + tan_a0 * S));
}

// calc_a_from_cos with the float32 facet cosine
__device__ __forceinline__ double calc_a32(const Params &P, double tan_a0, float cost) {
    float c2f = cost * cost;
    double c2 = (double)c2f;
    double C = P.p32 ? (double)sqrtf(c2f + (float)P.pp) : sqrt(c2 + P.pp);
    double om = 1.0 - c2;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + P.pp);
    return P.mu_a * (1.0 + P.delta_a * (C + tan_a0 * S));
}

// calc_b_from_cos (:34-79)
__device__ __forceinline__ double calc_b(const Params &P, double c) {
    if (c > 1.0) c = 1.0;
    else if (c < -1.0) c = -1.0;
    double theta = acos(c);
    if (theta >= P.theta_c) return 1.0;
    double x = theta / P.theta_c;
    const double eps = 1.0e-6;
    const double hp = 0.5 * 3.14159265358979323846;
    double y = hp * x;
    if (y > hp - eps) y = hp - eps;
    if (y < eps) y = eps;
    double t = tan(y);
    return P.ksi + (1.0 - P.ksi) * t * tanh(1.0 / t);
}

// coef = (c/C) - tan(a0)*(c/S) of da_dphixy_A12 / torque_A11 (:256-259, :317-320)
__device__ __forceinline__ double dadc_coef(const Params &P, double tan_a0, float cs) {
    float ccf = cs * cs;
    double om = 1.0 - (double)ccf;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + P.pp);
    if (P.p32) {
        float Cf = sqrtf(ccf + (float)P.pp);
        return (double)(cs / Cf) - tan_a0 * ((double)cs / S);
    }
    double C = sqrt((double)ccf + P.pp);
    return ((double)cs / C) - tan_a0 * ((double)cs / S);
}

struct DA {
    float a, x, y;
};

// da_dphixy_A12 (:237-264) from the liquid gradient and facet at a point
__device__ __forceinline__ DA da_dphi(const Params &P, double tan_a0, const Vec2 &g, const Facet &f) {
    DA r;
    if (!f.valid) {
        r.a = r.x = r.y = 0.0f;
        return r;
    }
    double q = g.x * g.x + g.y * g.y;
    double a_val = calc_a32(P, tan_a0, f.ca);
    double gg = sqrt(q);
    double inv_g = 1.0 / gg;
    double inv_g3 = 1.0 / (q * gg);
    double udotg = g.x * (double)f.nx + g.y * (double)f.ny;
    double dcx = (double)f.nx * inv_g - udotg * g.x * inv_g3;
    double dcy = (double)f.ny * inv_g - udotg * g.y * inv_g3;
    double coef = dadc_coef(P, tan_a0, f.cs);
    r.a = (float)a_val;
    r.x = (float)(P.mu_da * coef * dcx);
    r.y = (float)(P.mu_da * coef * dcy);
    return r;
}

// kernel_update_nfmf (:337-358)
template <typename T>
__global__ void __launch_bounds__(256) apt_kernel(Field<T> phi, int N, int32_t *__restrict__ mf, int depth,
                                                  int32_t *__restrict__ nf, int32_t *__restrict__ err) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    int l = blockIdx.y * blockDim.y + threadIdx.y;
    if (m >= phi.ny || l >= phi.nx) return;
    int lp = ixp(l, phi.nx), lm = ixm(l, phi.nx), mp = iyp(m, phi.ny), mm = iym(m, phi.ny);
    size_t cell = (size_t)l * phi.ny + m;
    const T zero = (T)0;
    int n = 0;
    bool deep = false;
    for (int i = 0; i < N; ++i) {
        T v = phi.at(i, l, m);
        bool act = (v > zero) || ((v == zero) && ((phi.at(i, lp, m) > zero) || (phi.at(i, lm, m) > zero) ||
                                                  (phi.at(i, l, mp) > zero) || (phi.at(i, l, mm) > zero)));
        if (act) {
            n += 1;
            if (n <= depth) mf[(size_t)(n - 1) * phi.plane + cell] = i;
            else deep = true;
        }
    }
    nf[cell] = n > depth ? depth : n;
    if (deep && err) atomicOr(err, MPF3D_DEV_MF_DEPTH);
}

// kernel_update_phasefield_active (:361-517)
template <typename T, typename TT>
__global__ void __launch_bounds__(128) update_kernel(Field<T> phi, T *__restrict__ phi_new,
                                                     const TT *__restrict__ temp,
                                                     const int32_t *__restrict__ mf,
                                                     const int32_t *__restrict__ nf,
                                                     const float *__restrict__ wij,
                                                     const float *__restrict__ aij,
                                                     const float *__restrict__ mij,
                                                     const float *__restrict__ n111, Params P,
                                                     int32_t *__restrict__ err) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    int l = blockIdx.y * blockDim.y + threadIdx.y;
    if (m >= P.ny || l >= P.nx) return;
    const int N = P.N;
    const size_t plane = phi.plane;
    const size_t cell = (size_t)l * P.ny + m;
    const int n = nf[cell];
    if (n < 0 || n > KMAX) {
        if (err) atomicOr(err, MPF3D_DEV_NF_GT_KMAX);
        return;
    }
    if (n > P.depth) {
        if (err) atomicOr(err, MPF3D_DEV_MF_DEPTH);
        return;
    }
    int ids[KMAX];
    for (int t = 0; t < n; ++t) {
        int g = mf[(size_t)t * plane + cell];
        if (g < 0 || g >= N) {
            if (err) atomicOr(err, MPF3D_DEV_BAD_ID);
            return;
        }
        ids[t] = g;
    }
    const double tan_a0 = P.a0_32 ? (double)tanf((float)P.a0) : tan(P.a0);
    const int lp = ixp(l, P.nx), lm = ixm(l, P.nx), mp = iyp(m, P.ny), mm = iym(m, P.ny);
    // stencil points: 0 c, 1 x+, 2 x-, 3 y+, 4 y-
    const int pl[5] = {l, lp, lm, l, l};
    const int pm[5] = {m, m, m, mp, mm};

    float lap_sl[KMAX], b_sl[KMAX];
    bool any_solid = false;
    for (int t = 0; t < n; ++t) any_solid |= (ids[t] != LIQ);
    if (any_solid) {
        Vec2 G[5];
#pragma unroll
        for (int p = 0; p < 5; ++p) G[p] = grad_at(phi, LIQ, pl[p], pm[p], P.two_dx);
        const T pc = phi.at(LIQ, l, m);
        T pv[5];
#pragma unroll
        for (int p = 1; p < 5; ++p) pv[p] = phi.at(LIQ, pl[p], pm[p]);
        for (int t = 0; t < n; ++t) {
            const int gid = ids[t];
            if (gid == LIQ) {
                b_sl[t] = 1.0f;
                lap_sl[t] = 0.0f;
                continue;
            }
            const float *u = n111 + (size_t)gid * 24;
            Facet F[5];
#pragma unroll
            for (int p = 0; p < 5; ++p) F[p] = facet(G[p], u, P.g2_floor);
            // aniso_term1_solid (:155-179)
            double e2[5];
#pragma unroll
            for (int p = 0; p < 5; ++p) {
                double e = P.eps0 * calc_a64(P, tan_a0, F[p].best64);
                e2[p] = e * e;
            }
            double Fxp = (e2[0] + e2[1]) * (double)(T)(pv[1] - pc) / P.two_dx;
            double Fxm = (e2[0] + e2[2]) * (double)(T)(pc - pv[2]) / P.two_dx;
            double Fyp = (e2[0] + e2[3]) * (double)(T)(pv[3] - pc) / P.two_dx;
            double Fym = (e2[0] + e2[4]) * (double)(T)(pc - pv[4]) / P.two_dx;
            float lap = (float)((Fxp - Fxm) / P.dx + (Fyp - Fym) / P.dx);
            // torque_A11 (:290-332); the reference adds it to the stored
            // float32 value, so the sum is rounded twice.
            double tq = 0.0;
            if (F[0].valid) {
                const Vec2 g0 = G[0];
                double q = g0.x * g0.x + g0.y * g0.y;
                // d2_phi_xy (:184-202) of the liquid
                double pxx = ((double)pv[1] - 2.0 * (double)pc + (double)pv[2]) * P.inv_dx2;
                double pyy = ((double)pv[3] - 2.0 * (double)pc + (double)pv[4]) * P.inv_dx2;
                double pxy = (double)(T)(((T)(phi.at(LIQ, lp, mp) - phi.at(LIQ, lp, mm)) - phi.at(LIQ, lm, mp)) +
                                         phi.at(LIQ, lm, mm)) *
                             (0.25 * P.inv_dx2);
                double q_x = 2.0 * (g0.x * pxx + g0.y * pxy);
                double q_y = 2.0 * (g0.x * pxy + g0.y * pyy);
                DA d0 = da_dphi(P, tan_a0, g0, F[0]);
                const Facet &f0 = F[0];
                double gg = sqrt(q);
                double inv_g = 1.0 / gg;
                double inv_g3 = 1.0 / (q * gg);
                double udotg = g0.x * (double)f0.nx + g0.y * (double)f0.ny;
                double dcx = (double)f0.nx * inv_g - udotg * g0.x * inv_g3;
                double dcy = (double)f0.ny * inv_g - udotg * g0.y * inv_g3;
                double cxx = dcx * pxx + dcy * pxy;
                double cyy = dcx * pxy + dcy * pyy;
                double coef = dadc_coef(P, tan_a0, f0.cs);
                double da_dx = P.mu_da * coef * cxx;
                double da_dy = P.mu_da * coef * cyy;
                // d_dx_da_dphix_and_d_dy_da_dphiy_A13 (:269-285)
                float ddx = (float)((double)(da_dphi(P, tan_a0, G[1], F[1]).x - da_dphi(P, tan_a0, G[2], F[2]).x) *
                                    P.half_over_dx);
                float ddy = (float)((double)(da_dphi(P, tan_a0, G[3], F[3]).y - da_dphi(P, tan_a0, G[4], F[4]).y) *
                                    P.half_over_dx);
                float a = d0.a;
                double Ex = (da_dx * (double)d0.x * q) + ((double)(a * ddx) * q) + ((double)(a * d0.x) * q_x);
                double Ey = (da_dy * (double)d0.y * q) + ((double)(a * ddy) * q) + ((double)(a * d0.y) * q_y);
                tq = P.eps0sq * (Ex + Ey);
            }
            lap_sl[t] = (float)((double)lap + tq);
            b_sl[t] = (float)calc_b(P, F[0].best64);
        }
    } else {
        for (int t = 0; t < n; ++t) {
            b_sl[t] = 1.0f;
            lap_sl[t] = 0.0f;
        }
    }

    // dominant solid grain and anisotropic w_sl (:410-436): grain 1 unless an
    // active solid holds a positive fraction; always evaluated.
    int i_s = 1;
    double maxv = 0.0;
    for (int t = 0; t < n; ++t) {
        int gid = ids[t];
        if (gid == LIQ) continue;
        double v = (double)phi.at(gid, l, m);
        if (v > maxv) {
            maxv = v;
            i_s = gid;
        }
    }
    double w_sl;
    {
        double phx = (double)(T)(phi.at(i_s, lp, m) - phi.at(i_s, lm, m)) * P.half_over_dx;
        double phy = (double)(T)(phi.at(i_s, l, mp) - phi.at(i_s, l, mm)) * P.half_over_dx;
        double gn2 = phx * phx + phy * phy;
        double cmax = 0.0;
        if (gn2 >= P.g2_floor) {
            double inv_gn = 1.0 / sqrt(gn2);
            double ux = phx * inv_gn, uy = phy * inv_gn;
            const float *u = n111 + (size_t)i_s * 24;
#pragma unroll
            for (int tt = 0; tt < 8; ++tt) {
                double cv = fabs(ux * (double)u[3 * tt] + uy * (double)u[3 * tt + 1]);
                if (cv > cmax) cmax = cv;
            }
            if (cmax > 1.0) cmax = 1.0;
        }
        double al = calc_a64(P, tan_a0, cmax);
        w_sl = P.w0 * (al * al);
    }

    for (int g = 0; g < N; ++g) phi_new[(size_t)g * plane + cell] = (T)0;

    T phc[KMAX];
    double lapk[KMAX];
    for (int t = 0; t < n; ++t) {
        int g = ids[t];
        phc[t] = phi.at(g, l, m);
        T s = phi.at(g, lp, m) + phi.at(g, lm, m);
        s = s + phi.at(g, l, mp);
        s = s + phi.at(g, l, mm);
        lapk[t] = ((double)s - 4.0 * (double)phc[t]) * P.inv_dx2;
    }
    const double Tcur = (double)temp[cell];
    const double dTv = P.dT32 ? (double)((float)Tcur - (float)P.T_melt) : Tcur - P.T_melt;
    T outv[KMAX];
    for (int t1 = 0; t1 < n; ++t1) {
        const int i = ids[t1];
        double dpi = 0.0;
        for (int t2 = 0; t2 < n; ++t2) {
            const int j = ids[t2];
            if (i == j) continue;
            double df = 0.0;
            if (i != LIQ && j == LIQ)
                df = P.df32 ? (double)(-(float)P.Sf * (float)dTv) : (-P.Sf) * dTv;
            else if (i == LIQ && j != LIQ)
                df = P.df32 ? (double)((float)P.Sf * (float)dTv) : P.Sf * dTv;
            double ppp = 0.0;
            for (int t3 = 0; t3 < n; ++t3) {
                const int k = ids[t3];
                double wik = (double)__ldg(wij + i * N + k), wjk = (double)__ldg(wij + j * N + k);
                if (k == LIQ) {
                    if (i != LIQ) wik = w_sl;
                    if (j != LIQ) wjk = w_sl;
                }
                double term1 = (wik - wjk) * (double)phc[t3];
                double term2 = 0.0;
                if (j == LIQ && i != LIQ) {
                    if (k == i) term2 = 0.5 * (double)lap_sl[t1];
                } else if (i == LIQ && j != LIQ) {
                    if (k == j) term2 = -0.5 * (double)lap_sl[t2];
                } else {
                    float ai = __ldg(aij + i * N + k), aj = __ldg(aij + j * N + k);
                    float e2i = ai * ai, e2j = aj * aj;
                    term2 = 0.5 * (double)(e2i - e2j) * lapk[t3];
                }
                ppp += term1 + term2;
            }
            T pij = phc[t1] * phc[t2];
            double pijd = (double)pij;
            double tf = (8.0 / 3.1415926535) * sqrt(pijd > 0.0 ? pijd : 0.0) * df;
            float me = __ldg(mij + i * N + j);
            if (i != LIQ && j == LIQ) me = me * b_sl[t1];
            else if (i == LIQ && j != LIQ) me = me * b_sl[t2];
            dpi -= 2.0 * (double)me / (double)n * (ppp - tf);
        }
        outv[t1] = (T)((double)phc[t1] + P.dt * dpi);
    }
    // clip and renormalise (:499-517)
    double ssum = 0.0;
    for (int t = 0; t < n; ++t) {
        double v = (double)outv[t];
        if (v < 0.0) v = 0.0;
        if (v > 1.0) v = 1.0;
        outv[t] = (T)v;
        ssum += v;
    }
    if (ssum > 1e-20) {
        double invs = 1.0 / ssum;
        for (int t = 0; t < n; ++t) phi_new[(size_t)ids[t] * plane + cell] = (T)((double)outv[t] * invs);
    } else {
        for (int t = 0; t < n; ++t) phi_new[(size_t)ids[t] * plane + cell] = outv[t];
        phi_new[cell] = (T)1;
    }
}

}  // namespace dense2d
}  // namespace mpf3d

using namespace mpf3d;
using namespace mpf3d::dense2d;

static inline int bitset2(uint32_t m, int i) { return (int)((m >> i) & 1u); }

static bool grid2_ok(int nx, int ny) { return nx > 0 && ny > 0 && nx <= 65535 * 4; }

static dim3 grid2(int nx, int ny, dim3 blk) {
    return dim3((ny + blk.x - 1) / blk.x, (nx + blk.y - 1) / blk.y, 1);
}

extern "C" int mpf2d_dense_apt(const void *phi, int phi_dtype, int N, int nx, int ny, int32_t *mf, int depth,
                               int32_t *nf, int32_t *err, void *stream) {
    if (!phi || !mf || !nf || N <= 0 || depth <= 0 || !grid2_ok(nx, ny)) return MPF3D_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 blk(32, 4, 1);
    dim3 grd = grid2(nx, ny, blk);
    size_t plane = (size_t)nx * ny;
    if (phi_dtype == MPF3D_F32) {
        Field<float> f{(const float *)phi, nx, ny, plane};
        apt_kernel<float><<<grd, blk, 0, s>>>(f, N, mf, depth, nf, err);
    } else if (phi_dtype == MPF3D_F64) {
        Field<double> f{(const double *)phi, nx, ny, plane};
        apt_kernel<double><<<grd, blk, 0, s>>>(f, N, mf, depth, nf, err);
    } else {
        return MPF3D_ERR_DTYPE;
    }
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

template <typename T, typename TT>
static void launch_update2d(const void *phi, void *phi_new, const void *temp, const int32_t *mf, const int32_t *nf,
                            const float *wij, const float *aij, const float *mij, const float *n111,
                            const Params &P, int32_t *err, cudaStream_t s) {
    dim3 blk(32, 4, 1);
    dim3 grd = grid2(P.nx, P.ny, blk);
    Field<T> f{(const T *)phi, P.nx, P.ny, (size_t)P.nx * P.ny};
    update_kernel<T, TT><<<grd, blk, 0, s>>>(f, (T *)phi_new, (const TT *)temp, mf, nf, wij, aij, mij, n111, P, err);
}

extern "C" int mpf2d_dense_update(const void *phi, void *phi_new, int phi_dtype, const void *temp, int temp_dtype,
                                  const int32_t *mf, int depth, const int32_t *nf, const float *wij,
                                  const float *aij, const float *mij, const float *n111, int N, int nx, int ny,
                                  const mpf3d_scalars *sc, int32_t *err, void *stream) {
    if (!phi || !phi_new || !temp || !mf || !nf || !wij || !aij || !mij || !n111 || !sc) return MPF3D_ERR_ARG;
    // The reference's dominant-solid lookup defaults to grain 1, so N >= 2.
    if (N < 2 || N > 65535 || depth <= 0 || !grid2_ok(nx, ny)) return MPF3D_ERR_ARG;
    if ((phi_dtype != MPF3D_F32 && phi_dtype != MPF3D_F64) || (temp_dtype != MPF3D_F32 && temp_dtype != MPF3D_F64))
        return MPF3D_ERR_DTYPE;
    Params P;
    P.N = N; P.nx = nx; P.ny = ny; P.depth = depth;
    const double *v = sc->v;
    const uint32_t fm = sc->f32mask;
    P.dx = v[MPF3D_S_DX]; P.dt = v[MPF3D_S_DT]; P.T_melt = v[MPF3D_S_T_MELT]; P.Sf = v[MPF3D_S_SF];
    P.eps0 = v[MPF3D_S_EPS0_SL]; P.w0 = v[MPF3D_S_W0_SL]; P.a0 = v[MPF3D_S_A0]; P.delta_a = v[MPF3D_S_DELTA_A];
    P.mu_a = v[MPF3D_S_MU_A]; P.p_round = v[MPF3D_S_P_ROUND]; P.g2_floor = v[MPF3D_S_G2_FLOOR];
    P.ksi = v[MPF3D_S_KSI]; P.theta_c = v[MPF3D_S_THETA_C_RAD];
    P.two_dx = 2.0 * P.dx;
    P.half_over_dx = 0.5 / P.dx;
    if (bitset2(fm, MPF3D_S_DX)) {
        float d = (float)P.dx;
        P.inv_dx2 = 1.0 / (double)(d * d);
    } else {
        P.inv_dx2 = 1.0 / (P.dx * P.dx);
    }
    P.p32 = bitset2(fm, MPF3D_S_P_ROUND);
    P.pp = P.p32 ? (double)((float)P.p_round * (float)P.p_round) : P.p_round * P.p_round;
    P.mu_da = (bitset2(fm, MPF3D_S_MU_A) && bitset2(fm, MPF3D_S_DELTA_A))
                  ? (double)((float)P.mu_a * (float)P.delta_a)
                  : P.mu_a * P.delta_a;
    P.eps0sq = bitset2(fm, MPF3D_S_EPS0_SL) ? (double)((float)P.eps0 * (float)P.eps0) : P.eps0 * P.eps0;
    P.a0_32 = bitset2(fm, MPF3D_S_A0);
    P.dT32 = (temp_dtype == MPF3D_F32) && bitset2(fm, MPF3D_S_T_MELT);
    P.df32 = P.dT32 && bitset2(fm, MPF3D_S_SF);
    cudaStream_t s = (cudaStream_t)stream;
    if (phi_dtype == MPF3D_F32 && temp_dtype == MPF3D_F32)
        launch_update2d<float, float>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    else if (phi_dtype == MPF3D_F32)
        launch_update2d<float, double>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    else if (temp_dtype == MPF3D_F32)
        launch_update2d<double, float>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    else
        launch_update2d<double, double>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf2d_dense_temp(void *temp, int temp_dtype, double rate, int rate_is_f32, int nx, int ny,
                                void *stream) {
    if (nx < 0 || ny < 0) return MPF3D_ERR_ARG;
    return mpf3d_dense_temp(temp, temp_dtype, rate, rate_is_f32, (int64_t)nx * ny, stream);
}
