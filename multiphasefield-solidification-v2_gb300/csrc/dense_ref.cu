// dense_ref.cu -- dense drop-in tier: the reference's 3D kernels with the
// reference's numerics, on the reference's dense [N][nx][ny][nz] arrays.
//
// Replaces src/gpu_kernels_3d.py:462-838 (kernel_update_nfmf_3d[_checked],
// kernel_update_phasefield_active_3d[_switchable], kernel_update_temp_3d).
//
// Numerics: arithmetic types follow compiled Numba (float literals are
// float64, float32 op float64 -> float64, float32(...) casts, float32 local
// arrays lap_sl/b_sl).  This translation unit is compiled with -fmad=false
// because the reference's NVVM pipeline does not contract a*b+c without
// fastmath; with that, results match the reference up to the last-bit
// differences of libm transcendentals.
//
// GB300 layout choices (not the reference's): threadIdx.x runs along z, the
// contiguous axis, so every phi/mf/nf access of a warp is a 128-byte
// coalesced segment; the liquid gradient at the 7 stencil points and the
// facet search per (point, grain) are computed once per cell and reused by
// the anisotropic term, the torque term and b(theta), where the reference
// re-derives them 15-20 times per solid phase; the per-phase Laplacians
// are computed once per cell instead of n^2 times in the t3 loop.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mpf3d.h"
#include "mpf3d_internal.h"

namespace mpf3d {
namespace dense {

constexpr int KMAX = MPF3D_KMAX;
constexpr int LIQ = 0;

struct Params {
    int N, nx, ny, nz, depth;
    double dx, dt, T_melt, Sf, eps0, w0, a0, delta_a, mu_a, p_round, g2_floor, ksi, theta_c;
    double two_dx, half_over_dx, inv_dx2, pp, mu_da, eps0sq;
    int a0_32, p32, dT32, df32;
    int use_aniso, use_torque, switchable;
};

__device__ __forceinline__ int ixp(int l, int n) { return l < n - 1 ? l + 1 : 0; }
__device__ __forceinline__ int ixm(int l, int n) { return l > 0 ? l - 1 : n - 1; }
__device__ __forceinline__ int izp(int k, int n) { return k < n - 1 ? k + 1 : n - 1; }
__device__ __forceinline__ int izm(int k, int n) { return k > 0 ? k - 1 : 0; }

template <typename T>
struct Field {
    const T *__restrict__ p;
    int nx, ny, nz;
    size_t plane;
    __device__ __forceinline__ T at(int g, int l, int m, int k) const {
        return __ldg(p + (size_t)g * plane + ((size_t)l * ny + m) * nz + k);
    }
};

struct Vec3 {
    double x, y, z;
};

// grad_phi_xyz (:94-107) of phase g at cell (l,m,k)
template <typename T>
__device__ __forceinline__ Vec3 grad_at(const Field<T> &f, int g, int l, int m, int k, double two_dx) {
    int lp = ixp(l, f.nx), lm = ixm(l, f.nx), mp = ixp(m, f.ny), mm = ixm(m, f.ny);
    int kp = izp(k, f.nz), km = izm(k, f.nz);
    Vec3 r;
    r.x = (double)(T)(f.at(g, lp, m, k) - f.at(g, lm, m, k)) / two_dx;
    r.y = (double)(T)(f.at(g, l, mp, k) - f.at(g, l, mm, k)) / two_dx;
    r.z = (double)(T)(f.at(g, l, m, kp) - f.at(g, l, m, km)) / two_dx;
    return r;
}

// One search over the 8 rotated {111} normals gives both
// best_cos_from_grad_3d (:110-134, float64 result) and
// facet_cos_and_nxyz_from_grad (:251-301, float32 results): the two
// functions evaluate the same dot products in the same order.
struct Facet {
    int valid;           // q >= g2_floor
    double best64;       // best_cos_from_grad_3d
    float cs, ca, nx, ny, nz;
};

__device__ __forceinline__ Facet facet(const Vec3 &g, const float *__restrict__ u, double g2_floor) {
    Facet f;
    double q = g.x * g.x + g.y * g.y + g.z * g.z;
    if (q < g2_floor) {
        f.valid = 0; f.best64 = 0.0; f.cs = 0.0f; f.ca = 0.0f; f.nx = 1.0f; f.ny = 0.0f; f.nz = 0.0f;
        return f;
    }
    double inv_g = 1.0 / sqrt(q);
    double gx = g.x * inv_g, gy = g.y * inv_g, gz = g.z * inv_g;
    double best_abs = 0.0, best_signed = 0.0, bx = 1.0, by = 0.0, bz = 0.0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        double ux = (double)u[3 * t], uy = (double)u[3 * t + 1], uz = (double)u[3 * t + 2];
        double dot = gx * ux + gy * uy + gz * uz;
        double ad = fabs(dot);
        if (ad > best_abs) {
            best_abs = ad; best_signed = dot; bx = ux; by = uy; bz = uz;
        }
    }
    if (best_abs > 1.0) best_abs = 1.0;
    if (best_signed > 1.0) best_signed = 1.0;
    if (best_signed < -1.0) best_signed = -1.0;
    f.valid = 1;
    f.best64 = best_abs;
    f.cs = (float)best_signed; f.ca = (float)best_abs;
    f.nx = (float)bx; f.ny = (float)by; f.nz = (float)bz;
    return f;
}

// calc_a_from_cos (:24-30) with a float64 cosine
__device__ __forceinline__ double calc_a64(const Params &P, double tan_a0, double cost) {
    double c2 = cost * cost;
    double C = sqrt(c2 + P.pp);
    double om = 1.0 - c2;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + P.pp);
    return P.mu_a * (1.0 + P.delta_a * (C + tan_a0 * S));
}

// calc_a_from_cos with a float32 cosine (the f32-cast facet value)
__device__ __forceinline__ double calc_a32(const Params &P, double tan_a0, float cost) {
    float c2f = cost * cost;
    double c2 = (double)c2f;
    double C = P.p32 ? (double)sqrtf(c2f + (float)P.pp) : sqrt(c2 + P.pp);
    double om = 1.0 - c2;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + P.pp);
    return P.mu_a * (1.0 + P.delta_a * (C + tan_a0 * S));
}

// calc_b_from_cos (:33-55)
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

// coef = (c/C) - tan(a0)*(c/S) of da_dphixyz_A12 / torque_A11_3d (:327-330, :423-426)
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
    float a, x, y, z;
};

// da_dphixyz_A12 (:304-341) from the liquid gradient and facet at a point
__device__ __forceinline__ DA da_dphi(const Params &P, double tan_a0, const Vec3 &g, const Facet &f) {
    DA r;
    if (!f.valid) {
        r.a = r.x = r.y = r.z = 0.0f;
        return r;
    }
    double q = g.x * g.x + g.y * g.y + g.z * g.z;
    double a_val = calc_a32(P, tan_a0, f.ca);
    double inv_g = 1.0 / sqrt(q);
    double inv_g3 = 1.0 / (q * sqrt(q));
    double udotg = g.x * (double)f.nx + g.y * (double)f.ny + g.z * (double)f.nz;
    double dcx = (double)f.nx * inv_g - udotg * g.x * inv_g3;
    double dcy = (double)f.ny * inv_g - udotg * g.y * inv_g3;
    double dcz = (double)f.nz * inv_g - udotg * g.z * inv_g3;
    double coef = dadc_coef(P, tan_a0, f.cs);
    r.a = (float)a_val;
    r.x = (float)(P.mu_da * coef * dcx);
    r.y = (float)(P.mu_da * coef * dcy);
    r.z = (float)(P.mu_da * coef * dcz);
    return r;
}

// ---------------------------------------------------------------------------
// APT (:462-527)
template <typename T>
__global__ void __launch_bounds__(256) apt_kernel(Field<T> phi, int N, int32_t *__restrict__ mf,
                                                  int depth, int32_t *__restrict__ nf,
                                                  int32_t *__restrict__ status, int checked,
                                                  int32_t *__restrict__ err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int m = blockIdx.y * blockDim.y + threadIdx.y;
    int l = blockIdx.z * blockDim.z + threadIdx.z;
    bool inside = (k < phi.nz) && (m < phi.ny) && (l < phi.nx);
    int n = 0;
    bool ovf = false, deep = false;
    if (inside) {
        int lp = ixp(l, phi.nx), lm = ixm(l, phi.nx), mp = ixp(m, phi.ny), mm = ixm(m, phi.ny);
        int kp = izp(k, phi.nz), km = izm(k, phi.nz);
        size_t cell = ((size_t)l * phi.ny + m) * phi.nz + k;
        const T zero = (T)0;
        for (int i = 0; i < N; ++i) {
            T v = phi.at(i, l, m, k);
            bool act = (v > zero) ||
                       ((v == zero) && ((phi.at(i, lp, m, k) > zero) || (phi.at(i, lm, m, k) > zero) ||
                                        (phi.at(i, l, mp, k) > zero) || (phi.at(i, l, mm, k) > zero) ||
                                        (phi.at(i, l, m, kp) > zero) || (phi.at(i, l, m, km) > zero)));
            if (act) {
                n += 1;
                int lim = checked ? KMAX : depth;
                if (n <= lim && n <= depth) mf[(size_t)(n - 1) * phi.plane + cell] = i;
                else if (!checked) deep = true;
            }
        }
        if (checked && n > KMAX) {
            ovf = true;
            nf[cell] = KMAX;
        } else {
            nf[cell] = (!checked && n > depth) ? depth : n;
        }
    }
    if (checked) {
        // warp-aggregated atomic max: same final values as one atomic per cell
        int wmax = n;
        for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
        unsigned any_ovf = __ballot_sync(0xffffffffu, ovf);
        if ((threadIdx.x & 31) == 0 && blockDim.x >= 32) {
            if (any_ovf) atomicMax(status + 0, 1);
            atomicMax(status + 1, wmax);
        }
    }
    if (deep && err) atomicOr(err, MPF3D_DEV_MF_DEPTH);
}

// ---------------------------------------------------------------------------
// Phase update (:530-830)
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
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int m = blockIdx.y * blockDim.y + threadIdx.y;
    int l = blockIdx.z * blockDim.z + threadIdx.z;
    if (k >= P.nz || m >= P.ny || l >= P.nx) return;
    const int N = P.N;
    const size_t plane = phi.plane;
    const size_t cell = ((size_t)l * P.ny + m) * P.nz + k;
    const int n = nf[cell];
    if (n < 0 || n > KMAX) {
        if (err) atomicOr(err, MPF3D_DEV_NF_GT_KMAX);
        return;
    }
    if (n > P.depth) {  // mf holds fewer rows than nf claims
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
    const int lp = ixp(l, P.nx), lm = ixm(l, P.nx), mp = ixp(m, P.ny), mm = ixm(m, P.ny);
    const int kp = izp(k, P.nz), km = izm(k, P.nz);
    // stencil points: 0 c, 1 x+, 2 x-, 3 y+, 4 y-, 5 z+, 6 z- (clamped/periodic)
    const int pl[7] = {l, lp, lm, l, l, l, l};
    const int pm[7] = {m, m, m, mp, mm, m, m};
    const int pk[7] = {k, k, k, k, k, kp, km};

    float lap_sl[KMAX], b_sl[KMAX];
    bool any_solid = false;
    for (int t = 0; t < n; ++t) any_solid |= (ids[t] != LIQ);

    if (any_solid) {
        Vec3 G[7];
        if (P.use_aniso) {
#pragma unroll
            for (int p = 0; p < 7; ++p) G[p] = grad_at(phi, LIQ, pl[p], pm[p], pk[p], P.two_dx);
        }
        double lap_liq = 0.0;
        if (!P.use_aniso) {
            T s = phi.at(LIQ, lp, m, k) + phi.at(LIQ, lm, m, k);
            s = s + phi.at(LIQ, l, mp, k);
            s = s + phi.at(LIQ, l, mm, k);
            s = s + phi.at(LIQ, l, m, kp);
            s = s + phi.at(LIQ, l, m, km);
            lap_liq = ((double)s - 6.0 * (double)phi.at(LIQ, l, m, k)) * P.inv_dx2;
        }
        for (int t = 0; t < n; ++t) {
            int gid = ids[t];
            if (gid == LIQ) {
                b_sl[t] = 1.0f;
                lap_sl[t] = 0.0f;
                continue;
            }
            if (!P.use_aniso) {
                lap_sl[t] = (float)(P.eps0sq * lap_liq);
                b_sl[t] = 1.0f;
                continue;
            }
            const float *u = n111 + (size_t)gid * 24;
            Facet F[7];
#pragma unroll
            for (int p = 0; p < 7; ++p) F[p] = facet(G[p], u, P.g2_floor);
            // aniso_term1_solid_3d (:149-204)
            double e2[7];
#pragma unroll
            for (int p = 0; p < 7; ++p) {
                double e = P.eps0 * calc_a64(P, tan_a0, F[p].best64);
                e2[p] = e * e;
            }
            T pc = phi.at(LIQ, l, m, k);
            T pv[7];
#pragma unroll
            for (int p = 1; p < 7; ++p) pv[p] = phi.at(LIQ, pl[p], pm[p], pk[p]);
            double Fxp = (e2[0] + e2[1]) * (double)(T)(pv[1] - pc) / P.two_dx;
            double Fxm = (e2[0] + e2[2]) * (double)(T)(pc - pv[2]) / P.two_dx;
            double Fyp = (e2[0] + e2[3]) * (double)(T)(pv[3] - pc) / P.two_dx;
            double Fym = (e2[0] + e2[4]) * (double)(T)(pc - pv[4]) / P.two_dx;
            double Fzp = (e2[0] + e2[5]) * (double)(T)(pv[5] - pc) / P.two_dx;
            double Fzm = (e2[0] + e2[6]) * (double)(T)(pc - pv[6]) / P.two_dx;
            double lap_val = (Fxp - Fxm) / P.dx + (Fyp - Fym) / P.dx + (Fzp - Fzm) / P.dx;
            // torque_A11_3d (:386-441)
            if (P.use_torque && F[0].valid) {
                const Vec3 g0 = G[0];
                double q = g0.x * g0.x + g0.y * g0.y + g0.z * g0.z;
                // d2_phi_xyz (:207-248) of the liquid
                T xp = pv[1], xm = pv[2], yp = pv[3], ym = pv[4], zp = pv[5], zm = pv[6];
                double pxx = ((double)xp - 2.0 * (double)pc + (double)xm) * P.inv_dx2;
                double pyy = ((double)yp - 2.0 * (double)pc + (double)ym) * P.inv_dx2;
                double pzz = ((double)zp - 2.0 * (double)pc + (double)zm) * P.inv_dx2;
                double qq = 0.25 * P.inv_dx2;
                double pxy = (double)(T)(((T)(phi.at(LIQ, lp, mp, k) - phi.at(LIQ, lp, mm, k)) - phi.at(LIQ, lm, mp, k)) +
                                         phi.at(LIQ, lm, mm, k)) * qq;
                double pxz = (double)(T)(((T)(phi.at(LIQ, lp, m, kp) - phi.at(LIQ, lp, m, km)) - phi.at(LIQ, lm, m, kp)) +
                                         phi.at(LIQ, lm, m, km)) * qq;
                double pyz = (double)(T)(((T)(phi.at(LIQ, l, mp, kp) - phi.at(LIQ, l, mp, km)) - phi.at(LIQ, l, mm, kp)) +
                                         phi.at(LIQ, l, mm, km)) * qq;
                double q_x = 2.0 * (g0.x * pxx + g0.y * pxy + g0.z * pxz);
                double q_y = 2.0 * (g0.x * pxy + g0.y * pyy + g0.z * pyz);
                double q_z = 2.0 * (g0.x * pxz + g0.y * pyz + g0.z * pzz);
                DA d0 = da_dphi(P, tan_a0, g0, F[0]);
                const Facet &f0 = F[0];
                double inv_g = 1.0 / sqrt(q);
                double inv_g3 = 1.0 / (q * sqrt(q));
                double udotg = g0.x * (double)f0.nx + g0.y * (double)f0.ny + g0.z * (double)f0.nz;
                double dcx = (double)f0.nx * inv_g - udotg * g0.x * inv_g3;
                double dcy = (double)f0.ny * inv_g - udotg * g0.y * inv_g3;
                double dcz = (double)f0.nz * inv_g - udotg * g0.z * inv_g3;
                double cxx = dcx * pxx + dcy * pxy + dcz * pxz;
                double cyy = dcx * pxy + dcy * pyy + dcz * pyz;
                double czz = dcx * pxz + dcy * pyz + dcz * pzz;
                double coef = dadc_coef(P, tan_a0, f0.cs);
                double da_dx = P.mu_da * coef * cxx;
                double da_dy = P.mu_da * coef * cyy;
                double da_dz = P.mu_da * coef * czz;
                // A13_divergence_3d (:344-383)
                float ddx = (float)((double)(da_dphi(P, tan_a0, G[1], F[1]).x - da_dphi(P, tan_a0, G[2], F[2]).x) *
                                    P.half_over_dx);
                float ddy = (float)((double)(da_dphi(P, tan_a0, G[3], F[3]).y - da_dphi(P, tan_a0, G[4], F[4]).y) *
                                    P.half_over_dx);
                float ddz = (float)((double)(da_dphi(P, tan_a0, G[5], F[5]).z - da_dphi(P, tan_a0, G[6], F[6]).z) *
                                    P.half_over_dx);
                float a = d0.a;
                double Ex = (da_dx * (double)d0.x * q) + ((double)(a * ddx) * q) + ((double)(a * d0.x) * q_x);
                double Ey = (da_dy * (double)d0.y * q) + ((double)(a * ddy) * q) + ((double)(a * d0.y) * q_y);
                double Ez = (da_dz * (double)d0.z * q) + ((double)(a * ddz) * q) + ((double)(a * d0.z) * q_z);
                lap_val += P.eps0sq * (Ex + Ey + Ez);
            }
            lap_sl[t] = (float)lap_val;
            b_sl[t] = (float)calc_b(P, F[0].best64);
        }
    } else {
        for (int t = 0; t < n; ++t) {
            b_sl[t] = 1.0f;
            lap_sl[t] = 0.0f;
        }
    }

    // dominant solid and anisotropic w_sl (:579-595)
    int i_s = -1;
    double maxv = -1.0;
    for (int t = 0; t < n; ++t) {
        int gid = ids[t];
        if (gid == LIQ) continue;
        double v = (double)phi.at(gid, l, m, k);
        if (v > maxv) {
            maxv = v;
            i_s = gid;
        }
    }
    double w_sl = P.w0;
    if (P.use_aniso && i_s != -1) {
        Vec3 gs = grad_at(phi, i_s, l, m, k, P.two_dx);
        Facet fs = facet(gs, n111 + (size_t)i_s * 24, P.g2_floor);
        double al = calc_a64(P, tan_a0, fs.best64);
        w_sl = P.w0 * (al * al);
    }

    for (int g = 0; g < N; ++g) phi_new[(size_t)g * plane + cell] = (T)0;

    // per-phase value and Laplacian at the cell (laplacian_3d :444-459)
    T phc[KMAX];
    double lapk[KMAX];
    for (int t = 0; t < n; ++t) {
        int g = ids[t];
        phc[t] = phi.at(g, l, m, k);
        T s = phi.at(g, lp, m, k) + phi.at(g, lm, m, k);
        s = s + phi.at(g, l, mp, k);
        s = s + phi.at(g, l, mm, k);
        s = s + phi.at(g, l, m, kp);
        s = s + phi.at(g, l, m, km);
        lapk[t] = ((double)s - 6.0 * (double)phc[t]) * P.inv_dx2;
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
                const int pk3 = ids[t3];
                double wik = (double)__ldg(wij + i * N + pk3), wjk = (double)__ldg(wij + j * N + pk3);
                if (pk3 == LIQ) {
                    if (i != LIQ) wik = w_sl;
                    if (j != LIQ) wjk = w_sl;
                }
                double term1 = (wik - wjk) * (double)phc[t3];
                double term2 = 0.0;
                if (j == LIQ && i != LIQ) {
                    if (pk3 == i) term2 = 0.5 * (double)lap_sl[t1];
                } else if (i == LIQ && j != LIQ) {
                    if (pk3 == j) term2 = -0.5 * (double)lap_sl[t2];
                } else {
                    float ai = __ldg(aij + i * N + pk3), aj = __ldg(aij + j * N + pk3);
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
    // clip and renormalise (:663-680)
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

// kernel_update_temp_3d (:833-838)
template <typename TT>
__global__ void temp_kernel(TT *__restrict__ temp, double rate, int rate32, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        if (sizeof(TT) == 4 && rate32)
            temp[i] = (TT)((float)temp[i] - (float)rate);
        else
            temp[i] = (TT)((double)temp[i] - rate);
    }
}

}  // namespace dense
}  // namespace mpf3d

using namespace mpf3d;
using namespace mpf3d::dense;

static inline int bitset(uint32_t m, int i) { return (int)((m >> i) & 1u); }

static dim3 cell_grid(int nx, int ny, int nz, dim3 blk) {
    return dim3((nz + blk.x - 1) / blk.x, (ny + blk.y - 1) / blk.y, (nx + blk.z - 1) / blk.z);
}

static bool grid_ok(int nx, int ny, int nz) {
    return nx > 0 && ny > 0 && nz > 0 && ny <= 65535 * 4 && nx <= 65535;
}

extern "C" int mpf3d_version(void) { return MPF3D_VERSION; }

extern "C" int mpf3d_dense_apt(const void *phi, int phi_dtype, int N, int nx, int ny, int nz, int32_t *mf,
                               int depth, int32_t *nf, int32_t *status, int checked, int32_t *err,
                               void *stream) {
    if (!phi || !mf || !nf || N <= 0 || depth <= 0 || !grid_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    if (checked && !status) return MPF3D_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 blk(32, 4, 2);
    dim3 grd = cell_grid(nx, ny, nz, blk);
    size_t plane = (size_t)nx * ny * nz;
    if (phi_dtype == MPF3D_F32) {
        Field<float> f{(const float *)phi, nx, ny, nz, plane};
        apt_kernel<float><<<grd, blk, 0, s>>>(f, N, mf, depth, nf, status, checked, err);
    } else if (phi_dtype == MPF3D_F64) {
        Field<double> f{(const double *)phi, nx, ny, nz, plane};
        apt_kernel<double><<<grd, blk, 0, s>>>(f, N, mf, depth, nf, status, checked, err);
    } else {
        return MPF3D_ERR_DTYPE;
    }
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

template <typename T, typename TT>
static void launch_update(const void *phi, void *phi_new, const void *temp, const int32_t *mf, const int32_t *nf,
                          const float *wij, const float *aij, const float *mij, const float *n111, const Params &P,
                          int32_t *err, cudaStream_t s) {
    dim3 blk(32, 4, 1);
    dim3 grd = cell_grid(P.nx, P.ny, P.nz, blk);
    Field<T> f{(const T *)phi, P.nx, P.ny, P.nz, (size_t)P.nx * P.ny * P.nz};
    update_kernel<T, TT><<<grd, blk, 0, s>>>(f, (T *)phi_new, (const TT *)temp, mf, nf, wij, aij, mij, n111, P, err);
}

extern "C" int mpf3d_dense_update(const void *phi, void *phi_new, int phi_dtype, const void *temp, int temp_dtype,
                                  const int32_t *mf, int depth, const int32_t *nf, const float *wij,
                                  const float *aij, const float *mij, const float *n111, int N, int nx, int ny,
                                  int nz, const mpf3d_scalars *sc, int switchable, int enable_anisotropy,
                                  int enable_torque, int32_t *err, void *stream) {
    if (!phi || !phi_new || !temp || !mf || !nf || !wij || !aij || !mij || !n111 || !sc) return MPF3D_ERR_ARG;
    if (N <= 0 || N > 65535 || depth <= 0 || !grid_ok(nx, ny, nz)) return MPF3D_ERR_ARG;
    if ((phi_dtype != MPF3D_F32 && phi_dtype != MPF3D_F64) || (temp_dtype != MPF3D_F32 && temp_dtype != MPF3D_F64))
        return MPF3D_ERR_DTYPE;
    Params P;
    P.N = N; P.nx = nx; P.ny = ny; P.nz = nz; P.depth = depth;
    const double *v = sc->v;
    const uint32_t fm = sc->f32mask;
    P.dx = v[MPF3D_S_DX]; P.dt = v[MPF3D_S_DT]; P.T_melt = v[MPF3D_S_T_MELT]; P.Sf = v[MPF3D_S_SF];
    P.eps0 = v[MPF3D_S_EPS0_SL]; P.w0 = v[MPF3D_S_W0_SL]; P.a0 = v[MPF3D_S_A0]; P.delta_a = v[MPF3D_S_DELTA_A];
    P.mu_a = v[MPF3D_S_MU_A]; P.p_round = v[MPF3D_S_P_ROUND]; P.g2_floor = v[MPF3D_S_G2_FLOOR];
    P.ksi = v[MPF3D_S_KSI]; P.theta_c = v[MPF3D_S_THETA_C_RAD];
    P.two_dx = 2.0 * P.dx;
    P.half_over_dx = 0.5 / P.dx;
    if (bitset(fm, MPF3D_S_DX)) {
        float d = (float)P.dx;
        P.inv_dx2 = 1.0 / (double)(d * d);
    } else {
        P.inv_dx2 = 1.0 / (P.dx * P.dx);
    }
    P.p32 = bitset(fm, MPF3D_S_P_ROUND);
    P.pp = P.p32 ? (double)((float)P.p_round * (float)P.p_round) : P.p_round * P.p_round;
    P.mu_da = (bitset(fm, MPF3D_S_MU_A) && bitset(fm, MPF3D_S_DELTA_A))
                  ? (double)((float)P.mu_a * (float)P.delta_a)
                  : P.mu_a * P.delta_a;
    P.eps0sq = bitset(fm, MPF3D_S_EPS0_SL) ? (double)((float)P.eps0 * (float)P.eps0) : P.eps0 * P.eps0;
    P.a0_32 = bitset(fm, MPF3D_S_A0);
    P.dT32 = (temp_dtype == MPF3D_F32) && bitset(fm, MPF3D_S_T_MELT);
    P.df32 = P.dT32 && bitset(fm, MPF3D_S_SF);
    P.switchable = switchable;
    P.use_aniso = switchable ? (enable_anisotropy != 0) : 1;
    P.use_torque = switchable ? (enable_anisotropy != 0 && enable_torque != 0) : 1;
    cudaStream_t s = (cudaStream_t)stream;
    if (phi_dtype == MPF3D_F32 && temp_dtype == MPF3D_F32)
        launch_update<float, float>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    else if (phi_dtype == MPF3D_F32)
        launch_update<float, double>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    else if (temp_dtype == MPF3D_F32)
        launch_update<double, float>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    else
        launch_update<double, double>(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, P, err, s);
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}

extern "C" int mpf3d_dense_temp(void *temp, int temp_dtype, double rate, int rate_is_f32, int64_t n, void *stream) {
    if (!temp || n < 0) return MPF3D_ERR_ARG;
    if (n == 0) return MPF3D_OK;
    if (rate_is_f32) rate = (double)(float)rate;
    cudaStream_t s = (cudaStream_t)stream;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (temp_dtype == MPF3D_F32)
        temp_kernel<float><<<blocks, 256, 0, s>>>((float *)temp, rate, rate_is_f32, n);
    else if (temp_dtype == MPF3D_F64)
        temp_kernel<double><<<blocks, 256, 0, s>>>((double *)temp, rate, rate_is_f32, n);
    else
        return MPF3D_ERR_DTYPE;
    return cudaGetLastError() == cudaSuccess ? MPF3D_OK : MPF3D_ERR_CUDA;
}
