/*
 * mpf3d_oracle.c -- CPU oracle for the 3D multi-phase-field step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA kernels of
 * the package and the CPU baseline of bench.py; no product code links it.
 *
 * It restates, cell by cell and expression by expression, the reference's
 * src/gpu_kernels_3d.py (daikihatanaka0327/multiphasefield-solidification-v2):
 *   calc_a_from_cos            :24-30      calc_b_from_cos          :33-55
 *   idx_xp/xm/yp/ym/zp/zm      :58-91      grad_phi_xyz             :94-107
 *   best_cos_from_grad_3d      :110-134    eps2_at_cell_from_liquid :137-146
 *   aniso_term1_solid_3d       :149-204    d2_phi_xyz               :207-248
 *   facet_cos_and_nxyz         :251-301    da_dphixyz_A12           :304-341
 *   A13_divergence_3d          :344-383    torque_A11_3d            :386-441
 *   laplacian_3d               :444-459    kernel_update_nfmf_3d    :462-486
 *   kernel_update_nfmf_3d_checked :489-527
 *   kernel_update_phasefield_active_3d            :530-680
 *   kernel_update_phasefield_active_3d_switchable :683-830
 *   kernel_update_temp_3d      :833-838
 *
 * Arithmetic types follow compiled Numba: Python float literals are float64
 * and float32 op float64 promotes to float64, so most arithmetic is double;
 * float32 survives where the reference casts with float32(...), stores into
 * its float32 local arrays lap_sl/b_sl, or combines two float32 values
 * (phi differences when phi is float32, aij*aij, mij*b_sl, the f32-cast
 * cosine squared, ...).  Which scalar arguments were float32 is carried in
 * a bit mask, because it changes the type of several expressions.
 *
 * Build with -ffp-contract=off (no fused multiply-add), as the reference's
 * NVVM pipeline does not contract without fastmath.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define LIQ 0
#define MPF_PI 3.14159265358979323846

enum {
    S_DX = 0, S_DT, S_TMELT, S_SF, S_EPS0, S_W0, S_A0, S_DELTA_A, S_MU_A, S_P_ROUND,
    S_G2_FLOOR, S_KSI, S_THETA_C, S_COUNT
};

typedef struct {
    double v[S_COUNT];   /* scalar values (exactly representable as float when marked f32) */
    uint32_t f32mask;    /* bit i set: scalar i was passed as a float32 */
} mpf3d_oracle_scalars;

typedef struct {
    const void *phi;
    int phi64;
    int N, nx, ny, nz;
    const float *n111;
    /* derived, typed as the reference computes them */
    double dx, two_dx, half_over_dx, inv_dx2;
    double pp;       /* p_round*p_round */
    int p32;         /* p_round is float32 */
    double tan_a0;   /* math.tan(a0) */
    double mu_a, delta_a, mu_da; /* mu_a*delta_a */
    double eps0, eps0sq;
    double g2_floor, ksi, theta_c;
} ctx_t;

static inline int bit(const mpf3d_oracle_scalars *s, int i) { return (s->f32mask >> i) & 1u; }

static inline int ixp(int l, int n) { return l < n - 1 ? l + 1 : 0; }
static inline int ixm(int l, int n) { return l > 0 ? l - 1 : n - 1; }
static inline int izp(int k, int n) { return k < n - 1 ? k + 1 : n - 1; }
static inline int izm(int k, int n) { return k > 0 ? k - 1 : 0; }

static inline size_t cidx(const ctx_t *c, int g, int l, int m, int k) {
    return (((size_t)g * c->nx + l) * c->ny + m) * c->nz + k;
}

static inline double P(const ctx_t *c, int g, int l, int m, int k) {
    size_t i = cidx(c, g, l, m, k);
    return c->phi64 ? ((const double *)c->phi)[i] : (double)((const float *)c->phi)[i];
}

/* a - b of two phi values: float32 subtraction when phi is float32 */
static inline double psub(const ctx_t *c, double a, double b) {
    return c->phi64 ? a - b : (double)((float)a - (float)b);
}
static inline double padd(const ctx_t *c, double a, double b) {
    return c->phi64 ? a + b : (double)((float)a + (float)b);
}
static inline double pmul(const ctx_t *c, double a, double b) {
    return c->phi64 ? a * b : (double)((float)a * (float)b);
}

static void ctx_init(ctx_t *c, const mpf3d_oracle_scalars *s) {
    c->dx = s->v[S_DX];
    c->two_dx = 2.0 * c->dx;
    c->half_over_dx = 0.5 / c->dx;
    if (bit(s, S_DX)) {
        float d = (float)c->dx;
        c->inv_dx2 = 1.0 / (double)(d * d);
    } else {
        c->inv_dx2 = 1.0 / (c->dx * c->dx);
    }
    double p = s->v[S_P_ROUND];
    c->p32 = bit(s, S_P_ROUND);
    c->pp = c->p32 ? (double)((float)p * (float)p) : p * p;
    double a0 = s->v[S_A0];
    c->tan_a0 = bit(s, S_A0) ? (double)tanf((float)a0) : tan(a0);
    c->mu_a = s->v[S_MU_A];
    c->delta_a = s->v[S_DELTA_A];
    c->mu_da = (bit(s, S_MU_A) && bit(s, S_DELTA_A)) ? (double)((float)c->mu_a * (float)c->delta_a)
                                                     : c->mu_a * c->delta_a;
    c->eps0 = s->v[S_EPS0];
    c->eps0sq = bit(s, S_EPS0) ? (double)((float)c->eps0 * (float)c->eps0) : c->eps0 * c->eps0;
    c->g2_floor = s->v[S_G2_FLOOR];
    c->ksi = s->v[S_KSI];
    c->theta_c = s->v[S_THETA_C];
}

/* calc_a_from_cos (:24-30).  cost32: the cosine argument is a float32 value. */
static double calc_a(const ctx_t *c, double cost, int cost32) {
    double c2, C;
    if (cost32) {
        float c2f = (float)cost * (float)cost;
        c2 = (double)c2f;
        C = c->p32 ? (double)sqrtf(c2f + (float)c->pp) : sqrt(c2 + c->pp);
    } else {
        c2 = cost * cost;
        C = sqrt(c2 + c->pp);
    }
    double om = 1.0 - c2;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + c->pp);
    return c->mu_a * (1.0 + c->delta_a * (C + c->tan_a0 * S));
}

/* calc_b_from_cos (:33-55) */
static double calc_b(const ctx_t *cx, double best_cost) {
    double c = best_cost;
    if (c > 1.0) c = 1.0;
    else if (c < -1.0) c = -1.0;
    double theta = acos(c);
    if (theta >= cx->theta_c) return 1.0;
    double x = theta / cx->theta_c;
    double eps = 1.0e-6;
    double hp = 0.5 * MPF_PI;
    double y = hp * x;
    if (y > hp - eps) y = hp - eps;
    if (y < eps) y = eps;
    double t = tan(y);
    return cx->ksi + (1.0 - cx->ksi) * t * tanh(1.0 / t);
}

/* grad_phi_xyz (:94-107) */
static void grad(const ctx_t *c, int g, int l, int m, int k, double *gx, double *gy, double *gz) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = ixp(m, c->ny), mm = ixm(m, c->ny);
    int kp = izp(k, c->nz), km = izm(k, c->nz);
    *gx = psub(c, P(c, g, lp, m, k), P(c, g, lm, m, k)) / c->two_dx;
    *gy = psub(c, P(c, g, l, mp, k), P(c, g, l, mm, k)) / c->two_dx;
    *gz = psub(c, P(c, g, l, m, kp), P(c, g, l, m, km)) / c->two_dx;
}

/* best_cos_from_grad_3d (:110-134) */
static double best_cos(const ctx_t *c, double gx, double gy, double gz, int sid) {
    double g2 = gx * gx + gy * gy + gz * gz;
    if (g2 < c->g2_floor) return 0.0;
    double inv_g = 1.0 / sqrt(g2);
    double nxn = gx * inv_g, nyn = gy * inv_g, nzn = gz * inv_g;
    double best = 0.0;
    const float *u = c->n111 + (size_t)sid * 24;
    for (int t = 0; t < 8; ++t) {
        double v = fabs(nxn * (double)u[3 * t] + nyn * (double)u[3 * t + 1] + nzn * (double)u[3 * t + 2]);
        if (v > best) best = v;
    }
    if (best > 1.0) best = 1.0;
    return best;
}

/* eps2_at_cell_from_liquid_3d (:137-146) */
static double eps2_at(const ctx_t *c, int l, int m, int k, int sid) {
    double gx, gy, gz;
    grad(c, LIQ, l, m, k, &gx, &gy, &gz);
    double bc = best_cos(c, gx, gy, gz, sid);
    double a = calc_a(c, bc, 0);
    double e = c->eps0 * a;
    return e * e;
}

/* aniso_term1_solid_3d (:149-204) */
static double aniso_term1(const ctx_t *c, int l, int m, int k, int sid) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = ixp(m, c->ny), mm = ixm(m, c->ny);
    int kp = izp(k, c->nz), km = izm(k, c->nz);
    double ec = eps2_at(c, l, m, k, sid);
    double exp_ = eps2_at(c, lp, m, k, sid), exm = eps2_at(c, lm, m, k, sid);
    double eyp = eps2_at(c, l, mp, k, sid), eym = eps2_at(c, l, mm, k, sid);
    double ezp = eps2_at(c, l, m, kp, sid), ezm = eps2_at(c, l, m, km, sid);
    double pc = P(c, LIQ, l, m, k);
    double pxp = P(c, LIQ, lp, m, k), pxm = P(c, LIQ, lm, m, k);
    double pyp = P(c, LIQ, l, mp, k), pym = P(c, LIQ, l, mm, k);
    double pzp = P(c, LIQ, l, m, kp), pzm = P(c, LIQ, l, m, km);
    double Fxp = (ec + exp_) * psub(c, pxp, pc) / c->two_dx;
    double Fxm = (ec + exm) * psub(c, pc, pxm) / c->two_dx;
    double Fyp = (ec + eyp) * psub(c, pyp, pc) / c->two_dx;
    double Fym = (ec + eym) * psub(c, pc, pym) / c->two_dx;
    double Fzp = (ec + ezp) * psub(c, pzp, pc) / c->two_dx;
    double Fzm = (ec + ezm) * psub(c, pc, pzm) / c->two_dx;
    return (Fxp - Fxm) / c->dx + (Fyp - Fym) / c->dx + (Fzp - Fzm) / c->dx;
}

/* d2_phi_xyz (:207-248) */
static void d2(const ctx_t *c, int g, int l, int m, int k, double o[6]) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = ixp(m, c->ny), mm = ixm(m, c->ny);
    int kp = izp(k, c->nz), km = izm(k, c->nz);
    double pc = P(c, g, l, m, k);
    double xp = P(c, g, lp, m, k), xm = P(c, g, lm, m, k);
    double yp = P(c, g, l, mp, k), ym = P(c, g, l, mm, k);
    double zp = P(c, g, l, m, kp), zm = P(c, g, l, m, km);
    double inv = c->inv_dx2;
    o[0] = (xp - 2.0 * pc + xm) * inv;
    o[1] = (yp - 2.0 * pc + ym) * inv;
    o[2] = (zp - 2.0 * pc + zm) * inv;
    double q = 0.25 * inv;
    o[3] = padd(c, psub(c, psub(c, P(c, g, lp, mp, k), P(c, g, lp, mm, k)), P(c, g, lm, mp, k)),
                P(c, g, lm, mm, k)) * q;
    o[4] = padd(c, psub(c, psub(c, P(c, g, lp, m, kp), P(c, g, lp, m, km)), P(c, g, lm, m, kp)),
                P(c, g, lm, m, km)) * q;
    o[5] = padd(c, psub(c, psub(c, P(c, g, l, mp, kp), P(c, g, l, mp, km)), P(c, g, l, mm, kp)),
                P(c, g, l, mm, km)) * q;
}

/* facet_cos_and_nxyz_from_grad (:251-301): float32 results */
static void facet(const ctx_t *c, double phix, double phiy, double phiz, int sid, float o[5]) {
    double q = phix * phix + phiy * phiy + phiz * phiz;
    if (q < c->g2_floor) {
        o[0] = 0.0f; o[1] = 0.0f; o[2] = 1.0f; o[3] = 0.0f; o[4] = 0.0f;
        return;
    }
    double inv_g = 1.0 / sqrt(q);
    double gx = phix * inv_g, gy = phiy * inv_g, gz = phiz * inv_g;
    double best_abs = 0.0, best_signed = 0.0, bnx = 1.0, bny = 0.0, bnz = 0.0;
    const float *u = c->n111 + (size_t)sid * 24;
    for (int t = 0; t < 8; ++t) {
        double ux = u[3 * t], uy = u[3 * t + 1], uz = u[3 * t + 2];
        double dot = gx * ux + gy * uy + gz * uz;
        double ad = fabs(dot);
        if (ad > best_abs) {
            best_abs = ad; best_signed = dot; bnx = ux; bny = uy; bnz = uz;
        }
    }
    if (best_abs > 1.0) best_abs = 1.0;
    if (best_signed > 1.0) best_signed = 1.0;
    if (best_signed < -1.0) best_signed = -1.0;
    o[0] = (float)best_signed; o[1] = (float)best_abs;
    o[2] = (float)bnx; o[3] = (float)bny; o[4] = (float)bnz;
}

/* coef = (c / C) - tan(a0) * (c / S) with c the float32 signed cosine */
static double dadc_coef(const ctx_t *cx, float cs) {
    float ccf = cs * cs;
    double C, coef;
    if (cx->p32) {
        float Cf = sqrtf(ccf + (float)cx->pp);
        C = Cf;
        double om = 1.0 - (double)ccf;
        if (!(om >= 0.0)) om = 0.0;
        double S = sqrt(om + cx->pp);
        coef = (double)(cs / Cf) - cx->tan_a0 * ((double)cs / S);
    } else {
        C = sqrt((double)ccf + cx->pp);
        double om = 1.0 - (double)ccf;
        if (!(om >= 0.0)) om = 0.0;
        double S = sqrt(om + cx->pp);
        coef = ((double)cs / C) - cx->tan_a0 * ((double)cs / S);
    }
    (void)C;
    return coef;
}

/* da_dphixyz_A12 (:304-341): (a, da/dphix, da/dphiy, da/dphiz) as float32 */
static void da_dphi(const ctx_t *c, int l, int m, int k, int sid, float o[4]) {
    double phix, phiy, phiz;
    grad(c, LIQ, l, m, k, &phix, &phiy, &phiz);
    double q = phix * phix + phiy * phiy + phiz * phiz;
    if (q < c->g2_floor) {
        o[0] = o[1] = o[2] = o[3] = 0.0f;
        return;
    }
    float f[5];
    facet(c, phix, phiy, phiz, sid, f);
    double a_val = calc_a(c, (double)f[1], 1);
    double inv_g = 1.0 / sqrt(q);
    double inv_g3 = 1.0 / (q * sqrt(q));
    double udotg = phix * (double)f[2] + phiy * (double)f[3] + phiz * (double)f[4];
    double dcx = (double)f[2] * inv_g - udotg * phix * inv_g3;
    double dcy = (double)f[3] * inv_g - udotg * phiy * inv_g3;
    double dcz = (double)f[4] * inv_g - udotg * phiz * inv_g3;
    double coef = dadc_coef(c, f[0]);
    o[0] = (float)a_val;
    o[1] = (float)(c->mu_da * coef * dcx);
    o[2] = (float)(c->mu_da * coef * dcy);
    o[3] = (float)(c->mu_da * coef * dcz);
}

/* A13_divergence_3d (:344-383) */
static void a13(const ctx_t *c, int l, int m, int k, int sid, float o[3]) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = ixp(m, c->ny), mm = ixm(m, c->ny);
    int kp = izp(k, c->nz), km = izm(k, c->nz);
    float a[4], b[4];
    da_dphi(c, lp, m, k, sid, a);
    da_dphi(c, lm, m, k, sid, b);
    o[0] = (float)((double)(a[1] - b[1]) * c->half_over_dx);
    da_dphi(c, l, mp, k, sid, a);
    da_dphi(c, l, mm, k, sid, b);
    o[1] = (float)((double)(a[2] - b[2]) * c->half_over_dx);
    da_dphi(c, l, m, kp, sid, a);
    da_dphi(c, l, m, km, sid, b);
    o[2] = (float)((double)(a[3] - b[3]) * c->half_over_dx);
}

/* torque_A11_3d (:386-441) */
static double torque(const ctx_t *c, int l, int m, int k, int sid) {
    double phix, phiy, phiz;
    grad(c, LIQ, l, m, k, &phix, &phiy, &phiz);
    double q = phix * phix + phiy * phiy + phiz * phiz;
    if (q < c->g2_floor) return 0.0;
    double h[6];
    d2(c, LIQ, l, m, k, h);
    double pxx = h[0], pyy = h[1], pzz = h[2], pxy = h[3], pxz = h[4], pyz = h[5];
    double q_x = 2.0 * (phix * pxx + phiy * pxy + phiz * pxz);
    double q_y = 2.0 * (phix * pxy + phiy * pyy + phiz * pyz);
    double q_z = 2.0 * (phix * pxz + phiy * pyz + phiz * pzz);
    float da[4];
    da_dphi(c, l, m, k, sid, da);
    float f[5];
    facet(c, phix, phiy, phiz, sid, f);
    double inv_g = 1.0 / sqrt(q);
    double inv_g3 = 1.0 / (q * sqrt(q));
    double udotg = phix * (double)f[2] + phiy * (double)f[3] + phiz * (double)f[4];
    double dcx = (double)f[2] * inv_g - udotg * phix * inv_g3;
    double dcy = (double)f[3] * inv_g - udotg * phiy * inv_g3;
    double dcz = (double)f[4] * inv_g - udotg * phiz * inv_g3;
    double cxx = dcx * pxx + dcy * pxy + dcz * pxz;
    double cyy = dcx * pxy + dcy * pyy + dcz * pyz;
    double czz = dcx * pxz + dcy * pyz + dcz * pzz;
    double coef = dadc_coef(c, f[0]);
    double da_dx = c->mu_da * coef * cxx;
    double da_dy = c->mu_da * coef * cyy;
    double da_dz = c->mu_da * coef * czz;
    float dd[3];
    a13(c, l, m, k, sid, dd);
    float a = da[0];
    double Ex = (da_dx * (double)da[1] * q) + ((double)(a * dd[0]) * q) + ((double)(a * da[1]) * q_x);
    double Ey = (da_dy * (double)da[2] * q) + ((double)(a * dd[1]) * q) + ((double)(a * da[2]) * q_y);
    double Ez = (da_dz * (double)da[3] * q) + ((double)(a * dd[2]) * q) + ((double)(a * da[3]) * q_z);
    return c->eps0sq * (Ex + Ey + Ez);
}

/* laplacian_3d (:444-459), also the inline Laplacian of :620-625 */
static double lap(const ctx_t *c, int g, int l, int m, int k) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = ixp(m, c->ny), mm = ixm(m, c->ny);
    int kp = izp(k, c->nz), km = izm(k, c->nz);
    double s = padd(c, P(c, g, lp, m, k), P(c, g, lm, m, k));
    s = padd(c, s, P(c, g, l, mp, k));
    s = padd(c, s, P(c, g, l, mm, k));
    s = padd(c, s, P(c, g, l, m, kp));
    s = padd(c, s, P(c, g, l, m, km));
    return (s - 6.0 * P(c, g, l, m, k)) * c->inv_dx2;
}

/* ------------------------------------------------------------------------ */
/* APT: kernel_update_nfmf_3d (:462-486) and the checked variant (:489-527).
 * Returns 0, or -1 when an unchecked rebuild would write past mf's depth
 * (the reference has no guard there).  status may be NULL when unchecked. */
int mpf3d_oracle_apt(const void *phi, int phi64, int N, int nx, int ny, int nz, int32_t *mf,
                     int depth, int32_t *nf, int32_t *status, int checked, int kmax) {
    ctx_t c;
    memset(&c, 0, sizeof c);
    c.phi = phi; c.phi64 = phi64; c.N = N; c.nx = nx; c.ny = ny; c.nz = nz;
    size_t plane = (size_t)nx * ny * nz;
    int err = 0, ovf = 0, nmax = 0;
#pragma omp parallel for collapse(2) schedule(static) reduction(| : err, ovf) reduction(max : nmax)
    for (int l = 0; l < nx; ++l)
        for (int m = 0; m < ny; ++m)
            for (int k = 0; k < nz; ++k) {
                int lp = ixp(l, nx), lm = ixm(l, nx), mp = ixp(m, ny), mm = ixm(m, ny);
                int kp = izp(k, nz), km = izm(k, nz);
                size_t cell = ((size_t)l * ny + m) * nz + k;
                int n = 0;
                for (int i = 0; i < N; ++i) {
                    double v = P(&c, i, l, m, k);
                    int act = (v > 0.0) || ((v == 0.0) && ((P(&c, i, lp, m, k) > 0.0) || (P(&c, i, lm, m, k) > 0.0) ||
                                                         (P(&c, i, l, mp, k) > 0.0) || (P(&c, i, l, mm, k) > 0.0) ||
                                                         (P(&c, i, l, m, kp) > 0.0) || (P(&c, i, l, m, km) > 0.0)));
                    if (act) {
                        n += 1;
                        if (checked) {
                            if (n <= kmax) mf[(size_t)(n - 1) * plane + cell] = i;
                        } else if (n <= depth) {
                            mf[(size_t)(n - 1) * plane + cell] = i;
                        } else {
                            err = 1;
                        }
                    }
                }
                if (checked && n > kmax) {
                    ovf = 1;
                    nf[cell] = kmax;
                } else {
                    nf[cell] = n;
                }
                if (n > nmax) nmax = n;
            }
    if (checked && status) {
        if (ovf && status[0] < 1) status[0] = 1;
        if (nmax > status[1]) status[1] = nmax;
    }
    return err ? -1 : 0;
}

/* kernel_update_temp_3d (:833-838) */
void mpf3d_oracle_temp(void *temp, int temp64, double rate, int rate32, int64_t n) {
    if (rate32) rate = (double)(float)rate;
    if (temp64) {
        double *t = (double *)temp;
        for (int64_t i = 0; i < n; ++i) t[i] -= rate;
    } else {
        float *t = (float *)temp;
        for (int64_t i = 0; i < n; ++i)
            t[i] = rate32 ? t[i] - (float)rate : (float)((double)t[i] - rate);
    }
}

/* Phase update: kernel_update_phasefield_active_3d (:530-680) when
 * switchable == 0, else kernel_update_phasefield_active_3d_switchable
 * (:683-830) with the two toggles.  Returns 0, -2 for nf > kmax, -3 for an
 * mf entry outside [0, N). */
int mpf3d_oracle_update(const void *phi, void *phi_new, int phi64, const void *temp, int temp64,
                        const int32_t *mf, int depth, const int32_t *nf, const float *wij,
                        const float *aij, const float *mij, const float *n111, int N, int nx,
                        int ny, int nz, const mpf3d_oracle_scalars *s, int switchable, int aniso,
                        int torque_on, int kmax) {
    ctx_t c;
    memset(&c, 0, sizeof c);
    c.phi = phi; c.phi64 = phi64; c.N = N; c.nx = nx; c.ny = ny; c.nz = nz; c.n111 = n111;
    ctx_init(&c, s);
    size_t plane = (size_t)nx * ny * nz;
    const double dt = s->v[S_DT], Tm = s->v[S_TMELT], Sf = s->v[S_SF], w0 = s->v[S_W0];
    const int dT32 = !temp64 && bit(s, S_TMELT);
    const int df32 = dT32 && bit(s, S_SF);
    const int use_aniso = switchable ? (aniso != 0) : 1;
    const int use_torque = switchable ? (aniso != 0 && torque_on != 0) : 1;
    int err = 0;
    (void)depth;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(min : err)
    for (int l = 0; l < nx; ++l)
        for (int m = 0; m < ny; ++m)
            for (int k = 0; k < nz; ++k) {
                size_t cell = ((size_t)l * ny + m) * nz + k;
                double Tcur = temp64 ? ((const double *)temp)[cell] : (double)((const float *)temp)[cell];
                int n = nf[cell];
                if (n > kmax || n < 0) { err = -2; continue; }
                int ids[64];
                int bad = 0;
                for (int t = 0; t < n; ++t) {
                    ids[t] = mf[(size_t)t * plane + cell];
                    if (ids[t] < 0 || ids[t] >= N) bad = 1;
                }
                if (bad) { err = -3; continue; }
                float lap_sl[64], b_sl[64];
                double gxl, gyl, gzl;
                grad(&c, LIQ, l, m, k, &gxl, &gyl, &gzl);
                double lap_liq = switchable ? lap(&c, LIQ, l, m, k) : 0.0;
                for (int t = 0; t < n; ++t) {
                    int gid = ids[t];
                    if (gid == LIQ) {
                        b_sl[t] = 1.0f;
                        lap_sl[t] = 0.0f;
                    } else if (use_aniso) {
                        double lv = aniso_term1(&c, l, m, k, gid);
                        if (use_torque) lv += torque(&c, l, m, k, gid);
                        lap_sl[t] = (float)lv;
                        b_sl[t] = (float)calc_b(&c, best_cos(&c, gxl, gyl, gzl, gid));
                    } else {
                        lap_sl[t] = (float)(c.eps0sq * lap_liq);
                        b_sl[t] = 1.0f;
                    }
                }
                int i_s = -1;
                double maxv = -1.0;
                for (int t = 0; t < n; ++t) {
                    int gid = ids[t];
                    if (gid == LIQ) continue;
                    double v = P(&c, gid, l, m, k);
                    if (v > maxv) { maxv = v; i_s = gid; }
                }
                double w_sl = w0;
                if (use_aniso && i_s != -1) {
                    double px, py, pz;
                    grad(&c, i_s, l, m, k, &px, &py, &pz);
                    double cm = best_cos(&c, px, py, pz, i_s);
                    double al = calc_a(&c, cm, 0);
                    w_sl = w0 * (al * al);
                }
                for (int g = 0; g < N; ++g) {
                    size_t o = (size_t)g * plane + cell;
                    if (phi64) ((double *)phi_new)[o] = 0.0; else ((float *)phi_new)[o] = 0.0f;
                }
                double dTv = dT32 ? (double)((float)Tcur - (float)Tm) : Tcur - Tm;
                for (int t1 = 0; t1 < n; ++t1) {
                    int i = ids[t1];
                    double dpi = 0.0;
                    for (int t2 = 0; t2 < n; ++t2) {
                        int j = ids[t2];
                        if (i == j) continue;
                        double df = 0.0;
                        if (i != LIQ && j == LIQ)
                            df = df32 ? (double)(-(float)Sf * (float)dTv) : (-Sf) * dTv;
                        else if (i == LIQ && j != LIQ)
                            df = df32 ? (double)((float)Sf * (float)dTv) : Sf * dTv;
                        double ppp = 0.0;
                        for (int t3 = 0; t3 < n; ++t3) {
                            int pk = ids[t3];
                            double phk = P(&c, pk, l, m, k);
                            double lapk = lap(&c, pk, l, m, k);
                            double wik = wij[i * N + pk], wjk = wij[j * N + pk];
                            if (pk == LIQ) {
                                if (i != LIQ) wik = w_sl;
                                if (j != LIQ) wjk = w_sl;
                            }
                            double term1 = (wik - wjk) * phk;
                            double term2 = 0.0;
                            if (j == LIQ && i != LIQ) {
                                if (pk == i) term2 = 0.5 * (double)lap_sl[t1];
                            } else if (i == LIQ && j != LIQ) {
                                if (pk == j) term2 = -0.5 * (double)lap_sl[t2];
                            } else {
                                float e2i = aij[i * N + pk] * aij[i * N + pk];
                                float e2j = aij[j * N + pk] * aij[j * N + pk];
                                term2 = 0.5 * (double)(e2i - e2j) * lapk;
                            }
                            ppp += term1 + term2;
                        }
                        double pij = pmul(&c, P(&c, i, l, m, k), P(&c, j, l, m, k));
                        double tf = (8.0 / 3.1415926535) * sqrt(pij > 0.0 ? pij : 0.0) * df;
                        float me = mij[i * N + j];
                        if (i != LIQ && j == LIQ) me = mij[i * N + j] * b_sl[t1];
                        else if (i == LIQ && j != LIQ) me = mij[i * N + j] * b_sl[t2];
                        dpi -= 2.0 * (double)me / (double)n * (ppp - tf);
                    }
                    double nv = P(&c, i, l, m, k) + dt * dpi;
                    size_t o = (size_t)i * plane + cell;
                    if (phi64) ((double *)phi_new)[o] = nv; else ((float *)phi_new)[o] = (float)nv;
                }
                double ssum = 0.0;
                for (int t = 0; t < n; ++t) {
                    size_t o = (size_t)ids[t] * plane + cell;
                    double v = phi64 ? ((double *)phi_new)[o] : (double)((float *)phi_new)[o];
                    if (v < 0.0) v = 0.0;
                    if (v > 1.0) v = 1.0;
                    if (phi64) ((double *)phi_new)[o] = v; else ((float *)phi_new)[o] = (float)v;
                    ssum += v;
                }
                if (ssum > 1e-20) {
                    double invs = 1.0 / ssum;
                    for (int t = 0; t < n; ++t) {
                        size_t o = (size_t)ids[t] * plane + cell;
                        if (phi64) ((double *)phi_new)[o] *= invs;
                        else ((float *)phi_new)[o] = (float)((double)((float *)phi_new)[o] * invs);
                    }
                } else {
                    size_t o = cell;
                    if (phi64) ((double *)phi_new)[o] = 1.0; else ((float *)phi_new)[o] = 1.0f;
                }
            }
    return err;
}
