/*
 * mpf2d_oracle.c -- CPU oracle for the 2D multi-phase-field step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the 2D CUDA kernels
 * of the package; no product code links it.
 *
 * It restates the reference's src/gpu_kernels.py
 * (daikihatanaka0327/multiphasefield-solidification-v2), the 2D module that
 * the reference's tests/verification_3d.py:21-25 imports for its
 * two_d_limit_consistency case:
 *   calc_a_from_cos                 :25-31    calc_b_from_cos        :34-79
 *   idx_xp/xm (periodic x)          :84-93    idx_yp/ym (mirror y)   :96-105
 *   grad_phi_xy                     :108-115  best_cos_from_grad     :120-136
 *   eps2_at_cell_from_liquid        :141-150  aniso_term1_solid      :155-179
 *   d2_phi_xy                       :184-202  facet_cos_and_nxy      :207-232
 *   da_dphixy_A12                   :237-264  A13 differences        :269-285
 *   torque_A11                      :290-332  kernel_update_nfmf     :337-358
 *   kernel_update_phasefield_active :361-517  kernel_update_temp     :520-525
 *
 * Arithmetic types follow compiled Numba, as in the 3D oracle: Python float
 * literals are float64, float32 op float64 promotes to float64, float32
 * survives in float32(...) casts, the float32 local arrays lap_sl/b_sl and
 * products/differences of two float32 values.  Which scalar arguments were
 * float32 is carried in a bit mask.  Build with -ffp-contract=off.
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
    double v[S_COUNT];
    uint32_t f32mask;
} mpf2d_oracle_scalars;

typedef struct {
    const void *phi;
    int phi64;
    int N, nx, ny;
    const float *n111;
    double dx, two_dx, half_over_dx, inv_dx2, pp, tan_a0, mu_a, delta_a, mu_da, eps0, eps0sq;
    double g2_floor, ksi, theta_c;
    int p32;
} ctx2_t;

static inline int bit(const mpf2d_oracle_scalars *s, int i) { return (s->f32mask >> i) & 1u; }

static inline int ixp(int l, int n) { return l < n - 1 ? l + 1 : 0; }
static inline int ixm(int l, int n) { return l > 0 ? l - 1 : n - 1; }
static inline int iyp(int m, int n) { return m < n - 1 ? m + 1 : n - 1; }
static inline int iym(int m, int n) { return m > 0 ? m - 1 : 0; }

static inline size_t cidx(const ctx2_t *c, int g, int l, int m) {
    return ((size_t)g * c->nx + l) * c->ny + m;
}

static inline double P(const ctx2_t *c, int g, int l, int m) {
    size_t i = cidx(c, g, l, m);
    return c->phi64 ? ((const double *)c->phi)[i] : (double)((const float *)c->phi)[i];
}

/* phi op phi in phi's type */
static inline double psub(const ctx2_t *c, double a, double b) {
    return c->phi64 ? a - b : (double)((float)a - (float)b);
}
static inline double padd(const ctx2_t *c, double a, double b) {
    return c->phi64 ? a + b : (double)((float)a + (float)b);
}
static inline double pmul(const ctx2_t *c, double a, double b) {
    return c->phi64 ? a * b : (double)((float)a * (float)b);
}

static void ctx_init(ctx2_t *c, const mpf2d_oracle_scalars *s) {
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

/* calc_a_from_cos (:25-31); cost32: the cosine is a float32 value */
static double calc_a(const ctx2_t *c, double cost, int cost32) {
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

/* calc_b_from_cos (:34-79) */
static double calc_b(const ctx2_t *cx, double best_cost) {
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

/* grad_phi_xy (:108-115) */
static void grad(const ctx2_t *c, int g, int l, int m, double *gx, double *gy) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = iyp(m, c->ny), mm = iym(m, c->ny);
    *gx = psub(c, P(c, g, lp, m), P(c, g, lm, m)) / c->two_dx;
    *gy = psub(c, P(c, g, l, mp), P(c, g, l, mm)) / c->two_dx;
}

/* best_cos_from_grad (:120-136): only the x and y components of the normals */
static double best_cos(const ctx2_t *c, double gx, double gy, int sid) {
    double g2 = gx * gx + gy * gy;
    if (g2 < c->g2_floor) return 0.0;
    double inv_g = 1.0 / sqrt(g2);
    double nxn = gx * inv_g, nyn = gy * inv_g;
    double best = 0.0;
    const float *u = c->n111 + (size_t)sid * 24;
    for (int t = 0; t < 8; ++t) {
        double v = fabs(nxn * (double)u[3 * t] + nyn * (double)u[3 * t + 1]);
        if (v > best) best = v;
    }
    if (best > 1.0) best = 1.0;
    return best;
}

/* eps2_at_cell_from_liquid (:141-150) */
static double eps2_at(const ctx2_t *c, int l, int m, int sid) {
    double gx, gy;
    grad(c, LIQ, l, m, &gx, &gy);
    double a = calc_a(c, best_cos(c, gx, gy, sid), 0);
    double e = c->eps0 * a;
    return e * e;
}

/* aniso_term1_solid (:155-179) */
static double aniso_term1(const ctx2_t *c, int l, int m, int sid) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = iyp(m, c->ny), mm = iym(m, c->ny);
    double ec = eps2_at(c, l, m, sid);
    double exp_ = eps2_at(c, lp, m, sid), exm = eps2_at(c, lm, m, sid);
    double eyp = eps2_at(c, l, mp, sid), eym = eps2_at(c, l, mm, sid);
    double pc = P(c, LIQ, l, m);
    double pxp = P(c, LIQ, lp, m), pxm = P(c, LIQ, lm, m);
    double pyp = P(c, LIQ, l, mp), pym = P(c, LIQ, l, mm);
    double Fxp = (ec + exp_) * psub(c, pxp, pc) / c->two_dx;
    double Fxm = (ec + exm) * psub(c, pc, pxm) / c->two_dx;
    double Fyp = (ec + eyp) * psub(c, pyp, pc) / c->two_dx;
    double Fym = (ec + eym) * psub(c, pc, pym) / c->two_dx;
    return (Fxp - Fxm) / c->dx + (Fyp - Fym) / c->dx;
}

/* d2_phi_xy (:184-202) */
static void d2(const ctx2_t *c, int g, int l, int m, double *pxx, double *pyy, double *pxy) {
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = iyp(m, c->ny), mm = iym(m, c->ny);
    double cc = P(c, g, l, m);
    double xp = P(c, g, lp, m), xm = P(c, g, lm, m), yp = P(c, g, l, mp), ym = P(c, g, l, mm);
    *pxx = (xp - 2.0 * cc + xm) * c->inv_dx2;
    *pyy = (yp - 2.0 * cc + ym) * c->inv_dx2;
    double s = psub(c, P(c, g, lp, mp), P(c, g, lp, mm));
    s = psub(c, s, P(c, g, lm, mp));
    s = padd(c, s, P(c, g, lm, mm));
    *pxy = s * (0.25 * c->inv_dx2);
}

typedef struct {
    int valid;
    float cs, ca, nx, ny;
} facet_t;

/* facet_cos_and_nxy_from_grad (:207-232) */
static facet_t facet(const ctx2_t *c, double phix, double phiy, int sid) {
    facet_t f;
    double q = phix * phix + phiy * phiy;
    if (q < c->g2_floor) {
        f.valid = 0; f.cs = 0.0f; f.ca = 0.0f; f.nx = 1.0f; f.ny = 0.0f;
        return f;
    }
    double inv_g = 1.0 / sqrt(q);
    double gx = phix * inv_g, gy = phiy * inv_g;
    double best_abs = 0.0, best_signed = 0.0, bx = 1.0, by = 0.0;
    const float *u = c->n111 + (size_t)sid * 24;
    for (int t = 0; t < 8; ++t) {
        double ux = (double)u[3 * t], uy = (double)u[3 * t + 1];
        double dot = gx * ux + gy * uy;
        double ad = fabs(dot);
        if (ad > best_abs) { best_abs = ad; best_signed = dot; bx = ux; by = uy; }
    }
    if (best_abs > 1.0) best_abs = 1.0;
    if (best_signed > 1.0) best_signed = 1.0;
    if (best_signed < -1.0) best_signed = -1.0;
    f.valid = 1;
    f.cs = (float)best_signed; f.ca = (float)best_abs; f.nx = (float)bx; f.ny = (float)by;
    return f;
}

/* coef = (c/C) - tan(a0)*(c/S) with the float32 signed cosine c */
static double dadc_coef(const ctx2_t *c, float cs) {
    float ccf = cs * cs;
    double om = 1.0 - (double)ccf;
    if (!(om >= 0.0)) om = 0.0;
    double S = sqrt(om + c->pp);
    if (c->p32) {
        float Cf = sqrtf(ccf + (float)c->pp);
        return (double)(cs / Cf) - c->tan_a0 * ((double)cs / S);
    }
    double C = sqrt((double)ccf + c->pp);
    return ((double)cs / C) - c->tan_a0 * ((double)cs / S);
}

/* da_dphixy_A12 (:237-264): float32 (a, da/dphix, da/dphiy) */
static void da_dphi(const ctx2_t *c, int l, int m, int sid, float *a, float *dx_, float *dy_) {
    double phix, phiy;
    grad(c, LIQ, l, m, &phix, &phiy);
    double q = phix * phix + phiy * phiy;
    if (q < c->g2_floor) { *a = *dx_ = *dy_ = 0.0f; return; }
    facet_t f = facet(c, phix, phiy, sid);
    double a_val = calc_a(c, (double)f.ca, 1);
    double g = sqrt(q), inv_g = 1.0 / g, inv_g3 = 1.0 / (q * g);
    double udotg = phix * (double)f.nx + phiy * (double)f.ny;
    double dcx = (double)f.nx * inv_g - udotg * phix * inv_g3;
    double dcy = (double)f.ny * inv_g - udotg * phiy * inv_g3;
    double coef = dadc_coef(c, f.cs);
    *a = (float)a_val;
    *dx_ = (float)(c->mu_da * coef * dcx);
    *dy_ = (float)(c->mu_da * coef * dcy);
}

/* torque_A11 (:290-332) with the A13 differences (:269-285) */
static double torque(const ctx2_t *c, int l, int m, int sid) {
    double phix, phiy;
    grad(c, LIQ, l, m, &phix, &phiy);
    double q = phix * phix + phiy * phiy;
    if (q < c->g2_floor) return 0.0;
    double pxx, pyy, pxy;
    d2(c, LIQ, l, m, &pxx, &pyy, &pxy);
    double q_x = 2.0 * (phix * pxx + phiy * pxy);
    double q_y = 2.0 * (phix * pxy + phiy * pyy);
    float a_val, dax, day;
    da_dphi(c, l, m, sid, &a_val, &dax, &day);
    facet_t f = facet(c, phix, phiy, sid);
    double g = sqrt(q), inv_g = 1.0 / g, inv_g3 = 1.0 / (q * g);
    double udotg = phix * (double)f.nx + phiy * (double)f.ny;
    double dcx = (double)f.nx * inv_g - udotg * phix * inv_g3;
    double dcy = (double)f.ny * inv_g - udotg * phiy * inv_g3;
    double cx = dcx * pxx + dcy * pxy;
    double cy = dcx * pxy + dcy * pyy;
    double coef = dadc_coef(c, f.cs);
    double da_dx = c->mu_da * coef * cx;
    double da_dy = c->mu_da * coef * cy;
    int lp = ixp(l, c->nx), lm = ixm(l, c->nx), mp = iyp(m, c->ny), mm = iym(m, c->ny);
    float t0, t1, xp_, xm_, yp_, ym_;
    da_dphi(c, lp, m, sid, &t0, &xp_, &t1);
    da_dphi(c, lm, m, sid, &t0, &xm_, &t1);
    da_dphi(c, l, mp, sid, &t0, &t1, &yp_);
    da_dphi(c, l, mm, sid, &t0, &t1, &ym_);
    float ddx = (float)((double)(xp_ - xm_) * c->half_over_dx);
    float ddy = (float)((double)(yp_ - ym_) * c->half_over_dx);
    double Ex = (da_dx * (double)dax * q) + ((double)(a_val * ddx) * q) + ((double)(a_val * dax) * q_x);
    double Ey = (da_dy * (double)day * q) + ((double)(a_val * ddy) * q) + ((double)(a_val * day) * q_y);
    return c->eps0sq * (Ex + Ey);
}

/* kernel_update_nfmf (:337-358).  Returns -1 when a cell has more active
 * phases than mf's depth (the reference would write past mf). */
int mpf2d_oracle_apt(const void *phi, int phi64, int N, int nx, int ny, int32_t *mf, int depth, int32_t *nf) {
    ctx2_t c;
    memset(&c, 0, sizeof c);
    c.phi = phi; c.phi64 = phi64; c.N = N; c.nx = nx; c.ny = ny;
    size_t plane = (size_t)nx * ny;
    int err = 0;
    for (int l = 0; l < nx; ++l)
        for (int m = 0; m < ny; ++m) {
            int lp = ixp(l, nx), lm = ixm(l, nx), mp = iyp(m, ny), mm = iym(m, ny);
            size_t cell = (size_t)l * ny + m;
            int n = 0;
            for (int i = 0; i < N; ++i) {
                double v = P(&c, i, l, m);
                int act = (v > 0.0) || ((v == 0.0) && ((P(&c, i, lp, m) > 0.0) || (P(&c, i, lm, m) > 0.0) ||
                                                     (P(&c, i, l, mp) > 0.0) || (P(&c, i, l, mm) > 0.0)));
                if (act) {
                    n += 1;
                    if (n <= depth) mf[(size_t)(n - 1) * plane + cell] = i;
                    else err = 1;
                }
            }
            nf[cell] = n;
        }
    return err ? -1 : 0;
}

/* kernel_update_phasefield_active (:361-517).  Returns 0, -2 for nf > kmax,
 * -3 for an mf entry outside [0, N). */
int mpf2d_oracle_update(const void *phi, void *phi_new, int phi64, const void *temp, int temp64,
                        const int32_t *mf, const int32_t *nf, const float *wij, const float *aij,
                        const float *mij, const float *n111, int N, int nx, int ny,
                        const mpf2d_oracle_scalars *s, int kmax) {
    ctx2_t c;
    memset(&c, 0, sizeof c);
    c.phi = phi; c.phi64 = phi64; c.N = N; c.nx = nx; c.ny = ny; c.n111 = n111;
    ctx_init(&c, s);
    size_t plane = (size_t)nx * ny;
    const double dt = s->v[S_DT], Tm = s->v[S_TMELT], Sf = s->v[S_SF], w0 = s->v[S_W0];
    const int dT32 = !temp64 && bit(s, S_TMELT);
    const int df32 = dT32 && bit(s, S_SF);
    int err = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(min : err)
    for (int l = 0; l < nx; ++l)
        for (int m = 0; m < ny; ++m) {
            size_t cell = (size_t)l * ny + m;
            int lp = ixp(l, nx), lm = ixm(l, nx), mp = iyp(m, ny), mm = iym(m, ny);
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
            for (int t = 0; t < n; ++t) {
                int gid = ids[t];
                if (gid == LIQ) {
                    b_sl[t] = 1.0f;
                    lap_sl[t] = 0.0f;
                } else {
                    lap_sl[t] = (float)aniso_term1(&c, l, m, gid);
                    lap_sl[t] = (float)((double)lap_sl[t] + torque(&c, l, m, gid));
                    double gx, gy;
                    grad(&c, LIQ, l, m, &gx, &gy);
                    b_sl[t] = (float)calc_b(&c, best_cos(&c, gx, gy, gid));
                }
            }
            /* dominant solid grain for the anisotropic w_sl (:410-436) */
            int i_s = 1;
            double maxv = 0.0;
            for (int t = 0; t < n; ++t) {
                int gid = ids[t];
                if (gid == LIQ) continue;
                double v = P(&c, gid, l, m);
                if (v > maxv) { maxv = v; i_s = gid; }
            }
            double phx = psub(&c, P(&c, i_s, lp, m), P(&c, i_s, lm, m)) * c.half_over_dx;
            double phy = psub(&c, P(&c, i_s, l, mp), P(&c, i_s, l, mm)) * c.half_over_dx;
            double gn2 = phx * phx + phy * phy;
            double cmax = 0.0;
            if (gn2 >= c.g2_floor) {
                double inv_gn = 1.0 / sqrt(gn2);
                double ux = phx * inv_gn, uy = phy * inv_gn;
                const float *u = n111 + (size_t)i_s * 24;
                for (int tt = 0; tt < 8; ++tt) {
                    double cv = fabs(ux * (double)u[3 * tt] + uy * (double)u[3 * tt + 1]);
                    if (cv > cmax) cmax = cv;
                }
                if (cmax > 1.0) cmax = 1.0;
            }
            double a_loc = calc_a(&c, cmax, 0);
            double w_sl = w0 * (a_loc * a_loc);
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
                        int k = ids[t3];
                        double sum4 = padd(&c, P(&c, k, lp, m), P(&c, k, lm, m));
                        sum4 = padd(&c, sum4, P(&c, k, l, mp));
                        sum4 = padd(&c, sum4, P(&c, k, l, mm));
                        double phk = P(&c, k, l, m);
                        double lap_k = (sum4 - 4.0 * phk) * c.inv_dx2;
                        double wik = wij[i * N + k], wjk = wij[j * N + k];
                        if (k == LIQ) {
                            if (i != LIQ) wik = w_sl;
                            if (j != LIQ) wjk = w_sl;
                        }
                        double term1 = (wik - wjk) * phk;
                        double term2 = 0.0;
                        if (j == LIQ && i != LIQ) {
                            if (k == i) term2 = 0.5 * (double)lap_sl[t1];
                        } else if (i == LIQ && j != LIQ) {
                            if (k == j) term2 = -0.5 * (double)lap_sl[t2];
                        } else {
                            float e2i = aij[i * N + k] * aij[i * N + k];
                            float e2j = aij[j * N + k] * aij[j * N + k];
                            term2 = 0.5 * (double)(e2i - e2j) * lap_k;
                        }
                        ppp += term1 + term2;
                    }
                    double pij = pmul(&c, P(&c, i, l, m), P(&c, j, l, m));
                    double tf = (8.0 / 3.1415926535) * sqrt(pij > 0.0 ? pij : 0.0) * df;
                    float me = mij[i * N + j];
                    if (i != LIQ && j == LIQ) me = mij[i * N + j] * b_sl[t1];
                    else if (i == LIQ && j != LIQ) me = mij[i * N + j] * b_sl[t2];
                    dpi -= 2.0 * (double)me / (double)n * (ppp - tf);
                }
                double nv = P(&c, i, l, m) + dt * dpi;
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
                if (phi64) ((double *)phi_new)[cell] = 1.0; else ((float *)phi_new)[cell] = 1.0f;
            }
        }
    return err;
}
