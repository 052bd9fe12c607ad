/*
 * adjoint64.c -- TEST INFRASTRUCTURE ONLY: FP64 model of the SPH step with
 * frozen integer structure, and its hand-written reverse-mode adjoint.
 *
 * The step is the reference's (fluids4.0/fluid_kernels.cu: computePressure
 * 112-149, computeForce 180-217, advanceParticles 332-420) evaluated in
 * double, with the per-step sort permutation and the neighbour pairs taken
 * as given ("frozen": the integer path carries no gradient). The adjoint
 * here checks the GPU adjoint, and is itself checked against central finite
 * differences of adj64_forward (tests/test_adjoint_oracle.py).
 *
 * Layout: n points, T steps. For step t, in sorted-slot order s:
 *   perm[t*n + s]   pre-sort index gathered into slot s
 *   inr[t*n + s]    1 if the point is inside the scan range
 *   poff[t*(n+1) + s] .. poff[t*(n+1) + s + 1]: its pairs in pnbr (slot ids)
 *   time[t]         the simulation time of step t
 * States are n x 3 doubles in the order before the step.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/fluids_gb300.h"

#define EPSD 0.00001   /* EPSILON, fluids4.0/fluid_kernels.cuh:17 */

typedef struct {
    double m, poly6, spiky, lap, visc, rho0, kap, h, ss, d2, rd2;
    double pr, slope, kb, damp, fric, wf, wfreq, bmin[3], bmax[3], g[3], AL, VL, dt;
} P64;

static P64 p64(const fl_params *p, const double *theta) {
    P64 q;
    q.m = p->pmass;
    q.h = p->psmoothradius;
    q.ss = p->sim_scale;
    q.d2 = q.ss * q.ss;
    q.rd2 = (q.h * q.h) / q.d2;
    q.poly6 = 315.0 / (64.0 * M_PI * pow(q.h, 9.0));
    q.spiky = -45.0 / (M_PI * pow(q.h, 6.0));
    q.lap = 45.0 / (M_PI * pow(q.h, 6.0));
    q.visc = theta ? theta[0] : p->pvisc;
    q.rho0 = theta ? theta[1] : p->prest_dens;
    q.kap = theta ? theta[2] : p->pintstiff;
    q.pr = p->pradius; q.slope = p->bound_slope; q.kb = p->bound_stiff; q.damp = p->bound_damp;
    q.fric = p->bound_friction; q.wf = p->bound_wall_force; q.wfreq = p->bound_wall_freq;
    for (int k = 0; k < 3; k++) {
        q.bmin[k] = p->bound_min[k]; q.bmax[k] = p->bound_max[k]; q.g[k] = p->gravity[k];
    }
    q.AL = p->AL; q.VL = p->VL; q.dt = p->dt;
    return q;
}

/* ---- one step, forward ---------------------------------------------------- */

/* Accumulated wall acceleration and the values the adjoint needs. */
typedef struct {
    double a[3];      /* before the accel clamp */
    double ac[3];     /* after */
    double vc[3];     /* clamped velocity */
    int aclamp, vclamp;
} AdvTape;

/* Branch decisions of one point's advance: bits 0-5 the walls (Y-, Y+, X-,
 * X+, Z-, Z+) acting, bit 6 the AccelLimit clamp, bit 7 the VelLimit clamp.
 * mode 0 decides from the values; 1 decides and records into *mk; 2 takes
 * the recorded decisions (the decisions frozen, as the adjoint treats them). */
static int decide(int mode, uint8_t *mk, int bit, int cond) {
    if (mode == 2) return (*mk >> bit) & 1;
    if (mode == 1) *mk = (uint8_t)((*mk & ~(1u << bit)) | ((cond ? 1u : 0u) << bit));
    return cond;
}

static void walls(const P64 *q, double t, const double *X, const double *E, double *a, uint8_t *mk, int mode) {
    double diff, adj, nx, ny, nz;
    diff = q->pr - (X[1] - (q->bmin[1] + (X[0] - q->bmin[0]) * q->slope)) * q->ss;
    if (decide(mode, mk, 0, diff > EPSD)) {
        nx = -q->slope; ny = 1.0 - q->slope; nz = 0.0;
        adj = q->kb * diff - q->damp * (nx * E[0] + ny * E[1] + nz * E[2]);
        a[0] += nx * adj - E[0] * q->fric; a[1] += ny * adj - E[1] * q->fric; a[2] += nz * adj - E[2] * q->fric;
    }
    diff = q->pr - (q->bmax[1] - X[1]) * q->ss;
    if (decide(mode, mk, 1, diff > EPSD)) {
        adj = q->kb * diff - q->damp * (-E[1]);
        a[0] += -E[0] * q->fric; a[1] += -adj - E[1] * q->fric; a[2] += -E[2] * q->fric;
    }
    const double wall = (sin(t * q->wfreq + X[2] / 400.0) * 0.5 + 0.5) * q->wf;
    diff = q->pr - (X[0] - (q->bmin[0] + wall)) * q->ss;
    if (decide(mode, mk, 2, diff > EPSD)) a[0] += wall * q->kb * diff - q->damp * E[0];
    diff = q->pr - (q->bmax[0] - X[0]) * q->ss;
    if (decide(mode, mk, 3, diff > EPSD)) a[0] += -(q->kb * diff - q->damp * (-E[0]));
    diff = q->pr - (X[2] - q->bmin[2]) * q->ss;
    if (decide(mode, mk, 4, diff > EPSD)) a[2] += q->kb * diff - q->damp * E[2];
    diff = q->pr - (q->bmax[2] - X[2]) * q->ss;
    if (decide(mode, mk, 5, diff > EPSD)) a[2] += -(q->kb * diff - q->damp * (-E[2]));
}

/* The adjoint of walls(): given abar, add d(a)/dX^T abar to Xbar and
 * d(a)/dE^T abar to Ebar (branch decisions taken from X as in the forward). */
static void walls_adj(const P64 *q, double t, const double *X, const double *E, const double *ab,
                      double *Xb, double *Eb) {
    double diff, nx, ny;
    (void)E;
    diff = q->pr - (X[1] - (q->bmin[1] + (X[0] - q->bmin[0]) * q->slope)) * q->ss;
    if (diff > EPSD) {
        nx = -q->slope; ny = 1.0 - q->slope;
        const double nab = nx * ab[0] + ny * ab[1];           /* d(a)/d(adj) . abar */
        /* d diff / dX = -ss * (-slope, 1, 0) */
        Xb[0] += q->kb * nab * (q->ss * q->slope);
        Xb[1] += q->kb * nab * (-q->ss);
        Eb[0] += -q->damp * nx * nab - q->fric * ab[0];
        Eb[1] += -q->damp * ny * nab - q->fric * ab[1];
        Eb[2] += -q->fric * ab[2];
    }
    diff = q->pr - (q->bmax[1] - X[1]) * q->ss;
    if (diff > EPSD) {
        const double nab = -ab[1];
        Xb[1] += q->kb * nab * q->ss;
        Eb[1] += -q->damp * (-1.0) * nab - q->fric * ab[1];
        Eb[0] += -q->fric * ab[0];
        Eb[2] += -q->fric * ab[2];
    }
    const double ph = t * q->wfreq + X[2] / 400.0;
    const double wall = (sin(ph) * 0.5 + 0.5) * q->wf;
    const double dwall_dz = cos(ph) * 0.5 * q->wf / 400.0;
    diff = q->pr - (X[0] - (q->bmin[0] + wall)) * q->ss;
    if (diff > EPSD) {
        /* a0 += wall*kb*diff - damp*E0; diff depends on X0 (-ss) and wall (+ss) */
        Xb[0] += ab[0] * wall * q->kb * (-q->ss);
        Xb[2] += ab[0] * q->kb * dwall_dz * (diff + wall * q->ss);
        Eb[0] += -q->damp * ab[0];
    }
    diff = q->pr - (q->bmax[0] - X[0]) * q->ss;
    if (diff > EPSD) {
        Xb[0] += -ab[0] * q->kb * q->ss;
        Eb[0] += -q->damp * ab[0];
    }
    diff = q->pr - (X[2] - q->bmin[2]) * q->ss;
    if (diff > EPSD) {
        Xb[2] += ab[2] * q->kb * (-q->ss);
        Eb[2] += -q->damp * ab[2];
    }
    diff = q->pr - (q->bmax[2] - X[2]) * q->ss;
    if (diff > EPSD) {
        Xb[2] += -ab[2] * q->kb * q->ss;
        Eb[2] += -q->damp * ab[2];
    }
}

/* Per-step tape (sorted order). */
typedef struct {
    double *X, *V, *E, *rho, *F;
    AdvTape *adv;
    uint8_t *mask;   /* n branch-decision bytes of this step (mode 1/2), else null */
    int mode;
} Tape;

static void step_forward(const P64 *q, int n, const uint32_t *perm, const uint8_t *inr, const uint32_t *poff,
                         const uint32_t *pnbr, double t, double *x, double *v, double *e, Tape *tp) {
    double *X = tp->X, *V = tp->V, *E = tp->E, *rho = tp->rho, *F = tp->F;
    for (int s = 0; s < n; s++)
        for (int k = 0; k < 3; k++) {
            X[3 * s + k] = x[3 * perm[s] + k];
            V[3 * s + k] = v[3 * perm[s] + k];
            E[3 * s + k] = e[3 * perm[s] + k];
        }
    for (int s = 0; s < n; s++) {
        rho[s] = 0.0;
        if (!inr[s]) continue;
        double S = 0.0;
        for (uint32_t u = poff[s]; u < poff[s + 1]; u++) {
            const int j = (int)pnbr[u];
            double qd = 0.0;
            for (int k = 0; k < 3; k++) { const double d = X[3 * s + k] - X[3 * j + k]; qd += d * d; }
            const double w = (q->rd2 - qd) * q->d2;
            S += w * w * w;
        }
        rho[s] = (S == 0.0) ? 1.0 : S * q->m * q->poly6;
    }
    for (int s = 0; s < n; s++) {
        F[3 * s] = F[3 * s + 1] = F[3 * s + 2] = 0.0;
        if (!inr[s]) continue;
        const double pi = (rho[s] - q->rho0) * q->kap;
        for (uint32_t u = poff[s]; u < poff[s + 1]; u++) {
            const int j = (int)pnbr[u];
            double D[3], qd = 0.0;
            for (int k = 0; k < 3; k++) { D[k] = X[3 * s + k] - X[3 * j + k]; qd += D[k] * D[k]; }
            const double r = sqrt(qd * q->d2), c = q->h - r;
            const double pj = (rho[j] - q->rho0) * q->kap;
            const double pterm = q->ss * -0.5 * c * q->spiky * (pi + pj) / r;
            const double B = c / (rho[s] * rho[j]);
            for (int k = 0; k < 3; k++)
                F[3 * s + k] += (pterm * D[k] + q->lap * q->visc * (E[3 * j + k] - E[3 * s + k])) * B;
        }
    }
    for (int s = 0; s < n; s++) {
        double *xo = x + 3 * s, *vo = v + 3 * s, *eo = e + 3 * s;
        AdvTape *at = &tp->adv[s];
        if (!inr[s]) {
            for (int k = 0; k < 3; k++) { xo[k] = -1000.0; vo[k] = 0.0; eo[k] = E[3 * s + k]; }
            continue;
        }
        double a[3];
        uint8_t scratch = 0, *mk = tp->mask ? tp->mask + s : &scratch;
        const int mode = tp->mask ? tp->mode : 0;
        for (int k = 0; k < 3; k++) a[k] = F[3 * s + k] * q->m;
        walls(q, t, X + 3 * s, E + 3 * s, a, mk, mode);
        for (int k = 0; k < 3; k++) a[k] += q->g[k];
        for (int k = 0; k < 3; k++) at->a[k] = a[k];
        const double sa = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        at->aclamp = decide(mode, mk, 6, sa > q->AL * q->AL);
        for (int k = 0; k < 3; k++) at->ac[k] = at->aclamp ? a[k] * q->AL / sqrt(sa) : a[k];
        const double sv = V[3 * s] * V[3 * s] + V[3 * s + 1] * V[3 * s + 1] + V[3 * s + 2] * V[3 * s + 2];
        at->vclamp = decide(mode, mk, 7, sv > q->VL * q->VL);
        for (int k = 0; k < 3; k++) at->vc[k] = at->vclamp ? V[3 * s + k] * q->VL / sqrt(sv) : V[3 * s + k];
        for (int k = 0; k < 3; k++) {
            const double vn = at->ac[k] * q->dt + at->vc[k];
            eo[k] = (at->vc[k] + vn) * 0.5;
            vo[k] = vn;
            xo[k] = X[3 * s + k] + vn * (q->dt / q->ss);
        }
    }
}

/* Adjoint of u -> u * L / |u| (applied when the clamp fired). */
static void clamp_adj(const double *u, double L, const double *ub, double *out) {
    const double nn = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    const double dot = (u[0] * ub[0] + u[1] * ub[1] + u[2] * ub[2]) / (nn * nn);
    for (int k = 0; k < 3; k++) out[k] = (L / nn) * (ub[k] - u[k] * dot);
}

static void step_backward(const P64 *q, int n, const uint32_t *perm, const uint8_t *inr, const uint32_t *poff,
                          const uint32_t *pnbr, double t, const Tape *tp, double *xb, double *vb, double *eb,
                          double *gparam) {
    const double *X = tp->X, *E = tp->E, *rho = tp->rho, *V = tp->V;
    double *Xb = calloc((size_t)n * 3, sizeof(double));
    double *Vb = calloc((size_t)n * 3, sizeof(double));
    double *Eb = calloc((size_t)n * 3, sizeof(double));
    double *Fb = calloc((size_t)n * 3, sizeof(double));
    double *rb = calloc((size_t)n, sizeof(double));
    /* advance */
    for (int s = 0; s < n; s++) {
        const double *xo = xb + 3 * s, *vo = vb + 3 * s, *eo = eb + 3 * s;
        if (!inr[s]) {
            for (int k = 0; k < 3; k++) Eb[3 * s + k] += eo[k];
            continue;
        }
        const AdvTape *at = &tp->adv[s];
        double vt[3], acb[3], vcb[3], ab[3], vbar[3];
        for (int k = 0; k < 3; k++) {
            vt[k] = vo[k] + 0.5 * eo[k] + (q->dt / q->ss) * xo[k];
            acb[k] = q->dt * vt[k];
            vcb[k] = vt[k] + 0.5 * eo[k];
            Xb[3 * s + k] += xo[k];
        }
        if (at->aclamp) clamp_adj(at->a, q->AL, acb, ab); else memcpy(ab, acb, sizeof(ab));
        if (at->vclamp) clamp_adj(V + 3 * s, q->VL, vcb, vbar); else memcpy(vbar, vcb, sizeof(vbar));
        for (int k = 0; k < 3; k++) { Vb[3 * s + k] += vbar[k]; Fb[3 * s + k] += q->m * ab[k]; }
        walls_adj(q, t, X + 3 * s, E + 3 * s, ab, Xb + 3 * s, Eb + 3 * s);
    }
    /* force */
    for (int s = 0; s < n; s++) {
        if (!inr[s]) continue;
        const double *Fs = Fb + 3 * s;
        const double pi = (rho[s] - q->rho0) * q->kap;
        for (uint32_t u = poff[s]; u < poff[s + 1]; u++) {
            const int j = (int)pnbr[u];
            double D[3], qd = 0.0, dE[3];
            for (int k = 0; k < 3; k++) {
                D[k] = X[3 * s + k] - X[3 * j + k]; qd += D[k] * D[k];
                dE[k] = E[3 * j + k] - E[3 * s + k];
            }
            const double r = sqrt(qd * q->d2), c = q->h - r;
            const double pj = (rho[j] - q->rho0) * q->kap;
            const double A = q->ss * -0.5 * q->spiky;
            const double P = pi + pj;
            const double pterm = A * c * P / r;
            const double RR = rho[s] * rho[j];
            const double B = c / RR;
            const double vterm = q->lap * q->visc;
            double sv[3];
            for (int k = 0; k < 3; k++) sv[k] = pterm * D[k] + vterm * dE[k];
            const double DF = D[0] * Fs[0] + D[1] * Fs[1] + D[2] * Fs[2];
            const double SF = sv[0] * Fs[0] + sv[1] * Fs[1] + sv[2] * Fs[2];
            const double dEF = dE[0] * Fs[0] + dE[1] * Fs[1] + dE[2] * Fs[2];
            const double dpt_coef = -A * P * q->d2 * q->h / (r * r * r);   /* d pterm / dD = coef * D */
            const double dB_coef = -(q->d2 / r) / RR;                        /* d B / dD = coef * D */
            for (int k = 0; k < 3; k++) {
                const double Db = B * pterm * Fs[k] + B * DF * dpt_coef * D[k] + SF * dB_coef * D[k];
                Xb[3 * s + k] += Db;
                Xb[3 * j + k] -= Db;
                Eb[3 * j + k] += vterm * B * Fs[k];
                Eb[3 * s + k] -= vterm * B * Fs[k];
            }
            const double dpt_drho = A * c * q->kap / r;      /* d pterm / d rho_s (= d rho_j) */
            rb[s] += B * DF * dpt_drho - SF * B / rho[s];
            rb[j] += B * DF * dpt_drho - SF * B / rho[j];
            gparam[0] += q->lap * dEF * B;                                   /* visc */
            gparam[1] += B * DF * (A * c * (-2.0 * q->kap) / r);             /* rest density */
            gparam[2] += B * DF * (A * c * ((rho[s] - q->rho0) + (rho[j] - q->rho0)) / r);   /* IntStiff */
        }
    }
    /* density */
    for (int s = 0; s < n; s++) {
        if (!inr[s] || rb[s] == 0.0) continue;
        double S = 0.0;
        for (uint32_t u = poff[s]; u < poff[s + 1]; u++) {
            const int j = (int)pnbr[u];
            double qd = 0.0;
            for (int k = 0; k < 3; k++) { const double d = X[3 * s + k] - X[3 * j + k]; qd += d * d; }
            const double w = (q->rd2 - qd) * q->d2;
            S += w * w * w;
        }
        if (S == 0.0) continue;
        const double Sb = rb[s] * q->m * q->poly6;
        for (uint32_t u = poff[s]; u < poff[s + 1]; u++) {
            const int j = (int)pnbr[u];
            double D[3], qd = 0.0;
            for (int k = 0; k < 3; k++) { D[k] = X[3 * s + k] - X[3 * j + k]; qd += D[k] * D[k]; }
            const double w = (q->rd2 - qd) * q->d2;
            const double dS_dq = 3.0 * w * w * (-q->d2);
            for (int k = 0; k < 3; k++) {
                Xb[3 * s + k] += Sb * dS_dq * 2.0 * D[k];
                Xb[3 * j + k] -= Sb * dS_dq * 2.0 * D[k];
            }
        }
    }
    /* permutation transpose: slot s came from pre-sort index perm[s] */
    for (int s = 0; s < n; s++)
        for (int k = 0; k < 3; k++) {
            xb[3 * perm[s] + k] = Xb[3 * s + k];
            vb[3 * perm[s] + k] = Vb[3 * s + k];
            eb[3 * perm[s] + k] = Eb[3 * s + k];
        }
    free(Xb); free(Vb); free(Eb); free(Fb); free(rb);
}

/* T steps forward from (x, v, e) in place (doubles, n x 3). theta =
 * (visc, rest density, IntStiff) overrides the parameter block's values.
 * masks (nullable, T x n bytes) with mask_mode 1 records each step's wall
 * and clamp decisions, with mask_mode 2 replays them (see decide()). */
void adj64_forward(const fl_params *p, const double *theta, int n, int T, const uint32_t *perm,
                   const uint8_t *inr, const uint32_t *poff, const uint32_t *pnbr, const uint64_t *pbase,
                   const double *time, double *x, double *v, double *e, uint8_t *masks, int mask_mode) {
    const P64 q = p64(p, theta);
    Tape tp;
    tp.X = malloc(sizeof(double) * 3 * n); tp.V = malloc(sizeof(double) * 3 * n);
    tp.E = malloc(sizeof(double) * 3 * n); tp.rho = malloc(sizeof(double) * n);
    tp.F = malloc(sizeof(double) * 3 * n); tp.adv = malloc(sizeof(AdvTape) * n);
    tp.mode = mask_mode;
    for (int t = 0; t < T; t++) {
        tp.mask = masks ? masks + (size_t)t * n : NULL;
        step_forward(&q, n, perm + (size_t)t * n, inr + (size_t)t * n, poff + (size_t)t * (n + 1),
                     pnbr + pbase[t], time[t], x, v, e, &tp);
    }
    free(tp.X); free(tp.V); free(tp.E); free(tp.rho); free(tp.F); free(tp.adv);
}

/* Reverse pass: xb/vb/eb hold dL/d(final state) on entry and dL/d(initial
 * state) on return; gparam[3] += dL/d(visc, rest density, IntStiff).
 * states (nullable): T x {x, v, e} (n x 3 each), the state before every
 * step, to linearise around (e.g. an FP32 trajectory); null re-runs the
 * FP64 forward from (x0, v0, e0). */
void adj64_backward(const fl_params *p, const double *theta, int n, int T, const uint32_t *perm,
                    const uint8_t *inr, const uint32_t *poff, const uint32_t *pnbr, const uint64_t *pbase,
                    const double *time, const double *states, const double *x0, const double *v0,
                    const double *e0, double *xb, double *vb, double *eb, double *gparam) {
    const P64 q = p64(p, theta);
    const size_t n3 = (size_t)n * 3;
    Tape tp;
    tp.mask = NULL;
    tp.mode = 0;
    tp.X = malloc(sizeof(double) * n3); tp.V = malloc(sizeof(double) * n3);
    tp.E = malloc(sizeof(double) * n3); tp.rho = malloc(sizeof(double) * (n ? n : 1));
    tp.F = malloc(sizeof(double) * n3); tp.adv = malloc(sizeof(AdvTape) * (n ? n : 1));
    double *st = (double *)states;
    if (!st) {
        st = malloc(sizeof(double) * 3 * n3 * (size_t)(T ? T : 1));
        double *x = malloc(sizeof(double) * n3), *v = malloc(sizeof(double) * n3),
               *e = malloc(sizeof(double) * n3);
        memcpy(x, x0, sizeof(double) * n3); memcpy(v, v0, sizeof(double) * n3);
        memcpy(e, e0, sizeof(double) * n3);
        for (int t = 0; t < T; t++) {
            memcpy(st + (size_t)t * 3 * n3, x, sizeof(double) * n3);
            memcpy(st + (size_t)t * 3 * n3 + n3, v, sizeof(double) * n3);
            memcpy(st + (size_t)t * 3 * n3 + 2 * n3, e, sizeof(double) * n3);
            step_forward(&q, n, perm + (size_t)t * n, inr + (size_t)t * n, poff + (size_t)t * (n + 1),
                         pnbr + pbase[t], time[t], x, v, e, &tp);
        }
        free(x); free(v); free(e);
    }
    double *x = malloc(sizeof(double) * n3), *v = malloc(sizeof(double) * n3),
           *e = malloc(sizeof(double) * n3);
    for (int t = T - 1; t >= 0; t--) {
        /* re-evaluate step t from its saved state to rebuild its tape */
        memcpy(x, st + (size_t)t * 3 * n3, sizeof(double) * n3);
        memcpy(v, st + (size_t)t * 3 * n3 + n3, sizeof(double) * n3);
        memcpy(e, st + (size_t)t * 3 * n3 + 2 * n3, sizeof(double) * n3);
        step_forward(&q, n, perm + (size_t)t * n, inr + (size_t)t * n, poff + (size_t)t * (n + 1),
                     pnbr + pbase[t], time[t], x, v, e, &tp);
        step_backward(&q, n, perm + (size_t)t * n, inr + (size_t)t * n, poff + (size_t)t * (n + 1),
                      pnbr + pbase[t], time[t], &tp, xb, vb, eb, gparam);
    }
    if (st != states) free(st);
    free(x); free(v); free(e);
    free(tp.X); free(tp.V); free(tp.E); free(tp.rho); free(tp.F); free(tp.adv);
}
