/* CPU oracle for the GliomaUQ hot path -- TEST INFRASTRUCTURE ONLY.
 * See gliomauq_oracle.h for what each function restates. Built with
 * -ffp-contract=off so every + and * rounds on its own, as the reference's
 * source writes them. Pinned against the reference compiled in place
 * (oracle/Makefile -> oracle/_ref/) through tests/golden/.
 */
#define _GNU_SOURCE
#include "gliomauq_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static int resolve_threads(int nthreads) {
    if (nthreads > 0) return nthreads;
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

/* std::max(a,b) / std::min(a,b) as UpdateTumor calls them (MRAG undefines its
 * own max/min macros, source/MRAGHeaders.h:30-31): max(0,x) = (0<x)?x:0 maps
 * NaN to 0; min(1,x) = (x<1)?x:1. */
static inline double clamp01_d(double x) {
    x = (0.0 < x) ? x : 0.0;
    return (x < 1.0) ? x : 1.0;
}
static inline float clamp01_f(float x) {
    x = (0.0f < x) ? x : 0.0f;
    return (x < 1.0f) ? x : 1.0f;
}

/* ---------------- per-cell operator, FP64 build ----------------------------
 * c[0] centre, c[1..6] = W, E, S, N, B, F neighbours (ix-1, ix+1, iy-1, iy+1,
 * iz-1, iz+1) -- the order of df[0..5] at Glioma_ReactionDiffusionOperator.h:183-188. */
static inline double rhs_f64(const double pw[7], const double pg[7], const double ph[7],
                             double Dw, double Dg, double rho, double ih2) {
    double df[6] = {0, 0, 0, 0, 0, 0};
    const double tissue = pw[0] + pg[0] + ph[0];
    if (tissue > 0.) {
        const double b0 = pw[0] + pg[0];
        const double inv0 = 1.0 / ((pw[0] * Dw + pg[0] * Dg) / b0);
        for (int f = 0; f < 6; ++f) {
            const double bn = pw[f + 1] + pg[f + 1];
            df[f] = 2.0 * (1.0 / (inv0 + (1.0 / ((pw[f + 1] * Dw + pg[f + 1] * Dg) / bn))));
        }
    }
    /* :198-203, evaluated in order */
    if (df[0] == 0 && ph[1] > 0.) df[1] *= 2.0;
    if (df[1] == 0 && ph[2] > 0.) df[0] *= 2.0;
    if (df[2] == 0 && ph[3] > 0.) df[3] *= 2.0;
    if (df[3] == 0 && ph[4] > 0.) df[2] *= 2.0;
    if (df[4] == 0 && ph[5] > 0.) df[5] *= 2.0;
    if (df[5] == 0 && ph[6] > 0.) df[4] *= 2.0;
    const double in = ih2 * (df[0] * ph[1] + df[1] * ph[2] + df[2] * ph[3] + df[3] * ph[4] +
                             df[4] * ph[5] + df[5] * ph[6]);
    const double out = -((df[0] + df[1] + df[2] + df[3] + df[4] + df[5]) * ph[0] * ih2);
    const double react = rho * ph[0] * (1. - ph[0]);
    return out + in + react;
}

/* ---------------- per-cell operator, FP32 (default) build ------------------
 * Real=float: lab fields, Dw, Dg, rho and brain sums are float; df[] and the
 * fluxes are double (Glioma_ReactionDiffusionOperator.h:40-42,155,174-188,206-214). */
static inline float rhs_f32ref(const float pw[7], const float pg[7], const float ph[7], float Dw,
                               float Dg, float rho, double ih2) {
    double df[6] = {0, 0, 0, 0, 0, 0};
    const float tissue = pw[0] + pg[0] + ph[0];
    if (tissue > 0.) {
        const float b0 = pw[0] + pg[0];
        const float k0 = (pw[0] * Dw + pg[0] * Dg) / b0;
        const double inv0 = 1.0 / (double)k0;
        for (int f = 0; f < 6; ++f) {
            const float bn = pw[f + 1] + pg[f + 1];
            const float kn = (pw[f + 1] * Dw + pg[f + 1] * Dg) / bn;
            df[f] = 2.0 * (1.0 / (inv0 + (1.0 / (double)kn)));
        }
    }
    if (df[0] == 0 && ph[1] > 0.) df[1] *= 2.0;
    if (df[1] == 0 && ph[2] > 0.) df[0] *= 2.0;
    if (df[2] == 0 && ph[3] > 0.) df[3] *= 2.0;
    if (df[3] == 0 && ph[4] > 0.) df[2] *= 2.0;
    if (df[4] == 0 && ph[5] > 0.) df[5] *= 2.0;
    if (df[5] == 0 && ph[6] > 0.) df[4] *= 2.0;
    const double in = ih2 * (df[0] * (double)ph[1] + df[1] * (double)ph[2] + df[2] * (double)ph[3] +
                             df[3] * (double)ph[4] + df[4] * (double)ph[5] + df[5] * (double)ph[6]);
    const double out = -((df[0] + df[1] + df[2] + df[3] + df[4] + df[5]) * (double)ph[0] * ih2);
    const float rp = rho * ph[0]; /* float * float */
    const double react = (double)rp * (1. - (double)ph[0]);
    return (float)(out + in + react);
}

/* ---------------- uniform periodic grid, threaded over z-slabs ------------- */
typedef struct {
    int n, prec; /* prec 0: f64, 1: f32ref */
    const void *pw, *pg, *phi_in;
    void *phi_out;
    double Dw, Dg, rho, dt, ih2;
    int z0, z1;
} step_job;

#define IDX(x, y, z) ((size_t)(x) + (size_t)n * ((size_t)(y) + (size_t)n * (size_t)(z)))

static void *step_worker(void *arg) {
    const step_job *j = (const step_job *)arg;
    const int n = j->n;
    for (int z = j->z0; z < j->z1; ++z) {
        const int zm = (z + n - 1) % n, zp = (z + 1) % n;
        for (int y = 0; y < n; ++y) {
            const int ym = (y + n - 1) % n, yp = (y + 1) % n;
            for (int x = 0; x < n; ++x) {
                const int xm = (x + n - 1) % n, xp = (x + 1) % n;
                const size_t id[7] = {IDX(x, y, z),  IDX(xm, y, z), IDX(xp, y, z), IDX(x, ym, z),
                                      IDX(x, yp, z), IDX(x, y, zm), IDX(x, y, zp)};
                if (j->prec == 0) {
                    const double *pw = (const double *)j->pw, *pg = (const double *)j->pg,
                                 *ph = (const double *)j->phi_in;
                    double a[7], b[7], c[7];
                    for (int k = 0; k < 7; ++k) { a[k] = pw[id[k]]; b[k] = pg[id[k]]; c[k] = ph[id[k]]; }
                    const double dphidt = rhs_f64(a, b, c, j->Dw, j->Dg, j->rho, j->ih2);
                    ((double *)j->phi_out)[id[0]] = clamp01_d(c[0] + j->dt * dphidt);
                } else {
                    const float *pw = (const float *)j->pw, *pg = (const float *)j->pg,
                                *ph = (const float *)j->phi_in;
                    float a[7], b[7], c[7];
                    for (int k = 0; k < 7; ++k) { a[k] = pw[id[k]]; b[k] = pg[id[k]]; c[k] = ph[id[k]]; }
                    const float dphidt =
                        rhs_f32ref(a, b, c, (float)j->Dw, (float)j->Dg, (float)j->rho, j->ih2);
                    /* phi += dt * dphidt with phi float, dt double (:258) */
                    const float upd = (float)((double)c[0] + j->dt * (double)dphidt);
                    ((float *)j->phi_out)[id[0]] = clamp01_f(upd);
                }
            }
        }
    }
    return NULL;
}

static void run_step(step_job base, int nthreads) {
    const int n = base.n;
    int nt = resolve_threads(nthreads);
    if (nt > n) nt = n;
    pthread_t th[256];
    step_job jobs[256];
    if (nt > 256) nt = 256;
    for (int t = 0; t < nt; ++t) {
        jobs[t] = base;
        jobs[t].z0 = (int)((long)n * t / nt);
        jobs[t].z1 = (int)((long)n * (t + 1) / nt);
    }
    for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, step_worker, &jobs[t]);
    step_worker(&jobs[0]);
    for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
}

void orc_rd_step_f64(int n, const double *pw, const double *pg, const double *phi_in,
                     double *phi_out, double Dw, double Dg, double rho, double dt, double h,
                     int nthreads) {
    step_job j = {n, 0, pw, pg, phi_in, phi_out, Dw, Dg, rho, dt, 1. / (h * h), 0, 0};
    run_step(j, nthreads);
}

void orc_rd_step_f32ref(int n, const float *pw, const float *pg, const float *phi_in,
                        float *phi_out, float Dw, float Dg, float rho, double dt, double h,
                        int nthreads) {
    step_job j = {n, 1, pw, pg, phi_in, phi_out, Dw, Dg, rho, dt, 1. / (h * h), 0, 0};
    run_step(j, nthreads);
}

void orc_rd_solve_f64(int n, const double *pw, const double *pg, double *phi, double Dw,
                      double Dg, double rho, double dt, double h, long nsteps, int nthreads) {
    size_t N = (size_t)n * n * n;
    double *tmp = (double *)malloc(N * sizeof(double));
    double *a = phi, *b = tmp;
    for (long s = 0; s < nsteps; ++s) {
        orc_rd_step_f64(n, pw, pg, a, b, Dw, Dg, rho, dt, h, nthreads);
        double *t = a; a = b; b = t;
    }
    if (a != phi) memcpy(phi, a, N * sizeof(double));
    free(tmp);
}

void orc_rd_solve_f32ref(int n, const float *pw, const float *pg, float *phi, float Dw,
                         float Dg, float rho, double dt, double h, long nsteps, int nthreads) {
    size_t N = (size_t)n * n * n;
    float *tmp = (float *)malloc(N * sizeof(float));
    float *a = phi, *b = tmp;
    for (long s = 0; s < nsteps; ++s) {
        orc_rd_step_f32ref(n, pw, pg, a, b, Dw, Dg, rho, dt, h, nthreads);
        float *t = a; a = b; b = t;
    }
    if (a != phi) memcpy(phi, a, N * sizeof(float));
    free(tmp);
}

/* ---------------- MALA slopes (Glioma_MALA_SlopesOperator.h) -------------
 * Tissue tensor of one cell, :131-148: tt[f] = 2/(1/a_c + 1/a_f) with
 * a = p_w + p_g * ratioD (1/0 = inf makes a face to a cell outside the
 * tissue 0), all zero outside the tissue, then the Neumann doubling in order.
 * a_c, a_f are computed by the caller (double; from float fields in the
 * default build). */
static void slopes_tt(int inside, const double a[7], double tt[6]) {
    for (int f = 0; f < 6; ++f) tt[f] = 0.0;
    if (inside) {
        for (int f = 0; f < 6; ++f) tt[f] = 2.0 * (1.0 / ((1.0 / a[0]) + (1.0 / a[f + 1])));
        if (tt[0] == 0) tt[1] *= 2.0;
        if (tt[1] == 0) tt[0] *= 2.0;
        if (tt[2] == 0) tt[3] *= 2.0;
        if (tt[3] == 0) tt[2] *= 2.0;
        if (tt[4] == 0) tt[5] *= 2.0;
        if (tt[5] == 0) tt[4] *= 2.0;
    }
}

/* :152-182: the two rates, in the reference's evaluation order; s, d, p are
 * sRho, sD and phi at (c, W, E, S, N, B, F) widened to double, DwR = Dw as
 * stored (Real). */
static void slopes_rates(const double tt[6], const double s[7], const double d[7], const double p[7],
                         double DwR, double ih2, double *dsr, double *dsd) {
    const double tsum = tt[0] + tt[1] + tt[2] + tt[3] + tt[4] + tt[5];
    const double inR = ih2 * DwR * (tt[0] * s[1] + tt[1] * s[2] + tt[2] * s[3] + tt[3] * s[4] +
                                    tt[4] * s[5] + tt[5] * s[6]);
    const double outR = -ih2 * DwR * tsum * s[0];
    const double reR = p[0] * (1. - p[0]);
    *dsr = outR + inR + reR;
    const double inD = ih2 * DwR * (tt[0] * d[1] + tt[1] * d[2] + tt[2] * d[3] + tt[3] * d[4] +
                                    tt[4] * d[5] + tt[5] * d[6]);
    const double outD = -ih2 * DwR * tsum * d[0];
    const double rin = ih2 * (tt[0] * p[1] + tt[1] * p[2] + tt[2] * p[3] + tt[3] * p[4] +
                              tt[4] * p[5] + tt[5] * p[6]);
    const double rout = -ih2 * tsum * p[0];
    *dsd = outD + inD + rin + rout;
}

void orc_mala_step_f64(int n, const double *pw, const double *pg, const double *phi_in,
                       const double *sr_in, const double *sd_in, double *phi_out,
                       double *sr_out, double *sd_out, double Dw, double Dg, double rho,
                       double dt, double h) {
    orc_rd_step_f64(n, pw, pg, phi_in, phi_out, Dw, Dg, rho, dt, h, 1);
    const double ih2 = 1. / (h * h), ratioD = Dg / Dw;
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                const size_t id[7] = {IDX(x, y, z), IDX((x + n - 1) % n, y, z), IDX((x + 1) % n, y, z),
                                      IDX(x, (y + n - 1) % n, z), IDX(x, (y + 1) % n, z),
                                      IDX(x, y, (z + n - 1) % n), IDX(x, y, (z + 1) % n)};
                double a[7], s[7], d[7], p[7], tt[6], dsr, dsd;
                for (int k = 0; k < 7; ++k) {
                    a[k] = pw[id[k]] + pg[id[k]] * ratioD;
                    s[k] = sr_in[id[k]];
                    d[k] = sd_in[id[k]];
                    p[k] = phi_in[id[k]];
                }
                slopes_tt(pw[id[0]] > 0.0 || pg[id[0]] > 0.0, a, tt);
                slopes_rates(tt, s, d, p, Dw, ih2, &dsr, &dsd);
                sr_out[id[0]] = s[0] + dt * dsr;
                sd_out[id[0]] = d[0] + dt * dsd;
            }
}

void orc_mala_step_f32ref(int n, const float *pw, const float *pg, const float *phi_in,
                          const float *sr_in, const float *sd_in, float *phi_out, float *sr_out,
                          float *sd_out, float Dw, float Dg, float rho, double dt, double h) {
    orc_rd_step_f32ref(n, pw, pg, phi_in, phi_out, Dw, Dg, rho, dt, h, 1);
    const double ih2 = 1. / (h * h);
    const double ratioD = (double)(Dg / Dw); /* Real / Real, then widened (:117) */
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                const size_t id[7] = {IDX(x, y, z), IDX((x + n - 1) % n, y, z), IDX((x + 1) % n, y, z),
                                      IDX(x, (y + n - 1) % n, z), IDX(x, (y + 1) % n, z),
                                      IDX(x, y, (z + n - 1) % n), IDX(x, y, (z + 1) % n)};
                double a[7], s[7], d[7], p[7], tt[6], dsr, dsd;
                for (int k = 0; k < 7; ++k) {
                    a[k] = (double)pw[id[k]] + (double)pg[id[k]] * ratioD;
                    s[k] = sr_in[id[k]];
                    d[k] = sd_in[id[k]];
                    p[k] = phi_in[id[k]];
                }
                slopes_tt(pw[id[0]] > 0.0 || pg[id[0]] > 0.0, a, tt);
                slopes_rates(tt, s, d, p, (double)Dw, ih2, &dsr, &dsd);
                /* the rates are stored as Real (:162,:182), the update in double (:221-222) */
                const float fr = (float)dsr, fd = (float)dsd;
                sr_out[id[0]] = (float)((double)sr_in[id[0]] + dt * (double)fr);
                sd_out[id[0]] = (float)((double)sd_in[id[0]] + dt * (double)fd);
            }
}

long orc_num_steps(double dt, double tend) {
    double t = 0.0;
    long k = 0;
    while (t <= tend) {
        t += dt;
        ++k;
    }
    return k;
}

/* ---------------- block-lab restatement (CPU baseline) ---------------------
 * 41 Real fields per cell as CCell_extended (source/Glioma/Glioma_Types.h:22-70);
 * only phi, dphidt, p_g, p_w are used, at the same offsets (0, 1, 2, 3). */
#define BS 16
#define LAB (BS + 2)
#define NFIELDS 41
typedef struct {
    float phi, dphidt, p_g, p_w;
    float other[NFIELDS - 4];
} orc_cell;

struct orc_blockgrid {
    int n, bpd, nblocks;
    orc_cell *cells; /* nblocks * BS^3, block-major, x-fastest inside a block */
};

orc_blockgrid *orc_blockgrid_create(int n, const float *pw, const float *pg, const float *phi) {
    if (n % BS) return NULL;
    orc_blockgrid *g = (orc_blockgrid *)calloc(1, sizeof(orc_blockgrid));
    g->n = n;
    g->bpd = n / BS;
    g->nblocks = g->bpd * g->bpd * g->bpd;
    g->cells = (orc_cell *)calloc((size_t)g->nblocks * BS * BS * BS, sizeof(orc_cell));
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                int b = (x / BS) + g->bpd * ((y / BS) + g->bpd * (z / BS));
                orc_cell *c = &g->cells[(size_t)b * BS * BS * BS + (x % BS) + BS * ((y % BS) + BS * (z % BS))];
                size_t gi = IDX(x, y, z);
                c->p_w = pw[gi];
                c->p_g = pg[gi];
                c->phi = phi[gi];
            }
    return g;
}

void orc_blockgrid_get_phi(const orc_blockgrid *g, float *phi) {
    const int n = g->n;
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                int b = (x / BS) + g->bpd * ((y / BS) + g->bpd * (z / BS));
                phi[IDX(x, y, z)] =
                    g->cells[(size_t)b * BS * BS * BS + (x % BS) + BS * ((y % BS) + BS * (z % BS))].phi;
            }
}

void orc_blockgrid_destroy(orc_blockgrid *g) {
    if (!g) return;
    free(g->cells);
    free(g);
}

typedef struct {
    orc_blockgrid *g;
    atomic_int *next;
    int phase; /* 0 = RHS through the lab, 1 = update */
    float Dw, Dg, rho;
    double dt, ih2;
} lab_job;

static orc_cell *block_cell(orc_blockgrid *g, int bx, int by, int bz, int x, int y, int z) {
    const int p = g->bpd;
    bx = (bx + p) % p; by = (by + p) % p; bz = (bz + p) % p;
    int b = bx + p * (by + p * bz);
    return &g->cells[(size_t)b * BS * BS * BS + x + BS * (y + BS * z)];
}

static void *lab_worker(void *arg) {
    lab_job *j = (lab_job *)arg;
    orc_blockgrid *g = j->g;
    const int p = g->bpd;
    orc_cell *lab = (orc_cell *)malloc(sizeof(orc_cell) * LAB * LAB * LAB);
    for (;;) {
        int b = atomic_fetch_add(j->next, 1);
        if (b >= g->nblocks) break;
        const int bx = b % p, by = (b / p) % p, bz = b / (p * p);
        orc_cell *blk = &g->cells[(size_t)b * BS * BS * BS];
        if (j->phase == 1) {
            for (int c = 0; c < BS * BS * BS; ++c) {
                float v = (float)((double)blk[c].phi + j->dt * (double)blk[c].dphidt);
                blk[c].phi = clamp01_f(v);
            }
            continue;
        }
        /* lab fill: interior rows, then every ghost cell of the 26 regions,
         * each a same-level periodic copy */
        for (int z = -1; z <= BS; ++z)
            for (int y = -1; y <= BS; ++y)
                for (int x = -1; x <= BS; ++x) {
                    const int ox = x < 0 ? -1 : (x >= BS ? 1 : 0);
                    const int oy = y < 0 ? -1 : (y >= BS ? 1 : 0);
                    const int oz = z < 0 ? -1 : (z >= BS ? 1 : 0);
                    const orc_cell *src = block_cell(g, bx + ox, by + oy, bz + oz, x - ox * BS,
                                                     y - oy * BS, z - oz * BS);
                    lab[(x + 1) + LAB * ((y + 1) + LAB * (z + 1))] = *src;
                }
        for (int z = 0; z < BS; ++z)
            for (int y = 0; y < BS; ++y)
                for (int x = 0; x < BS; ++x) {
                    const int l = (x + 1) + LAB * ((y + 1) + LAB * (z + 1));
                    const int off[7] = {0, -1, 1, -LAB, LAB, -LAB * LAB, LAB * LAB};
                    float a[7], bb[7], c[7];
                    for (int k = 0; k < 7; ++k) {
                        a[k] = lab[l + off[k]].p_w;
                        bb[k] = lab[l + off[k]].p_g;
                        c[k] = lab[l + off[k]].phi;
                    }
                    blk[x + BS * (y + BS * z)].dphidt = rhs_f32ref(a, bb, c, j->Dw, j->Dg, j->rho, j->ih2);
                }
    }
    free(lab);
    return NULL;
}

void orc_blockgrid_steps(orc_blockgrid *g, float Dw, float Dg, float rho, double dt, double h,
                         long nsteps, int nthreads) {
    int nt = resolve_threads(nthreads);
    if (nt > 256) nt = 256;
    pthread_t th[256];
    for (long s = 0; s < nsteps; ++s) {
        for (int phase = 0; phase < 2; ++phase) {
            atomic_int next;
            atomic_init(&next, 0);
            lab_job j = {g, &next, phase, Dw, Dg, rho, dt, 1. / (h * h)};
            for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, lab_worker, &j);
            lab_worker(&j);
            for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
        }
    }
}

/* ---------------- HGG_Likelihood ------------------------------------------- */
static int sgn_d(double d) { /* HGG_Likelihood.cpp:155-160 */
    const double eps = 0.0;
    if (d < -eps) return -1;
    return d > eps;
}

static long double log_bernoulli(double u, double y, double uc, double slope) {
    /* HGG_Likelihood.cpp:136-153 */
    const double is2 = 1. / slope;
    const double diff = u - uc;
    const long double alpha = 0.5 + 0.5 * sgn_d(diff) * (1. - exp(-diff * diff * is2));
    return (y == 1) ? logl(alpha) : logl(1. - alpha);
}

void orc_loglik(int nx, int ny, int nz, const double *model, const double *pet, const double *t1,
                const double *t2, const double *points, long npoints, const orc_lik_params *p,
                int step_pet, int step_ti, int selective, orc_lik_result *out) {
    /* PET, :40-75 */
    long N = 0;
    long double sum = 0.;
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                if ((ix % step_pet == 0) && (iy % step_pet == 0) && (iz % step_pet == 0)) {
                    size_t g = (size_t)ix + (size_t)nx * ((size_t)iy + (size_t)ny * iz);
                    if (pet[g] > 0.) {
                        sum += (model[g] - p->pet_scale * pet[g]) * (model[g] - p->pet_scale * pet[g]);
                        N++;
                    }
                }
            }
    const long double p1 = -0.5 * N * log(2. * M_PI * p->pet_sigma2);
    const long double p2 = -0.5 * (1. / p->pet_sigma2) * sum;
    const long double lpet = p1 + p2;

    /* T1 / T2, :77-128 */
    long double lt[2] = {0., 0.};
    for (int ti = 0; ti < 2; ++ti) {
        const double *data = ti == 0 ? t1 : t2;
        const double uc = ti == 0 ? p->t1_uc : p->t2_uc;
        long double s = 0.;
        if (!selective) {
            for (int iz = 0; iz < nz; iz++)
                for (int iy = 0; iy < ny; iy++)
                    for (int ix = 0; ix < nx; ix++) {
                        size_t g = (size_t)ix + (size_t)nx * ((size_t)iy + (size_t)ny * iz);
                        s += log_bernoulli(model[g], data[g], uc, p->slope);
                    }
        } else {
            for (long i = 0; i < npoints; i++) {
                const int ix = (int)points[i], iy = (int)points[i + npoints],
                          iz = (int)points[i + 2 * npoints];
                if ((ix % step_ti == 0) && (iy % step_ti == 0) && (iz % step_ti == 0)) {
                    size_t g = (size_t)ix + (size_t)nx * ((size_t)iy + (size_t)ny * iz);
                    s += log_bernoulli(model[g], data[g], uc, p->slope);
                }
            }
        }
        lt[ti] = s;
    }
    out->l_pet = (double)lpet;
    out->l_t1 = (double)lt[0];
    out->l_t2 = (double)lt[1];
    out->total = (double)(lpet + lt[0] + lt[1]);
    out->n_pet = N;
}
