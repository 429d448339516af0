/*
 * Oracle: plain-C restatement of the reference lattice-Boltzmann time step.
 * TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline); see bclbm_oracle.h.
 *
 * Each function cites the reference code it restates.  Expressions keep the
 * reference's evaluation order (C evaluates a + b + c as (a + b) + c, as C++
 * does for the valarray element loops of the reference); build with
 * -ffp-contract=off.
 */
#include "bclbm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- lattice constants (src/lbsolver/LBd2q9.h:19-40, LBd3q19.h:19-40) ---- */
static const double C2INV = 3.0;
static const double C4INV = 9.0;
#define C2 (1.0 / 3.0)
static const double C4INV0_5 = 0.5 * 9.0;
#define SQRT2_REF 1.4142135623730950488 /* LBglobal.h:11 */
static const double EPS = 2.220446049250313080847e-16; /* lbBaseEps, LBglobal.h:14 */

typedef struct {
    int nq, nd, npairs;
    double w[19];
    int c[19][3];
    int rev[19];
    double B[19];
    double cnorm[19];
    double w1c2inv, w2c2inv;
} lattice_t;

static void lattice_init(lattice_t* L, int nq) {
    memset(L, 0, sizeof(*L));
    L->nq = nq;
    if (nq == 9) {
        const double w0 = 16.0 / 36.0, w1 = 4.0 / 36.0, w2 = 1.0 / 36.0;
        const double B0 = -16.0 / 108.0, B1 = 8.0 / 108.0, B2 = 5.0 / 108.0;
        static const int c[9][2] = {{1, 0}, {1, 1}, {0, 1}, {-1, 1}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {0, 0}};
        L->nd = 2;
        L->npairs = 4;
        for (int q = 0; q < 9; ++q) {
            L->c[q][0] = c[q][0];
            L->c[q][1] = c[q][1];
            int diag = (q % 2) == 1;
            L->w[q] = q == 8 ? w0 : (diag ? w2 : w1);
            L->B[q] = q == 8 ? B0 : (diag ? B2 : B1);
            L->cnorm[q] = q == 8 ? 0.0 : (diag ? SQRT2_REF : 1.0);
            L->rev[q] = q == 8 ? 8 : (q + 4) % 8;
        }
        L->w1c2inv = w1 * 3.0;
        L->w2c2inv = w2 * 3.0;
    } else {
        const double w0 = 12.0 / 36.0, w1 = 2.0 / 36.0, w2 = 1.0 / 36.0;
        const double B0 = -12.0 / 54.0, B1 = 1.0 / 54.0, B2 = 2.0 / 54.0;
        static const int c[19][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1},
                                     {0, 1, 1}, {0, 1, -1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0},
                                     {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1}, {0, -1, -1}, {0, -1, 1}, {0, 0, 0}};
        L->nd = 3;
        L->npairs = 9;
        for (int q = 0; q < 19; ++q) {
            for (int d = 0; d < 3; ++d) L->c[q][d] = c[q][d];
            int axis = (q % 9) < 3;
            L->w[q] = q == 18 ? w0 : (axis ? w1 : w2);
            L->B[q] = q == 18 ? B0 : (axis ? B1 : B2);
            L->cnorm[q] = q == 18 ? 0.0 : (axis ? 1.0 : SQRT2_REF);
            L->rev[q] = q == 18 ? 18 : (q + 9) % 18;
        }
        L->w1c2inv = w1 * 3.0;
        L->w2c2inv = w2 * 3.0;
    }
}

/* qSum (LBd2q9.h:161-168, LBd3q19.h:173-180) */
static double qsum(const lattice_t* L, const double* f) {
    double r = 0.0;
    for (int q = 0; q < L->nq; ++q) r += f[q];
    return r;
}

/* qSumC (LBd2q9.h:170-177, LBd3q19.h:182-190) */
static void qsumc(const lattice_t* L, const double* d, double* r) {
    if (L->nq == 9) {
        r[0] = d[0] + d[1] - d[3] - d[4] - d[5] + d[7];
        r[1] = d[1] + d[2] + d[3] - d[5] - d[6] - d[7];
    } else {
        r[0] = d[0] + d[3] + d[4] + d[5] + d[6] - d[9] - d[12] - d[13] - d[14] - d[15];
        r[1] = d[1] + d[3] - d[4] + d[7] + d[8] - d[10] - d[12] + d[13] - d[16] - d[17];
        r[2] = d[2] + d[5] - d[6] + d[7] - d[8] - d[11] - d[14] + d[15] - d[16] + d[17];
    }
}

/* cDotAll (LBd2q9.h:128-142, LBd3q19.h:129-153) */
static void cdotall(const lattice_t* L, const double* v, double* r) {
    if (L->nq == 9) {
        r[0] = +v[0];
        r[1] = +v[0] + v[1];
        r[2] = +v[1];
        r[3] = -v[0] + v[1];
        r[4] = -v[0];
        r[5] = -v[0] - v[1];
        r[6] = -v[1];
        r[7] = +v[0] - v[1];
        r[8] = 0.0;
    } else {
        r[0] = +v[0];
        r[1] = +v[1];
        r[2] = +v[2];
        r[3] = +v[0] + v[1];
        r[4] = +v[0] - v[1];
        r[5] = +v[0] + v[2];
        r[6] = +v[0] - v[2];
        r[7] = +v[1] + v[2];
        r[8] = +v[1] - v[2];
        r[9] = -v[0];
        r[10] = -v[1];
        r[11] = -v[2];
        r[12] = -v[0] - v[1];
        r[13] = -v[0] + v[1];
        r[14] = -v[0] - v[2];
        r[15] = -v[0] + v[2];
        r[16] = -v[1] - v[2];
        r[17] = -v[1] + v[2];
        r[18] = 0.0;
    }
}

/* dot (LBd2q9.h dot, LBd3q19.h:111-115) */
static double dotv(const lattice_t* L, const double* a, const double* b) {
    if (L->nd == 2) return a[0] * b[0] + a[1] * b[1];
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* grad (LBd2q9.h:144-151, LBd3q19.h:155-163) */
static void gradq(const lattice_t* L, const double* s, double* r) {
    const double a = L->w1c2inv, b = L->w2c2inv;
    if (L->nq == 9) {
        r[0] = a * (s[0] - s[4]) + b * (s[1] - s[3] - s[5] + s[7]);
        r[1] = a * (s[2] - s[6]) + b * (s[1] + s[3] - s[5] - s[7]);
    } else {
        r[0] = a * (s[0] - s[9]) + b * (s[3] + s[4] + s[5] + s[6] - s[12] - s[13] - s[14] - s[15]);
        r[1] = a * (s[1] - s[10]) + b * (s[3] - s[4] + s[7] + s[8] - s[12] + s[13] - s[16] - s[17]);
        r[2] = a * (s[2] - s[11]) + b * (s[5] - s[6] + s[7] - s[8] - s[14] + s[15] - s[16] + s[17]);
    }
}

/* ---- node-loop threading: contiguous slices of the bulk list ---- */
typedef void (*slice_fn)(void* ctx, int begin, int end);
typedef struct {
    slice_fn fn;
    void* ctx;
    int begin, end;
} slice_job;

static void* slice_thread(void* p) {
    slice_job* j = (slice_job*)p;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

static void parallel_for(int n, int nthreads, slice_fn fn, void* ctx) {
    if (nthreads <= 1 || n < 4096) {
        fn(ctx, 0, n);
        return;
    }
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    slice_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].begin = (int)((long long)n * t / nthreads);
        jobs[t].end = (int)((long long)n * (t + 1) / nthreads);
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, slice_thread, &jobs[t]);
    fn(ctx, jobs[0].begin, jobs[0].end);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* ---- half-way bounce-back (LBhalfwayhelperclass.h:128-159, LBhalfwaybb.h:49-62) ---- */
typedef struct {
    int n;            /* boundary nodes */
    int32_t* node;    /* node numbers */
    int8_t* kind;     /* per node and pair: 0 gamma, 1 beta(q), 2 beta(rev q), 3 delta */
} bb_links;

static int bb_build(const lattice_t* L, const oracle_grid* g, const int32_t* list, int n, bb_links* bb) {
    bb->n = n;
    bb->node = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    bb->kind = (int8_t*)malloc((size_t)(n > 0 ? n : 1) * (size_t)L->npairs);
    if (!bb->node || !bb->kind) return -1;
    for (int b = 0; b < n; ++b) {
        int node = list[b];
        bb->node[b] = node;
        for (int q = 0; q < L->npairs; ++q) {
            int a = g->types[g->neigh[(size_t)node * L->nq + q]] > 1;
            int r = g->types[g->neigh[(size_t)node * L->nq + L->rev[q]]] > 1;
            bb->kind[(size_t)b * L->npairs + q] = (int8_t)(a ? (r ? 0 : 1) : (r ? 2 : 3));
        }
    }
    return 0;
}

static void bb_free(bb_links* bb) {
    free(bb->node);
    free(bb->kind);
}

typedef struct {
    const lattice_t* L;
    const oracle_grid* g;
    const bb_links* bb;
    double* f;
    int nfields, field;
} bb_ctx;

static void bb_slice(void* p, int begin, int end) {
    bb_ctx* c = (bb_ctx*)p;
    const lattice_t* L = c->L;
    const int nq = L->nq, es = c->nfields * nq, sh = c->field * nq;
    double* f = c->f;
    for (int b = begin; b < end; ++b) {
        const size_t node = (size_t)c->bb->node[b];
        const int32_t* nb = c->g->neigh + node * nq;
        const int8_t* kind = c->bb->kind + (size_t)b * L->npairs;
        /* beta links first, then delta links, in pair order (LBhalfwaybb.h:52-61) */
        for (int q = 0; q < L->npairs; ++q) {
            int beta;
            if (kind[q] == 1) beta = q;
            else if (kind[q] == 2) beta = L->rev[q];
            else continue;
            int br = L->rev[beta];
            f[es * node + sh + beta] = f[es * (size_t)nb[br] + sh + br];
        }
        for (int q = 0; q < L->npairs; ++q) {
            if (kind[q] != 3) continue;
            int dr = L->rev[q];
            f[es * node + sh + q] = f[es * (size_t)nb[dr] + sh + dr];
            f[es * node + sh + dr] = f[es * (size_t)nb[q] + sh + q];
        }
    }
}

static int check_grid(const oracle_grid* g) {
    if (!g || (g->nq != 9 && g->nq != 19) || g->n_nodes < 1 || !g->neigh || !g->types || !g->bulk) return -1;
    for (size_t i = 0; i < (size_t)g->n_nodes * g->nq; ++i)
        if (g->neigh[i] < 0 || g->neigh[i] >= g->n_nodes) return -2;
    for (int b = 0; b < g->n_bulk; ++b)
        if (g->bulk[b] < 1 || g->bulk[b] >= g->n_nodes) return -3;
    return 0;
}

/* ---- std_case collision + propagation (src/std_case/main.cpp:110-135) ---- */
typedef struct {
    const lattice_t* L;
    const oracle_grid* g;
    int trt;
    double tau, tau_anti;
    const double* F;
    const double* f;
    double* ftmp;
    double* rho;
    double* vel;
    double cF[19];
} single_ctx;

static void single_slice(void* p, int begin, int end) {
    single_ctx* c = (single_ctx*)p;
    const lattice_t* L = c->L;
    const int nq = L->nq, nd = L->nd;
    double fn[19], cu[19], om[19], dF[19], vel[3], j[3];
    for (int b = begin; b < end; ++b) {
        const size_t node = (size_t)c->g->bulk[b];
        memcpy(fn, c->f + node * nq, sizeof(double) * nq);
        /* calcRho, calcVel (LBmacroscopic.h:53-61, 77-86) */
        const double rho = qsum(L, fn);
        qsumc(L, fn, j);
        for (int d = 0; d < nd; ++d) vel[d] = (j[d] + 0.5 * c->F[d]) / rho;
        if (c->rho) c->rho[node] = rho;
        if (c->vel)
            for (int d = 0; d < nd; ++d) c->vel[node * nd + d] = vel[d];
        const double u2 = dotv(L, vel, vel);
        cdotall(L, vel, cu);
        const double uF = dotv(L, vel, c->F);
        if (!c->trt) {
            /* calcOmegaBGK (LBcollision.h:38-45) */
            const double tau_inv = 1.0 / c->tau;
            for (int q = 0; q < nq; ++q)
                om[q] = -tau_inv * (fn[q] - rho * L->w[q] * (1.0 + C2INV * cu[q] + C4INV0_5 * (cu[q] * cu[q] - C2 * u2)));
            /* calcDeltaOmegaF (LBcollision.h:205-212) */
            const double tf = (1 - 0.5 / c->tau);
            for (int q = 0; q < nq; ++q)
                dF[q] = L->w[q] * tf * (C2INV * c->cF[q] + C4INV * (c->cF[q] * cu[q] - C2 * uF));
        } else {
            /* calcOmegaBGKTRT (LBcollision.h:63-74) */
            const double ts_inv = 1.0 / c->tau;
            const double ta_inv = 1.0 / c->tau_anti;
            for (int q = 0; q < nq; ++q) {
                const double fs = 0.5 * (fn[q] + fn[L->rev[q]]);
                const double fa = 0.5 * (fn[q] - fn[L->rev[q]]);
                om[q] = -ts_inv * (fs - rho * L->w[q] * (1.0 + C4INV0_5 * (cu[q] * cu[q] - C2 * u2)))
                        - ta_inv * (fa - rho * L->w[q] * C2INV * cu[q]);
            }
            /* calcDeltaOmegaFTRT with phi = 1 (LBcollision.h:227-235) */
            const double tsf = (1 - 0.5 / c->tau);
            const double taf = (1 - 0.5 / c->tau_anti);
            const double phi = 1.0;
            for (int q = 0; q < nq; ++q)
                dF[q] = L->w[q] * phi * (taf * C2INV * c->cF[q] + tsf * C4INV * (c->cF[q] * cu[q] - C2 * uF));
        }
        /* propagateTo (LBfield.h:350-357) with fNode + omega + deltaOmegaF */
        const int32_t* nb = c->g->neigh + node * nq;
        for (int q = 0; q < nq; ++q) c->ftmp[(size_t)nb[q] * nq + q] = fn[q] + om[q] + dF[q];
    }
}

int oracle_single_run(const oracle_grid* g, int nsteps, int trt, double tau, double tau_anti,
                      const double* force, double* f, double* ftmp, double* rho, double* vel,
                      int nthreads) {
    int rc = check_grid(g);
    if (rc) return rc;
    lattice_t L;
    lattice_init(&L, g->nq);
    /* HalfWayBounceBack over findFluidBndNodes (main.cpp:84, LBgeometry.h:49-56) */
    int nb = 0;
    for (int n = 1; n < g->n_nodes; ++n) nb += g->types[n] == 2;
    int32_t* list = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    if (!list) return -10;
    nb = 0;
    for (int n = 1; n < g->n_nodes; ++n)
        if (g->types[n] == 2) list[nb++] = n;
    bb_links bb;
    if (bb_build(&L, g, list, nb, &bb)) return -10;
    free(list);

    single_ctx c;
    memset(&c, 0, sizeof(c));
    c.L = &L;
    c.g = g;
    c.trt = trt;
    c.tau = tau;
    c.tau_anti = tau_anti;
    c.F = force;
    c.rho = rho;
    c.vel = vel;
    cdotall(&L, force, c.cF);
    double* cur = f;
    double* nxt = ftmp;
    for (int i = 0; i < nsteps; ++i) {
        c.f = cur;
        c.ftmp = nxt;
        parallel_for(g->n_bulk, nthreads, single_slice, &c);
        double* t = cur; cur = nxt; nxt = t; /* swapData (LBfield.h:359) */
        bb_ctx bc = {&L, g, &bb, cur, 1, 0};
        parallel_for(bb.n, nthreads, bb_slice, &bc);
    }
    bb_free(&bb);
    return cur == f ? 0 : 1;
}

/* ---- twophase (src/twophase/main_TWOPHASE.cpp:238-392) ---- */
typedef struct {
    const lattice_t* L;
    const oracle_grid* g;
    const double* f;
    double* ftmp;
    double* rho;
    double* vel;
    const double* cg;
    double* cgw;
    double nu0inv, nu1inv, sigma, beta;
    const double* F;
} tp_ctx;

/* PASS 1: densities and colour field (main_TWOPHASE.cpp:238-246) */
static void tp_density_slice(void* p, int begin, int end) {
    tp_ctx* c = (tp_ctx*)p;
    const lattice_t* L = c->L;
    const int nq = L->nq;
    for (int b = begin; b < end; ++b) {
        const size_t node = (size_t)c->g->bulk[b];
        const double r0 = qsum(L, c->f + node * 2 * nq);
        const double r1 = qsum(L, c->f + node * 2 * nq + nq);
        c->rho[node * 2] = r0;
        c->rho[node * 2 + 1] = r1;
        c->cgw[node] = (r0 - r1) / (r0 + r1);
    }
}

/* PASS 2: RK collision, recolouring and propagation (main_TWOPHASE.cpp:312-376) */
static void tp_collide_slice(void* p, int begin, int end) {
    tp_ctx* c = (tp_ctx*)p;
    const lattice_t* L = c->L;
    const int nq = L->nq, nd = L->nd;
    double ft[19], cu[19], cF[19], om[19], dF[19], dQ0[19], dQ1[19], sc[19], cn[19], dST[19], dRC[19];
    double j[3], vel[3], G[3];
    cdotall(L, c->F, cF);
    for (int b = begin; b < end; ++b) {
        const size_t node = (size_t)c->g->bulk[b];
        const double* f0 = c->f + node * 2 * nq;
        const double* f1 = f0 + nq;
        for (int q = 0; q < nq; ++q) ft[q] = f0[q] + f1[q];
        double rho0 = c->rho[node * 2];
        double rho1 = c->rho[node * 2 + 1];
        const double rho = rho0 + rho1;
        qsumc(L, ft, j);
        for (int d = 0; d < nd; ++d) vel[d] = (j[d] + 0.5 * c->F[d]) / rho;
        for (int d = 0; d < nd; ++d) c->vel[node * nd + d] = vel[d];
        const double q0 = 0.0, q1 = 0.0;
        c->rho[node * 2] = rho0 += 0.5 * q0;
        c->rho[node * 2 + 1] = rho1 += 0.5 * q1;
        const double tau = C2INV * rho / (rho0 * c->nu0inv + rho1 * c->nu1inv) + 0.5;
        const double uu = dotv(L, vel, vel);
        cdotall(L, vel, cu);
        const double tau_inv = 1.0 / tau;
        for (int q = 0; q < nq; ++q)
            om[q] = -tau_inv * (ft[q] - rho * L->w[q] * (1.0 + C2INV * cu[q] + C4INV0_5 * (cu[q] * cu[q] - C2 * uu)));
        const double uF = dotv(L, vel, c->F);
        const double tf = (1 - 0.5 / tau);
        for (int q = 0; q < nq; ++q)
            dF[q] = L->w[q] * tf * (C2INV * cF[q] + C4INV * (cF[q] * cu[q] - C2 * uF));
        /* calcDeltaOmegaQ with zero sources (LBcollision.h:90-97) */
        for (int q = 0; q < nq; ++q) {
            const double e = (1.0 + C2INV * cu[q] + C4INV0_5 * (cu[q] * cu[q] - C2 * uu));
            dQ0[q] = tf * q0 * L->w[q] * e;
            dQ1[q] = tf * q1 * L->w[q] * e;
        }
        /* grad (LButilities.h:12-22), vecNorm (:62-66) */
        const int32_t* nb = c->g->neigh + node * nq;
        for (int q = 0; q < nq; ++q) sc[q] = c->cg[nb[q]];
        gradq(L, sc, G);
        const double cgn = sqrt(dotv(L, G, G));
        const double sc_inv = 1.0 / (cgn + (double)(cgn < EPS));
        for (int d = 0; d < nd; ++d) G[d] *= sc_inv;
        cdotall(L, G, cn);
        /* calcDeltaOmegaST (LBcollision2phase.h:7-20) */
        const double af = 1.125 * cgn * c->sigma / tau;
        for (int q = 0; q < nq - 1; ++q) dST[q] = af * (L->w[q] * cn[q] * cn[q] - L->B[q]);
        dST[nq - 1] = -af * L->B[nq - 1];
        /* calcDeltaOmegaRC (LBcollision2phase.h:70-86) */
        const double rfb = c->beta * rho0 * rho1 / rho;
        for (int q = 0; q < nq - 1; ++q) dRC[q] = rfb * L->w[q] * cn[q] / L->cnorm[q];
        dRC[nq - 1] = 0.0;
        const double c0 = (rho0 / rho);
        const double c1 = (rho1 / rho);
        for (int q = 0; q < nq; ++q) {
            const size_t t = (size_t)nb[q] * 2 * nq;
            c->ftmp[t + q] = c0 * (ft[q] + om[q] + dF[q] + dST[q]) + dRC[q] + dQ0[q];
            c->ftmp[t + nq + q] = c1 * (ft[q] + om[q] + dF[q] + dST[q]) - dRC[q] + dQ1[q];
        }
    }
}

int oracle_twophase_run(const oracle_grid* g, int nsteps, double tau0, double tau1, double sigma,
                        double beta, int flux_control, double mom_x, double* force,
                        double* f, double* ftmp, double* rho, double* vel, double* cg,
                        double* force_log, int nthreads) {
    int rc = check_grid(g);
    if (rc) return rc;
    lattice_t L;
    lattice_init(&L, g->nq);
    const int nq = L.nq;
    /* HalfWayBounceBack over all bulk nodes (main_TWOPHASE.cpp:81) */
    bb_links bb;
    if (bb_build(&L, g, g->bulk, g->n_bulk, &bb)) return -10;
    int nsb = 0;
    for (int n = 1; n < g->n_nodes; ++n) nsb += g->types[n] == 1;
    int32_t* solid = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsb > 0 ? nsb : 1));
    if (!solid) return -10;
    nsb = 0;
    for (int n = 1; n < g->n_nodes; ++n)
        if (g->types[n] == 1) solid[nsb++] = n;

    tp_ctx c;
    memset(&c, 0, sizeof(c));
    c.L = &L;
    c.g = g;
    c.rho = rho;
    c.vel = vel;
    c.cg = cg;
    c.cgw = cg;
    c.nu0inv = 1.0 / (C2 * (tau0 - 0.5));
    c.nu1inv = 1.0 / (C2 * (tau1 - 0.5));
    c.sigma = sigma;
    c.beta = beta;
    c.F = force;
    double* cur = f;
    double* nxt = ftmp;
    for (int i = 0; i < nsteps; ++i) {
        c.f = cur;
        c.ftmp = nxt;
        parallel_for(g->n_bulk, nthreads, tp_density_slice, &c);
        for (int s = 0; s < nsb; ++s) {
            const size_t node = (size_t)solid[s];
            const double r0 = rho[node * 2], r1 = rho[node * 2 + 1];
            cg[node] = (r0 - r1) / (r0 + r1);
        }
        if (flux_control) {
            /* flux controller, serial sum in bulk order (main_TWOPHASE.cpp:292-308) */
            double mean = 0.0;
            double ft[19], j[3];
            for (int b = 0; b < g->n_bulk; ++b) {
                const double* f0 = cur + (size_t)g->bulk[b] * 2 * nq;
                for (int q = 0; q < nq; ++q) ft[q] = f0[q] + f0[nq + q];
                qsumc(&L, ft, j);
                mean += j[0];
            }
            mean /= g->n_bulk;
            force[0] = 2 * (mom_x - mean);
        }
        if (force_log) force_log[i] = force[0];
        parallel_for(g->n_bulk, nthreads, tp_collide_slice, &c);
        double* t = cur; cur = nxt; nxt = t;
        for (int field = 0; field < 2; ++field) {
            bb_ctx bc = {&L, g, &bb, cur, 2, field};
            parallel_for(bb.n, nthreads, bb_slice, &bc);
        }
    }
    bb_free(&bb);
    free(solid);
    return cur == f ? 0 : 1;
}


/* ---- std_one_phase (src/std_one_phase/main.cpp:24-203, 318-575) ---- */
typedef struct {
    const lattice_t* L;
    const oracle_grid* g;
    double tau;
    const double* bf;
    const int32_t* labels;
    const int32_t* force_on;
    const double* scale;
    const double* mchange;
    const double* add;
    const double* f;
    double* ftmp;
    double* rho;
    double* vel;
} links_ctx;

static void links_slice(void* p, int begin, int end) {
    links_ctx* c = (links_ctx*)p;
    const lattice_t* L = c->L;
    double fn[19], cu[19], cF[19], vel[3], j[3], F[3];
    for (int b = begin; b < end; ++b) {
        const size_t node = (size_t)c->g->bulk[b];
        memcpy(fn, c->f + node * 19, sizeof(double) * 19);
        double rho = qsum(L, fn);
        const int label = c->labels[node];
        /* main.cpp:504-507 */
        const double qm = 0.9 * 2 * c->scale[label] * c->mchange[label] * c->add[node];
        rho += 0.5 * qm;
        for (int d = 0; d < 3; ++d) F[d] = c->bf[d] * (double)c->force_on[node];
        qsumc(L, fn, j);
        for (int d = 0; d < 3; ++d) vel[d] = (j[d] + 0.5 * F[d]) / rho;
        c->rho[node] = rho;
        for (int d = 0; d < 3; ++d) c->vel[node * 3 + d] = vel[d];
        const double u2 = dotv(L, vel, vel);
        cdotall(L, vel, cu);
        const double uF = dotv(L, vel, F);
        cdotall(L, F, cF);
        const double tau_inv = 1.0 / c->tau;
        const double tf = (1 - 0.5 / c->tau);
        const int32_t* nb = c->g->neigh + node * 19;
        for (int q = 0; q < 19; ++q) {
            /* calcOmegaBGK, calcDeltaOmegaF, calcDeltaOmegaQ (LBcollision.h:38-45, 80-98, 205-212) */
            const double om = -tau_inv * (fn[q] - rho * L->w[q] * (1.0 + C2INV * cu[q] + C4INV0_5 * (cu[q] * cu[q] - C2 * u2)));
            const double dF = L->w[q] * tf * (C2INV * cF[q] + C4INV * (cF[q] * cu[q] - C2 * uF));
            const double dQ = tf * qm * L->w[q] * (1.0 + C2INV * cu[q] + C4INV0_5 * (cu[q] * cu[q] - C2 * u2));
            c->ftmp[(size_t)nb[q] * 19 + q] = fn[q] + om + dF + dQ;
        }
    }
}

int oracle_links_run(const oracle_grid* g, int nsteps, double tau, const double* force, const int32_t* tags,
                     const int32_t* labels, const int32_t* force_on, double rho_w, double* f, double* ftmp,
                     double* rho, double* vel, double* flux, int nthreads) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (g->nq != 19 || !tags || !labels || !force_on) return -1;
    lattice_t L;
    lattice_init(&L, 19);
    const int N = g->n_nodes;
#define TAG(n) ((n) == 0 ? -1 : tags[(n)])
    /* link lists (findSolidFluidLinks, findPressureFluidLinks, findFluidFluidLinks):
     * {node, qUnknown, neighbour, qKnown} */
    int nsf = 0, npf = 0, nff = 0, cap = 0;
    for (int n = 1; n < N; ++n) cap += 18;
    int32_t* sf = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)cap);
    int32_t* pf = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)cap);
    int32_t* ff = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)cap);
    int lmax = 0;
    for (int n = 1; n < N; ++n)
        if (labels[n] > lmax) lmax = labels[n];
    double* scale = (double*)calloc((size_t)lmax + 1, sizeof(double));
    double* mchange = (double*)calloc((size_t)lmax + 1, sizeof(double));
    double* add = (double*)calloc((size_t)N, sizeof(double));
    if (!sf || !pf || !ff || !scale || !mchange || !add) return -10;
    for (int n = 1; n < N; ++n) {
        const int t = TAG(n);
        for (int q = 0; q < 18; ++q) {
            const int nn = g->neigh[(size_t)n * 19 + q];
            const int tn = TAG(nn);
            int32_t* rec = NULL;
            if (((t >> 3) & 1) && (tn & 3) == 0) rec = sf + 4 * nsf++;
            if (rec) { rec[0] = n; rec[1] = L.rev[q]; rec[2] = nn; rec[3] = q; }
            rec = NULL;
            if (((t >> 4) & 1) && (tn & 3) == 3) rec = pf + 4 * npf++;
            if (rec) { rec[0] = n; rec[1] = L.rev[q]; rec[2] = nn; rec[3] = q; }
            rec = NULL;
            if (((t >> 2) & 1) && (t & 3) == 1 && (tn & 3) == 2) rec = ff + 4 * nff++;
            if (rec) { rec[0] = n; rec[1] = L.rev[q]; rec[2] = nn; rec[3] = q; }
        }
    }
    /* interior-domain sources (main.cpp:331-358) */
    for (int n = 1; n < N; ++n)
        if (labels[n] > 0 && TAG(n) < 3) {
            scale[labels[n]] += 1;
            add[n] = 1.0;
        }
    for (int i = 1; i <= lmax; ++i) {
        if (scale[i] == 0.0) return -20;
        scale[i] = 1.0 / scale[i];
    }
    links_ctx c;
    memset(&c, 0, sizeof(c));
    c.L = &L;
    c.g = g;
    c.tau = tau;
    c.bf = force;
    c.labels = labels;
    c.force_on = force_on;
    c.scale = scale;
    c.mchange = mchange;
    c.add = add;
    c.rho = rho;
    c.vel = vel;
    double* cur = f;
    double* nxt = ftmp;
    for (int it = 0; it < nsteps; ++it) {
        /* main.cpp:486-495 */
        for (int l = 0; l <= lmax; ++l) mchange[l] = 0.0;
        for (int b = 0; b < g->n_bulk; ++b) {
            const int n = g->bulk[b];
            mchange[labels[n]] += 1.0 - qsum(&L, cur + (size_t)n * 19);
        }
        c.f = cur;
        c.ftmp = nxt;
        parallel_for(g->n_bulk, nthreads, links_slice, &c);
        double* t = cur; cur = nxt; nxt = t;
        for (int k = 0; k < nsf; ++k) {  /* applySolidFluidBoundary */
            const int32_t* r = sf + 4 * k;
            cur[(size_t)r[0] * 19 + r[1]] = cur[(size_t)r[2] * 19 + r[3]];
        }
        for (int k = 0; k < npf; ++k) {  /* applyPressureFluidBoundary (anti-bounce-back) */
            const int32_t* r = pf + 4 * k;
            const double* u = vel + (size_t)r[0] * 3;
            const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
            const double cu = L.c[r[3]][0] * u[0] + L.c[r[3]][1] * u[1] + L.c[r[3]][2] * u[2];
            const double w = L.w[r[3]];
            cur[(size_t)r[0] * 19 + r[1]] = -cur[(size_t)r[2] * 19 + r[3]] + 2 * w * rho_w * (1 + 0.5 * (C4INV * cu * cu - C2INV * u2));
        }
        for (int k = 0; k < nff; ++k) {  /* applyFluidFluidBoundary (its correction is 0) */
            const int32_t* r = ff + 4 * k;
            const double f1 = cur[(size_t)r[0] * 19 + r[1]];
            cur[(size_t)r[0] * 19 + r[1]] = cur[(size_t)r[2] * 19 + r[3]];
            cur[(size_t)r[2] * 19 + r[3]] = f1;
        }
    }
    if (flux) {  /* main.cpp:550-562 */
        double s[2] = {0.0, 0.0};
        for (int n = 1; n < N; ++n)
            if ((TAG(n) >> 4) & 1) {
                const int ph = (TAG(n) & 3) - 1;
                if (ph != 0 && ph != 1) return -21;
                s[ph] += vel[(size_t)n * 3 + 2] * rho[n];
            }
        flux[0] = 0.5 * s[0];
        flux[1] = 0.5 * s[1];
    }
#undef TAG
    free(sf); free(pf); free(ff); free(scale); free(mchange); free(add);
    return cur == f ? 0 : 1;
}
