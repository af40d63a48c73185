/*
 * hmec_oracle.c -- CPU restatement of the H-MEC per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle; never part of the product path).
 *
 * Follows cpp/h_mec_rsf_v9.cpp of lucadalzilio/H-MECs-2D section by section;
 * each function cites the lines it restates.  Conventions carried over so
 * the numbers agree with the reference as written:
 *   - grids are column-major, element (i, j) at j*rows + i (Eigen MatrixXd);
 *   - every Eigen 2x2 block .sum() is taken in column-major order
 *     (0,0)+(1,0)+(0,1)+(1,1) (Eigen's vectorised reduction may order the
 *     four terms differently, a last-bit effect);
 *   - std::min/std::max are (b<a?b:a) and (a<b?b:a), which decide NaN
 *     cases the way the reference's calls do;
 *   - pow(x, 2) is x*x (correctly rounded either way);
 *   - compiled with -ffp-contract=off so no multiply-add is fused on any
 *     host (aarch64 GCC fuses by default).
 * Quirks of the reference reproduced here (they change numbers):
 *   Q1 the per-step reset of the marker sums (:377-381) runs on copies and
 *      does nothing, so sums accumulate over timesteps (flag
 *      quirk_accumulate_sums; default off = sums restart each step, as the
 *      evident intent and as the GPU does);
 *   Q2 copy_bounds() on range-for copies (:1130-1132) is a no-op, so the
 *      ghost rows/columns of SXX, SYY stay zero;
 *   Q4 the as-written RK stage shift of the (dead) advection loop
 *      (:1622-1630), behind rk4_as_written;
 *   Q6 every field starts at zero;
 *   Q7 duplicate triplets are summed (Eigen setFromTriplets, :1047);
 *   Q8 the bisection only runs on a sign change of the stress residual;
 *   Q9 node coordinates follow Eigen's LinSpaced: low + i*step with
 *      step = (high-low)/(n-1) and the last point exactly `high`.
 * The fault-stress bisection (:1224) has no cap in the reference; here it
 * stops after rsf_maxit iterations and raises a flag.
 */
#include "hmec_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define DMIN(a, b) ((b) < (a) ? (b) : (a))
#define DMAX(a, b) ((a) < (b) ? (b) : (a))

/* Marker sums kept across steps (quirk Q1). */
enum { SB_RHO, SB_KKK, SB_TTT, SB_GGG, SB_ETA0, SB_COHT, SB_FRIT, SB_COHC, SB_FRIC, SB_DILC, SB_WT, SB_N };
enum { SP_ETAP, SP_POR, SP_ETAB0, SP_ETAP0, SP_GGGP, SP_WT, SP_N };
enum { SV_RHO, SV_ETAD, SV_RHOF, SV_POR, SV_WT, SV_N };

struct hmo_state {
    hmec_params p;
    int Nx, Ny, Nx1, Ny1, N, line_fault;
    double dx, dy, dx2, dy2, dx_dy, lower_block, upper_block, dy_faultw;
    double* crd[8]; /* x, y, xvx, yvx, xvy, yvy, xp, yp */
    int64_t marknum;
    double* mk[HMEC_M_COUNT];
    double* f[HMEC_F_COUNT];
    double* sb[SB_N];
    double* sp[SP_N];
    double* sx[SV_N];
    double* sy[SV_N];
    double sc[HMEC_S_COUNT];
    double* DSYLSQ;
    double maxvxy0;
    double ptscale, pfscale;
    double* R;
    /* triplets and CSR */
    int64_t ntrip, tcap;
    int32_t* ti;
    int32_t* tj;
    double* tv;
    int64_t* indptr;
    int32_t* indices;
    double* data;
    int64_t nnz;
    int32_t last_ynpl;
    double last_dsylsq;
    int32_t rsf_noconv;
    int nthreads; /* threads of the marker loop (1: the serial loop) */
};

/* ------------------------------------------------------------ constants */

void hmo_params_default(hmec_params* p) {
    /* cpp/constants.hpp:13-146 */
    memset(p, 0, sizeof(*p));
    p->Nx = 401;
    p->Ny = 51;
    p->xsize = 40000.;
    p->ysize = 10000.;
    p->mx = 4;
    p->my = 4;
    p->TS_1 = 2e3;
    p->TS_2 = 4e3;
    p->TS_3 = 34e3;
    p->TS_4 = 38e3;
    p->dtelastic0 = 5e8;
    p->dtmin = 1e-4;
    p->inertia = 1.;
    p->arsfm[0] = .025; p->arsfm[1] = .006;
    p->brsfm[0] = .001; p->brsfm[1] = .015;
    p->lrsfm[0] = .020; p->lrsfm[1] = .0085;
    p->omm[0] = 10; p->omm[1] = -10;
    p->V0 = 1.e-9;
    p->alpha = 29;
    p->POR0 = .01;
    p->cohes = 0.;
    p->friction = .6;
    p->dilatation = 0.;
    p->tensile = 1.;
    p->shearmod = 3.e10;
    p->BETAFLUID = 1.e-8;
    p->BETASOLID = 2.e-11;
    p->gx = 0.;
    p->gy = 0.;
    p->PCONF = 1.e7;
    p->PTFDIFF = 3.e7;
    p->etamin = 1e-3;
    p->etamax = 1e50;
    p->kkkmin = 1e-22;
    p->kkkmax = 1e-12;
    p->stpmax = 2e-4;
    p->stpmax1 = 6e-5;
    p->bcupper = -1e-9;
    p->bclower = 1e-9;
    p->bcvyflower = 0;
    p->niterglobal = 10000;
    p->ynlastmax = 499;
    p->dtstep = 5;
    p->vratiomax = 0.001;
    p->dtkoef = 1.1;
    p->dtkoefup = 1.2;
    p->dtkoefv = 1.001;
    p->errmin = 1e2;
    p->etawt = 0.0;
    p->syieldmin = 1e-3;
    p->tyield = 1;
    p->num_timesteps = 100000;
    p->form = HMEC_FORM_FP64;
    p->krylov_rtol = 1e-15;
    p->krylov_restart = 40;
    p->krylov_maxit = 2000;
    p->mg_levels = 5;
    p->mg_pre = 2;
    p->mg_post = 2;
    p->mg_coarse_sweeps = 8;
    p->rsf_maxit = 10000;
    p->advect_markers = 0;
    p->rk4_as_written = 0;
    p->quirk_accumulate_sums = 0;
    p->bounds_check = 0;
    p->mg_flags = 1; /* HMEC_MG_DARCY_HARMONIC */
    p->graph = 1;
    p->autotune = 1;
    p->invariants_every = 1;
}

/* Eigen 3.3 LinSpaced(n, low, high) for |high| >= |low| (all grids here). */
static void linspaced(double* out, int n, double low, double high) {
    double step = (n == 1) ? 0. : (high - low) / (double)(n - 1);
    for (int i = 0; i < n; i++) out[i] = (i == n - 1) ? high : low + (double)i * step;
}

/* h_mec_rsf_v9.cpp:119-121 -- truncation toward zero. */
static int fix_(double t) { return t < 0. ? (int)ceil(t) : (int)floor(t); }
/* :144-151 */
static int check_bounds(int k, int bound) {
    if (k < 0) k = 0;
    else if (k > bound - 2) k = bound - 2;
    return k;
}
/* :124-131 */
static double enforce_bounds(double v, double lo, double hi) {
    if (v < lo) v = lo;
    else if (v > hi) v = hi;
    return v;
}
/* :139-141 */
static double divplus(double x, double y) { return x / (x + y); }

#define BI(F, i, j) (st->f[HMEC_F_##F][(size_t)(j) * Ny + (i)])
#define SI(F, i, j) (st->f[HMEC_F_##F][(size_t)(j) * Ny1 + (i)])
/* column-major sum of the 2x2 block starting at (i, j) of a grid with `rows` rows */
static double block_sum(const double* a, int rows, int i, int j) {
    const double* c0 = a + (size_t)j * rows + i;
    const double* c1 = c0 + rows;
    return ((c0[0] + c0[1]) + c1[0]) + c1[1];
}
/* Eigen square_block (:134-136): row-major comma order m00, m01, m10, m11 */
static double square4(double m00, double m01, double m10, double m11) {
    return ((m00 * m00 + m01 * m01) + m10 * m10) + m11 * m11;
}

hmo_state* hmo_create(const hmec_params* pin) {
    hmo_state* st = (hmo_state*)calloc(1, sizeof(hmo_state));
    if (!st) return NULL;
    st->p = *pin;
    const hmec_params* p = &st->p;
    int Nx = p->Nx, Ny = p->Ny;
    st->Nx = Nx;
    st->Ny = Ny;
    st->Nx1 = Nx + 1;
    st->Ny1 = Ny + 1;
    st->N = st->Nx1 * st->Ny1 * 6;
    st->line_fault = (int)((Ny - 1) / 2.);
    st->dx = p->xsize / (Nx - 1);
    st->dy = p->ysize / (Ny - 1);
    st->dx2 = st->dx * st->dx;
    st->dy2 = st->dy * st->dy;
    st->dx_dy = st->dx * st->dy;
    st->lower_block = p->ysize / 2. + st->dy;
    st->upper_block = p->ysize / 2. - st->dy;
    st->dy_faultw = st->dy / st->dx; /* faultwidth = dx, constants.hpp:66, :175 */
    double dx = st->dx, dy = st->dy;
    int n1[8] = {Nx, Ny, Nx + 1, Ny + 1, Nx + 1, Ny + 1, Nx + 1, Ny + 1};
    for (int k = 0; k < 8; k++) st->crd[k] = (double*)calloc(n1[k], sizeof(double));
    /* constants.hpp:57-64 */
    linspaced(st->crd[0], Nx, 0, p->xsize);
    linspaced(st->crd[1], Ny, 0, p->ysize);
    linspaced(st->crd[2], Nx + 1, 0, p->xsize + dx);
    linspaced(st->crd[3], Ny + 1, 0 - dy / 2., p->ysize + dy / 2.);
    linspaced(st->crd[4], Nx + 1, 0 - dx / 2., p->xsize + dx / 2.);
    linspaced(st->crd[5], Ny + 1, 0, p->ysize + dy);
    linspaced(st->crd[6], Nx + 1, 0 - dx / 2., p->xsize + dx / 2.);
    linspaced(st->crd[7], Ny + 1, 0 - dy / 2., p->ysize + dy / 2.);
    st->marknum = (int64_t)(Nx - 1) * p->mx * (int64_t)(Ny - 1) * p->my;
    for (int k = 0; k < HMEC_M_COUNT; k++) st->mk[k] = (double*)calloc((size_t)st->marknum, sizeof(double));
    size_t nb = (size_t)Nx * Ny, ns = (size_t)(Nx + 1) * (Ny + 1);
#define HMO_ALLOC(name, grid) st->f[HMEC_F_##name] = (double*)calloc(grid ? ns : nb, sizeof(double));
    HMEC_FIELD_LIST(HMO_ALLOC)
#undef HMO_ALLOC
    for (int k = 0; k < SB_N; k++) st->sb[k] = (double*)calloc(nb, sizeof(double));
    for (int k = 0; k < SP_N; k++) st->sp[k] = (double*)calloc(ns, sizeof(double));
    for (int k = 0; k < SV_N; k++) st->sx[k] = (double*)calloc(ns, sizeof(double));
    for (int k = 0; k < SV_N; k++) st->sy[k] = (double*)calloc(ns, sizeof(double));
    st->DSYLSQ = (double*)calloc((size_t)p->niterglobal + 1, sizeof(double));
    st->R = (double*)calloc((size_t)st->N, sizeof(double));
    st->tcap = (int64_t)st->N * 10;
    st->ti = (int32_t*)malloc(sizeof(int32_t) * st->tcap);
    st->tj = (int32_t*)malloc(sizeof(int32_t) * st->tcap);
    st->tv = (double*)malloc(sizeof(double) * st->tcap);
    st->indptr = (int64_t*)calloc((size_t)st->N + 1, sizeof(int64_t));
    st->indices = NULL;
    st->data = NULL;
    /* h_mec_rsf_v9.cpp:101-103 */
    st->sc[HMEC_S_timesum] = 0;
    st->sc[HMEC_S_dt] = p->dtelastic0;
    st->sc[HMEC_S_yndtdecrease] = 1;
    st->sc[HMEC_S_timestep] = 1;
    st->nthreads = 1;
    return st;
}

void hmo_destroy(hmo_state* st) {
    if (!st) return;
    for (int k = 0; k < 8; k++) free(st->crd[k]);
    for (int k = 0; k < HMEC_M_COUNT; k++) free(st->mk[k]);
    for (int k = 0; k < HMEC_F_COUNT; k++) free(st->f[k]);
    for (int k = 0; k < SB_N; k++) free(st->sb[k]);
    for (int k = 0; k < SP_N; k++) free(st->sp[k]);
    for (int k = 0; k < SV_N; k++) free(st->sx[k]);
    for (int k = 0; k < SV_N; k++) free(st->sy[k]);
    free(st->DSYLSQ);
    free(st->R);
    free(st->ti);
    free(st->tj);
    free(st->tv);
    free(st->indptr);
    free(st->indices);
    free(st->data);
    free(st);
}

int64_t hmo_marknum(const hmo_state* st) { return st->marknum; }
int32_t hmo_unknowns(const hmo_state* st) { return st->N; }
double* hmo_field(hmo_state* st, int32_t f) { return (f >= 0 && f < HMEC_F_COUNT) ? st->f[f] : NULL; }
double* hmo_marker(hmo_state* st, int32_t f) { return (f >= 0 && f < HMEC_M_COUNT) ? st->mk[f] : NULL; }
double hmo_get_scalar(const hmo_state* st, int32_t id) { return (id >= 0 && id < HMEC_S_COUNT) ? st->sc[id] : NAN; }
void hmo_set_scalar(hmo_state* st, int32_t id, double v) {
    if (id >= 0 && id < HMEC_S_COUNT) st->sc[id] = v;
}
const double* hmo_coords(const hmo_state* st, int32_t w) { return (w >= 0 && w < 8) ? st->crd[w] : NULL; }
int32_t hmo_last_ynpl(const hmo_state* st) { return st->last_ynpl; }
double hmo_last_dsylsq(const hmo_state* st) { return st->last_dsylsq; }
int32_t hmo_rsf_noconv(const hmo_state* st) { return st->rsf_noconv; }

/* ------------------------------------------------ a1-a4: markers -> nodes */

static void add_block(double* s, int rows, int i, int j, double v, const double w[4]) {
    /* Sub-block += v * wtm, wtm = [w00 w01; w10 w11] (comma init, :444) */
    double* c0 = s + (size_t)j * rows + i;
    double* c1 = c0 + rows;
    c0[0] += v * w[0];
    c1[0] += v * w[1];
    c0[1] += v * w[2];
    c1[1] += v * w[3];
}
static void add_wt(double* s, int rows, int i, int j, const double w[4]) {
    double* c0 = s + (size_t)j * rows + i;
    double* c1 = c0 + rows;
    c0[0] += w[0];
    c1[0] += w[1];
    c0[1] += w[2];
    c1[1] += w[3];
}
static void weights(double dxm, double dym, double w[4]) {
    w[0] = (1 - dxm) * (1 - dym);
    w[1] = dxm * (1 - dym);
    w[2] = (1 - dxm) * dym;
    w[3] = dxm * dym;
}

/* The marker sums of one pass: the node sums the loop adds into. */
typedef struct {
    double* sb[SB_N];
    double* sp[SP_N];
    double* sx[SV_N];
    double* sy[SV_N];
} hmo_sums;

/* Markers m0 .. m1-1 added into the sums s (:385-529). */
static void accumulate_markers(const hmo_state* st, int64_t m0, int64_t m1, const hmo_sums* s) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Ny1 = st->Ny1;
    const double dx = st->dx, dy = st->dy;
    const double *x = st->crd[0], *y = st->crd[1], *xvx = st->crd[2], *yvx = st->crd[3];
    const double *xvy = st->crd[4], *yvy = st->crd[5], *xp = st->crd[6], *yp = st->crd[7];
    double* const* mk = st->mk;
    for (int64_t m = m0; m < m1; m++) { /* :385-529, in marker order */
        const double por = mk[HMEC_M_porm][m];
        double kkkmm = mk[HMEC_M_kkkm][m] * pow(por / p->POR0, 3);
        kkkmm = enforce_bounds(kkkmm, p->kkkmin, p->kkkmax);
        double cohescmm, cohestmm, frictcmm, dilatcmm, fricttmm, etasmm0, etamm0, etamm, rhomm;
        if (mk[HMEC_M_t_marker][m] != 0) {
            cohescmm = mk[HMEC_M_cohescm][m] * (1 - por);
            cohestmm = mk[HMEC_M_cohestm][m] * (1 - por);
            frictcmm = mk[HMEC_M_frictcm][m];
            dilatcmm = mk[HMEC_M_dilatcm][m];
            fricttmm = mk[HMEC_M_fricttm][m];
            etasmm0 = mk[HMEC_M_etasm][m];
            etamm0 = mk[HMEC_M_etasm][m] * exp(-p->alpha * por);
            etamm = mk[HMEC_M_etam][m];
            rhomm = mk[HMEC_M_rhom][m] * (1 - por) + mk[HMEC_M_rhofm][m] * por;
        } else {
            cohescmm = mk[HMEC_M_cohescm][m];
            cohestmm = mk[HMEC_M_cohestm][m];
            frictcmm = mk[HMEC_M_frictcm][m];
            dilatcmm = 0;
            fricttmm = mk[HMEC_M_fricttm][m];
            etasmm0 = mk[HMEC_M_etasm][m];
            etamm0 = mk[HMEC_M_etasm][m];
            etamm = mk[HMEC_M_etam][m];
            rhomm = mk[HMEC_M_rhom][m];
        }
        etamm0 = enforce_bounds(etamm0, p->etamin, p->etamax);
        etamm = enforce_bounds(etamm, p->etamin, p->etamax);
        const double etadm = mk[HMEC_M_etafm][m] / kkkmm;
        const double xmm = mk[HMEC_M_xm][m], ymm = mk[HMEC_M_ym][m];
        const double invg = 1. / mk[HMEC_M_gm][m];
        double w[4];
        /* basic nodes :432-459 */
        int j = check_bounds(fix_(xmm / dx), Nx);
        int i = check_bounds(fix_(ymm / dy), Ny);
        weights((xmm - x[j]) / dx, (ymm - y[i]) / dy, w);
        add_block(s->sb[SB_RHO], Ny, i, j, rhomm, w);
        add_block(s->sb[SB_KKK], Ny, i, j, kkkmm, w);
        add_block(s->sb[SB_TTT], Ny, i, j, mk[HMEC_M_t_marker][m], w);
        add_block(s->sb[SB_GGG], Ny, i, j, invg, w);
        add_block(s->sb[SB_ETA0], Ny, i, j, etamm0, w);
        add_block(s->sb[SB_COHT], Ny, i, j, cohestmm, w);
        add_block(s->sb[SB_FRIT], Ny, i, j, fricttmm, w);
        add_block(s->sb[SB_COHC], Ny, i, j, cohescmm, w);
        add_block(s->sb[SB_FRIC], Ny, i, j, frictcmm, w);
        add_block(s->sb[SB_DILC], Ny, i, j, dilatcmm, w);
        add_wt(s->sb[SB_WT], Ny, i, j, w);
        /* pressure nodes :468-484 */
        j = check_bounds(fix_((xmm + dx / 2.) / dx), Nx);
        i = check_bounds(fix_((ymm + dy / 2.) / dy), Ny);
        weights((xmm - xp[j]) / dx, (ymm - yp[i]) / dy, w);
        add_block(s->sp[SP_ETAP], Ny1, i, j, etamm, w);
        add_block(s->sp[SP_POR], Ny1, i, j, por, w);
        add_block(s->sp[SP_GGGP], Ny1, i, j, invg, w);
        add_block(s->sp[SP_ETAP0], Ny1, i, j, etamm0, w);
        add_block(s->sp[SP_ETAB0], Ny1, i, j, etasmm0, w);
        add_wt(s->sp[SP_WT], Ny1, i, j, w);
        /* Vx nodes :493-506 */
        j = check_bounds(fix_(xmm / dx), Nx);
        i = check_bounds(fix_((ymm + dy / 2.) / dy), Ny);
        weights((xmm - xvx[j]) / dx, (ymm - yvx[i]) / dy, w);
        add_block(s->sx[SV_RHO], Ny1, i, j, rhomm, w);
        add_block(s->sx[SV_ETAD], Ny1, i, j, 1. / etadm, w);
        add_block(s->sx[SV_RHOF], Ny1, i, j, mk[HMEC_M_rhofm][m], w);
        add_block(s->sx[SV_POR], Ny1, i, j, por, w);
        add_wt(s->sx[SV_WT], Ny1, i, j, w);
        /* Vy nodes :515-528 */
        j = check_bounds(fix_((xmm + dx / 2.) / dx), Nx);
        i = check_bounds(fix_(ymm / dy), Ny);
        weights((xmm - xvy[j]) / dx, (ymm - yvy[i]) / dy, w);
        add_block(s->sy[SV_RHO], Ny1, i, j, rhomm, w);
        add_block(s->sy[SV_ETAD], Ny1, i, j, 1. / etadm, w);
        add_block(s->sy[SV_RHOF], Ny1, i, j, mk[HMEC_M_rhofm][m], w);
        add_block(s->sy[SV_POR], Ny1, i, j, por, w);
        add_wt(s->sy[SV_WT], Ny1, i, j, w);
    }
}

/* The marker loop on several threads (the reference runs it as an OpenMP
 * parallel loop, :384, whose threads add into shared sums without
 * synchronisation).  Here thread t takes the t-th contiguous share of the
 * markers into sums of its own (thread 0 into the state's), and the shares
 * are then added in thread order, each thread over its own slice of the
 * nodes: deterministic for a given thread count, equal to the serial loop
 * up to the order of the additions. */
typedef struct {
    const hmo_state* st;
    int64_t m0, m1;
    hmo_sums s;
    int t, T;
    hmo_sums* all;
    size_t nb, ns;
} hmo_job;

static void* accumulate_job(void* arg) {
    hmo_job* j = (hmo_job*)arg;
    accumulate_markers(j->st, j->m0, j->m1, &j->s);
    return NULL;
}

static void add_slice(double* dst, double* const* src, int T, size_t n, int t) {
    const size_t a = n * (size_t)t / (size_t)T, b = n * (size_t)(t + 1) / (size_t)T;
    for (size_t k = a; k < b; k++) {
        double v = dst[k];
        for (int u = 1; u < T; u++) v += src[u][k];
        dst[k] = v;
    }
}

static void* reduce_job(void* arg) {
    hmo_job* j = (hmo_job*)arg;
    double* src[256];
    for (int k = 0; k < SB_N; k++) {
        for (int u = 1; u < j->T; u++) src[u] = j->all[u].sb[k];
        add_slice(j->all[0].sb[k], src, j->T, j->nb, j->t);
    }
    for (int k = 0; k < SP_N; k++) {
        for (int u = 1; u < j->T; u++) src[u] = j->all[u].sp[k];
        add_slice(j->all[0].sp[k], src, j->T, j->ns, j->t);
    }
    for (int k = 0; k < SV_N; k++) {
        for (int u = 1; u < j->T; u++) src[u] = j->all[u].sx[k];
        add_slice(j->all[0].sx[k], src, j->T, j->ns, j->t);
        for (int u = 1; u < j->T; u++) src[u] = j->all[u].sy[k];
        add_slice(j->all[0].sy[k], src, j->T, j->ns, j->t);
    }
    return NULL;
}

/* Returns 0, or -1 when a buffer or a thread could not be had (the sums are
 * then formed by the serial loop). */
static int accumulate_threaded(hmo_state* st, int T, size_t nb, size_t ns) {
    hmo_sums* all = (hmo_sums*)calloc((size_t)T, sizeof(hmo_sums));
    hmo_job* job = (hmo_job*)calloc((size_t)T, sizeof(hmo_job));
    pthread_t* th = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
    int ok = all && job && th, started = 0;
    if (!ok) {
        free(all);
        free(job);
        free(th);
        return -1;
    }
    for (int k = 0; k < SB_N; k++) all[0].sb[k] = st->sb[k];
    for (int k = 0; k < SP_N; k++) all[0].sp[k] = st->sp[k];
    for (int k = 0; k < SV_N; k++) all[0].sx[k] = st->sx[k];
    for (int k = 0; k < SV_N; k++) all[0].sy[k] = st->sy[k];
    for (int u = 1; u < T && ok; u++) {
        for (int k = 0; k < SB_N; k++) ok = ok && (all[u].sb[k] = (double*)calloc(nb, sizeof(double)));
        for (int k = 0; k < SP_N; k++) ok = ok && (all[u].sp[k] = (double*)calloc(ns, sizeof(double)));
        for (int k = 0; k < SV_N; k++) ok = ok && (all[u].sx[k] = (double*)calloc(ns, sizeof(double)));
        for (int k = 0; k < SV_N; k++) ok = ok && (all[u].sy[k] = (double*)calloc(ns, sizeof(double)));
    }
    if (ok) {
        for (int t = 0; t < T; t++) {
            job[t].st = st;
            job[t].m0 = st->marknum * t / T;
            job[t].m1 = st->marknum * (t + 1) / T;
            job[t].s = all[t];
            job[t].t = t;
            job[t].T = T;
            job[t].all = all;
            job[t].nb = nb;
            job[t].ns = ns;
        }
        for (; started < T; started++)
            if (pthread_create(&th[started], NULL, accumulate_job, &job[started]) != 0) break;
        for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
        if (started < T) {
            /* the shares of the threads that never started, on this thread */
            for (int t = started; t < T; t++) accumulate_markers(st, job[t].m0, job[t].m1, &job[t].s);
        }
        started = 0;
        for (; started < T; started++)
            if (pthread_create(&th[started], NULL, reduce_job, &job[started]) != 0) break;
        for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
        for (int t = started; t < T; t++) reduce_job(&job[t]);
    }
    for (int u = 1; u < T; u++) {
        for (int k = 0; k < SB_N; k++) free(all[u].sb[k]);
        for (int k = 0; k < SP_N; k++) free(all[u].sp[k]);
        for (int k = 0; k < SV_N; k++) free(all[u].sx[k]);
        for (int k = 0; k < SV_N; k++) free(all[u].sy[k]);
    }
    free(all);
    free(job);
    free(th);
    return ok ? 0 : -1;
}

void hmo_set_threads(hmo_state* st, int32_t n) { st->nthreads = n < 1 ? 1 : (n > 256 ? 256 : n); }

void hmo_markers_to_nodes(hmo_state* st) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Ny1 = st->Ny1, Nx1 = st->Nx1;
    size_t nb = (size_t)Nx * Ny, ns = (size_t)Nx1 * Ny1;
    if (!p->quirk_accumulate_sums) { /* :377-381 as intended */
        for (int k = 0; k < SB_N; k++) memset(st->sb[k], 0, nb * sizeof(double));
        for (int k = 0; k < SP_N; k++) memset(st->sp[k], 0, ns * sizeof(double));
        for (int k = 0; k < SV_N; k++) memset(st->sx[k], 0, ns * sizeof(double));
        for (int k = 0; k < SV_N; k++) memset(st->sy[k], 0, ns * sizeof(double));
    }
    hmo_sums own;
    for (int k = 0; k < SB_N; k++) own.sb[k] = st->sb[k];
    for (int k = 0; k < SP_N; k++) own.sp[k] = st->sp[k];
    for (int k = 0; k < SV_N; k++) own.sx[k] = st->sx[k];
    for (int k = 0; k < SV_N; k++) own.sy[k] = st->sy[k];
    const int T = st->marknum >= 2 * (int64_t)st->nthreads ? st->nthreads : 1;
    if (T < 2 || accumulate_threaded(st, T, nb, ns) != 0) accumulate_markers(st, 0, st->marknum, &own);
    /* normalisation :531-583 */
    for (int i = 0; i < Ny; i++) {
        for (int j = 0; j < Nx; j++) {
            size_t k = (size_t)j * Ny + i;
            double wt = st->sb[SB_WT][k];
            if (wt > 0) {
                BI(RHO, i, j) = st->sb[SB_RHO][k] / wt;
                BI(KKK, i, j) = st->sb[SB_KKK][k] / wt;
                BI(TTT, i, j) = st->sb[SB_TTT][k] / wt;
                BI(GGG, i, j) = 1. / (st->sb[SB_GGG][k] / wt);
                BI(ETA0, i, j) = st->sb[SB_ETA0][k] / wt;
                BI(COHT, i, j) = st->sb[SB_COHT][k] / wt;
                BI(FRIT, i, j) = st->sb[SB_FRIT][k] / wt;
                BI(COHC, i, j) = st->sb[SB_COHC][k] / wt;
                BI(FRIC, i, j) = st->sb[SB_FRIC][k] / wt;
                BI(DILC, i, j) = st->sb[SB_DILC][k] / wt;
            }
        }
        for (int j = 0; j < Nx1; j++) {
            size_t k = (size_t)j * Ny1 + i;
            double wt = st->sy[SV_WT][k];
            if (wt > 0) {
                SI(RHOY, i, j) = st->sy[SV_RHO][k] / wt;
                SI(ETADY, i, j) = 1. / (st->sy[SV_ETAD][k] / wt);
                SI(RHOFY, i, j) = st->sy[SV_RHOF][k] / wt;
                SI(PORY, i, j) = st->sy[SV_POR][k] / wt;
            }
        }
    }
    for (int i = 0; i < Ny1; i++) {
        for (int j = 0; j < Nx; j++) {
            size_t k = (size_t)j * Ny1 + i;
            double wt = st->sx[SV_WT][k];
            if (wt > 0) {
                SI(RHOX, i, j) = st->sx[SV_RHO][k] / wt;
                SI(ETADX, i, j) = 1. / (st->sx[SV_ETAD][k] / wt);
                SI(RHOFX, i, j) = st->sx[SV_RHOF][k] / wt;
                SI(PORX, i, j) = st->sx[SV_POR][k] / wt;
            }
        }
        for (int j = 0; j < Nx1; j++) {
            size_t k = (size_t)j * Ny1 + i;
            double wt = st->sp[SP_WT][k];
            if (wt > 0) {
                SI(ETAP, i, j) = st->sp[SP_ETAP][k] / wt;
                SI(POR, i, j) = st->sp[SP_POR][k] / wt;
                SI(ETAB0, i, j) = st->sp[SP_ETAB0][k] / wt / SI(POR, i, j);
                SI(ETAP0, i, j) = st->sp[SP_ETAP0][k] / wt;
                SI(GGGP, i, j) = 1. / (st->sp[SP_GGGP][k] / wt);
            }
        }
    }
}

/* ------------------------------------------------------ a5: step begin */

void hmo_timestep_begin(hmo_state* st) {
    const hmec_params* p = &st->p;
    size_t nb = (size_t)st->Nx * st->Ny;
    const double* src = (st->sc[HMEC_S_timestep] == 1) ? st->f[HMEC_F_ETA0] : st->f[HMEC_F_ETA00];
    memmove(st->f[HMEC_F_ETA1], src, nb * sizeof(double));
    memmove(st->f[HMEC_F_ETA], src, nb * sizeof(double));
    memmove(st->f[HMEC_F_ETA50], src, nb * sizeof(double));
    memcpy(st->f[HMEC_F_OM], st->f[HMEC_F_OM0], nb * sizeof(double));
    double dt = st->sc[HMEC_S_dt];
    if (!st->sc[HMEC_S_yndtdecrease]) dt = DMAX(DMIN(dt * p->dtkoefup, p->dtelastic0), p->dtmin);
    else dt = DMAX(DMIN(dt, p->dtelastic0), p->dtmin);
    st->sc[HMEC_S_dt] = dt;
    st->sc[HMEC_S_yndtdecrease] = 0;
    st->sc[HMEC_S_dt00] = dt;
    st->sc[HMEC_S_ynlast] = 0;
    st->sc[HMEC_S_iterstep] = 0;
    memset(st->DSYLSQ, 0, sizeof(double) * ((size_t)p->niterglobal + 1));
}

/* ------------------------------------------------- a6-a8: iteration prep */

static void copy_bounds(hmo_state* st, double* T) {
    /* :154-159 (applied to the real matrix, as at :616-617) */
    const int Ny1 = st->Ny1, Nx = st->Nx, Ny = st->Ny;
    for (int i = 0; i < Ny1; i++) T[i] = T[(size_t)1 * Ny1 + i];
    for (int i = 0; i < Ny1; i++) T[(size_t)Nx * Ny1 + i] = T[(size_t)(Nx - 1) * Ny1 + i];
    for (int j = 0; j < Nx + 1; j++) T[(size_t)j * Ny1] = T[(size_t)j * Ny1 + 1];
    for (int j = 0; j < Nx + 1; j++) T[(size_t)j * Ny1 + Ny] = T[(size_t)j * Ny1 + Ny - 1];
}

void hmo_iter_prepare(hmo_state* st) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Ny1 = st->Ny1;
    const double dt = st->sc[HMEC_S_dt];
    const double etamincur = dt * p->shearmod * 1e-4; /* :612 */
    copy_bounds(st, st->f[HMEC_F_pt]);                /* :616-617 */
    copy_bounds(st, st->f[HMEC_F_pf]);
    for (int i = 0; i < Ny; i++) { /* :620-636 */
        for (int j = 0; j < Nx; j++) {
            if (BI(ETA, i, j) < etamincur) BI(ETA, i, j) = etamincur;
            if (BI(ETA, i, j) < BI(ETA0, i, j)) {
                const double sxx = block_sum(st->f[HMEC_F_SXX], Ny1, i, j);
                const double syy = block_sum(st->f[HMEC_F_SYY], Ny1, i, j);
                const double sxy = BI(SXY, i, j);
                BI(SIIB, i, j) = sqrt(sxy * sxy + (sxx * sxx + syy * syy + (sxx + syy) * (sxx + syy)) / 32.);
                BI(IETAPLB, i, j) = (1. / BI(ETA, i, j) - 1. / BI(ETA0, i, j));
                BI(EIIB, i, j) = st->dy_faultw * BI(SIIB, i, j) * BI(IETAPLB, i, j) / 2.;
            } else {
                BI(EIIB, i, j) = 0;
                BI(IETAPLB, i, j) = 0;
            }
        }
    }
    for (int i = 1; i < Ny; i++) { /* :639-669 */
        for (int j = 1; j < Nx; j++) {
            const double IETAPL = block_sum(st->f[HMEC_F_IETAPLB], Ny, i - 1, j - 1) / 4.;
            if (BI(YNY0, i - 1, j - 1) > 0 || BI(YNY0, i, j - 1) > 0 || BI(YNY0, i - 1, j) > 0 || BI(YNY0, i, j) > 0) {
                SI(ETAP, i, j) = 1. / (1. / SI(ETAP0, i, j) + IETAPL);
                SI(ETAB, i, j) = 1. / (1. / SI(ETAB0, i, j) + st->dy_faultw * IETAPL * SI(POR, i, j));
            } else {
                SI(ETAP, i, j) = SI(ETAP0, i, j);
                SI(ETAB, i, j) = SI(ETAB0, i, j);
            }
            if (SI(ETAP, i, j) < etamincur) SI(ETAP, i, j) = etamincur;
            if (SI(ETAB, i, j) * SI(POR, i, j) < etamincur) SI(ETAB, i, j) = etamincur / SI(POR, i, j);
            SI(GGGB, i, j) = SI(GGGP, i, j) / SI(POR, i, j);
            SI(DILP, i, j) = 0;
        }
    }
    /* :671-677 */
    double mn = INFINITY;
    for (int j = 0; j < Nx; j++)
        for (int i = 1; i < Ny; i++) mn = DMIN(mn, SI(ETADX, i, j));
    if (dt > 2e5) st->pfscale = mn * st->dx * 1e17 / (dt * dt);
    else st->pfscale = mn * st->dx;
    st->ptscale = st->pfscale;
}

/* ------------------------------------------------------ a9: assembly */

static void trp(hmo_state* st, int r, int c, double v) {
    if (st->ntrip == st->tcap) {
        st->tcap *= 2;
        st->ti = (int32_t*)realloc(st->ti, sizeof(int32_t) * st->tcap);
        st->tj = (int32_t*)realloc(st->tj, sizeof(int32_t) * st->tcap);
        st->tv = (double*)realloc(st->tv, sizeof(double) * st->tcap);
    }
    st->ti[st->ntrip] = r;
    st->tj[st->ntrip] = c;
    st->tv[st->ntrip] = v;
    st->ntrip++;
}

/* CSR from the triplet list, duplicates summed in list order (Eigen setFromTriplets). */
static void build_csr(hmo_state* st) {
    const int N = st->N;
    int64_t* cnt = (int64_t*)calloc((size_t)N + 1, sizeof(int64_t));
    for (int64_t t = 0; t < st->ntrip; t++) cnt[st->ti[t] + 1]++;
    for (int r = 0; r < N; r++) cnt[r + 1] += cnt[r];
    int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * ((size_t)N + 1));
    memcpy(pos, cnt, sizeof(int64_t) * ((size_t)N + 1));
    int32_t* cj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(st->ntrip + 1));
    double* cv = (double*)malloc(sizeof(double) * (size_t)(st->ntrip + 1));
    for (int64_t t = 0; t < st->ntrip; t++) {
        int64_t q = pos[st->ti[t]]++;
        cj[q] = st->tj[t];
        cv[q] = st->tv[t];
    }
    free(st->indices);
    free(st->data);
    st->indices = (int32_t*)malloc(sizeof(int32_t) * (size_t)(st->ntrip + 1));
    st->data = (double*)malloc(sizeof(double) * (size_t)(st->ntrip + 1));
    int64_t nnz = 0;
    st->indptr[0] = 0;
    for (int r = 0; r < N; r++) {
        int64_t b = cnt[r], e = cnt[r + 1];
        /* stable insertion sort by column within the row (rows are short) */
        for (int64_t a = b + 1; a < e; a++) {
            int32_t c = cj[a];
            double v = cv[a];
            int64_t q = a;
            while (q > b && cj[q - 1] > c) {
                cj[q] = cj[q - 1];
                cv[q] = cv[q - 1];
                q--;
            }
            cj[q] = c;
            cv[q] = v;
        }
        for (int64_t a = b; a < e; a++) {
            if (nnz > st->indptr[r] && st->indices[nnz - 1] == cj[a]) {
                st->data[nnz - 1] += cv[a];
            } else {
                st->indices[nnz] = cj[a];
                st->data[nnz] = cv[a];
                nnz++;
            }
        }
        st->indptr[r + 1] = nnz;
    }
    st->nnz = nnz;
    free(cnt);
    free(pos);
    free(cj);
    free(cv);
}

int64_t hmo_assemble(hmo_state* st) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Nx1 = st->Nx1, Ny1 = st->Ny1;
    const double dx = st->dx, dy = st->dy, dx2 = st->dx2, dy2 = st->dy2, dx_dy = st->dx_dy;
    const double dt = st->sc[HMEC_S_dt];
    const double ptscale = st->ptscale, pfscale = st->pfscale;
    const double gx = p->gx, gy = p->gy, inertia = p->inertia;
    const int NV = 6, RS = Ny1 * 6; /* Num_var, row stride of one grid column */
    double* R = st->R;
    st->ntrip = 0;
    memset(R, 0, sizeof(double) * (size_t)st->N); /* :685 */
    for (int j = 0; j < Nx1; j++) {
        for (int i = 0; i < Ny1; i++) {
            const int kp = (j * Ny1 + i) * NV; /* :690-695 */
            const int kx = kp + 1, ky = kp + 2, kpf = kp + 3, kxf = kp + 4, kyf = kp + 5;
            /* 5a) vxs :698-768 */
            if (i == 0 || i == Ny || j == 0 || j >= Nx - 1) {
                if (j == Nx) trp(st, kx, kx, 1);
                if (i == 0 && j < Nx) {
                    trp(st, kx, kx, 1);
                    trp(st, kx, kx + NV, 1);
                    R[kx] = 2 * p->bcupper;
                }
                if (i == Ny && j < Nx) {
                    trp(st, kx, kx, 1);
                    trp(st, kx, kx - NV, 1);
                    R[kx] = 2 * p->bclower;
                }
                if (j == 0 && i > 0 && i < Ny) {
                    trp(st, kx, kx, 1);
                    trp(st, kx, kx + RS, -1);
                }
                if (j == Nx - 1 && i > 0 && i < Ny) {
                    trp(st, kx, kx, 1);
                    trp(st, kx, kx - RS, -1);
                }
            } else {
                double ETAXY1 = BI(ETA, i - 1, j), ETAXY2 = BI(ETA, i, j);
                double ETAXX1 = SI(ETAP, i, j), ETAXX2 = SI(ETAP, i, j + 1);
                const double GXY1 = BI(GGG, i - 1, j), GXY2 = BI(GGG, i, j);
                const double GXX1 = SI(GGGP, i, j), GXX2 = SI(GGGP, i, j + 1);
                const double KXY1 = divplus(dt * GXY1, ETAXY1), KXY2 = divplus(dt * GXY2, ETAXY2);
                const double KXX1 = divplus(dt * GXX1, ETAXX1), KXX2 = divplus(dt * GXX2, ETAXX2);
                ETAXY1 *= KXY1;
                ETAXY2 *= KXY2;
                ETAXX1 *= KXX1;
                ETAXX2 *= KXX2;
                const double SXY1 = BI(SXY0, i - 1, j) * (1 - KXY1), SXY2 = BI(SXY0, i, j) * (1 - KXY2);
                const double SXX1 = SI(SXX0, i, j) * (1 - KXX1), SXX2 = SI(SXX0, i, j + 1) * (1 - KXX2);
                const double dRHOdx = (SI(RHOX, i, j + 1) - SI(RHOX, i, j - 1)) / (2. * dx);
                const double dRHOdy = (BI(RHO, i, j) - BI(RHO, i - 1, j)) / dy;
                const double temp = gx * dt * dRHOdy / 4.;
                trp(st, kx, kx, -(ETAXX1 + ETAXX2) / dx2 - (ETAXY1 + ETAXY2) / dy2 - gx * dt * dRHOdx - inertia * SI(RHOX, i, j) / dt);
                trp(st, kx, kx - RS, ETAXX1 / dx2);
                trp(st, kx, kx + RS, ETAXX2 / dx2);
                trp(st, kx, kx - NV, ETAXY1 / dy2);
                trp(st, kx, kx + NV, ETAXY2 / dy2);
                trp(st, kx, ky - NV, (ETAXY1 - ETAXX1) / dx_dy - temp);
                trp(st, kx, ky, (ETAXX1 - ETAXY2) / dx_dy - temp);
                trp(st, kx, ky - NV + RS, (ETAXX2 - ETAXY1) / dx_dy - temp);
                trp(st, kx, ky + RS, (ETAXY2 - ETAXX2) / dx_dy - temp);
                trp(st, kx, kp, ptscale / dx);
                trp(st, kx, kp + RS, -ptscale / dx);
                R[kx] = -SI(RHOX, i, j) * (inertia * SI(VX0, i, j) / dt + gx) - (SXX2 - SXX1) / dx - (SXY2 - SXY1) / dy;
            }
            /* 5b) vys :770-840 */
            if (j == 0 || j == Nx || i == 0 || i >= Ny - 1) {
                if (i == Ny) trp(st, ky, ky, 1);
                if (j == 0) {
                    trp(st, ky, ky, 1);
                    trp(st, ky, ky + RS, 1);
                }
                if (j == Nx) {
                    trp(st, ky, ky, 1);
                    trp(st, ky, ky - RS, 1);
                }
                if (i == 0 && j > 0 && j < Nx) trp(st, ky, ky, 1);
                if (i == Ny - 1 && j > 0 && j < Nx) trp(st, ky, ky, 1);
            } else {
                double ETAXY1 = BI(ETA, i, j - 1), ETAXY2 = BI(ETA, i, j);
                double ETAYY1 = SI(ETAP, i, j), ETAYY2 = SI(ETAP, i + 1, j);
                const double GXY1 = BI(GGG, i, j - 1), GXY2 = BI(GGG, i, j);
                const double GYY1 = SI(GGGP, i, j), GYY2 = SI(GGGP, i + 1, j);
                const double KXY1 = divplus(dt * GXY1, ETAXY1), KXY2 = divplus(dt * GXY2, ETAXY2);
                const double KYY1 = divplus(dt * GYY1, ETAYY1), KYY2 = divplus(dt * GYY2, ETAYY2);
                ETAXY1 *= KXY1;
                ETAXY2 *= KXY2;
                ETAYY1 *= KYY1;
                ETAYY2 *= KYY2;
                const double SXY1 = BI(SXY0, i, j - 1) * (1 - KXY1), SXY2 = BI(SXY0, i, j) * (1 - KXY2);
                const double SYY1 = SI(SYY0, i, j) * (1 - KYY1), SYY2 = SI(SYY0, i + 1, j) * (1 - KYY2);
                const double dRHOdy = (SI(RHOY, i + 1, j) - SI(RHOY, i - 1, j)) / 2. / dy;
                const double dRHOdx = (BI(RHO, i, j) - BI(RHO, i, j - 1)) / dx;
                const double temp = gy * dt * dRHOdx / 4.;
                trp(st, ky, ky, -(ETAYY1 + ETAYY2) / dy2 - (ETAXY1 + ETAXY2) / dx2 - gy * dt * dRHOdy - inertia * SI(RHOY, i, j) / dt);
                trp(st, ky, ky - RS, ETAXY1 / dx2);
                trp(st, ky, ky + RS, ETAXY2 / dx2);
                trp(st, ky, ky - NV, ETAYY1 / dy2);
                trp(st, ky, ky + NV, ETAYY2 / dy2);
                trp(st, ky, kx - RS, (ETAXY1 - ETAYY1) / dx_dy - temp);
                trp(st, ky, kx + NV - RS, (ETAYY2 - ETAXY1) / dx_dy - temp);
                trp(st, ky, kx, (ETAYY1 - ETAXY2) / dx_dy - temp);
                trp(st, ky, kx + NV, (ETAXY2 - ETAYY2) / dx_dy - temp);
                trp(st, ky, kp, ptscale / dy);
                trp(st, ky, kp + NV, -ptscale / dy);
                R[ky] = -SI(RHOY, i, j) * (inertia * SI(VY0, i, j) / dt + gy) - (SYY2 - SYY1) / dy - (SXY2 - SXY1) / dx;
            }
            /* 5c) Pt :842-862 */
            if (i == 0 || j == 0 || i == Ny || j == Nx) {
                trp(st, kp, kp, 1);
            } else {
                const double por = SI(POR, i, j);
                const double BETADRAINED = (1. / SI(GGGB, i, j) + p->BETASOLID) / (1 - por);
                const double KBW = 1 - p->BETASOLID / BETADRAINED;
                trp(st, kp, kx - RS, -1. / dx);
                trp(st, kp, kx, 1. / dx);
                trp(st, kp, ky - NV, -1. / dy);
                trp(st, kp, ky, 1. / dy);
                trp(st, kp, kp, ptscale * (1. / SI(ETAB, i, j) / (1 - por) + BETADRAINED / dt));
                trp(st, kp, kpf, -pfscale * (1. / SI(ETAB, i, j) / (1 - por) + BETADRAINED * KBW / dt));
                R[kp] = BETADRAINED * (SI(PT0, i, j) - KBW * SI(PF0, i, j)) / dt + SI(DILP, i, j);
            }
            /* 5d) vxD :864-903 */
            if (i == 0 || i == Ny || j == 0 || j >= Nx - 1) {
                if (j == Nx) trp(st, kxf, kxf, 1);
                if (i == 0 && j < Nx) {
                    trp(st, kxf, kxf, 1);
                    trp(st, kxf, kxf + NV, -1);
                }
                if (i == Ny && j < Nx) {
                    trp(st, kxf, kxf, 1);
                    trp(st, kxf, kxf - NV, -1);
                }
                if (j == 0) trp(st, kxf, kxf, 1);
                if (j == Nx - 1) trp(st, kxf, kxf, 1);
            } else {
                trp(st, kxf, kxf, -SI(ETADX, i, j) - SI(RHOFX, i, j) / SI(PORX, i, j) * inertia / dt);
                trp(st, kxf, kx, -SI(RHOFX, i, j) * inertia / dt);
                trp(st, kxf, kpf, pfscale / dx);
                trp(st, kxf, kpf + RS, -pfscale / dx);
                R[kxf] = -SI(RHOFX, i, j) * (inertia * SI(VXF0, i, j) / dt + gx);
            }
            /* 5e) vyD :905-949 */
            if (j == 0 || j == Nx || i == 0 || i >= Ny - 1) {
                if (i == Ny) trp(st, kyf, kyf, 1);
                if (j == 0 && i > 0 && i < Ny - 1) {
                    trp(st, kyf, kyf, 1);
                    trp(st, kyf, kyf + RS, -1);
                }
                if (j == Nx && i > 0 && i < Ny - 1) {
                    trp(st, kyf, kyf, 1);
                    trp(st, kyf, kyf - RS, -1);
                }
                if (i == 0) {
                    trp(st, kyf, kyf, 1);
                    R[kyf] = p->bcvyflower;
                }
                if (i == Ny - 1) {
                    trp(st, kyf, kyf, 1);
                    R[kyf] = p->bcvyflower;
                }
            } else {
                trp(st, kyf, kyf, -SI(ETADY, i, j) - SI(RHOFY, i, j) / SI(PORY, i, j) * inertia / dt);
                trp(st, kyf, ky, -SI(RHOFY, i, j) * inertia / dt);
                trp(st, kyf, kpf, pfscale / dy);
                trp(st, kyf, kpf + NV, -pfscale / dy);
                R[kyf] = -SI(RHOFY, i, j) * (inertia * SI(VYF0, i, j) / dt + gy);
            }
            /* 5f) Pf :951-980 */
            if (j == 0 || j == Nx || i <= 1 || i >= Ny - 1) {
                if (i == 1 || i == Ny - 1) {
                    trp(st, kpf, kpf, pfscale);
                    trp(st, kpf, kp, -ptscale);
                    R[kpf] = -p->PTFDIFF;
                } else {
                    trp(st, kpf, kpf, 1);
                }
            } else {
                const double por = SI(POR, i, j);
                const double BETADRAINED = (1 / SI(GGGB, i, j) + p->BETASOLID) / (1 - por);
                const double KBW = 1 - p->BETASOLID / BETADRAINED;
                const double KSK = (BETADRAINED - p->BETASOLID) / (BETADRAINED - p->BETASOLID + por * (p->BETAFLUID - p->BETASOLID));
                trp(st, kpf, kxf - RS, -1. / dx);
                trp(st, kpf, kxf, 1. / dx);
                trp(st, kpf, kyf - NV, -1. / dy);
                trp(st, kpf, kyf, 1. / dy);
                trp(st, kpf, kp, -ptscale * (1 / SI(ETAB, i, j) / (1 - por) + BETADRAINED * KBW / dt));
                trp(st, kpf, kpf, pfscale * (1 / SI(ETAB, i, j) / (1 - por) + BETADRAINED * KBW / KSK / dt));
                R[kpf] = -BETADRAINED * KBW * (SI(PT0, i, j) - 1. / KSK * SI(PF0, i, j)) / dt - SI(DILP, i, j);
            }
        }
    }
    build_csr(st);
    return st->nnz;
}

void hmo_csr(const hmo_state* st, const int64_t** indptr, const int32_t** indices, const double** data, const double** rhs) {
    *indptr = st->indptr;
    *indices = st->indices;
    *data = st->data;
    *rhs = st->R;
}

/* ------------------------------------------- a11-a15: after the solve */

int32_t hmo_iter_finish(hmo_state* st, const double* S) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Nx1 = st->Nx1, Ny1 = st->Ny1;
    const double dx = st->dx, dy = st->dy;
    const int iterstep = (int)st->sc[HMEC_S_iterstep];
    int ynlast = (int)st->sc[HMEC_S_ynlast];
    double dt = st->sc[HMEC_S_dt];
    const double ptscale = st->ptscale, pfscale = st->pfscale;
    size_t nb = (size_t)Nx * Ny;
    /* 7) reload :1060-1075 */
    for (int j = 0; j < Nx1; j++) {
        for (int i = 0; i < Ny1; i++) {
            const int kp = (j * Ny1 + i) * 6;
            SI(pt, i, j) = S[kp] * ptscale;
            SI(vxs, i, j) = S[kp + 1];
            SI(vys, i, j) = S[kp + 2];
            SI(pf, i, j) = S[kp + 3] * pfscale;
            SI(vxD, i, j) = S[kp + 4];
            SI(vyD, i, j) = S[kp + 5];
        }
    }
    double vmax = -INFINITY; /* :1077 */
    for (size_t k = 0; k < nb; k++) vmax = DMAX(vmax, st->f[HMEC_F_VSLIPB][k]);
    st->sc[HMEC_S_Vmax] = vmax;
    int yn = 0;
    /* stress :1102-1127 */
    for (int i = 0; i < Ny; i++) {
        for (int j = 0; j < Nx; j++) {
            BI(EXY, i, j) = .5 * ((SI(vxs, i + 1, j) - SI(vxs, i, j)) / dy + (SI(vys, i, j + 1) - SI(vys, i, j)) / dx);
            const double KXY = divplus(dt * BI(GGG, i, j), BI(ETA, i, j));
            BI(SXY, i, j) = 2 * BI(ETA, i, j) * BI(EXY, i, j) * KXY + BI(SXY0, i, j) * (1 - KXY);
        }
    }
    for (int i = 1; i < Ny; i++) {
        for (int j = 1; j < Nx; j++) {
            SI(EXX, i, j) = (2 * (SI(vxs, i, j) - SI(vxs, i, j - 1)) / dx - (SI(vys, i, j) - SI(vys, i - 1, j)) / dy) / 3.;
            SI(EYY, i, j) = (2 * (SI(vys, i, j) - SI(vys, i - 1, j)) / dy - (SI(vxs, i, j) - SI(vxs, i, j - 1)) / dx) / 3.;
            const double KXX = divplus(dt * SI(GGGP, i, j), SI(ETAP, i, j));
            SI(SXX, i, j) = 2 * SI(ETAP, i, j) * SI(EXX, i, j) * KXX + SI(SXX0, i, j) * (1 - KXX);
            SI(SYY, i, j) = 2 * SI(ETAP, i, j) * SI(EYY, i, j) * KXX + SI(SYY0, i, j) * (1 - KXX);
        }
    }
    /* :1130-1132 copy_bounds on copies: no-op (Q2) */
    /* RSF :1154-1308 */
    memcpy(st->f[HMEC_F_ETA5], st->f[HMEC_F_ETA0], nb * sizeof(double));
    memset(st->f[HMEC_F_DSY], 0, nb * sizeof(double));
    memset(st->f[HMEC_F_YNY], 0, nb * sizeof(double));
    memset(st->f[HMEC_F_SigmaY], 0, nb * sizeof(double));
    memset(st->f[HMEC_F_SII_fault], 0, nb * sizeof(double));
    int ynpl = 0;
    double ddd = 0;
    double dtlapusta = 1e7;
    memcpy(st->f[HMEC_F_OM5], st->f[HMEC_F_OM], nb * sizeof(double));
    double dtslip = 1e30;
    if (st->sc[HMEC_S_timestep] > p->tyield) {
        const int i = st->line_fault;
        for (int j = 0; j < Nx; j++) {
            const double arsf = BI(ARSF, i, j), brsf = BI(BRSF, i, j), lrsf = BI(LRSF, i, j);
            const double fric = BI(FRIC, i, j), eta0 = BI(ETA0, i, j);
            const double sxx = block_sum(st->f[HMEC_F_SXX], Ny1, i, j);
            const double syy = block_sum(st->f[HMEC_F_SYY], Ny1, i, j);
            const double sxy = BI(SXY, i, j);
            BI(SIIB, i, j) = sqrt(sxy * sxy + (sxx * sxx + syy * syy + (sxx + syy) * (sxx + syy)) / 32.);
            const double G = BI(GGG, i, j), ETAij = BI(ETA, i, j), OMij = BI(OM, i, j);
            const double siiel = BI(SIIB, i, j) / (ETAij / (G * dt + ETAij));
            const double prB_temp = (block_sum(st->f[HMEC_F_pt], Ny1, i, j) - block_sum(st->f[HMEC_F_pf], Ny1, i, j)) / 4.;
            double prB = prB_temp;
            if (prB < 1e3) prB = 1e3;
            double SIIB1 = BI(SIIB, i, j);
            const double eom = exp(-(brsf * OMij + fric) / arsf);
            double EIISLIP = p->V0 * sinh(DMAX(SIIB1, 0.) / arsf / prB) * eom / dx;
            double ETAPL = SIIB1 / 2. / EIISLIP;
            double ETAVP = 1. / (1. / eta0 + 1. / ETAPL);
            double SIIB2 = siiel * ETAVP / (G * dt + ETAVP);
            const double DSIIB1 = SIIB2 - SIIB1;
            double V = 2 * p->V0 * sinh(DMAX(SIIB2, 0.) / arsf / prB) * eom;
            EIISLIP = V / dx / 2.;
            ETAPL = SIIB2 / 2. / EIISLIP;
            ETAVP = 1. / (1. / eta0 + 1. / ETAPL);
            const double DSIIB2 = siiel * ETAVP / (G * dt + ETAVP) - SIIB2;
            double SIIB4 = 0.;
            if ((DSIIB1 >= 0 && DSIIB2 <= 0) || (DSIIB1 <= 0 && DSIIB2 >= 0)) {
                double DSIIB = 1e9;
                int it = 0;
                while (fabs(DSIIB) > 1e-3) {
                    if (it++ >= p->rsf_maxit) {
                        st->rsf_noconv = 1;
                        break;
                    }
                    SIIB4 = (SIIB1 + SIIB2) / 2.;
                    V = 2 * p->V0 * sinh(DMAX(SIIB4, 0.) / arsf / prB) * eom;
                    EIISLIP = V / dx / 2.;
                    ETAPL = SIIB4 / 2. / EIISLIP;
                    ETAVP = 1. / (1. / eta0 + 1. / ETAPL);
                    DSIIB = siiel * ETAVP / (G * dt + ETAVP) - SIIB4;
                    if ((DSIIB >= 0 && DSIIB1 >= 0) || (DSIIB <= 0 && DSIIB1 <= 0)) SIIB1 = SIIB4;
                    else SIIB2 = SIIB4;
                }
            }
            /* aging law :1245-1249 */
            if (V * dt / lrsf > 1e-6) {
                BI(OM5, i, j) = log(p->V0 / V + (exp(BI(OM0, i, j)) - p->V0 / V) * exp(-V * dt / lrsf));
            } else {
                BI(OM5, i, j) = log(exp(BI(OM0, i, j)) * (1 - V * dt / lrsf) + p->V0 * dt / lrsf);
            }
            const double syield = DMAX(p->syieldmin, prB_temp * arsf * asinh(V / 2. / p->V0 * exp((brsf * BI(OM5, i, j) + fric) / arsf)));
            double etapl = eta0 * syield / (eta0 * V + syield);
            BI(SigmaY, i, j) = syield;
            BI(VSLIPB, i, j) = V;
            BI(SII_fault, i, j) = SIIB4;
            const double g_temp = 2 * G;
            const double k = g_temp / (M_PI * (1 - ((3. / p->BETASOLID - g_temp) / (6. / p->BETASOLID + g_temp))) * dx);
            double dTETAmax;
            const double q = (k * lrsf / prB - brsf) / arsf - 1;
            if ((q * q / 4. - k * lrsf / arsf / prB) < 0) {
                dTETAmax = DMIN(1. - (brsf - arsf) * prB / (k * lrsf), .2);
            } else {
                dTETAmax = DMIN(arsf * prB / (k * lrsf - (brsf - arsf) * prB), .2);
            }
            dtlapusta = DMIN(dtlapusta, dTETAmax * lrsf / V);
            int ynn = 0;
            if (BI(YNY0, i, j) > 0) {
                ynn = 1;
                BI(DSY, i, j) = BI(SIIB, i, j) - syield;
                ddd += BI(DSY, i, j) * BI(DSY, i, j);
                ynpl++;
            }
            const double A = syield / siiel;
            if (A < 1) {
                etapl = dt * G * A / (1 - A);
                if (etapl < eta0) {
                    BI(ETA5, i, j) = pow(etapl, 1 - p->etawt) * pow(ETAij, p->etawt);
                    BI(YNY, i, j) = 1;
                    if (!ynn) {
                        BI(DSY, i, j) = BI(SIIB, i, j) - syield;
                        ddd += BI(DSY, i, j) * BI(DSY, i, j);
                        ynpl++;
                    }
                } else {
                    BI(ETA5, i, j) = eta0;
                }
            } else {
                BI(ETA5, i, j) = eta0;
            }
        }
    }
    /* error :1311-1325 */
    st->DSYLSQ[iterstep] = 0;
    if (ynpl > 0) st->DSYLSQ[iterstep] = sqrt(ddd / ynpl);
    if (ynpl == 0) memcpy(st->f[HMEC_F_ETA], st->f[HMEC_F_ETA0], nb * sizeof(double));
    const double D_iter = st->DSYLSQ[iterstep];
    double D_iter_quot = 0;
    if (iterstep != 0) D_iter_quot = D_iter / st->DSYLSQ[iterstep - 1];
    /* adaptive dt :1329-1427 */
    double dtpl = dt;
    if (ynpl > 0 && iterstep < p->niterglobal && ynlast >= p->dtstep &&
        (ynlast > p->ynlastmax || log10(D_iter_quot) >= 0 ||
         log10(D_iter_quot) > log10(p->errmin / D_iter) / (double)(p->ynlastmax - ynlast))) {
        dtpl = dt / p->dtkoef;
        yn = 1;
    }
    if (iterstep > 0) st->maxvxy0 = st->sc[HMEC_S_maxvxy];
    double vxmax = -INFINITY, vxmin = INFINITY, vymax = -INFINITY, vymin = INFINITY;
    size_t ns = (size_t)Nx1 * Ny1;
    for (size_t k = 0; k < ns; k++) {
        vxmax = DMAX(vxmax, st->f[HMEC_F_vxs][k]);
        vxmin = DMIN(vxmin, st->f[HMEC_F_vxs][k]);
        vymax = DMAX(vymax, st->f[HMEC_F_vys][k]);
        vymin = DMIN(vymin, st->f[HMEC_F_vys][k]);
    }
    double maxvxs = DMAX(vxmax, fabs(vxmin));
    double maxvys = DMAX(vymax, fabs(vymin));
    const double maxvxy = sqrt((vxmax - vxmin) * (vxmax - vxmin) + (vymax - vymin) * (vymax - vymin));
    st->sc[HMEC_S_maxvxy] = maxvxy;
    double stpmaxcur = p->stpmax1;
    double dtx = dt;
    if (dt > dx * stpmaxcur / maxvxs) {
        dtx = dx / p->dtkoefv * stpmaxcur / maxvxs;
        yn = 1;
    }
    double dty = dt;
    if (dt > dy * stpmaxcur / maxvys) {
        dty = dy / p->dtkoefv * stpmaxcur / maxvys;
        yn = 1;
    }
    maxvxs = 0;
    maxvys = 0;
    const double* yvx = st->crd[3];
    const double* yvy = st->crd[5];
    for (int i = 0; i < Ny1; i++) {
        for (int j = 0; j < Nx1; j++) {
            if (yvx[i] >= st->upper_block && yvx[i] <= st->lower_block) maxvxs = DMAX(maxvxs, fabs(SI(vxs, i, j)));
            if (yvy[i] >= st->upper_block && yvy[i] <= st->lower_block) maxvys = DMAX(maxvys, fabs(SI(vys, i, j)));
        }
    }
    stpmaxcur = p->stpmax;
    if (dt > dx * stpmaxcur / maxvxs) {
        dtx = dx / p->dtkoefv * stpmaxcur / maxvxs;
        yn = 1;
    }
    if (dt > dy * stpmaxcur / maxvys) {
        dty = dy / p->dtkoefv * stpmaxcur / maxvys;
        yn = 1;
    }
    dtslip = 1e30;
    for (size_t k = 0; k < nb; k++) {
        const double v = st->f[HMEC_F_VSLIPB][k];
        if (v > 0) dtslip = DMIN(dtslip, dx * p->stpmax / v);
    }
    if (ynpl > 0 && dtslip < dt) {
        yn = 1;
        dtslip = dtslip / p->dtkoefv;
    }
    if (yn && dt > p->dtmin) {
        const double dtold = dt;
        dt = DMAX(DMIN(DMIN(dtx, dty), DMIN(DMIN(dtpl, dtslip), dtlapusta)), p->dtmin);
        if (dt < dtold) ynlast = 0;
    } else {
        yn = 0;
    }
    /* exit :1430-1456 */
    int ynstop = 0;
    double vratio = 0;
    if (iterstep > 0) vratio = log10(maxvxy / st->maxvxy0);
    if (!yn && (ynpl == 0 || (st->DSYLSQ[iterstep] < p->errmin && iterstep > 0 && fabs(vratio) < p->vratiomax))) {
        ynstop = 1;
    } else {
        for (size_t k = 0; k < nb; k++)
            st->f[HMEC_F_ETA][k] = DMAX(DMIN(st->f[HMEC_F_ETA5][k], st->f[HMEC_F_ETA0][k]), p->etamin);
        memcpy(st->f[HMEC_F_ETA50], st->f[HMEC_F_ETA], nb * sizeof(double));
        memcpy(st->f[HMEC_F_YNY0], st->f[HMEC_F_YNY], nb * sizeof(double));
        memcpy(st->f[HMEC_F_OM], st->f[HMEC_F_OM5], nb * sizeof(double));
    }
    st->sc[HMEC_S_dt] = dt;
    st->sc[HMEC_S_dtx] = dtx;
    st->sc[HMEC_S_dty] = dty;
    st->sc[HMEC_S_dtlapusta] = dtlapusta;
    st->last_ynpl = ynpl;
    st->last_dsylsq = st->DSYLSQ[iterstep];
    if (!ynstop) {
        ynlast++;
        st->sc[HMEC_S_iterstep] = iterstep + 1;
    }
    st->sc[HMEC_S_ynlast] = ynlast;
    return ynstop;
}

int32_t hmo_global_iteration(hmo_state* st, hmo_solve_fn solve, void* user) {
    hmo_iter_prepare(st);
    hmo_assemble(st);
    double* S = (double*)calloc((size_t)st->N, sizeof(double));
    int rc = solve(user, st->N, st->indptr, st->indices, st->data, st->R, S);
    if (rc != 0) {
        free(S);
        return -1;
    }
    int32_t stop = hmo_iter_finish(st, S);
    free(S);
    return stop;
}

/* ------------------------------------------- a16, a17, a19: step end */

void hmo_timestep_end(hmo_state* st) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Nx1 = st->Nx1, Ny1 = st->Ny1;
    const double dx = st->dx, dy = st->dy;
    size_t nb = (size_t)Nx * Ny, ns = (size_t)Nx1 * Ny1;
    /* :1464-1472 */
    if (st->sc[HMEC_S_dt00] > st->sc[HMEC_S_dt]) st->sc[HMEC_S_yndtdecrease] = 1;
    memcpy(st->f[HMEC_F_ETA00], st->f[HMEC_F_ETA50], nb * sizeof(double));
    memcpy(st->f[HMEC_F_OM0], st->f[HMEC_F_OM], nb * sizeof(double));
    const double dt = DMIN(DMIN(st->sc[HMEC_S_dtx], st->sc[HMEC_S_dty]), DMIN(st->sc[HMEC_S_dt], st->sc[HMEC_S_dtlapusta]));
    st->sc[HMEC_S_dt] = dt;
    /* :1475-1477 setZero on copies: no-op (Q2 family) */
    for (int i = 0; i < Ny; i++) { /* :1480-1495 */
        for (int j = 0; j < Nx; j++) {
            BI(ESP, i, j) = .5 * ((SI(vys, i, j + 1) - SI(vys, i, j)) / dx - (SI(vxs, i + 1, j) - SI(vxs, i, j)) / dy);
            BI(EXY, i, j) = .5 * ((SI(vxs, i + 1, j) - SI(vxs, i, j)) / dy + (SI(vys, i, j + 1) - SI(vys, i, j)) / dx);
            const double KXY = divplus(dt * BI(GGG, i, j), BI(ETA, i, j));
            BI(SXY, i, j) = 2 * BI(ETA, i, j) * BI(EXY, i, j) * KXY + BI(SXY0, i, j) * (1 - KXY);
        }
    }
    for (int i = 1; i < Ny; i++) { /* :1499-1559 */
        for (int j = 1; j < Nx; j++) {
            SI(EXX, i, j) = (2 * (SI(vxs, i, j) - SI(vxs, i, j - 1)) / dx - (SI(vys, i, j) - SI(vys, i - 1, j)) / dy) / 3.;
            SI(EYY, i, j) = (2 * (SI(vys, i, j) - SI(vys, i - 1, j)) / dy - (SI(vxs, i, j) - SI(vxs, i, j - 1)) / dx) / 3.;
            const double KXX = divplus(dt * SI(GGGP, i, j), SI(ETAP, i, j));
            SI(SXX, i, j) = 2 * SI(ETAP, i, j) * SI(EXX, i, j) * KXX + SI(SXX0, i, j) * (1 - KXX);
            SI(SYY, i, j) = 2 * SI(ETAP, i, j) * SI(EYY, i, j) * KXX + SI(SYY0, i, j) * (1 - KXX);
            const double t00 = BI(SXY, i - 1, j - 1) / BI(ETA, i - 1, j - 1), t01 = BI(SXY, i - 1, j) / BI(ETA, i - 1, j);
            const double t10 = BI(SXY, i, j - 1) / BI(ETA, i, j - 1), t11 = BI(SXY, i, j) / BI(ETA, i, j);
            const double exx = SI(EXX, i, j), sxx = SI(SXX, i, j), syy = SI(SYY, i, j), etap = SI(ETAP, i, j);
            SI(EII, i, j) = sqrt(exx * exx + square4(BI(EXY, i - 1, j - 1), BI(EXY, i - 1, j), BI(EXY, i, j - 1), BI(EXY, i, j)) / 4.);
            const double a = sxx / (2 * etap), b = syy / (2 * etap);
            SI(EIIVP, i, j) = sqrt(.5 * (a * a + b * b) + square4(t00, t01, t10, t11) / 16.);
            SI(SII, i, j) = sqrt(.5 * (sxx * sxx + syy * syy) + square4(BI(SXY, i - 1, j - 1), BI(SXY, i - 1, j), BI(SXY, i, j - 1), BI(SXY, i, j)) / 4.);
            const double s11 = BI(SXY, i, j), s01 = BI(SXY, i - 1, j), s10 = BI(SXY, i, j - 1), s00 = BI(SXY, i - 1, j - 1);
            const double DISXY = (s11 * s11 / BI(ETA, i, j) + s01 * s01 / BI(ETA, i - 1, j) + s10 * s10 / BI(ETA, i, j - 1) +
                                  s00 * s00 / BI(ETA, i - 1, j - 1)) / 2.;
            SI(DIS, i, j) = sxx * sxx / (2 * etap) + syy * syy / (2 * etap) + DISXY;
            double PT0_ave, PF0_ave;
            if (i < Ny - 1) {
                SI(pt_ave, i, j) = (SI(pt, i, j) + SI(pt, i + 1, j)) / 2.;
                SI(pf_ave, i, j) = (SI(pf, i, j) + SI(pf, i + 1, j)) / 2.;
                PT0_ave = (SI(PT0, i, j) + SI(PT0, i + 1, j)) / 2.;
                PF0_ave = (SI(PF0, i, j) + SI(PF0, i + 1, j)) / 2.;
            } else {
                SI(pt_ave, i, j) = SI(pt, i, j);
                SI(pf_ave, i, j) = SI(pf, i, j);
                PT0_ave = SI(PT0, i, j);
                PF0_ave = SI(PF0, i, j);
            }
            const double por = SI(POR, i, j);
            SI(VIS_COMP, i, j) = (SI(pt_ave, i, j) - SI(pf_ave, i, j)) / (SI(ETAB, i, j) * (1 - por));
            const double BETADRAINED = (1 / SI(GGGB, i, j) + p->BETASOLID) / (1 - por);
            const double KBW = 1 - p->BETASOLID / BETADRAINED;
            SI(EL_DECOM, i, j) = BETADRAINED * (SI(pt_ave, i, j) - PT0_ave - KBW * SI(pf_ave, i, j) + KBW * PF0_ave) / dt;
        }
    }
    /* rollover :1658-1726 */
    st->sc[HMEC_S_timesum] += dt;
    double mxx = -1e30, mnx = 1e30, mxy = -1e30, mny = 1e30;
    memcpy(st->f[HMEC_F_VX0], st->f[HMEC_F_vxs], ns * sizeof(double));
    memcpy(st->f[HMEC_F_VY0], st->f[HMEC_F_vys], ns * sizeof(double));
    for (int i = 0; i < Ny; i++) {
        for (int j = 0; j < Nx; j++) {
            if (SI(RHOX, i, j) > 2000 && i != 0) {
                mxx = DMAX(mxx, SI(vxs, i, j));
                mnx = DMIN(mnx, SI(vxs, i, j));
            }
            if (SI(RHOY, i, j) > 2000 && j != 0) {
                mxy = DMAX(mxy, SI(vys, i, j));
                mny = DMIN(mny, SI(vys, i, j));
            }
        }
    }
    st->sc[HMEC_S_maxvxsmod] = mxx;
    st->sc[HMEC_S_minvxsmod] = mnx;
    st->sc[HMEC_S_maxvysmod] = mxy;
    st->sc[HMEC_S_minvysmod] = mny;
    for (int i = 0; i < Ny1; i++) {
        for (int j = 0; j < Nx1; j++) {
            if (SI(PORX, i, j) > 0) SI(VXF0, i, j) = SI(vxs, i, j) + SI(vxD, i, j) / SI(PORX, i, j);
            if (SI(PORY, i, j) > 0) SI(VYF0, i, j) = SI(vys, i, j) + SI(vyD, i, j) / SI(PORY, i, j);
        }
    }
    memcpy(st->f[HMEC_F_SXX0], st->f[HMEC_F_SXX], ns * sizeof(double));
    memcpy(st->f[HMEC_F_SYY0], st->f[HMEC_F_SYY], ns * sizeof(double));
    memcpy(st->f[HMEC_F_SXY0], st->f[HMEC_F_SXY], nb * sizeof(double));
    for (size_t k = 0; k < ns; k++) st->f[HMEC_F_PTF0][k] = st->f[HMEC_F_pt][k] - st->f[HMEC_F_pf][k];
    memcpy(st->f[HMEC_F_PT0], st->f[HMEC_F_pt], ns * sizeof(double));
    memcpy(st->f[HMEC_F_PF0], st->f[HMEC_F_pf], ns * sizeof(double));
    st->sc[HMEC_S_timestep] += 1; /* the for-loop increment of :376 */
}

/* ------------------------------------------ a18, a20: marker advection */

static double bilin(const double* F, int rows, int i, int j, double dxm, double dym) {
    const double* c0 = F + (size_t)j * rows + i;
    const double* c1 = c0 + rows;
    return c0[0] * (1 - dxm) * (1 - dym) + c0[1] * (1 - dxm) * dym + c1[0] * dxm * (1 - dym) + c1[1] * dxm * dym;
}

void hmo_advect_markers(hmo_state* st) {
    const hmec_params* p = &st->p;
    const int Nx = st->Nx, Ny = st->Ny, Ny1 = st->Ny1;
    const double dx = st->dx, dy = st->dy;
    const double dt = st->sc[HMEC_S_dt];
    const double *x = st->crd[0], *y = st->crd[1], *xvx = st->crd[2], *yvx = st->crd[3];
    const double *xvy = st->crd[4], *yvy = st->crd[5];
    double* xm = st->mk[HMEC_M_xm];
    double* ym = st->mk[HMEC_M_ym];
    for (int64_t m = 0; m < st->marknum; m++) { /* :1563-1656 */
        double vxm[4], vym[4], spm[4];
        const double xold = xm[m], yold = ym[m];
        double xc = xold, yc = yold;
        for (int rk = 0; rk < 4; rk++) {
            int j = check_bounds(fix_(xc / dx), Nx);
            int i = check_bounds(fix_((yc + dy / 2.) / dy), Ny);
            vxm[rk] = bilin(st->f[HMEC_F_vxs], Ny1, i, j, (xc - xvx[j]) / dx, (yc - yvx[i]) / dy);
            j = check_bounds(fix_((xc + dx / 2.) / dx), Nx);
            i = check_bounds(fix_(yc / dy), Ny);
            vym[rk] = bilin(st->f[HMEC_F_vys], Ny1, i, j, (xc - xvy[j]) / dx, (yc - yvy[i]) / dy);
            j = check_bounds(fix_(xc / dx), Nx);
            i = check_bounds(fix_(yc / dy), Ny);
            spm[rk] = bilin(st->f[HMEC_F_ESP], Ny, i, j, (xc - x[j]) / dx, (yc - y[i]) / dy);
            if (p->rk4_as_written) { /* :1622-1630 */
                if (rk < 2) {
                    xc = xold + vxm[rk] * dt / 2.;
                    yc = yold + vym[rk] * dt / 2.;
                } else if (rk == 3) {
                    xc = xold + vxm[rk] * dt;
                    yc = yold + vym[rk] * dt;
                }
            } else { /* classic RK4 (the comment's A->B, A->C, A->D) */
                if (rk < 2) {
                    xc = xold + vxm[rk] * dt / 2.;
                    yc = yold + vym[rk] * dt / 2.;
                } else if (rk == 2) {
                    xc = xold + vxm[rk] * dt;
                    yc = yold + vym[rk] * dt;
                }
            }
        }
        const double dspeff = spm[0] * dt; /* :1636-1643 */
        double* sxx = st->mk[HMEC_M_sxxm];
        double* syy = st->mk[HMEC_M_syym];
        double* sxy = st->mk[HMEC_M_sxym];
        const double o_xx = sxx[m], o_yy = syy[m], o_xy = sxy[m];
        const double s2 = sin(2 * dspeff), c2 = cos(2 * dspeff), s1 = sin(dspeff), c1 = cos(dspeff);
        sxy[m] = .5 * (o_xx - o_yy) * s2 + o_xy * c2;
        sxx[m] = o_xx * (c1 * c1) + o_yy * (s1 * s1) - o_xy * s2;
        syy[m] = o_xx * (s1 * s1) + o_yy * (c1 * c1) + o_xy * s2;
        double xn = xold + (vxm[0] + 2 * vxm[1] + 2 * vxm[2] + vxm[3]) / 6. * dt; /* :1646-1647 */
        double yn = yold + (vym[0] + 2 * vym[1] + 2 * vym[2] + vym[3]) / 6. * dt;
        if (xn < 0) xn = xn + p->xsize; /* :1650-1655 */
        if (xn > p->xsize) xn = xn - p->xsize;
        xm[m] = xn;
        ym[m] = yn;
    }
}

/* ------------------------------------------------------- whole timestep */

int32_t hmo_timestep(hmo_state* st, hmo_solve_fn solve, void* user) {
    hmo_markers_to_nodes(st);
    hmo_timestep_begin(st);
    int iters = 0;
    for (;;) { /* :610 */
        if ((int)st->sc[HMEC_S_iterstep] >= st->p.niterglobal) break;
        int rc = hmo_global_iteration(st, solve, user);
        iters++;
        if (rc < 0) return -1;
        if (rc == 1) break;
    }
    hmo_timestep_end(st);
    if (st->p.advect_markers) hmo_advect_markers(st);
    return iters;
}
