/*
 * oracle.c — CPU oracle for the segment-attenuation sweep (declared in oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: never linked into or called by the product library.
 *
 * Build with -ffp-contract=off (oracle/Makefile): the FP32 restatement must round each
 * operation exactly as the reference's C does, so that it matches the reference's own
 * attenuate_segment bit for bit (tests/test_oracle_pin.py).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------
 * Exponential table — restates buildExponentialTable, src/cpu/init.c:81-117:
 *   dx = maxVal / N (float); for n < N: exponential = (float) exp(-(n*dx));
 *   values[2n] = -exponential; values[2n+1] = 1 + (n*dx - 1) * exponential;
 *   lookup bound = maxVal - dx.
 * The slope sign is the reference's (the tangent of 1-exp(-x) has slope +exp(-x)).
 * ---------------------------------------------------------------------------------- */
void oracle_build_table(int32_t n_points, float max_val, float *values, float *dx,
                        float *lookup_max)
{
    const float d = max_val / (float)n_points;
    for (int n = 0; n < n_points; n++) {
        const float nd = (float)n * d;                 /* int * float in float    */
        const float exponential = (float)exp((double)(-nd));
        values[2 * n] = -exponential;
        const float a = nd - 1.0f;
        const float b = a * exponential;
        values[2 * n + 1] = 1.0f + b;
    }
    *dx = d;
    *lookup_max = max_val - d;
}

/* Restates interpolateTable, src/cpu/kernel.c:337-361. The interval index is
 * (int)(x / dx + 0.5f * dx), as written there (not x/dx + 0.5). */
float oracle_table_lookup(const float *values, float dx, float lookup_max, float x)
{
    if (x > lookup_max) return 1.0f;
    const float q = x / dx;
    const float h = 0.5f * dx;
    int interval = (int)(q + h);
    interval = interval * 2;
    const float slope = values[interval];
    const float intercept = values[interval + 1];
    const float sx = slope * x;
    return sx + intercept;
}

/* ------------------------------------------------------------------------------------
 * Validation shared by every entry point (host pointers).
 * ---------------------------------------------------------------------------------- */
static int problem_ok(const moc_problem_t *p, const moc_fwd_opts_t *o)
{
    if (!p || !o) return 0;
    if (p->n_regions < 1 || p->n_intervals < 2 || p->n_intervals > 255) return 0;
    if (p->n_groups < 1 || p->group_stride < p->n_groups || p->n_tracks < 0) return 0;
    if (p->n_segments < 0 || !p->track_offsets) return 0;
    if (p->n_segments > 0 && (!p->seg_region || !p->seg_interval || !p->seg_ds)) return 0;
    if (!p->sigT || !p->source || !p->fine_flux || (p->n_tracks > 0 && !p->psi)) return 0;
    if (p->track_offsets[0] != 0 || p->track_offsets[p->n_tracks] != p->n_segments) return 0;
    for (int32_t t = 0; t < p->n_tracks; t++)
        if (p->track_offsets[t + 1] < p->track_offsets[t]) return 0;
    for (int64_t j = 0; j < p->n_segments; j++)
        if (p->seg_region[j] < 0 || p->seg_region[j] >= p->n_regions ||
            p->seg_interval[j] >= p->n_intervals)
            return 0;
    if (o->exp_mode == MOC_EXP_TABLE && o->table_points < 2) return 0;
    return 1;
}

typedef struct {
    float *values;
    float dx, lookup_max;
} table_t;

static int table_make(const moc_fwd_opts_t *o, table_t *t)
{
    t->values = NULL;
    if (o->exp_mode != MOC_EXP_TABLE) return 0;
    t->values = (float *)malloc(2 * (size_t)o->table_points * sizeof(float));
    if (!t->values) return -1;
    oracle_build_table(o->table_points, o->table_max, t->values, &t->dx, &t->lookup_max);
    return 0;
}

/* ------------------------------------------------------------------------------------
 * FP32 restatement of attenuate_segment, src/cpu/kernel.c:99-332.
 * Every expression keeps the reference's operand order and grouping (C evaluates
 * a*b*c as (a*b)*c), so the rounding is the same; ds is the segment's own length
 * where the reference hard-codes 0.7f (kernel.c:104). The work is split into the same
 * per-group passes over scratch vectors as the reference's (one pass per quantity), so
 * that a build with the reference's optimisation flags vectorises it the way it
 * vectorises the reference; per element the operations are unchanged.
 * ---------------------------------------------------------------------------------- */
typedef struct {
    float *q0, *q1, *q2, *sig, *tau, *sig2, *ev, *reuse, *fi, *tally, *t1, *t2, *t3, *t4;
    float *mem;
} vecs_t;

static int vecs_make(vecs_t *v, int64_t n)
{
    v->mem = (float *)malloc((size_t)(14 * n) * sizeof(float));
    if (!v->mem) return -1;
    float **f[] = {&v->q0, &v->q1, &v->q2, &v->sig, &v->tau, &v->sig2, &v->ev, &v->reuse,
                   &v->fi, &v->tally, &v->t1, &v->t2, &v->t3, &v->t4};
    for (int k = 0; k < 14; k++) *f[k] = v->mem + k * n;
    return 0;
}

/* Fills v->tally (weight * flux integral per group) and updates state_flux. */
static void attenuate_fp32(const moc_problem_t *p, const moc_fwd_opts_t *o,
                           const table_t *tab, int32_t region, int32_t fai, float ds,
                           float *restrict state_flux, const vecs_t *v)
{
    const float dz = o->dz, zin = o->zin, weight = o->weight, mu = o->mu, mu2 = o->mu2;
    const int64_t Gs = p->group_stride;
    const int G = p->n_groups, I = p->n_intervals;
    const float *restrict src = p->source + (int64_t)region * I * Gs;
    const float *restrict sg = p->sigT + (int64_t)region * Gs;
    float *restrict q0 = v->q0, *restrict q1 = v->q1, *restrict q2 = v->q2;
    float *restrict sigT = v->sig, *restrict tau = v->tau, *restrict sigT2 = v->sig2;
    float *restrict expVal = v->ev, *restrict reuse = v->reuse, *restrict fi = v->fi;
    float *restrict tally = v->tally, *restrict t1 = v->t1, *restrict t2 = v->t2;
    float *restrict t3 = v->t3, *restrict t4 = v->t4;

    if (fai == 0) {                                          /* kernel.c:111-133 */
        const float *restrict f2 = src + (int64_t)fai * Gs;
        const float *restrict f3 = src + (int64_t)(fai + 1) * Gs;
        for (int g = 0; g < G; g++) {
            const float y2 = f2[g], y3 = f3[g];
            const float c0 = y2;
            const float c1 = (y3 - y2) / dz;
            q0[g] = c0 + c1 * zin;
            q1[g] = c1;
            q2[g] = 0;
        }
    } else if (fai == I - 1) {                               /* kernel.c:134-156 */
        const float *restrict f1 = src + (int64_t)(fai - 1) * Gs;
        const float *restrict f2 = src + (int64_t)fai * Gs;
        for (int g = 0; g < G; g++) {
            const float y1 = f1[g], y2 = f2[g];
            const float c0 = y2;
            const float c1 = (y2 - y1) / dz;
            q0[g] = c0 + c1 * zin;
            q1[g] = c1;
            q2[g] = 0;
        }
    } else {                                                 /* kernel.c:157-191 */
        const float *restrict f1 = src + (int64_t)(fai - 1) * Gs;
        const float *restrict f2 = src + (int64_t)fai * Gs;
        const float *restrict f3 = src + (int64_t)(fai + 1) * Gs;
        for (int g = 0; g < G; g++) {
            const float y1 = f1[g], y2 = f2[g], y3 = f3[g];
            const float c0 = y2;
            const float c1 = (y1 - y3) / (2.f * dz);
            const float c2 = (y1 - 2.f * y2 + y3) / (2.f * dz * dz);
            q0[g] = c0 + c1 * zin + c2 * zin * zin;
            q1[g] = c1 + 2.f * c2 * zin;
            q2[g] = c2;
        }
    }
    for (int g = 0; g < G; g++) {                            /* kernel.c:200-208 */
        sigT[g] = sg[g];
        tau[g] = sigT[g] * ds;
        sigT2[g] = sigT[g] * sigT[g];
    }
    if (tab->values) {                                       /* kernel.c:216-223 */
        for (int g = 0; g < G; g++)
            expVal[g] = oracle_table_lookup(tab->values, tab->dx, tab->lookup_max, tau[g]);
    } else {
        for (int g = 0; g < G; g++) expVal[g] = 1.f - expf(-tau[g]);
    }
    /* kernel.c:233-237: only the last term is divided (C precedence) */
    for (int g = 0; g < G; g++)
        reuse[g] = tau[g] * (tau[g] - 2.f) + 2.f * expVal[g] / (sigT[g] * sigT2[g]);
    for (int g = 0; g < G; g++)                              /* kernel.c:245-252 */
        fi[g] = (q0[g] * tau[g] + (sigT[g] * state_flux[g] - q0[g]) * expVal[g]) / sigT2[g] +
                q1[g] * mu * reuse[g] +
                q2[g] * mu2 * (tau[g] * (tau[g] * (tau[g] - 3.f) + 6.f) - 6.f * expVal[g]) /
                    (3.f * sigT2[g] * sigT2[g]);
    for (int g = 0; g < G; g++) tally[g] = weight * fi[g];  /* kernel.c:259-263 */
    for (int g = 0; g < G; g++) t1[g] = q0[g] * expVal[g] / sigT[g];  /* kernel.c:289-331 */
    for (int g = 0; g < G; g++) t2[g] = q1[g] * mu * (tau[g] - expVal[g]) / sigT2[g];
    for (int g = 0; g < G; g++) t3[g] = q2[g] * mu2 * reuse[g];
    for (int g = 0; g < G; g++) t4[g] = state_flux[g] * (1.f - expVal[g]);
    for (int g = 0; g < G; g++) state_flux[g] = t1[g] + t2[g] + t3[g] + t4[g];
}

int oracle_fwd_fp32(const moc_problem_t *p, const moc_fwd_opts_t *o)
{
    if (!problem_ok(p, o)) return -1;
    table_t tab;
    if (table_make(o, &tab)) return -1;
    vecs_t v;
    if (vecs_make(&v, p->group_stride)) {
        free(tab.values);
        return -1;
    }
    const int64_t Gs = p->group_stride;
    for (int32_t t = 0; t < p->n_tracks; t++) {
        float *psi = p->psi + (int64_t)t * Gs;
        for (int64_t j = p->track_offsets[t]; j < p->track_offsets[t + 1]; j++) {
            const int32_t r = p->seg_region[j];
            const int32_t i = p->seg_interval[j];
            float *ff = p->fine_flux + ((int64_t)r * p->n_intervals + i) * Gs;
            attenuate_fp32(p, o, &tab, r, i, p->seg_ds[j], psi, &v);
            for (int g = 0; g < p->n_groups; g++) ff[g] += v.tally[g];  /* kernel.c:275-278 */
        }
    }
    free(v.mem);
    free(tab.values);
    return 0;
}

int oracle_fwd_fp32_omp(const moc_problem_t *p, const moc_fwd_opts_t *o, int nthreads)
{
    if (!problem_ok(p, o)) return -1;
#ifndef _OPENMP
    (void)nthreads;
    return oracle_fwd_fp32(p, o);
#else
    table_t tab;
    if (table_make(o, &tab)) return -1;
    const int64_t Gs = p->group_stride;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    omp_lock_t *locks = (omp_lock_t *)malloc((size_t)ncell * sizeof(omp_lock_t));
    if (!locks) {
        free(tab.values);
        return -1;
    }
    for (int64_t c = 0; c < ncell; c++) omp_init_lock(&locks[c]);
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    int failed = 0;
#pragma omp parallel num_threads(nthreads) reduction(| : failed)
    {
        vecs_t v;
        if (vecs_make(&v, Gs)) {
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 16)
            for (int32_t t = 0; t < p->n_tracks; t++) {
                float *psi = p->psi + (int64_t)t * Gs;
                for (int64_t j = p->track_offsets[t]; j < p->track_offsets[t + 1]; j++) {
                    const int32_t r = p->seg_region[j];
                    const int32_t i = p->seg_interval[j];
                    const int64_t c = (int64_t)r * p->n_intervals + i;
                    /* The tally is formed into a private row and added under the cell's
                     * lock, as kernel.c:265-281 does. */
                    attenuate_fp32(p, o, &tab, r, i, p->seg_ds[j], psi, &v);
                    float *ff = p->fine_flux + c * Gs;
                    omp_set_lock(&locks[c]);
                    for (int g = 0; g < p->n_groups; g++) ff[g] += v.tally[g];
                    omp_unset_lock(&locks[c]);
                }
            }
            free(v.mem);
        }
    }
    for (int64_t c = 0; c < ncell; c++) omp_destroy_lock(&locks[c]);
    free(locks);
    free(tab.values);
    return failed ? -1 : 0;
#endif
}

/* ------------------------------------------------------------------------------------
 * FP64 oracle.
 * ---------------------------------------------------------------------------------- */

/* d q_k / d y_{i+m} of the axial fit (src/cpu/kernel.c:111-191) for interval i of I:
 * a[k][m+1], k = 0,1,2 (q0,q1,q2), m = -1,0,+1. The fit is linear in the sources. */
static void qfit_coeffs(int i, int I, double dz, double zin, double a[3][3])
{
    memset(a, 0, 9 * sizeof(double));
    if (i == 0) {               /* c0 = y2, c1 = (y3-y2)/dz; q0 = c0+c1 zin, q1 = c1 */
        a[0][1] = 1.0 - zin / dz;
        a[0][2] = zin / dz;
        a[1][1] = -1.0 / dz;
        a[1][2] = 1.0 / dz;
    } else if (i == I - 1) {    /* c0 = y2, c1 = (y2-y1)/dz */
        a[0][0] = -zin / dz;
        a[0][1] = 1.0 + zin / dz;
        a[1][0] = -1.0 / dz;
        a[1][1] = 1.0 / dz;
    } else {                    /* c1 = (y1-y3)/(2dz), c2 = (y1-2y2+y3)/(2dz^2) */
        const double h1 = 1.0 / (2.0 * dz), h2 = 1.0 / (2.0 * dz * dz);
        /* q0 = y2 + c1 zin + c2 zin^2 */
        a[0][0] = h1 * zin + h2 * zin * zin;
        a[0][1] = 1.0 - 2.0 * h2 * zin * zin;
        a[0][2] = -h1 * zin + h2 * zin * zin;
        /* q1 = c1 + 2 c2 zin */
        a[1][0] = h1 + 2.0 * h2 * zin;
        a[1][1] = -4.0 * h2 * zin;
        a[1][2] = -h1 + 2.0 * h2 * zin;
        /* q2 = c2 */
        a[2][0] = h2;
        a[2][1] = -2.0 * h2;
        a[2][2] = h2;
    }
}

/* e = 1 - exp(-tau), E = exp(-tau), tme = tau - e, cub = tau(tau(tau-3)+6) - 6e, and
 * dcub = d cub / d tau = 3tau^2 - 6tau + 6 - 6E. Below tau = 1 the last three come
 * from their Taylor series (tau - e = sum_{k>=2} (-1)^k tau^k/k!,
 * cub = 6 sum_{k>=4} (-1)^k tau^k/k!, dcub = -6 sum_{k>=3} (-1)^k tau^k/k!), because
 * the direct forms cancel catastrophically for small tau. */
typedef struct {
    double e, E, tme, cub, dcub;
} expo_t;

static expo_t expo_exact(double tau)
{
    expo_t x;
    if (tau < 1.0) {
        /* s4 = sum_{k=4}^{22} (-1)^k tau^k / k! by Horner in -tau (the first omitted term
         * is below 1e-20 of s4 for tau < 1; the sum alternates with shrinking terms, so
         * it does not cancel) */
        static const double inv_fact[23] = {  /* 1/k!, k = 0..22, rounded to double */
            1.0, 1.0, 0.5, 0.16666666666666666,
            0.041666666666666664, 0.008333333333333333, 0.001388888888888889,
            0.0001984126984126984, 2.48015873015873e-05, 2.7557319223985893e-06,
            2.755731922398589e-07, 2.505210838544172e-08, 2.08767569878681e-09,
            1.6059043836821613e-10, 1.1470745597729725e-11, 7.647163731819816e-13,
            4.779477332387385e-14, 2.8114572543455206e-15, 1.5619206968586225e-16,
            8.22063524662433e-18, 4.110317623312165e-19, 1.9572941063391263e-20,
            8.896791392450574e-22};
        double h = inv_fact[22];
        for (int k = 21; k >= 4; k--) h = h * -tau + inv_fact[k];
        const double t2 = tau * tau, t3 = t2 * tau;
        const double s4 = h * t2 * t2;
        const double s3 = s4 - t3 * inv_fact[3];
        const double s2 = s3 + t2 * inv_fact[2];
        x.tme = s2;
        x.cub = 6.0 * s4;
        x.dcub = -6.0 * s3;
        /* e = tau - (tau - e) keeps full relative accuracy (tau - e <= tau^2/2), and
         * E = 1 - e does too while e < 1 - 1/e_Napier */
        x.e = tau - s2;
        x.E = 1.0 - x.e;
    } else {
        x.E = exp(-tau);
        x.e = 1.0 - x.E;
        x.tme = tau - x.e;
        x.cub = tau * (tau * (tau - 3.0) + 6.0) - 6.0 * x.e;
        x.dcub = 3.0 * tau * tau - 6.0 * tau + 6.0 - 6.0 * x.E;
    }
    return x;
}

/* Table mode: e is the reference's FP32 lookup at the FP32 tau (the table is a
 * discontinuous function, so its interval choice is taken exactly as the FP32 code
 * makes it); the rest is evaluated directly in double. */
static expo_t expo_table(const table_t *tab, float tau_f, double tau)
{
    expo_t x;
    x.e = (double)oracle_table_lookup(tab->values, tab->dx, tab->lookup_max, tau_f);
    x.E = 1.0 - x.e;
    x.tme = tau - x.e;
    x.cub = tau * (tau * (tau - 3.0) + 6.0) - 6.0 * x.e;
    x.dcub = 0.0; /* the table has no adjoint */
    return x;
}

typedef struct {
    const moc_problem_t *p;
    const moc_fwd_opts_t *o;
    const double *sigT;   /* [R][Gs] */
    const double *source; /* [R][I][Gs] */
    table_t tab;
    double dz, zin, weight, mu, mu2;
    double *q;            /* [R*I][3][Gs] fitted q0, q1, q2           */
    double *aq;           /* [R*I][3][Gs] their error magnitudes       */
} ctx64_t;

/* q0,q1,q2 of cell (r, i) for group g, and their error magnitudes. */
static inline void q_of(const ctx64_t *c, int32_t r, int32_t i, int g, double q[3],
                        double aq[3])
{
    const int64_t Gs = c->p->group_stride;
    const int64_t b = ((int64_t)r * c->p->n_intervals + i) * 3 * Gs + g;
    for (int k = 0; k < 3; k++) {
        q[k] = c->q[b + k * Gs];
        aq[k] = c->aq[b + k * Gs];
    }
}

static void ctx_free(ctx64_t *c)
{
    free(c->tab.values);
    free(c->q);
    free(c->aq);
    c->tab.values = NULL;
    c->q = c->aq = NULL;
}

static int ctx_init(ctx64_t *c, const moc_problem_t *p, const moc_fwd_opts_t *o,
                    const double *sigT, const double *source)
{
    c->p = p;
    c->o = o;
    c->sigT = sigT;
    c->source = source;
    c->dz = o->dz;
    c->zin = o->zin;
    c->weight = o->weight;
    c->mu = o->mu;
    c->mu2 = o->mu2;
    const int64_t I = p->n_intervals, Gs = p->group_stride, G = p->n_groups;
    const int64_t ncell = (int64_t)p->n_regions * I;
    c->q = (double *)calloc((size_t)(ncell * 3 * Gs), sizeof(double));
    c->aq = (double *)calloc((size_t)(ncell * 3 * Gs), sizeof(double));
    c->tab.values = NULL;
    if (!c->q || !c->aq || table_make(o, &c->tab)) {
        ctx_free(c);
        return -1;
    }
    for (int64_t cell = 0; cell < ncell; cell++) {
        const int i = (int)(cell % I);
        double a[3][3];
        qfit_coeffs(i, (int)I, c->dz, c->zin, a);
        for (int k = 0; k < 3; k++)
            for (int64_t g = 0; g < G; g++) {
                double q = 0.0, aq = 0.0;
                for (int m = -1; m <= 1; m++) {
                    if (a[k][m + 1] == 0.0) continue;
                    const double y = source[(cell + m) * Gs + g];
                    q += a[k][m + 1] * y;
                    aq += fabs(a[k][m + 1] * y);
                }
                c->q[(cell * 3 + k) * Gs + g] = q;
                c->aq[(cell * 3 + k) * Gs + g] = aq;
            }
    }
    return 0;
}

static double *promote(const float *x, int64_t n)
{
    double *d = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (d)
        for (int64_t k = 0; k < n; k++) d[k] = x[k];
    return d;
}

/* FP32 coefficients a0 = q0, a1 = q1*mu, a2 = q2*mu2 of every cell, rounded as the
 * reference's FP32 code rounds them (src/cpu/kernel.c:111-191 and the first product of
 * kernel.c:250-251, 311-322). */
int oracle_fit_fp32(const moc_problem_t *p, const moc_fwd_opts_t *o, float *coef)
{
    if (!problem_ok(p, o) || !coef) return -1;
    const float dz = o->dz, zin = o->zin, mu = o->mu, mu2 = o->mu2;
    const int64_t Gs = p->group_stride, I = p->n_intervals;
    for (int64_t cell = 0; cell < (int64_t)p->n_regions * I; cell++) {
        const int i = (int)(cell % I);
        const float *row = p->source + cell * Gs;
        for (int64_t g = 0; g < Gs; g++) {
            float q0 = 0, q1 = 0, q2 = 0;
            if (g < p->n_groups) {
                if (i == 0) {
                    const float y2 = row[g], y3 = row[Gs + g];
                    const float c1 = (y3 - y2) / dz;
                    q0 = y2 + c1 * zin;
                    q1 = c1;
                } else if (i == I - 1) {
                    const float y1 = row[g - Gs], y2 = row[g];
                    const float c1 = (y2 - y1) / dz;
                    q0 = y2 + c1 * zin;
                    q1 = c1;
                } else {
                    const float y1 = row[g - Gs], y2 = row[g], y3 = row[Gs + g];
                    const float c1 = (y1 - y3) / (2.f * dz);
                    const float c2 = (y1 - 2.f * y2 + y3) / (2.f * dz * dz);
                    q0 = y2 + c1 * zin + c2 * zin * zin;
                    q1 = c1 + 2.f * c2 * zin;
                    q2 = c2;
                }
            }
            coef[(cell * 3 + 0) * Gs + g] = q0;
            coef[(cell * 3 + 1) * Gs + g] = q1 * mu;
            coef[(cell * 3 + 2) * Gs + g] = q2 * mu2;
        }
    }
    return 0;
}

static int fwd64(const moc_problem_t *p, const moc_fwd_opts_t *o, const float *coef,
                 double *psi_out, double *ff_out, double *a_psi, double *a_ff,
                 double *abs_tally, int64_t *hits, int nthreads);

int oracle_fwd_fp64(const moc_problem_t *p, const moc_fwd_opts_t *o, double *psi_out,
                    double *ff_out, double *a_psi, double *a_ff, double *abs_tally,
                    int64_t *hits, int nthreads)
{
    return fwd64(p, o, NULL, psi_out, ff_out, a_psi, a_ff, abs_tally, hits, nthreads);
}

int oracle_fwd_fp64_coef(const moc_problem_t *p, const moc_fwd_opts_t *o, const float *coef,
                         double *psi_out, double *ff_out, double *a_psi, double *a_ff,
                         double *abs_tally, int64_t *hits, int nthreads)
{
    if (!coef) return -1;
    return fwd64(p, o, coef, psi_out, ff_out, a_psi, a_ff, abs_tally, hits, nthreads);
}

static int fwd64(const moc_problem_t *p, const moc_fwd_opts_t *o, const float *coef,
                 double *psi_out, double *ff_out, double *a_psi, double *a_ff,
                 double *abs_tally, int64_t *hits, int nthreads)
{
    if (!problem_ok(p, o)) return -1;
    const int64_t Gs = p->group_stride, G = p->n_groups;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    const int64_t nff = ncell * Gs;
    double *sig = promote(p->sigT, (int64_t)p->n_regions * Gs);
    double *src = promote(p->source, nff);
    double *ff = (double *)calloc((size_t)nff, sizeof(double));
    double *aff = (double *)calloc((size_t)nff, sizeof(double));
    double *atal = (double *)calloc((size_t)nff, sizeof(double));
    int64_t *nh = (int64_t *)calloc((size_t)ncell, sizeof(int64_t));
    ctx64_t c;
    if (!sig || !src || !ff || !aff || !atal || !nh || ctx_init(&c, p, o, sig, src)) {
        free(sig); free(src); free(ff); free(aff); free(atal); free(nh);
        return -1;
    }
    if (coef) {
        /* given coefficients a0 = q0, a1 = q1*mu, a2 = q2*mu2 replace the fit */
        const double scale[3] = {1.0, 1.0 / c.mu, 1.0 / c.mu2};
        for (int64_t k = 0; k < ncell * 3 * Gs; k++) {
            const int64_t kk = (k / Gs) % 3;
            c.q[k] = (double)coef[k] * scale[kk];
            c.aq[k] = fabs(c.q[k]);
        }
    }
    for (int64_t k = 0; k < nff; k++) {
        ff[k] = p->fine_flux[k];
        aff[k] = fabs((double)p->fine_flux[k]);
    }
#ifdef _OPENMP
    omp_lock_t *locks = (omp_lock_t *)malloc((size_t)ncell * sizeof(omp_lock_t));
    for (int64_t k = 0; k < ncell; k++) omp_init_lock(&locks[k]);
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    (void)nthreads;
#endif

#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        double *psi = (double *)malloc((size_t)Gs * 6 * sizeof(double));
        double *apsi = psi + Gs, *tl = psi + 2 * Gs, *atl = psi + 3 * Gs, *abt = psi + 4 * Gs;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int32_t t = 0; t < p->n_tracks; t++) {
            for (int64_t g = 0; g < G; g++) {
                psi[g] = p->psi[(int64_t)t * Gs + g];
                apsi[g] = fabs(psi[g]);
            }
            for (int64_t j = p->track_offsets[t]; j < p->track_offsets[t + 1]; j++) {
                const int32_t r = p->seg_region[j];
                const int32_t i = p->seg_interval[j];
                const double ds = p->seg_ds[j];
                for (int64_t g = 0; g < G; g++) {
                    double q[3], aq[3];
                    q_of(&c, r, i, (int)g, q, aq);
                    const double s = sig[(int64_t)r * Gs + g];
                    const double tau = s * ds; /* exact: 24 x 24 bit product */
                    const expo_t x = c.tab.values
                                         ? expo_table(&c.tab, (float)s * (float)ds, tau)
                                         : expo_exact(tau);
                    /* reciprocal powers of s (one division; double rounding of 1/s^k is
                     * far below the FP32 errors this oracle measures) */
                    const double r1 = 1.0 / s, r2 = r1 * r1, r3 = r2 * r1;
                    const double r4_3 = r2 * r2 * (1.0 / 3.0);
                    const double reuse = tau * (tau - 2.0) + 2.0 * x.e * r3;
                    const double fi = q[0] * x.tme * r2 + psi[g] * x.e * r1 +
                                      q[1] * c.mu * reuse + q[2] * c.mu2 * x.cub * r4_3;
                    const double pn = q[0] * x.e * r1 + q[1] * c.mu * x.tme * r2 +
                                      q[2] * c.mu2 * reuse + psi[g] * x.E;
                    /* error magnitudes (see oracle.h); em bounds |e| plus its absolute
                     * evaluation error (1 - expf(-tau) is off by ~2^-24 absolutely) */
                    const double em = 1.0 + fabs(x.e);
                    const double areuse = tau * (tau + 2.0) + 2.0 * em * r3;
                    const double afi = (aq[0] * tau + (s * fabs(psi[g]) + aq[0]) * em) * r2 +
                                       apsi[g] * fabs(x.e) * r1 + aq[1] * c.mu * areuse +
                                       aq[2] * c.mu2 *
                                           (tau * tau * tau + 3.0 * tau * tau + 6.0 * tau +
                                            6.0 * em) * r4_3;
                    const double apn = aq[0] * em * r1 + aq[1] * c.mu * (tau + em) * r2 +
                                       aq[2] * c.mu2 * areuse +
                                       fabs(psi[g]) * (x.E + em) + apsi[g] * x.E;
                    tl[g] = c.weight * fi;
                    atl[g] = c.weight * afi;
                    abt[g] = fabs(c.weight * fi);
                    psi[g] = pn;
                    apsi[g] = apn;
                }
                const int64_t cell = (int64_t)r * p->n_intervals + i;
#ifdef _OPENMP
                omp_set_lock(&locks[cell]);
#endif
                for (int64_t g = 0; g < G; g++) {
                    ff[cell * Gs + g] += tl[g];
                    aff[cell * Gs + g] += atl[g];
                    atal[cell * Gs + g] += abt[g];
                }
                nh[cell]++;
#ifdef _OPENMP
                omp_unset_lock(&locks[cell]);
#endif
            }
            for (int64_t g = 0; g < Gs; g++) {
                if (psi_out) psi_out[(int64_t)t * Gs + g] = g < G ? psi[g] : 0.0;
                if (a_psi) a_psi[(int64_t)t * Gs + g] = g < G ? apsi[g] : 0.0;
            }
        }
        free(psi);
    }
#ifdef _OPENMP
    for (int64_t k = 0; k < ncell; k++) omp_destroy_lock(&locks[k]);
    free(locks);
#endif
    if (ff_out) memcpy(ff_out, ff, (size_t)nff * sizeof(double));
    if (a_ff) memcpy(a_ff, aff, (size_t)nff * sizeof(double));
    if (abs_tally) memcpy(abs_tally, atal, (size_t)nff * sizeof(double));
    if (hits) memcpy(hits, nh, (size_t)ncell * sizeof(int64_t));
    free(sig); free(src); free(ff); free(aff); free(atal); free(nh);
    ctx_free(&c);
    return 0;
}

/* ------------------------------------------------------------------------------------
 * FP64 adjoint. Per segment and group, with tau = s ds, e = 1-exp(-tau), E = exp(-tau):
 *   FI   = q0 tme/s^2 + psi e/s + q1 mu reuse + q2 mu2 cub/(3 s^4)
 *   psi' = q0 e/s + q1 mu tme/s^2 + q2 mu2 reuse + psi E
 *   reuse = tau(tau-2) + 2e/s^3
 * (the reference's expressions, src/cpu/kernel.c:233-331, rewritten with
 * (q0 tau + (s psi - q0) e)/s^2 = q0 tme/s^2 + psi e/s, which is exact algebra).
 * With lambda = dL/dpsi' and W = weight * w[cell]:
 *   dL/dpsi += lambda E + W e/s                       (carried backwards)
 *   dL/ds   += lambda dpsi'/ds + W dFI/ds             (scattered to region)
 *   dL/dq_k += lambda dpsi'/dq_k + W dFI/dq_k         (scattered to cell, then
 *                                                      through the fit Jacobian)
 * ---------------------------------------------------------------------------------- */
typedef struct {
    double fi_s, pn_s;          /* d/ds */
    double fi_q[3], pn_q[3];    /* d/dq_k */
    double fi_psi, pn_psi;      /* d/dpsi */
} partials_t;

static partials_t partials(const ctx64_t *c, double s, double ds, const double q[3],
                           double psi)
{
    partials_t d;
    const double tau = s * ds;
    const expo_t x = expo_exact(tau);
    const double s2 = s * s, s3 = s2 * s, s4 = s2 * s2, s5 = s4 * s;
    const double reuse = tau * (tau - 2.0) + 2.0 * x.e / s3;
    const double de = x.E * ds;       /* de/ds   */
    const double dtme = ds * x.e;     /* dtme/ds */
    const double dreuse = (2.0 * tau - 2.0) * ds + 2.0 * de / s3 - 6.0 * x.e / s4;
    const double dcub = x.dcub * ds;
    d.fi_s = q[0] * (dtme / s2 - 2.0 * x.tme / s3) + psi * (de / s - x.e / s2) +
             q[1] * c->mu * dreuse +
             q[2] * c->mu2 * (dcub / (3.0 * s4) - 4.0 * x.cub / (3.0 * s5));
    d.pn_s = q[0] * (de / s - x.e / s2) + q[1] * c->mu * (dtme / s2 - 2.0 * x.tme / s3) +
             q[2] * c->mu2 * dreuse - psi * x.E * ds;
    d.fi_q[0] = x.tme / s2;
    d.fi_q[1] = c->mu * reuse;
    d.fi_q[2] = c->mu2 * x.cub / (3.0 * s4);
    d.pn_q[0] = x.e / s;
    d.pn_q[1] = c->mu * x.tme / s2;
    d.pn_q[2] = c->mu2 * reuse;
    d.fi_psi = x.e / s;
    d.pn_psi = x.E;
    return d;
}

int oracle_adj_fp64(const moc_problem_t *p, const moc_fwd_opts_t *o, const double *w,
                    const double *v, double *d_sigT, double *d_source, double *d_psi_in,
                    int nthreads)
{
    if (!problem_ok(p, o) || !w || !v || o->exp_mode != MOC_EXP_FULL) return -1;
    const int64_t Gs = p->group_stride, G = p->n_groups, I = p->n_intervals;
    const int64_t ncell = (int64_t)p->n_regions * I;
    double *sig = promote(p->sigT, (int64_t)p->n_regions * Gs);
    double *src = promote(p->source, ncell * Gs);
    double *dq = (double *)calloc((size_t)(ncell * 3 * Gs), sizeof(double));
    double *dsc = (double *)calloc((size_t)(ncell * Gs), sizeof(double));
    int64_t maxlen = 0;
    for (int32_t t = 0; t < p->n_tracks; t++) {
        const int64_t L = p->track_offsets[t + 1] - p->track_offsets[t];
        if (L > maxlen) maxlen = L;
    }
    ctx64_t c;
    if (!sig || !src || !dq || !dsc || ctx_init(&c, p, o, sig, src)) {
        free(sig); free(src); free(dq); free(dsc);
        return -1;
    }
#ifdef _OPENMP
    omp_lock_t *locks = (omp_lock_t *)malloc((size_t)ncell * sizeof(omp_lock_t));
    for (int64_t k = 0; k < ncell; k++) omp_init_lock(&locks[k]);
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    (void)nthreads;
#endif
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        /* psi history of one track: hist[k][g] = psi entering segment k */
        double *hist = (double *)malloc((size_t)((maxlen + 1) * Gs) * sizeof(double));
        double *lam = (double *)malloc((size_t)Gs * 5 * sizeof(double));
        double *cs = lam + Gs, *cq = lam + 2 * Gs; /* cq: 3*Gs */
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
        for (int32_t t = 0; t < p->n_tracks; t++) {
            const int64_t b = p->track_offsets[t], n = p->track_offsets[t + 1] - b;
            for (int64_t g = 0; g < G; g++) hist[g] = p->psi[(int64_t)t * Gs + g];
            for (int64_t k = 0; k < n; k++) {
                const int32_t r = p->seg_region[b + k], i = p->seg_interval[b + k];
                const double ds = p->seg_ds[b + k];
                for (int64_t g = 0; g < G; g++) {
                    double q[3], aq[3];
                    q_of(&c, r, i, (int)g, q, aq);
                    const double s = sig[(int64_t)r * Gs + g];
                    const double tau = s * ds;
                    const expo_t x = expo_exact(tau);
                    const double s2 = s * s, s3 = s2 * s;
                    const double reuse = tau * (tau - 2.0) + 2.0 * x.e / s3;
                    const double ps = hist[k * Gs + g];
                    hist[(k + 1) * Gs + g] = q[0] * x.e / s + q[1] * c.mu * x.tme / s2 +
                                             q[2] * c.mu2 * reuse + ps * x.E;
                }
            }
            for (int64_t g = 0; g < G; g++) lam[g] = v[(int64_t)t * Gs + g];
            for (int64_t k = n - 1; k >= 0; k--) {
                const int32_t r = p->seg_region[b + k], i = p->seg_interval[b + k];
                const double ds = p->seg_ds[b + k];
                const int64_t cell = (int64_t)r * I + i;
                for (int64_t g = 0; g < G; g++) {
                    double q[3], aq[3];
                    q_of(&c, r, i, (int)g, q, aq);
                    const double s = sig[(int64_t)r * Gs + g];
                    const partials_t d = partials(&c, s, ds, q, hist[k * Gs + g]);
                    const double W = c.weight * w[cell * Gs + g];
                    cs[g] = lam[g] * d.pn_s + W * d.fi_s;
                    for (int kk = 0; kk < 3; kk++)
                        cq[kk * Gs + g] = lam[g] * d.pn_q[kk] + W * d.fi_q[kk];
                    lam[g] = lam[g] * d.pn_psi + W * d.fi_psi;
                }
#ifdef _OPENMP
                omp_set_lock(&locks[cell]);
#endif
                for (int64_t g = 0; g < G; g++) {
                    dsc[cell * Gs + g] += cs[g];
                    for (int kk = 0; kk < 3; kk++)
                        dq[(cell * 3 + kk) * Gs + g] += cq[kk * Gs + g];
                }
#ifdef _OPENMP
                omp_unset_lock(&locks[cell]);
#endif
            }
            for (int64_t g = 0; g < Gs; g++)
                d_psi_in[(int64_t)t * Gs + g] = g < G ? lam[g] : 0.0;
        }
        free(hist);
        free(lam);
    }
#ifdef _OPENMP
    for (int64_t k = 0; k < ncell; k++) omp_destroy_lock(&locks[k]);
    free(locks);
#endif
    /* sigT: sum the per-cell partials over the intervals of each region. */
    memset(d_sigT, 0, (size_t)((int64_t)p->n_regions * Gs) * sizeof(double));
    memset(d_source, 0, (size_t)(ncell * Gs) * sizeof(double));
    for (int32_t r = 0; r < p->n_regions; r++)
        for (int64_t i = 0; i < I; i++) {
            const int64_t cell = (int64_t)r * I + i;
            double a[3][3];
            qfit_coeffs((int)i, (int)I, c.dz, c.zin, a);
            for (int64_t g = 0; g < G; g++) {
                d_sigT[(int64_t)r * Gs + g] += dsc[cell * Gs + g];
                for (int kk = 0; kk < 3; kk++)
                    for (int m = -1; m <= 1; m++)
                        if (a[kk][m + 1] != 0.0)
                            d_source[(cell + m) * Gs + g] +=
                                a[kk][m + 1] * dq[(cell * 3 + kk) * Gs + g];
            }
        }
    free(sig); free(src); free(dq); free(dsc);
    ctx_free(&c);
    return 0;
}

double oracle_loss_fp64(const moc_problem_t *p, const moc_fwd_opts_t *o,
                        const double *sigT, const double *source, const double *psi_in,
                        const double *w, const double *v, int32_t group)
{
    if (!problem_ok(p, o) || o->exp_mode != MOC_EXP_FULL) return NAN;
    const int64_t Gs = p->group_stride, G = p->n_groups, I = p->n_intervals;
    ctx64_t c;
    if (ctx_init(&c, p, o, sigT, source)) return NAN;
    double L = 0.0;
    /* L = sum_cells w . (ff0 + tallies) + sum_tracks v . psi_out; the tally part is
     * accumulated per segment as w[cell] * weight * FI. */
    const int64_t g0 = group >= 0 ? group : 0, g1 = group >= 0 ? group + 1 : G;
    if (group >= G) return NAN;
    for (int64_t k = 0; k < (int64_t)p->n_regions * I * Gs; k++)
        if (k % Gs >= g0 && k % Gs < g1) L += w[k] * (double)p->fine_flux[k];
    for (int32_t t = 0; t < p->n_tracks; t++) {
        for (int64_t g = g0; g < g1; g++) {
            double psi = psi_in[(int64_t)t * Gs + g];
            for (int64_t j = p->track_offsets[t]; j < p->track_offsets[t + 1]; j++) {
                const int32_t r = p->seg_region[j], i = p->seg_interval[j];
                double q[3], aq[3];
                q_of(&c, r, i, (int)g, q, aq);
                const double s = sigT[(int64_t)r * Gs + g];
                const double tau = s * (double)p->seg_ds[j];
                const expo_t x = expo_exact(tau);
                const double s2 = s * s, s3 = s2 * s, s4 = s2 * s2;
                const double reuse = tau * (tau - 2.0) + 2.0 * x.e / s3;
                const double fi = q[0] * x.tme / s2 + psi * x.e / s + q[1] * c.mu * reuse +
                                  q[2] * c.mu2 * x.cub / (3.0 * s4);
                L += w[((int64_t)r * I + i) * Gs + g] * c.weight * fi;
                psi = q[0] * x.e / s + q[1] * c.mu * x.tme / s2 + q[2] * c.mu2 * reuse +
                      psi * x.E;
            }
            L += v[(int64_t)t * Gs + g] * psi;
        }
    }
    ctx_free(&c);
    return L;
}
