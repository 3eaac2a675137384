/*
 * tracks.c — CPU oracle of track generation (include/moc_tracks.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of libmocatt's moc_tracks_plan and of its GPU
 * walk (moc_trace_count / moc_trace_segments), and the timed CPU arm of the track
 * benchmark. Nothing in the product links or calls it.
 *
 * The reference has no ray tracer: its kernel draws segments at random
 * (src/cpu/kernel.c:47-50), so this row's parity is against this restatement, not
 * pinned to reference code. The plan is restated from the header's definition. The
 * segments come from a different algorithm than the GPU's: where the GPU walks pin cell
 * by pin cell, merging the next grid line, ring crossing and axial plane, this collects
 * every crossing of the track with every grid line, every ring of every pin and every
 * fine axial plane, sorts them, and classifies the midpoint of each gap. Both compute
 * each crossing with the same formula and round every FP64 operation on its own (built
 * with -ffp-contract=off), so the descriptors must agree bit for bit.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "moc_tracks.h"
#include "oracle.h"

typedef struct {
    int nx, ny, K, n_axial, n_int, NZ;
    double P, rP, dz, rdz;
    double r2[MOC_TRACKS_MAX_RINGS];
} geo_t;

static int geo_valid(const moc_geometry_t *g)
{
    return g && g->nx >= 1 && g->ny >= 1 && g->n_rings >= 1 &&
           g->n_rings <= MOC_TRACKS_MAX_RINGS && g->n_axial >= 1 && g->n_intervals >= 2 &&
           g->n_intervals <= 255 && g->pitch > 0.0 && g->fuel_radius > 0.0 &&
           g->fuel_radius < 0.45 * g->pitch && g->height > 0.0;
}

static geo_t geo_of(const moc_geometry_t *g)
{
    geo_t G;
    memset(&G, 0, sizeof(G));
    G.nx = g->nx;
    G.ny = g->ny;
    G.K = g->n_rings;
    G.n_axial = g->n_axial;
    G.n_int = g->n_intervals;
    G.NZ = g->n_axial * g->n_intervals;
    G.P = g->pitch;
    G.rP = 1.0 / g->pitch;
    G.dz = g->height / (double)G.NZ;
    G.rdz = (double)G.NZ / g->height;
    for (int k = 0; k < G.K; k++)
        G.r2[k] = (g->fuel_radius * g->fuel_radius) * ((double)(k + 1) / (double)G.K);
    return G;
}

int64_t oracle_tracks_plan(const moc_geometry_t *g, const moc_quadrature_t *q,
                           moc_track_t *out, int64_t cap)
{
    if (!geo_valid(g) || !q || q->n_azim < 2 || q->n_azim % 2 || q->n_polar < 2 ||
        q->n_polar % 2 || !(q->spacing > 0.0) || !(q->axial_spacing > 0.0))
        return -1;
    const double pi = 3.14159265358979323846;
    const double W = (double)g->nx * g->pitch, Y = (double)g->ny * g->pitch;
    const int NZ = g->n_axial * g->n_intervals;
    const double H = (double)NZ * (g->height / (double)NZ); /* the top fine plane */
    int64_t n = 0;
    for (int a = 0; a < q->n_azim; a++) {
        const double phi = pi * ((double)a + 0.5) / (double)q->n_azim;
        const double ux = cos(phi), uy = sin(phi);
        /* the lattice's corners projected on the normal (-uy, ux) */
        const double proj[4] = {0.0, W * -uy, Y * ux, W * -uy + Y * ux};
        double lo = proj[0], hi = proj[0];
        for (int i = 1; i < 4; i++) {
            if (proj[i] < lo) lo = proj[i];
            if (proj[i] > hi) hi = proj[i];
        }
        const int64_t nlines = (int64_t)floor((hi - lo) / q->spacing);
        const double margin = ((hi - lo) - (double)nlines * q->spacing) * 0.5;
        for (int64_t l = 0; l < nlines; l++) {
            const double c = lo + margin + ((double)l + 0.5) * q->spacing;
            const double px = c * -uy, py = c * ux;
            double tin = -INFINITY, tout = INFINITY;
            if (ux != 0.0) {
                const double t1 = (0.0 - px) / ux, t2 = (W - px) / ux;
                tin = fmax(tin, fmin(t1, t2));
                tout = fmin(tout, fmax(t1, t2));
            } else if (!(px >= 0.0 && px <= W)) {
                continue;
            }
            if (uy != 0.0) {
                const double t1 = (0.0 - py) / uy, t2 = (Y - py) / uy;
                tin = fmax(tin, fmin(t1, t2));
                tout = fmin(tout, fmax(t1, t2));
            } else if (!(py >= 0.0 && py <= Y)) {
                continue;
            }
            if (!(tout > tin)) continue;
            /* entry exactly on the entry face; length = the exit face's crossing */
            const double rux = 1.0 / ux, ruy = 1.0 / uy;
            double x0, y0;
            if (ux != 0.0 && tin == fmin((0.0 - px) / ux, (W - px) / ux)) {
                x0 = ux > 0.0 ? 0.0 : W;
                y0 = py + tin * uy;
            } else {
                x0 = px + tin * ux;
                y0 = 0.0;
            }
            const double ty = (Y - y0) * ruy;
            const double L = ux != 0.0 ? fmin(((ux > 0.0 ? W : 0.0) - x0) * rux, ty) : ty;
            if (!(L > 0.0)) continue;
            for (int p = 0; p < q->n_polar; p++) {
                const double mu = 1.0 - (2.0 * (double)p + 1.0) / (double)q->n_polar;
                const double s = sqrt(1.0 - mu * mu);
                const double cot = mu / s, rcot = s / mu;
                const double step = q->axial_spacing / s;
                const double zlo = mu > 0.0 ? -L * cot : 0.0;
                const double zhi = mu > 0.0 ? H : H - L * cot;
                const int64_t nz = (int64_t)floor((zhi - zlo) / step);
                const double zmargin = ((zhi - zlo) - (double)nz * step) * 0.5;
                for (int64_t j = 0; j < nz; j++) {
                    const double z0 = zlo + zmargin + ((double)j + 0.5) * step;
                    double ta, za, tb;
                    if (mu > 0.0) {
                        ta = z0 < 0.0 ? -z0 * rcot : 0.0;
                        za = z0 < 0.0 ? 0.0 : z0;
                        tb = fmin(L, ta + (H - za) * rcot);
                    } else {
                        ta = z0 > H ? (H - z0) * rcot : 0.0;
                        za = z0 > H ? H : z0;
                        tb = fmin(L, ta + (0.0 - za) * rcot);
                    }
                    if (!(tb > ta)) continue;
                    for (int rev = 0; rev <= (q->both_directions ? 1 : 0); rev++) {
                        if (n < cap) {
                            moc_track_t *r = &out[n];
                            memset(r, 0, sizeof(*r));
                            r->x0 = x0;
                            r->y0 = y0;
                            r->ux = ux;
                            r->uy = uy;
                            r->rux = rux;
                            r->ruy = ruy;
                            r->ta = ta;
                            r->tb = tb;
                            r->za = za;
                            r->cot = cot;
                            r->rcot = rcot;
                            r->rsin = 1.0 / s;
                            r->azim = a;
                            r->polar = p;
                            r->reversed = rev;
                        }
                        n++;
                    }
                }
            }
        }
    }
    return n;
}

static int cmp_double(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

static void midpoint_cell(const geo_t *G, const moc_track_t *tr, double tm, int32_t *region,
                          uint8_t *itv)
{
    const double xm = tr->x0 + tm * tr->ux, ym = tr->y0 + tm * tr->uy;
    const double zm = tr->za + (tm - tr->ta) * tr->cot;
    int ix = (int)floor(xm * G->rP), iy = (int)floor(ym * G->rP);
    if (ix < 0) ix = 0;
    if (ix >= G->nx) ix = G->nx - 1;
    if (iy < 0) iy = 0;
    if (iy >= G->ny) iy = G->ny - 1;
    const double ddx = xm - ((double)ix + 0.5) * G->P, ddy = ym - ((double)iy + 0.5) * G->P;
    const double rr = ddx * ddx + ddy * ddy;
    int k = G->K;
    for (int j = G->K - 1; j >= 0; j--)
        if (rr < G->r2[j]) k = j;
    int f = (int)floor(zm * G->rdz);
    if (f < 0) f = 0;
    if (f >= G->NZ) f = G->NZ - 1;
    const int a = f / G->n_int;
    *itv = (uint8_t)(f - a * G->n_int);
    *region = ((iy * G->nx + ix) * (G->K + 1) + k) * G->n_axial + a;
}

/* All crossings of one track strictly inside (ta, tb), with ta and tb; sorted. */
static int64_t crossings(const geo_t *G, const moc_track_t *tr, double *ev)
{
    int64_t n = 0;
    ev[n++] = tr->ta;
#define KEEP(t)                                 \
    do {                                        \
        const double t_ = (t);                  \
        if (t_ > tr->ta && t_ < tr->tb) ev[n++] = t_; \
    } while (0)
    if (tr->ux != 0.0)
        for (int i = 0; i <= G->nx; i++) KEEP(((double)i * G->P - tr->x0) * tr->rux);
    if (tr->uy != 0.0)
        for (int j = 0; j <= G->ny; j++) KEEP(((double)j * G->P - tr->y0) * tr->ruy);
    for (int j = 0; j < G->ny; j++)
        for (int i = 0; i < G->nx; i++) {
            const double dxc = ((double)i + 0.5) * G->P - tr->x0;
            const double dyc = ((double)j + 0.5) * G->P - tr->y0;
            const double w = dxc * tr->ux + dyc * tr->uy;
            const double d = dxc * tr->uy - dyc * tr->ux;
            const double d2 = d * d;
            for (int k = 0; k < G->K; k++) {
                const double h2 = G->r2[k] - d2;
                if (h2 > 0.0) {
                    const double h = sqrt(h2);
                    KEEP(w - h);
                    KEEP(w + h);
                }
            }
        }
    for (int m = 0; m <= G->NZ; m++) KEEP(tr->ta + ((double)m * G->dz - tr->za) * tr->rcot);
#undef KEEP
    ev[n++] = tr->tb;
    qsort(ev, (size_t)n, sizeof(double), cmp_double);
    return n;
}

static int64_t max_crossings(const geo_t *G)
{
    return 2 + (G->nx + 1) + (G->ny + 1) + 2 * (int64_t)G->K * G->nx * G->ny + G->NZ + 1;
}

/* Segments of track tr (reversed order for a reversed track) into reg/itv/ds from
 * position 0; returns the count. ev: scratch of max_crossings doubles. */
static int64_t trace_one(const geo_t *G, const moc_track_t *tr, double *ev, int32_t *reg,
                         uint8_t *itv, float *ds)
{
    const int64_t n = crossings(G, tr, ev);
    int64_t c = 0;
    for (int64_t i = 0; i + 1 < n; i++)
        if (ev[i + 1] > ev[i]) c++;
    if (!reg) return c;
    int64_t k = 0;
    for (int64_t i = 0; i + 1 < n; i++) {
        if (!(ev[i + 1] > ev[i])) continue;
        const int64_t pos = tr->reversed ? c - 1 - k : k;
        midpoint_cell(G, tr, (ev[i] + ev[i + 1]) * 0.5, &reg[pos], &itv[pos]);
        ds[pos] = (float)((ev[i + 1] - ev[i]) * tr->rsin);
        k++;
    }
    return c;
}

int64_t oracle_trace(const moc_geometry_t *g, const moc_track_t *tracks, int64_t n_tracks,
                     int64_t *offsets, int32_t *reg, uint8_t *itv, float *ds, int64_t cap)
{
    if (!geo_valid(g) || n_tracks < 0 || !offsets) return -1;
    const geo_t G = geo_of(g);
    double *ev = (double *)malloc((size_t)max_crossings(&G) * sizeof(double));
    if (!ev) return -1;
    offsets[0] = 0;
    for (int64_t t = 0; t < n_tracks; t++) {
        const int64_t base = offsets[t];
        int64_t c = trace_one(&G, &tracks[t], ev, NULL, NULL, NULL);
        if (reg && base + c <= cap)
            c = trace_one(&G, &tracks[t], ev, reg + base, itv + base, ds + base);
        offsets[t + 1] = base + c;
    }
    free(ev);
    return offsets[n_tracks];
}

int64_t oracle_trace_omp(const moc_geometry_t *g, const moc_track_t *tracks,
                         int64_t n_tracks, int nthreads)
{
    if (!geo_valid(g) || n_tracks < 0) return -1;
    const geo_t G = geo_of(g);
    const int64_t mc = max_crossings(&G);
    int64_t total = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : total)
    {
        double *ev = (double *)malloc((size_t)mc * sizeof(double));
#pragma omp for schedule(dynamic, 64)
        for (int64_t t = 0; t < n_tracks; t++)
            if (ev) total += trace_one(&G, &tracks[t], ev, NULL, NULL, NULL);
        free(ev);
    }
    return total;
}
