/*
 * pin_ref.c — drives the reference's UNMODIFIED attenuate_segment (src/cpu/kernel.c:75-333)
 * and buildExponentialTable (src/cpu/init.c:81-117) over a seeded CSR problem, so the
 * oracle's FP32 restatement can be checked against the reference bit for bit.
 *
 * TEST INFRASTRUCTURE ONLY. oracle/Makefile compiles this file together with the
 * reference's own kernel.c and init.c, read in place from the reference source tree,
 * into oracle/_ref/ (never committed). Built twice: without and with -DTABLE (the
 * reference's compile-time exp switch, src/cpu/Makefile:124-127).
 *
 * The reference hard-codes ds = 0.7f (src/cpu/kernel.c:104), so the pin holds for
 * problems whose seg_ds are all 0.7f; the restatement takes ds per segment.
 */
#include "SimpleMOC-kernel_header.h"
#include "moc_attenuate.h"

#include <stdlib.h>

/* Sweep every track in CSR order through the reference's attenuate_segment; psi and
 * fine_flux are updated in place. group_stride must equal n_groups (the reference's
 * rows are unpadded). Table mode (library built with -DTABLE) uses table_values /
 * table_dx / table_lookup_max as the reference's Table. Returns 0 or -1. */
int pinref_sweep(const moc_problem_t *p, const float *table_values, int32_t table_points,
                 float table_dx, float table_lookup_max)
{
    if (!p || p->group_stride != p->n_groups) return -1;
    Input in = {0};
    in.source_3D_regions = p->n_regions;
    in.fine_axial_intervals = p->n_intervals;
    in.egroups = p->n_groups;
    in.segments = p->n_segments;
    const long G = p->n_groups, I = p->n_intervals;
    Source *S = (Source *)calloc((size_t)p->n_regions, sizeof(Source));
    if (!S) return -1;
    for (int r = 0; r < p->n_regions; r++) {
        S[r].fine_source = (float *)p->source + (long)r * I * G;
        S[r].fine_flux = p->fine_flux + (long)r * I * G;
        S[r].sigT = (float *)p->sigT + (long)r * G;
    }
    Table table;
    table.values = (float *)table_values;
    table.dx = table_dx;
    table.maxVal = table_lookup_max;
    table.N = table_points;
    SIMD_Vectors v = allocate_simd_vectors(&in);
    for (int t = 0; t < p->n_tracks; t++) {
        float *state_flux = p->psi + (long)t * G;
        for (int64_t j = p->track_offsets[t]; j < p->track_offsets[t + 1]; j++)
            attenuate_segment(&in, S, p->seg_region[j], p->seg_interval[j], state_flux, &v,
                              &table);
    }
    free(v.q0); /* allocate_simd_vectors makes one block starting at q0 */
    free(S);
    return 0;
}

/* The reference's own table for a precision / maxVal pair: fills *n_points, *dx,
 * *lookup_max and up to cap values. Returns 0, or -1 if cap is too small. */
int pinref_build_table(float precision, float max_val, float *values, int32_t cap,
                       int32_t *n_points, float *dx, float *lookup_max)
{
    Input in = {0};
    Table *t = buildExponentialTable(precision, max_val, &in);
    int rc = -1;
    if (t && 2 * t->N <= cap) {
        for (int k = 0; k < 2 * t->N; k++) values[k] = t->values[k];
        *n_points = t->N;
        *dx = t->dx;
        *lookup_max = t->maxVal;
        rc = 0;
    }
    if (t) {
        free(t->values);
        free(t);
    }
    return rc;
}
