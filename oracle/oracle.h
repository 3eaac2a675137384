/*
 * oracle.h — CPU oracle for the segment-attenuation sweep.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product (libmocatt.so, its Python wrapper)
 * links, loads or calls this code. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it, and only as the checker or the timed CPU reference arm.
 *
 * Pinning: oracle_fwd_fp32 is checked bit for bit against the reference's own
 * attenuate_segment (src/cpu/kernel.c:75-333), compiled unmodified from the reference
 * sources by oracle/Makefile into oracle/_ref/ (tests/test_oracle_pin.py). The golden
 * fixtures under tests/golden/ were produced by that pinned pair.
 *
 * Problem and option structs are the library's (moc_attenuate.h); here every pointer
 * is host memory.
 */
#ifndef MOC_ORACLE_H
#define MOC_ORACLE_H

#include <stdint.h>
#include "moc_attenuate.h"
#include "moc_tracks.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Exponential table, restating buildExponentialTable (src/cpu/init.c:81-117) for a
 * given N: values[2N], dx, and the lookup bound maxVal - dx. */
void oracle_build_table(int32_t n_points, float max_val, float *values, float *dx,
                        float *lookup_max);
/* Table lookup, restating interpolateTable (src/cpu/kernel.c:337-361). */
float oracle_table_lookup(const float *values, float dx, float lookup_max, float x);

/* FP32 restatement of attenuate_segment (src/cpu/kernel.c:99-332), swept over tracks
 * in CSR order, one track after another (deterministic). Updates p->psi and
 * p->fine_flux in place. Returns 0, or -1 on invalid input. */
int oracle_fwd_fp32(const moc_problem_t *p, const moc_fwd_opts_t *o);

/* Same arithmetic, OpenMP over tracks with one omp_lock per (region, interval) around
 * the tally, as src/cpu/kernel.c:265-281. Tally order varies between runs. This is the
 * timed CPU reference arm. nthreads <= 0 uses all available threads. */
int oracle_fwd_fp32_omp(const moc_problem_t *p, const moc_fwd_opts_t *o, int nthreads);

/*
 * FP64 oracle of the same formula on the same FP32 inputs and FP32 constants, with
 * the cancelling small-tau terms (tau - e and tau(tau(tau-3)+6) - 6e, e = 1-exp(-tau))
 * evaluated by their Taylor series. Outputs (all [.][group_stride]):
 *   psi_out   outgoing psi per track          ff_out  fine_flux (initial + tallies)
 *   a_psi     error-magnitude companion of psi_out
 *   a_ff      error-magnitude companion of ff_out (|initial| + sum of tally companions)
 *   abs_tally sum of |tally| per fine_flux entry
 *   hits      [R*I] number of segments that tallied into each (region, interval)
 * The companion A bounds the rounding error of an FP32 evaluation of the reference
 * formula: |x_fp32 - x| <= c * 2^-24 * A for a small operation count c (tally sums add
 * hits * 2^-24 * abs_tally). Any output pointer may be NULL. nthreads <= 0: all.
 */
int oracle_fwd_fp64(const moc_problem_t *p, const moc_fwd_opts_t *o, double *psi_out,
                    double *ff_out, double *a_psi, double *a_ff, double *abs_tally,
                    int64_t *hits, int nthreads);

/* FP32 axial coefficients a0 = q0, a1 = q1*mu, a2 = q2*mu2 per cell ([R*I][3][Gs]),
 * rounded as the reference's FP32 code rounds them. */
int oracle_fit_fp32(const moc_problem_t *p, const moc_fwd_opts_t *o, float *coef);

/* oracle_fwd_fp64 with the axial coefficients given ([R*I][3][Gs], as oracle_fit_fp32
 * lays them out) instead of fitted from p->source: the FP64 reference for a form that
 * stores rounded coefficients, evaluated on exactly the values it stored. */
int oracle_fwd_fp64_coef(const moc_problem_t *p, const moc_fwd_opts_t *o, const float *coef,
                         double *psi_out, double *ff_out, double *a_psi, double *a_ff,
                         double *abs_tally, int64_t *hits, int nthreads);

/*
 * FP64 adjoint of the sweep for L = sum w . fine_flux_out + sum v . psi_out
 * (w [R][I][group_stride], v [T][group_stride]). Outputs dL/dsigT [R][group_stride],
 * dL/dsource [R][I][group_stride], dL/dpsi_in [T][group_stride] (overwritten).
 * Hand-derived reverse sweep over each track; exp terms as in oracle_fwd_fp64.
 */
int oracle_adj_fp64(const moc_problem_t *p, const moc_fwd_opts_t *o, const double *w,
                    const double *v, double *d_sigT, double *d_source, double *d_psi_in,
                    int nthreads);

/* FP64 forward loss only (for central differences): returns L for the given inputs,
 * with sigT/source/psi_in taken in double precision from the arrays given. Groups are
 * independent, so group >= 0 returns the part of L carried by that group alone (a
 * parameter of group g moves only that part); group < 0 returns all of L. */
double oracle_loss_fp64(const moc_problem_t *p, const moc_fwd_opts_t *o,
                        const double *sigT, const double *source, const double *psi_in,
                        const double *w, const double *v, int32_t group);

/* Track generation (include/moc_tracks.h), oracle/tracks.c. The plan restated from the
 * header's definition: fills out[0 .. min(n, cap)) and returns n (-1 if invalid). */
int64_t oracle_tracks_plan(const moc_geometry_t *g, const moc_quadrature_t *q,
                           moc_track_t *out, int64_t cap);
/* Segments of every track by sorting all of its crossings: offsets[0 .. n_tracks], and
 * the descriptors when reg != NULL and they fit in cap. Returns the total (-1 if
 * invalid). */
int64_t oracle_trace(const moc_geometry_t *g, const moc_track_t *tracks, int64_t n_tracks,
                     int64_t *offsets, int32_t *reg, uint8_t *itv, float *ds, int64_t cap);
/* The same crossings counted with OpenMP over tracks (the timed CPU arm); returns the
 * total segment count. nthreads <= 0 uses all available threads. */
int64_t oracle_trace_omp(const moc_geometry_t *g, const moc_track_t *tracks,
                         int64_t n_tracks, int nthreads);

/* Source update (include/moc_transport.h), oracle/transport.c. Cross sections as host
 * arrays in moc_xs_t's layout. FP32: every source value the same fmaf chain, in the same
 * order, as the GPU kernel; fission = sum over cells (in cell order) of F V. FP64: the
 * same definition in double from double tallies. Return 0, or -1 on invalid input. */
int oracle_source_update_fp32(int32_t M, int32_t G, int32_t Gs, const float *scatter,
                              const float *nu_fission, const float *chi,
                              const int32_t *material, int32_t R, int32_t I,
                              const double *volume, const float *tally, double k,
                              float *source, double *fission);
int oracle_source_update_fp64(int32_t M, int32_t G, int32_t Gs, const float *scatter,
                              const float *nu_fission, const float *chi,
                              const int32_t *material, int32_t R, int32_t I,
                              const double *volume, const double *tally, double k,
                              double *source, double *fission);

/* The on-disk track format (include/moc_trackfile.h), oracle/trackfile.c: reads a file
 * into malloc'ed arrays (the caller frees them), checking the checksum, the offsets and
 * the cell indices. Returns 0, or -1 for a file that is not a valid track file. */
int oracle_trackfile_read(const char *path, int64_t *T, int64_t *S, int32_t *R, int32_t *I,
                          int64_t **offsets, int32_t **region, uint8_t **interval,
                          float **ds);

#ifdef __cplusplus
}
#endif
#endif
