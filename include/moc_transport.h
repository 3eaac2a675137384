/*
 * moc_transport.h — the source update and the power iteration around the sweep (C ABI).
 *
 * The step after the segment-attenuation sweep: its tallies (moc_attenuate_fwd's
 * fine_flux, each sum_tracks w * integral of psi over a fine cell) become a scalar flux,
 * the scalar flux a new fine source (scattering plus fission), and the fission rate a new
 * eigenvalue, iterated until k converges. The reference kernel stops at the tallies (its
 * parent application iterates); this is that iteration, with multigroup cross sections
 * per material:
 *
 *   phi[c][g]  = fine_flux[c][g] / V[c]                         (c: a fine cell r*I + i)
 *   F[c]       = sum_g' nu_fission[m][g'] phi[c][g']            (m = material of region r)
 *   q[c][g]    = ( sum_g' scatter[m][g'][g] phi[c][g'] + chi[m][g] F[c] / k ) / (4 pi)
 *   k_n        = k_(n-1) * sum_c V[c] F_n[c] / sum_c V[c] F_(n-1)[c]
 * where the source swept in iteration n + 1 is the one computed from the flux of sweep n
 * with the eigenvalue k_(n-1) (the fission source lags one eigenvalue update; at the
 * fixed point both agree).
 *
 * The sums over g' run in increasing g' as chains of fused multiply-adds in FP32, so the
 * GPU's sources equal the FP32 restatement of the oracle bit for bit; the fission totals
 * are summed in FP64.
 *
 * Sources for an iteration: the sweep's axial model (src/cpu/kernel.c:111-191) fits a
 * line or parabola through neighbouring fine intervals with the constants dz, zin, mu
 * and mu2 of moc_fwd_opts_t, which stand for one segment's entry height and one polar
 * cosine; with sources that differ from interval to interval that extrapolation is not a
 * transport solution (the tallies go negative). Iterate with flat sources: zin = 0 makes
 * q0 the interval's own source and mu = mu2 = 0 drop the linear and quadratic terms, so
 * every segment sees its fine cell's source and the flux integral is exact.
 */
#ifndef MOC_TRANSPORT_H
#define MOC_TRANSPORT_H

#include <stdint.h>

#include "moc_attenuate.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Multigroup cross sections of n_materials materials (device, float, rows of
 * group_stride like the problem's): total sigT[m][g], scatter[m][g'][g] (from group g'
 * into group g, G rows of group_stride), nu_fission[m][g], chi[m][g]. */
typedef struct {
    int32_t n_materials, n_groups, group_stride, reserved;
    const float *sigT;
    const float *scatter;
    const float *nu_fission;
    const float *chi;
} moc_xs_t;

/* The problem's sigT table from the materials: sigT[r][g] = xs->sigT[material[r]][g]
 * (device; material: int32 [n_regions]). Asynchronous on `stream`. */
moc_status_t moc_region_sigT(moc_handle_t h, const moc_xs_t *xs, const int32_t *material,
                             int32_t n_regions, float *sigT, void *stream);

/* One source update: from the tallies fine_flux[R*I][group_stride] and the fine-cell
 * volumes volume[R*I] (double), writes source[R*I][group_stride] (groups >= G untouched)
 * and adds sum_c V[c] F[c] into *fission (one device double, which the caller zeroes).
 * k: the eigenvalue the fission source is divided by. Device pointers, asynchronous. */
moc_status_t moc_source_update(moc_handle_t h, const moc_xs_t *xs, const int32_t *material,
                               int32_t n_regions, int32_t n_intervals, const double *volume,
                               const float *fine_flux, double k, float *source,
                               double *fission, void *stream);

typedef struct {
    int32_t max_iterations;  /* >= 1                                                        */
    int32_t reserved;
    double tolerance;        /* stop when |k_next - k| <= tolerance * k (0: run them all)   */
} moc_eigen_opts_t;

/* Power iteration. problem: a device problem whose sigT is the materials' (see
 * moc_region_sigT); its fine_flux holds the starting tallies (fine_flux[c][g] = V[c] for a
 * flat flux phi = 1), its source and psi are workspace. First the source of the starting
 * tallies with the starting eigenvalue *k; then each iteration: psi = 0 (vacuum
 * boundaries: nothing enters a track), fine_flux = 0, moc_attenuate_fwd with the current
 * source, moc_source_update of the new tallies into problem->source, k updated from the
 * fission totals. Stops after max_iterations or when |k_n - k_(n-1)| <= tolerance k_n.
 * On return *k is the last eigenvalue, *iterations the sweeps run, problem->fine_flux the
 * last sweep's tallies and problem->source the source of the next one. The call
 * synchronizes `stream` once per iteration (to read the fission total). */
moc_status_t moc_power_iteration(moc_handle_t h, const moc_problem_t *problem,
                                 const moc_fwd_opts_t *opts, const moc_xs_t *xs,
                                 const int32_t *material, const double *volume,
                                 const moc_eigen_opts_t *eopts, double *k,
                                 int32_t *iterations, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MOC_TRANSPORT_H */
