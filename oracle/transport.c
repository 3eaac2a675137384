/*
 * transport.c — CPU oracle of the source update (include/moc_transport.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of libmocatt's moc_source_update and, with the
 * sweep oracle, of its moc_power_iteration; nothing in the product links or calls it.
 *
 * The reference kernel stops at the tallies (its parent application iterates), so this
 * row's parity is against this restatement of the header's definition, not pinned to
 * reference code. oracle_source_update_fp32 evaluates every source value as the same
 * FP32 chain of fused multiply-adds, in the same order, as the GPU kernel, so the sources
 * must agree bit for bit (built with -ffp-contract=off: only the explicit fmaf fuse);
 * oracle_source_update_fp64 is the same definition in FP64, the accuracy reference.
 */
#include <math.h>
#include <stdint.h>

#include "oracle.h"

static const double PI = 3.14159265358979323846;

int oracle_source_update_fp32(int32_t M, int32_t G, int32_t Gs, const float *scatter,
                              const float *nu_fission, const float *chi,
                              const int32_t *material, int32_t R, int32_t I,
                              const double *volume, const float *tally, double k,
                              float *source, double *fission)
{
    if (M < 1 || G < 1 || Gs < G || R < 0 || I < 1 || !(k > 0.0)) return -1;
    const float rk = (float)(1.0 / k), rpi = (float)(1.0 / (4.0 * PI));
    double total = 0.0;
    float phi[1024], acc[1024];
    if (G > 1024) return -1;
    for (int64_t c = 0; c < (int64_t)R * I; c++) {
        const int32_t m = material[c / I];
        if (m < 0 || m >= M) return -1;
        const double V = volume[c];
        const float rv = (float)(1.0 / V);
        const float *row = tally + c * Gs;
        const float *S = scatter + (int64_t)m * G * Gs;
        const float *nuf = nu_fission + (int64_t)m * Gs;
        for (int g = 0; g < G; g++) {
            phi[g] = row[g] * rv;
            acc[g] = 0.0f;
        }
        float F = 0.0f;
        for (int gp = 0; gp < G; gp++) {
            F = fmaf(nuf[gp], phi[gp], F);
            for (int g = 0; g < G; g++) acc[g] = fmaf(S[(int64_t)gp * Gs + g], phi[gp], acc[g]);
        }
        const float f = F * rk;
        for (int g = 0; g < G; g++)
            source[c * Gs + g] = fmaf(chi[(int64_t)m * Gs + g], f, acc[g]) * rpi;
        total += (double)F * V;
    }
    *fission = total;
    return 0;
}

int oracle_source_update_fp64(int32_t M, int32_t G, int32_t Gs, const float *scatter,
                              const float *nu_fission, const float *chi,
                              const int32_t *material, int32_t R, int32_t I,
                              const double *volume, const double *tally, double k,
                              double *source, double *fission)
{
    if (M < 1 || G < 1 || Gs < G || R < 0 || I < 1 || !(k > 0.0) || G > 1024) return -1;
    double phi[1024];
    double total = 0.0;
    for (int64_t c = 0; c < (int64_t)R * I; c++) {
        const int32_t m = material[c / I];
        if (m < 0 || m >= M) return -1;
        const double V = volume[c];
        const double *row = tally + c * Gs;
        const float *S = scatter + (int64_t)m * G * Gs;
        double F = 0.0;
        for (int g = 0; g < G; g++) {
            phi[g] = row[g] / V;
            F += (double)nu_fission[(int64_t)m * Gs + g] * phi[g];
        }
        for (int g = 0; g < G; g++) {
            double s = 0.0;
            for (int gp = 0; gp < G; gp++) s += (double)S[(int64_t)gp * Gs + g] * phi[gp];
            source[c * Gs + g] = (s + (double)chi[(int64_t)m * Gs + g] * F / k) / (4.0 * PI);
        }
        total += F * V;
    }
    *fission = total;
    return 0;
}
