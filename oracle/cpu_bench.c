/*
 * cpu_bench.c — the timed CPU reference arm (test/bench infrastructure only).
 *
 * Generates a workload with the seeded generator (moc_synth.h), takes the first
 * `--sample-tracks` tracks of it as a bounded sample, and times the oracle's FP32
 * restatement of the reference sweep (OpenMP over tracks, one lock per
 * (region, interval) around each tally, as src/cpu/kernel.c:3-73,265-281) for
 * `--warmup` + `--steps` passes. Built with the reference's gnu optimisation flags.
 * Prints one JSON object with segment*group attenuations per second.
 *
 * Arguments (all optional except the sizes):
 *   --seed N --regions R --intervals I --groups G --tracks T --segments S
 *   --lognormal MEDIAN SIGMA MIN MAX     lognormal track lengths instead of uniform
 *   --logsigt LO HI                      sigT ~ logU(LO, HI) instead of U(0.1, 2.0)
 *   --ds LO HI                           ds ~ U(LO, HI) (default 0.01 1.0)
 *   --table N MAX                        table exp mode
 *   --sample-tracks K --threads N --steps K --warmup W
 *   --track-file PATH                    the segments of a track file
 *                                        (include/moc_trackfile.h), which sets the tracks,
 *                                        segments, regions and intervals; tables and psi
 *                                        stay seeded
 */
#include "moc_synth.h"
#include "oracle.h"

#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static double now(void) { return omp_get_wtime(); }

int main(int argc, char **argv)
{
    moc_synth_spec_t spec;
    moc_synth_spec_init(&spec, 1, 2000, 5, 64, 1000, 1000000);
    moc_fwd_opts_t opts;
    memset(&opts, 0, sizeof(opts));
    opts.exp_mode = MOC_EXP_FULL;
    opts.table_points = 353;
    opts.table_max = 10.0f;
    opts.dz = 0.1f; opts.zin = 0.3f; opts.weight = 0.5f; opts.mu = 0.9f; opts.mu2 = 0.3f;
    long sample = -1;
    const char *track_file = NULL;
    int threads = 0, steps = 3, warmup = 1;
    for (int a = 1; a < argc; a++) {
#define ARG(name) (strcmp(argv[a], name) == 0 && a + 1 < argc)
        if (ARG("--seed")) spec.seed = strtoull(argv[++a], 0, 10);
        else if (ARG("--regions")) spec.n_regions = atoi(argv[++a]);
        else if (ARG("--intervals")) spec.n_intervals = atoi(argv[++a]);
        else if (ARG("--groups")) spec.n_groups = atoi(argv[++a]);
        else if (ARG("--tracks")) spec.n_tracks = atoi(argv[++a]);
        else if (ARG("--segments")) spec.n_segments = atoll(argv[++a]);
        else if (strcmp(argv[a], "--lognormal") == 0 && a + 4 < argc) {
            spec.track_mode = MOC_SYNTH_TRACKS_LOGNORMAL;
            spec.len_median = (float)atof(argv[++a]);
            spec.len_sigma = (float)atof(argv[++a]);
            spec.len_min = atoi(argv[++a]);
            spec.len_max = atoi(argv[++a]);
        } else if (strcmp(argv[a], "--logsigt") == 0 && a + 2 < argc) {
            spec.sigT_mode = MOC_SYNTH_SIGT_LOGUNIFORM;
            spec.sigT_lo = (float)atof(argv[++a]);
            spec.sigT_hi = (float)atof(argv[++a]);
        } else if (strcmp(argv[a], "--ds") == 0 && a + 2 < argc) {
            spec.ds_lo = (float)atof(argv[++a]);
            spec.ds_hi = (float)atof(argv[++a]);
        } else if (strcmp(argv[a], "--table") == 0 && a + 2 < argc) {
            opts.exp_mode = MOC_EXP_TABLE;
            opts.table_points = atoi(argv[++a]);
            opts.table_max = (float)atof(argv[++a]);
        } else if (ARG("--sample-tracks")) sample = atol(argv[++a]);
        else if (ARG("--threads")) threads = atoi(argv[++a]);
        else if (ARG("--steps")) steps = atoi(argv[++a]);
        else if (ARG("--warmup")) warmup = atoi(argv[++a]);
        else if (ARG("--track-file")) track_file = argv[++a];
        else {
            fprintf(stderr, "cpu_bench: bad argument %s\n", argv[a]);
            return 2;
        }
#undef ARG
    }
    int64_t *foff = NULL, fT = 0, fS = 0;
    int32_t *freg = NULL, fR = 0, fI = 0;
    uint8_t *fitv = NULL;
    float *fds = NULL;
    if (track_file) {
        if (oracle_trackfile_read(track_file, &fT, &fS, &fR, &fI, &foff, &freg, &fitv, &fds) ||
            fT < 1 || fT > 2147483647 || fI < 2 || fI > 255) {
            fprintf(stderr, "cpu_bench: %s is not a usable track file\n", track_file);
            return 2;
        }
        spec.n_tracks = (int32_t)fT;
        spec.n_segments = fS;
        spec.n_regions = fR;
        spec.n_intervals = fI;
    }
    spec.group_stride = (spec.n_groups + 3) & ~3;
    const long T = spec.n_tracks, Gs = spec.group_stride;
    const long ncell = (long)spec.n_regions * spec.n_intervals;
    int64_t *off = foff ? foff : (int64_t *)malloc((size_t)(T + 1) * sizeof(int64_t));
    const int64_t S = foff ? fS : moc_synth_track_offsets(&spec, off);
    if (S < 0) {
        fprintf(stderr, "cpu_bench: invalid sizes\n");
        return 2;
    }
    float *psi0 = malloc((size_t)(T * Gs) * sizeof(float));
    float *psi = malloc((size_t)(T * Gs) * sizeof(float));
    float *sig = malloc((size_t)(spec.n_regions * Gs) * sizeof(float));
    float *src = malloc((size_t)(ncell * Gs) * sizeof(float));
    float *ff = calloc((size_t)(ncell * Gs), sizeof(float));
    int32_t *reg = freg ? freg : malloc((size_t)(S > 0 ? S : 1) * sizeof(int32_t));
    uint8_t *itv = fitv ? fitv : malloc((size_t)(S > 0 ? S : 1));
    float *ds = fds ? fds : malloc((size_t)(S > 0 ? S : 1) * sizeof(float));
    if (!psi0 || !psi || !sig || !src || !ff || !reg || !itv || !ds) {
        fprintf(stderr, "cpu_bench: out of memory\n");
        return 3;
    }
    if (track_file)
        moc_synth_fill(&spec, off, psi0, sig, src, NULL, NULL, NULL);
    else
        moc_synth_fill(&spec, off, psi0, sig, src, reg, itv, ds);
    if (sample < 0 || sample > T) sample = T;

    moc_problem_t p;
    memset(&p, 0, sizeof(p));
    p.n_regions = spec.n_regions;
    p.n_intervals = spec.n_intervals;
    p.n_groups = spec.n_groups;
    p.group_stride = (int32_t)Gs;
    p.n_tracks = (int32_t)sample;
    p.n_segments = off[sample];
    p.track_offsets = off;
    p.seg_region = reg;
    p.seg_interval = itv;
    p.seg_ds = ds;
    p.sigT = sig;
    p.source = src;
    p.fine_flux = ff;
    p.psi = psi;

    if (threads <= 0) threads = omp_get_max_threads();
    double total = 0.0;
    for (int it = 0; it < warmup + steps; it++) {
        memcpy(psi, psi0, (size_t)(sample * Gs) * sizeof(float));
        memset(ff, 0, (size_t)(ncell * Gs) * sizeof(float));
        const double t0 = now();
        if (oracle_fwd_fp32_omp(&p, &opts, threads) != 0) {
            fprintf(stderr, "cpu_bench: sweep rejected the problem\n");
            return 4;
        }
        const double t1 = now();
        if (it >= warmup) total += t1 - t0;
    }
    double checksum = 0.0;
    for (long k = 0; k < sample * Gs; k++) checksum += psi[k];
    const double units = (double)p.n_segments * (double)spec.n_groups;
    const double sec = steps > 0 ? total / steps : 0.0;
    printf("{\"value\": %.6e, \"unit\": \"segment*group attenuations/s\", \"cores\": %d, "
           "\"sample_tracks\": %ld, \"sample_segments\": %lld, \"groups\": %d, "
           "\"s_per_step\": %.6f, \"steps\": %d, \"warmup\": %d, \"psi_checksum\": %.9e, "
           "\"exp_mode\": \"%s\", \"compiler\": \"gcc %d.%d\"}\n",
           sec > 0 ? units / sec : 0.0, threads, sample, (long long)p.n_segments,
           spec.n_groups, sec, steps, warmup, checksum,
           opts.exp_mode == MOC_EXP_TABLE ? "table" : "full", __GNUC__, __GNUC_MINOR__);
    return 0;
}
