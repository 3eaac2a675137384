/*
 * mocatt_run — C host program that drives the GB300 sweep through the C ABI.
 *
 * Mirrors the reference program's flow (src/cpu/main.c:3-62): read the command line
 * (src/cpu/io.c:99-161: -t threads, -s segments, -e energy groups), build the source
 * regions and segments, run the sweep once, print the runtime and the time per
 * intersection = runtime / (segments * groups) (src/cpu/main.c:55-58). Where the
 * reference calls run_kernel(I, S, table) on host arrays (src/cpu/main.c:46), this calls
 * moc_attenuate_fwd_host on host arrays.
 *
 * Inputs are seeded (moc_synth.h) instead of rand()/time(NULL). Extra flags:
 *   -r regions   (default: the reference's ceil(5000 * 27 / 20) = 6750)
 *   -k tracks    (default: segments / 500)
 *   -x           table exp mode with the reference's table (N = 353, maxVal = 10)
 *   -d device    CUDA device index (default 0)
 *   -n repeats   sweeps to time (default 1)
 *   -f file      sweep the segments of a track file (include/moc_trackfile.h: its
 *                tracks, regions and intervals replace -s, -k and -r; the tables and psi
 *                stay seeded)
 *   -w file      write the generated segments to a track file before sweeping
 *   -W file      the same in the compact version (half lengths, 6 bytes per segment)
 * -t is accepted for command-line compatibility and ignored (the sweep runs on the GPU).
 */
#include "moc_attenuate.h"
#include "moc_synth.h"
#include "moc_trackfile.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void usage(void)
{
    printf("Usage: mocatt_run <options>\n"
           "  -s <segments>       Number of segments to process\n"
           "  -e <energy groups>  Number of energy groups\n"
           "  -r <regions>        Number of 3D source regions\n"
           "  -k <tracks>         Number of tracks\n"
           "  -x                  Use the exponential table\n"
           "  -d <device>         CUDA device\n"
           "  -n <repeats>        Sweeps to time\n"
           "  -f <file>           Sweep the segments of a track file\n"
           "  -w <file>           Write the generated segments to a track file\n"
           "  -W <file>           Same, compact (half lengths, 6 bytes per segment)\n"
           "  -t <threads>        Accepted and ignored\n");
}

static void *xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p) {
        fprintf(stderr, "out of host memory\n");
        exit(3);
    }
    return p;
}

int main(int argc, char **argv)
{
    long segments = 50000000;
    int groups = 128, regions = 6750, device = 0, repeats = 1, table = 0;
    long tracks = -1;
    int intervals = 5;
    const char *in_file = NULL, *out_file = NULL;
    int compact = 0;
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
        const int more = i + 1 < argc;
        if (!strcmp(a, "-s") && more) segments = atol(argv[++i]);
        else if (!strcmp(a, "-e") && more) groups = atoi(argv[++i]);
        else if (!strcmp(a, "-r") && more) regions = atoi(argv[++i]);
        else if (!strcmp(a, "-k") && more) tracks = atol(argv[++i]);
        else if (!strcmp(a, "-d") && more) device = atoi(argv[++i]);
        else if (!strcmp(a, "-n") && more) repeats = atoi(argv[++i]);
        else if (!strcmp(a, "-t") && more) ++i;
        else if (!strcmp(a, "-x")) table = 1;
        else if (!strcmp(a, "-f") && more) in_file = argv[++i];
        else if (!strcmp(a, "-w") && more) out_file = argv[++i];
        else if (!strcmp(a, "-W") && more) {
            out_file = argv[++i];
            compact = 1;
        }
        else {
            usage();
            return 1;
        }
    }
    moc_trackfile_info_t info;
    if (in_file) {
        const moc_status_t fs = moc_trackfile_info(in_file, &info);
        if (fs != MOC_OK) {
            fprintf(stderr, "%s: %s\n", in_file, moc_status_string(fs));
            return 1;
        }
        segments = info.n_segments;
        tracks = info.n_tracks;
        regions = info.n_regions;
        intervals = info.n_intervals;
    }
    if (tracks < 0) tracks = segments / 500 > 0 ? segments / 500 : 1;
    if (segments < 0 || groups < 1 || regions < 1 || tracks < 1 || repeats < 1 ||
        tracks > 2147483647L) {
        usage();
        return 1;
    }

    moc_synth_spec_t spec;
    moc_synth_spec_init(&spec, 1, regions, intervals, groups, (int32_t)tracks, segments);
    const long Gs = spec.group_stride, ncell = (long)regions * intervals;
    int64_t *off = xmalloc((size_t)(tracks + 1) * sizeof(int64_t));
    if (!in_file && moc_synth_track_offsets(&spec, off) < 0) {
        fprintf(stderr, "invalid sizes\n");
        return 1;
    }
    float *psi = xmalloc((size_t)(tracks * Gs) * sizeof(float));
    float *sigT = xmalloc((size_t)(regions * Gs) * sizeof(float));
    float *source = xmalloc((size_t)(ncell * Gs) * sizeof(float));
    float *flux = calloc((size_t)(ncell * Gs), sizeof(float));
    int32_t *reg = xmalloc((size_t)segments * sizeof(int32_t));
    uint8_t *itv = xmalloc((size_t)segments);
    float *ds = xmalloc((size_t)segments * sizeof(float));
    if (!flux) return 3;
    if (in_file) {
        const moc_status_t fs = moc_trackfile_read(in_file, off, reg, itv, ds);
        if (fs != MOC_OK || moc_synth_fill(&spec, off, psi, sigT, source, NULL, NULL, NULL)) {
            fprintf(stderr, "%s: %s\n", in_file, moc_status_string(fs ? fs : MOC_ERR_IO));
            return 1;
        }
    } else {
        moc_synth_fill(&spec, off, psi, sigT, source, reg, itv, ds);
    }
    if (out_file) {
        const moc_status_t fs =
            compact ? moc_trackfile_write_compact(out_file, tracks, segments, regions,
                                                  intervals, off, reg, itv, ds)
                    : moc_trackfile_write(out_file, tracks, segments, regions, intervals, off,
                                          reg, itv, ds);
        if (fs != MOC_OK) {
            fprintf(stderr, "%s: %s\n", out_file, moc_status_string(fs));
            return 1;
        }
    }

    moc_problem_t p = {0};
    p.n_regions = regions;
    p.n_intervals = intervals;
    p.n_groups = groups;
    p.group_stride = (int32_t)Gs;
    p.n_tracks = (int32_t)tracks;
    p.n_segments = segments;
    p.track_offsets = off;
    p.seg_region = reg;
    p.seg_interval = itv;
    p.seg_ds = ds;
    p.sigT = sigT;
    p.source = source;
    p.fine_flux = flux;
    p.psi = psi;
    moc_fwd_opts_t o;
    moc_fwd_opts_default(&o);
    if (table) o.exp_mode = MOC_EXP_TABLE;

    moc_handle_t h = NULL;
    moc_status_t st = moc_create(&h, device);
    if (st != MOC_OK) {
        fprintf(stderr, "moc_create: %s\n", moc_status_string(st));
        return 2;
    }
    /* one untimed call sizes the handle's device copies */
    st = moc_attenuate_fwd_host(h, &p, &o);
    double t0 = now();
    for (int r = 0; r < repeats && st == MOC_OK; r++) st = moc_attenuate_fwd_host(h, &p, &o);
    double t1 = now();
    if (st != MOC_OK) {
        fprintf(stderr, "moc_attenuate_fwd_host: %s %s\n", moc_status_string(st),
                moc_last_error(h));
        moc_destroy(h);
        return 2;
    }
    const double sec = (t1 - t0) / repeats;
    double check = 0.0;
    for (long k = 0; k < tracks * Gs; k++) check += psi[k];
    printf("Segments: %ld  Groups: %d  Regions: %d  Tracks: %ld  Exp: %s\n", segments, groups,
           regions, tracks, table ? "table" : "full");
    printf("%-25s%.6f seconds\n", "Runtime:", sec);
    printf("%-25s%.6f ns\n", "Time per Intersection:", sec / (double)segments / groups * 1e9);
    printf("%-25s%.6e\n", "psi checksum:", check);
    moc_destroy(h);
    return 0;
}
