/*
 * Seeded synthetic inputs for the segment-attenuation sweep (declared in moc_synth.h).
 *
 * Stands in for the reference's initialize_sources() (src/cpu/init.c:26-78) and the
 * rand_r draws of psi / QSR_id / FAI_id in run_kernel (src/cpu/kernel.c:29-30,47-50),
 * with a counter-based generator so the inputs are reproducible on every host.
 * Build with -ffp-contract=off: U(a,b) must round the same way on x86 and Arm.
 */
#include "moc_synth.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define GOLDEN 0x9E3779B97F4A7C15ULL

enum { TAG_PSI = 1, TAG_SIGT = 2, TAG_SOURCE = 3, TAG_SEG = 4, TAG_LEN = 5 };

static inline uint64_t fin64(uint64_t z)
{
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ULL;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return z;
}

static inline uint64_t stream_key(uint64_t seed, uint64_t tag)
{
    return fin64(fin64(seed) + tag * GOLDEN);
}

static inline uint64_t draw(uint64_t key, uint64_t k)
{
    return fin64(key + (k + 1) * GOLDEN);
}

static inline float u24(uint64_t x) { return (float)(x >> 40) * (1.0f / 16777216.0f); }
static inline double u53(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }
static inline uint32_t below(uint64_t x, uint32_t n)
{
    return (uint32_t)(((x >> 32) * (uint64_t)n) >> 32);
}
static inline float uab(uint64_t x, float a, float b)
{
    float d = b - a;
    float p = d * u24(x);
    return a + p;
}

void moc_synth_spec_init(moc_synth_spec_t *spec, uint64_t seed, int32_t n_regions,
                         int32_t n_intervals, int32_t n_groups, int32_t n_tracks,
                         int64_t n_segments)
{
    memset(spec, 0, sizeof(*spec));
    spec->seed = seed;
    spec->n_regions = n_regions;
    spec->n_intervals = n_intervals;
    spec->n_groups = n_groups;
    spec->group_stride = (n_groups + 3) & ~3;
    spec->n_tracks = n_tracks;
    spec->n_segments = n_segments;
    spec->track_mode = MOC_SYNTH_TRACKS_UNIFORM;
    spec->len_median = 200.0f;
    spec->len_sigma = 0.9005f;
    spec->len_min = 1;
    spec->len_max = 5000;
    spec->sigT_mode = MOC_SYNTH_SIGT_UNIFORM;
    spec->sigT_lo = 0.1f;
    spec->sigT_hi = 2.0f;
    spec->ds_lo = 0.01f;
    spec->ds_hi = 1.0f;
}

static int spec_ok(const moc_synth_spec_t *s)
{
    if (!s) return 0;
    if (s->n_regions < 1 || s->n_intervals < 2 || s->n_intervals > 255) return 0;
    if (s->n_groups < 1 || s->group_stride < s->n_groups || s->n_tracks < 1) return 0;
    if (s->track_mode == MOC_SYNTH_TRACKS_UNIFORM && s->n_segments < 0) return 0;
    if (s->track_mode == MOC_SYNTH_TRACKS_LOGNORMAL &&
        (s->len_min < 0 || s->len_max < s->len_min || !(s->len_median > 0.0f)))
        return 0;
    if (s->track_mode != MOC_SYNTH_TRACKS_UNIFORM &&
        s->track_mode != MOC_SYNTH_TRACKS_LOGNORMAL)
        return 0;
    if (s->sigT_mode == MOC_SYNTH_SIGT_LOGUNIFORM && !(s->sigT_lo > 0.0f)) return 0;
    return 1;
}

/* Box-Muller normal from draws 2k and 2k+1 of a stream. */
static double normal_pair(uint64_t key, uint64_t k)
{
    double d0 = u53(draw(key, 2 * k));
    double d1 = u53(draw(key, 2 * k + 1));
    double r = sqrt(-2.0 * log(1.0 - d0));
    return r * cos(6.283185307179586476925 * d1);
}

int64_t moc_synth_track_offsets(const moc_synth_spec_t *spec, int64_t *off)
{
    if (!spec_ok(spec) || !off) return -1;
    const int64_t T = spec->n_tracks;
    if (spec->track_mode == MOC_SYNTH_TRACKS_LOGNORMAL) {
        uint64_t key = stream_key(spec->seed, TAG_LEN);
        off[0] = 0;
        for (int64_t t = 0; t < T; t++) {
            double z = normal_pair(key, (uint64_t)t);
            double len = (double)spec->len_median * exp((double)spec->len_sigma * z);
            long long L = llround(len);
            if (L < spec->len_min) L = spec->len_min;
            if (L > spec->len_max) L = spec->len_max;
            off[t + 1] = off[t] + L;
        }
        return off[T];
    }
    /* UNIFORM: count the track draw of every segment, then prefix-sum. */
    const int64_t S = spec->n_segments;
    uint64_t key = stream_key(spec->seed, TAG_SEG);
    memset(off, 0, (size_t)(T + 1) * sizeof(int64_t));
    for (int64_t j = 0; j < S; j++) {
        uint32_t t = below(draw(key, 4 * (uint64_t)j), (uint32_t)T);
        off[t + 1]++;
    }
    for (int64_t t = 0; t < T; t++) off[t + 1] += off[t];
    return off[T];
}

int moc_synth_fill(const moc_synth_spec_t *spec, const int64_t *off, float *psi,
                   float *sigT, float *source, int32_t *seg_region, uint8_t *seg_interval,
                   float *seg_ds)
{
    if (!spec_ok(spec) || !off) return -1;
    const int64_t R = spec->n_regions, I = spec->n_intervals, G = spec->n_groups;
    const int64_t Gs = spec->group_stride, T = spec->n_tracks;
    const int64_t S = off[T];

    if (psi) {
        uint64_t key = stream_key(spec->seed, TAG_PSI);
        for (int64_t t = 0; t < T; t++)
            for (int64_t g = 0; g < Gs; g++)
                psi[t * Gs + g] = g < G ? u24(draw(key, (uint64_t)(t * G + g))) : 0.0f;
    }
    if (sigT) {
        uint64_t key = stream_key(spec->seed, TAG_SIGT);
        const double la = log((double)spec->sigT_lo), lb = log((double)spec->sigT_hi);
        for (int64_t r = 0; r < R; r++)
            for (int64_t g = 0; g < Gs; g++) {
                float v = 1.0f;
                if (g < G) {
                    uint64_t x = draw(key, (uint64_t)(r * G + g));
                    if (spec->sigT_mode == MOC_SYNTH_SIGT_LOGUNIFORM)
                        v = (float)exp(la + u53(x) * (lb - la));
                    else
                        v = uab(x, spec->sigT_lo, spec->sigT_hi);
                }
                sigT[r * Gs + g] = v;
            }
    }
    if (source) {
        uint64_t key = stream_key(spec->seed, TAG_SOURCE);
        for (int64_t c = 0; c < R * I; c++)
            for (int64_t g = 0; g < Gs; g++)
                source[c * Gs + g] = g < G ? u24(draw(key, (uint64_t)(c * G + g))) : 0.0f;
    }
    if (seg_region || seg_interval || seg_ds) {
        uint64_t key = stream_key(spec->seed, TAG_SEG);
        if (spec->track_mode == MOC_SYNTH_TRACKS_LOGNORMAL) {
            for (int64_t j = 0; j < S; j++) {
                uint64_t b = 4 * (uint64_t)j;
                if (seg_region) seg_region[j] = (int32_t)below(draw(key, b + 1), (uint32_t)R);
                if (seg_interval) seg_interval[j] = (uint8_t)below(draw(key, b + 2), (uint32_t)I);
                if (seg_ds) seg_ds[j] = uab(draw(key, b + 3), spec->ds_lo, spec->ds_hi);
            }
        } else {
            /* Stable placement: segment j goes to the next free slot of its track. */
            int64_t *cursor = (int64_t *)malloc((size_t)T * sizeof(int64_t));
            if (!cursor) return -1;
            memcpy(cursor, off, (size_t)T * sizeof(int64_t));
            for (int64_t j = 0; j < S; j++) {
                uint64_t b = 4 * (uint64_t)j;
                uint32_t t = below(draw(key, b), (uint32_t)T);
                int64_t p = cursor[t]++;
                if (seg_region) seg_region[p] = (int32_t)below(draw(key, b + 1), (uint32_t)R);
                if (seg_interval) seg_interval[p] = (uint8_t)below(draw(key, b + 2), (uint32_t)I);
                if (seg_ds) seg_ds[p] = uab(draw(key, b + 3), spec->ds_lo, spec->ds_hi);
            }
            free(cursor);
        }
    }
    return 0;
}

void moc_synth_uniform(uint64_t seed, uint64_t tag, int64_t n, float lo, float hi,
                       float *out)
{
    uint64_t key = stream_key(seed, tag);
    for (int64_t i = 0; i < n; i++) out[i] = uab(draw(key, (uint64_t)i), lo, hi);
}

void moc_synth_normal(uint64_t seed, uint64_t tag, int64_t n, float *out)
{
    uint64_t key = stream_key(seed, tag);
    for (int64_t i = 0; i < n; i++) out[i] = (float)normal_pair(key, (uint64_t)i);
}

void moc_synth_randint(uint64_t seed, uint64_t tag, int64_t n, int64_t bound, int64_t *out)
{
    uint64_t key = stream_key(seed, tag);
    for (int64_t i = 0; i < n; i++) {
        uint64_t x = draw(key, (uint64_t)i);
        /* 64x64 -> high 64 via two 32-bit halves (portable, no __int128). */
        uint64_t b = (uint64_t)bound;
        uint64_t xh = x >> 32, xl = x & 0xffffffffULL, bh = b >> 32, bl = b & 0xffffffffULL;
        uint64_t ll = xl * bl, lh = xl * bh, hl = xh * bl, hh = xh * bh;
        uint64_t mid = (ll >> 32) + (lh & 0xffffffffULL) + (hl & 0xffffffffULL);
        out[i] = (int64_t)(hh + (lh >> 32) + (hl >> 32) + (mid >> 32));
    }
}
