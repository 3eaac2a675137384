/*
 * moc_synth.h — seeded synthetic inputs for the segment-attenuation sweep.
 *
 * Replaces the reference's input synthesis:
 *   - initialize_sources()   src/cpu/init.c:26-78   (rand() U(0,1) fill of fine_source,
 *                                                     fine_flux and sigT)
 *   - the per-segment draws  src/cpu/kernel.c:29-30,47-50 (psi via rand_r, random
 *                                                     QSR_id / FAI_id per segment)
 * The reference seeds from time(NULL) and is not reproducible. This generator is
 * counter-based (SplitMix64 finaliser, Steele, Lea & Flood 2014), so every draw is a
 * pure function of (seed, stream, index): the same inputs come out on x86 and Arm,
 * single- or multi-threaded.
 *
 * Draw definition (all integer arithmetic modulo 2^64):
 *   fin(z)        = SplitMix64 finaliser
 *                   z ^= z>>30; z *= 0xBF58476D1CE4E5B9; z ^= z>>27;
 *                   z *= 0x94D049BB133111EB; z ^= z>>31
 *   key(seed,tag) = fin(fin(seed) + tag * 0x9E3779B97F4A7C15)
 *   x(seed,tag,k) = fin(key(seed,tag) + (k+1) * 0x9E3779B97F4A7C15)
 *   uniform float u in [0,1)  = (x >> 40) * 2^-24          (exact in FP32)
 *   uniform double d in [0,1) = (x >> 11) * 2^-53
 *   uniform int in [0,n)      = ((x >> 32) * n) >> 32      (multiply-shift)
 *   U(a,b) float              = a + (b - a) * u            (FP32, no contraction)
 *   logU(a,b) float           = (float) exp(log(a) + d * (log(b) - log(a)))
 *   N(0,1)                    = Box-Muller on draws 2k, 2k+1 of the stream:
 *                               sqrt(-2 ln(1-d0)) * cos(2 pi d1)
 *
 * Streams (tag): 1 psi[T][G], 2 sigT[R][G], 3 source[R][I][G],
 *   4 segments (draws 4j..4j+3 = track, region, interval, ds of segment j),
 *   5 track lengths (Box-Muller pair per track), 6.. free for callers
 *   (loss weights, parameter picks, initial tallies).
 *
 * Layout of what is filled (group_stride >= n_groups; padding lanes are set to 0,
 * except sigT padding which is set to 1 so padded lanes stay finite):
 *   psi    [T][group_stride]     sigT [R][group_stride]
 *   source [R][I][group_stride]
 *   seg_region[S] int32, seg_interval[S] uint8, seg_ds[S] float, grouped by track
 *   in CSR order: track t owns segments [track_offsets[t], track_offsets[t+1]).
 */
#ifndef MOC_SYNTH_H
#define MOC_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* How segments are assigned to tracks. */
enum {
    MOC_SYNTH_TRACKS_UNIFORM   = 0, /* each segment draws its track uniformly; CSR by a
                                       stable counting sort (original order kept)      */
    MOC_SYNTH_TRACKS_LOGNORMAL = 1  /* track t has round(median*exp(sigma*z_t)) segments,
                                       clipped to [len_min, len_max]                    */
};

/* Distribution of sigT. */
enum {
    MOC_SYNTH_SIGT_UNIFORM    = 0,  /* U(sigT_lo, sigT_hi)    */
    MOC_SYNTH_SIGT_LOGUNIFORM = 1   /* logU(sigT_lo, sigT_hi) */
};

typedef struct {
    uint64_t seed;
    int32_t  n_regions;     /* R */
    int32_t  n_intervals;   /* I (fine axial intervals, 2..255) */
    int32_t  n_groups;      /* G */
    int32_t  group_stride;  /* >= G */
    int32_t  n_tracks;      /* T */
    int64_t  n_segments;    /* S: input for UNIFORM mode, ignored (computed) for LOGNORMAL */
    int32_t  track_mode;    /* MOC_SYNTH_TRACKS_* */
    float    len_median;    /* LOGNORMAL only */
    float    len_sigma;
    int32_t  len_min, len_max;
    int32_t  sigT_mode;     /* MOC_SYNTH_SIGT_* */
    float    sigT_lo, sigT_hi;
    float    ds_lo, ds_hi;
} moc_synth_spec_t;

/* Fill a spec with the distributions shared by all workloads (sigT U(0.1,2.0),
 * ds U(0.01,1.0), uniform track assignment) and the given sizes. */
void moc_synth_spec_init(moc_synth_spec_t *spec, uint64_t seed, int32_t n_regions,
                         int32_t n_intervals, int32_t n_groups, int32_t n_tracks,
                         int64_t n_segments);

/* Compute the CSR track offsets [T+1]. Returns the total segment count S (>= 0), or -1
 * on invalid arguments. For UNIFORM mode this is spec->n_segments. */
int64_t moc_synth_track_offsets(const moc_synth_spec_t *spec, int64_t *track_offsets);

/* Fill every input array (any pointer may be NULL to skip that array). track_offsets
 * must come from moc_synth_track_offsets with the same spec. Returns 0 or -1. */
int moc_synth_fill(const moc_synth_spec_t *spec, const int64_t *track_offsets,
                   float *psi, float *sigT, float *source, int32_t *seg_region,
                   uint8_t *seg_interval, float *seg_ds);

/* n draws of U(lo,hi) / N(0,1) from stream `tag` (for loss weights, initial tallies). */
void moc_synth_uniform(uint64_t seed, uint64_t tag, int64_t n, float lo, float hi,
                       float *out);
void moc_synth_normal(uint64_t seed, uint64_t tag, int64_t n, float *out);
/* n draws of uniform integers in [0, bound) from stream `tag`. */
void moc_synth_randint(uint64_t seed, uint64_t tag, int64_t n, int64_t bound,
                       int64_t *out);

#ifdef __cplusplus
}
#endif
#endif /* MOC_SYNTH_H */
