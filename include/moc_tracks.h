/*
 * moc_tracks.h — track generation for the segment-attenuation sweep (C ABI).
 *
 * The step before the sweep: ray tracing of straight 3D characteristic tracks through a
 * source-region mesh, producing the sweep's segment descriptors (CSR by track:
 * track_offsets, seg_region, seg_interval, seg_ds of moc_problem_t). The reference
 * kernel stubs this step with random draws of the region, interval and length of every
 * segment (src/cpu/kernel.c:47-50, src/cuda/kernel.cu:52-60); its parent application
 * traces tracks through a reactor geometry. This is that step for a geometry of the
 * same kind:
 *
 *   radial: an nx x ny lattice of square pin cells of side `pitch`, each holding a fuel
 *           cylinder of radius `fuel_radius` (< 0.45 pitch) cut into `n_rings` rings of
 *           equal area, and the moderator around it (ring index n_rings);
 *   axial:  the height [0, height] cut into `n_axial` source regions, each of
 *           `n_intervals` fine axial intervals (the sweep's I) of equal thickness.
 *
 * Source region of (pin cell ix, iy; ring k; axial region a):
 *   region = ((iy * nx + ix) * (n_rings + 1) + k) * n_axial + a,
 * and n_regions = nx * ny * (n_rings + 1) * n_axial. A segment's interval is its fine
 * axial interval inside its axial region.
 *
 * Tracks: for each azimuth phi_a = pi (a + 1/2) / n_azim, 2D lines of direction
 * (cos phi, sin phi) at perpendicular spacing `spacing` cover the lattice; for each polar
 * cosine mu_p = 1 - (2p + 1) / n_polar (equal-weight cosine bins, none horizontal when
 * n_polar is even) 3D tracks over each 2D line are stacked at perpendicular spacing
 * `axial_spacing` (vertical spacing axial_spacing / sin(theta)) and clipped to the box.
 * Every direction bin carries the same solid angle and every track the same
 * cross-section, so all tracks share one weight (moc_tracks_weight). With
 * both_directions, every 3D track is followed by its reverse (same segments in reverse
 * order), so the directions cover the sphere.
 *
 * The plan (moc_tracks_plan, host) lists the tracks; moc_trace_count and
 * moc_trace_segments walk them on the GPU, one thread per track, in FP64 without
 * contraction. Crossings are the pin-cell grid lines, the ring circles and the fine axial
 * planes along the track; a segment runs between consecutive distinct crossings and is
 * classified by its midpoint; its length is the 3D distance, rounded to float.
 */
#ifndef MOC_TRACKS_H
#define MOC_TRACKS_H

#include <stdint.h>

#include "moc_attenuate.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MOC_TRACKS_MAX_RINGS 8

typedef struct {
    int32_t nx, ny;        /* pin cells in x and y (>= 1)                                  */
    int32_t n_rings;       /* equal-area rings per fuel cylinder, 1..MOC_TRACKS_MAX_RINGS  */
    int32_t n_axial;       /* axial source regions (>= 1)                                  */
    int32_t n_intervals;   /* fine axial intervals per source region, 2..255 (the sweep's I) */
    int32_t reserved;      /* 0                                                            */
    double pitch;          /* pin-cell side (> 0)                                          */
    double fuel_radius;    /* fuel cylinder radius, 0 < r < 0.45 pitch                     */
    double height;         /* axial extent (> 0)                                           */
} moc_geometry_t;

typedef struct {
    int32_t n_azim;          /* azimuthal angles in (0, pi), even, >= 2                    */
    int32_t n_polar;         /* polar cosine bins in (-1, 1), even, >= 2                   */
    int32_t both_directions; /* 1: every track followed by its reverse                     */
    int32_t reserved;        /* 0                                                          */
    double spacing;          /* perpendicular spacing of the 2D lines (> 0)                */
    double axial_spacing;    /* perpendicular spacing of the stacked 3D tracks (> 0)       */
} moc_quadrature_t;

/* One 3D track: points (x0 + t ux, y0 + t uy, za + (t - ta) cot) for t in [ta, tb], with
 * t the distance along the 2D line from its entry into the lattice; 3D length per unit
 * t is rsin = 1/sin(theta). rux = 1/ux, ruy = 1/uy (+-inf where the component is 0),
 * rcot = 1/cot. reversed = 1: the segments of this track are emitted last to first. */
typedef struct {
    double x0, y0, ux, uy, rux, ruy;
    double ta, tb, za, cot, rcot, rsin;
    int32_t azim, polar;   /* direction bin indices                                        */
    int32_t reversed;
    int32_t reserved;
} moc_track_t;

/* n_regions of the geometry (0 if invalid). */
int32_t moc_geometry_regions(const moc_geometry_t *g);

/* Volume of every (region, interval) cell, vol[n_regions * n_intervals]: ring areas
 * pi fuel_radius^2 / n_rings, moderator pitch^2 - pi fuel_radius^2, times the fine
 * interval thickness height / (n_axial n_intervals). */
moc_status_t moc_geometry_volumes(const moc_geometry_t *g, double *vol);

/* The plan: fills tracks[0 .. min(*n_tracks_out, cap)) in plan order (azimuth, 2D line,
 * polar bin, stack position, then the reverse if both_directions) and sets *n_tracks_out
 * to the full count. tracks = NULL, cap = 0 only counts. Host only, deterministic. */
moc_status_t moc_tracks_plan(const moc_geometry_t *g, const moc_quadrature_t *q,
                             moc_track_t *tracks, int64_t cap, int64_t *n_tracks_out);

/* Weight of every track for the sweep's tally (opts.weight): the solid angle of a
 * direction bin, 4 pi / (n_azim n_polar) (2 pi / (n_azim n_polar) with both_directions,
 * whose 2 n_azim azimuths cover the circle), times the track cross-section
 * spacing * axial_spacing. The tallies are then track-length estimates of the
 * volume-integrated scalar flux. */
double moc_tracks_weight(const moc_quadrature_t *q);

/* Segment count of every track (d_tracks: n_tracks device records), scanned into
 * d_track_offsets[0 .. n_tracks] (device, int64), and the total returned in *n_segments
 * (host; the call synchronizes `stream`). The tracks are walked once, into workspace of
 * the handle sized by a per-track upper bound of the counts; a following
 * moc_trace_segments with the same tracks, count and offsets (the records unchanged)
 * copies that walk out instead of walking again. */
moc_status_t moc_trace_count(moc_handle_t h, const moc_geometry_t *g,
                             const moc_track_t *d_tracks, int64_t n_tracks,
                             int64_t *d_track_offsets, int64_t *n_segments, void *stream);

/* The segments of every track into the CSR arrays sized by moc_trace_count
 * (d_seg_region int32, d_seg_interval uint8, d_seg_ds float; device, n_segments each),
 * asynchronous on `stream`. The descriptors are those moc_attenuate_fwd reads. Right
 * after moc_trace_count on the same handle and arguments this is a copy of that call's
 * walk; otherwise the tracks are walked again (a segment count that disagrees with the
 * offsets is then reported by moc_synchronize as MOC_ERR_BAD_TRACK). */
moc_status_t moc_trace_segments(moc_handle_t h, const moc_geometry_t *g,
                                const moc_track_t *d_tracks, int64_t n_tracks,
                                const int64_t *d_track_offsets, int32_t *d_seg_region,
                                uint8_t *d_seg_interval, float *d_seg_ds, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MOC_TRACKS_H */
