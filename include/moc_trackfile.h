/*
 * moc_trackfile.h — the on-disk track format (C ABI, host only).
 *
 * A problem's segment descriptors (CSR by track, as moc_problem_t takes them) in one
 * binary file that the GPU program (host/moc_driver.c, -f / -w / -W) and the CPU harness
 * (oracle/cpu_bench, --track-file) both read, so a traced or generated track set is made
 * once and swept by either. Region and interval are packed into one 32-bit cell index.
 * Two versions:
 *   1: lengths as FP32, 8 bytes per segment instead of the 9 of the three arrays; nothing
 *      is rounded;
 *   2 (compact): lengths as IEEE half (round to nearest even), 6 bytes per segment; the
 *      reader widens them exactly, so a length changes by at most 2^-11 of itself (2^-25
 *      absolute below 6.1e-5) and the sweep then computes with the rounded lengths.
 *
 * Layout (little-endian, no padding):
 *   offset  size  field
 *        0     8  magic "MOCTRK01"
 *        8     4  uint32 version (1 or 2)
 *       12     4  uint32 header bytes (48)
 *       16     8  int64 n_tracks T
 *       24     8  int64 n_segments S
 *       32     4  int32 n_regions R
 *       36     4  int32 n_intervals I
 *       40     8  uint64 checksum of the payload
 *       48        payload: int64 offsets[T + 1], uint32 cell[S] (region * I + interval),
 *                 then float ds[S] (version 1) or uint16 half ds[S] (version 2)
 * The checksum is FNV-1a over the payload read as little-endian 64-bit words (the last
 * one zero-padded): h = 14695981039346656037; for each word w: h = (h ^ w) *
 * 1099511628211 (mod 2^64).
 */
#ifndef MOC_TRACKFILE_H
#define MOC_TRACKFILE_H

#include <stdint.h>

#include "moc_attenuate.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t n_tracks, n_segments;
    int32_t n_regions, n_intervals;
    uint64_t checksum;
    int32_t version;              /* 1: FP32 lengths; 2: half lengths (compact)         */
    int32_t bytes_per_segment;    /* 8 or 6                                              */
} moc_trackfile_info_t;

/* Write T tracks of S segments (host arrays; offsets[T + 1] a partition of [0, S], every
 * region in [0, R), interval in [0, I), R * I < 2^32). MOC_ERR_INVALID_ARG for arrays that
 * break those rules, MOC_ERR_IO if the file cannot be written. */
moc_status_t moc_trackfile_write(const char *path, int64_t n_tracks, int64_t n_segments,
                                 int32_t n_regions, int32_t n_intervals,
                                 const int64_t *track_offsets, const int32_t *seg_region,
                                 const uint8_t *seg_interval, const float *seg_ds);

/* The same descriptors in the compact version 2: every length must be finite, >= 0 and
 * below 65520 (it is stored as an IEEE half, rounded to nearest even), else
 * MOC_ERR_INVALID_ARG. A further step of the on-disk format, with no counterpart in the
 * reference (whose segments are random draws, src/cpu/kernel.c:47-50). */
moc_status_t moc_trackfile_write_compact(const char *path, int64_t n_tracks, int64_t n_segments,
                                         int32_t n_regions, int32_t n_intervals,
                                         const int64_t *track_offsets,
                                         const int32_t *seg_region,
                                         const uint8_t *seg_interval, const float *seg_ds);

/* The header of a track file (checksum not verified). MOC_ERR_IO if it is not one. */
moc_status_t moc_trackfile_info(const char *path, moc_trackfile_info_t *info);

/* Read the descriptors (either version; half lengths widened exactly to FP32) into host
 * arrays sized from moc_trackfile_info (offsets T + 1, the others S), checking the
 * checksum, the offsets and every cell index: MOC_ERR_IO for
 * a file that is short, corrupt or inconsistent (the arrays' contents are then
 * unspecified). */
moc_status_t moc_trackfile_read(const char *path, int64_t *track_offsets, int32_t *seg_region,
                                uint8_t *seg_interval, float *seg_ds);

#ifdef __cplusplus
}
#endif

#endif /* MOC_TRACKFILE_H */
