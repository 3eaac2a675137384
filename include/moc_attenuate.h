/*
 * moc_attenuate.h — C ABI of the GB300 segment-attenuation sweep (libmocatt.so).
 *
 * What it replaces in the reference (ANL-CESAR/SimpleMOC-kernel):
 *   - void run_kernel(Input*, Source*, Table*)            src/cpu/SimpleMOC-kernel_header.h:81
 *       the OpenMP loop over segments, src/cpu/kernel.c:3-73, called once from
 *       src/cpu/main.c:46                                  -> moc_attenuate_fwd[_host]
 *   - void attenuate_segment(Input*, Source*, int QSR_id, int FAI_id, float* state_flux,
 *       SIMD_Vectors*, Table*)                             src/cpu/SimpleMOC-kernel_header.h:82-84
 *       the per-segment body, src/cpu/kernel.c:75-333      -> one (segment, group) lane of
 *                                                             the device sweep
 *   - __global__ run_kernel(Input, Source*, Source_Arrays, Table*, curandState*, float*, int)
 *                                                          src/cuda/SimpleMOC-kernel_header.h:66-68
 *   - Table* buildExponentialTable(float precision, float maxVal, Input*)
 *                                                          src/cpu/init.c:81-117
 *                                                          -> moc_build_exp_table
 *   - float interpolateTable(Table*, float x)              src/cpu/kernel.c:337-361
 *                                                          -> MOC_EXP_TABLE mode
 *
 * Differences in meaning, all deliberate:
 *   - Segments are explicit inputs (region, interval, ds per segment, grouped by track
 *     in CSR order) instead of rand_r draws inside the loop (src/cpu/kernel.c:47-50);
 *     ds is per segment instead of the constant 0.7f (src/cpu/kernel.c:104).
 *   - psi is carried per track (psi[T][G]) instead of per OpenMP thread
 *     (src/cpu/kernel.c:24-30).
 *   - The tally fine_flux[r][i][g] += weight * flux_integral is an atomic reduction on
 *     the device instead of a per-(region, interval) omp_lock (src/cpu/kernel.c:265-281).
 *   - Errors come back as moc_status_t; nothing exits (the reference has no error path).
 *
 * Conventions:
 *   - Every pointer in moc_problem_t is caller-owned device memory (moc_attenuate_fwd)
 *     or host memory (moc_attenuate_fwd_host); the library never frees them.
 *   - Float arrays must be 16-byte aligned and group_stride a multiple of 4, so each
 *     row is read as 128-bit vectors.
 *   - Device calls are asynchronous and ordered on `stream` (a cudaStream_t passed as
 *     void*; NULL = legacy default stream). A handle serves one host thread at a time;
 *     distinct handles are independent.
 */
#ifndef MOC_ATTENUATE_H
#define MOC_ATTENUATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MOC_ABI_VERSION 4

typedef enum {
    MOC_OK = 0,
    MOC_ERR_INVALID_ARG = 1,     /* NULL pointer, negative size, unknown enum value   */
    MOC_ERR_MISALIGNED = 2,      /* a float array is not 16-byte aligned             */
    MOC_ERR_UNSUPPORTED = 3,     /* valid but unsupported combination                */
    MOC_ERR_CUDA = 4,            /* a CUDA runtime call failed (see moc_last_error)   */
    MOC_ERR_NO_DEVICE = 5,       /* no CUDA device, or the device index is invalid   */
    MOC_ERR_OUT_OF_MEMORY = 6,   /* workspace allocation failed                      */
    MOC_ERR_BAD_INDEX = 7,       /* checked mode: a segment named a region, interval
                                    or track offset out of range; nothing was added  */
    MOC_ERR_DEVICE_TIMEOUT = 8,  /* a bounded device-side wait gave up               */
    MOC_ERR_TOO_LARGE = 9,       /* the problem exceeds the fixed scratch of
                                    moc_attenuate_fwd_noalloc                         */
    MOC_ERR_BAD_TRACK = 10,      /* track generation (moc_tracks.h): a track record is
                                    invalid or disagrees with the offsets             */
    MOC_ERR_IO = 11              /* a track file (moc_trackfile.h) cannot be written or
                                    read, or is short, corrupt or inconsistent        */
} moc_status_t;

typedef struct moc_handle_s *moc_handle_t;

/* Exponential evaluation: 1 - exp(-tau). */
typedef enum {
    MOC_EXP_FULL = 0,   /* range-reduced exp (the reference's 1.f - expf(-tau),
                           src/cpu/kernel.c:221)                                        */
    MOC_EXP_TABLE = 1   /* the reference's piecewise-linear table, built by
                           src/cpu/init.c:81-117 and read by src/cpu/kernel.c:337-361,
                           reproduced exactly (including its slope sign and index rule)   */
} moc_exp_mode_t;

/*
 * Storage precision of sigT and the axial source coefficients (math is always FP32).
 * The precision forms (all but MOC_PREC_FP32) evaluate 1 - exp(-tau), tau - (1 - exp(-tau))
 * and the cubic of src/cpu/kernel.c:250-251 from one Taylor sum below tau = 1, where the
 * reference's expressions cancel, and accept every moc_tally_t. MOC_PREC_FP32 is the
 * reference computation (drop-in) and takes MOC_TALLY_ATOMIC_FP32 only.
 */
typedef enum {
    MOC_PREC_FP32 = 0,       /* plain method: the reference computation in FP32          */
    MOC_PREC_BF16 = 1,       /* precision form: sigT and coefficients stored as bf16      */
    MOC_PREC_FP16 = 2,       /* precision form: sigT and coefficients stored as fp16      */
    MOC_PREC_FP32_STABLE = 3 /* precision form with FP32 storage                          */
} moc_precision_t;

/* How fine_flux tallies are accumulated. */
typedef enum {
    MOC_TALLY_ATOMIC_FP32 = 0,  /* vector red.global.add.f32 into fine_flux             */
    MOC_TALLY_COMPENSATED = 1,  /* FP32 atomics with an error-free-transform companion
                                   array (hi + lo), combined in FP64 at the end         */
    MOC_TALLY_FP64 = 2          /* FP64 atomics into a workspace, added at the end       */
} moc_tally_t;

/*
 * One sweep problem. Sizes follow the reference's Input (src/cpu/SimpleMOC-kernel_header.h:
 * 24-42): n_regions = source_3D_regions, n_intervals = fine_axial_intervals,
 * n_groups = egroups, n_segments = segments. Arrays follow Source
 * (src/cpu/SimpleMOC-kernel_header.h:45-52): fine_source, fine_flux and sigT, one
 * contiguous array each.
 */
typedef struct {
    int32_t n_regions;            /* R >= 1                                              */
    int32_t n_intervals;          /* I, 2..255                                           */
    int32_t n_groups;             /* G >= 1                                              */
    int32_t group_stride;         /* row stride in floats, >= G, multiple of 4          */
    int32_t n_tracks;             /* T >= 0                                              */
    int32_t reserved0;
    int64_t n_segments;           /* S >= 0                                              */
    const int64_t *track_offsets; /* [T+1], nondecreasing, track_offsets[0] = 0,
                                     track_offsets[T] = S                                */
    const int32_t *seg_region;    /* [S] region of each segment, in [0, R)               */
    const uint8_t *seg_interval;  /* [S] fine axial interval, in [0, I)                  */
    const float *seg_ds;          /* [S] segment length, >= 0                            */
    const float *sigT;            /* [R][group_stride] total cross section, > 0          */
    const float *source;          /* [R][I][group_stride] fine source                    */
    float *fine_flux;             /* [R][I][group_stride] tallies are ADDED here         */
    float *psi;                   /* [T][group_stride] in: incoming, out: outgoing flux  */
} moc_problem_t;

typedef struct {
    moc_exp_mode_t exp_mode;
    int32_t table_points;         /* N of the table (reference: 353), >= 2              */
    float table_max;              /* maxVal of the table (reference: 10.0f)              */
    moc_precision_t precision;
    moc_tally_t tally;
    /* Placeholder constants of src/cpu/kernel.c:99-103 (defaults are the reference's). */
    float dz, zin, weight, mu, mu2;
    int32_t checked;              /* 1: bounds-check every segment first (an extra pass)
                                     and return MOC_ERR_BAD_INDEX without touching
                                     fine_flux or psi (that return is the report:
                                     moc_synchronize has nothing left to report)          */
    int32_t vec;                  /* groups per lane: 0 = auto, else 1, 2 or 4          */
    int32_t warps_per_block;      /* 0 = auto (8; 16 in table mode), else 1..16          */
    int32_t profile;              /* 1: time each kernel of the call with CUDA events on
                                     the call's stream (read with moc_last_timings)      */
    int32_t prefetch;             /* how far ahead of the arithmetic segments' cell blocks
                                     are fetched: 0 = auto, 1 = one segment, in registers;
                                     2..16 = a ring of that many slots per warp in shared
                                     memory, filled by bulk copies (the TMA engine), so
                                     prefetch - 1 segments are in flight (FP32 storage with
                                     FP32 tallies: MOC_PREC_FP32, MOC_PREC_FP32_STABLE)  */
    int32_t track_chunk;          /* long tracks sweep in parallel chunks: a track of more
                                     than 4 * C segments is cut into chunks of C segments,
                                     joined through the affine form of the psi recursion.
                                     -1 = never cut; C in 32 .. 2^24 = that C (a track's
                                     psi then depends only on its own segments and C);
                                     0 = auto: C from the problem's size, so that no
                                     whole track takes more than about a quarter of the
                                     sweep (a power of two, >= 32). The no-allocation
                                     entry point never cuts tracks                         */
    int32_t reserved[1];
} moc_fwd_opts_t;

/* Device time of each kernel of the last call made with opts.profile = 1. */
typedef struct {
    float prep_ms;                /* axial-coefficient pass                              */
    float sweep_ms;               /* the sweep kernel                                    */
    float finish_ms;              /* tally finishing pass (0 when the form has none)     */
    int32_t launches;             /* kernels the call launched                           */
    float split_ms;               /* long-track split passes (records, chunk maps, chunk
                                     starts) of the forward sweep; 0 when none ran        */
} moc_timings_t;

/* Reference defaults: FULL exp, N=353 / maxVal=10 table, FP32, atomic tallies,
 * dz=0.1 zin=0.3 weight=0.5 mu=0.9 mu2=0.3. */
void moc_fwd_opts_default(moc_fwd_opts_t *opts);

/* Create a handle on CUDA device `device` (it becomes current for the handle's calls). */
moc_status_t moc_create(moc_handle_t *handle, int device);
/* Destroy a handle and free its workspace (synchronises its device). NULL is a no-op. */
moc_status_t moc_destroy(moc_handle_t handle);

/*
 * Attenuate every segment of every track, in track order, on device buffers.
 * For each track t and each segment j of it (in CSR order) and each group g:
 *   fine_flux[region_j][interval_j][g] += weight * flux_integral(psi[t][g])
 *   psi[t][g] = attenuated psi                       (src/cpu/kernel.c:111-332)
 * Asynchronous on `stream`; returns after enqueueing (checked mode waits for the
 * index check). The handle's workspace (axial coefficients, table) is reused by
 * later calls, so calls on one handle must not overlap on different streams.
 */
moc_status_t moc_attenuate_fwd(moc_handle_t handle, const moc_problem_t *problem,
                               const moc_fwd_opts_t *opts, void *stream);

/*
 * Compact segment descriptors: 6 bytes per segment instead of 9 (the on-disk compact track
 * format's payload, include/moc_trackfile.h). No counterpart in the reference, whose
 * segments are random draws (src/cpu/kernel.c:47-50).
 */
typedef struct {
    const uint32_t *seg_cell;     /* [S] region * n_intervals + interval, < R * I        */
    const uint16_t *seg_ds_half;  /* [S] segment length as IEEE half bits (>= 0)         */
} moc_compact_segments_t;

/*
 * moc_attenuate_fwd on compact descriptors: the problem's seg_region, seg_interval and
 * seg_ds are not used (they may be NULL); every segment's cell and half length come from
 * `segments` (device memory, 4- and 2-byte aligned). The sweep widens each length to FP32
 * exactly, so its results are moc_attenuate_fwd's on those widened lengths. Every form,
 * exp mode and option of moc_attenuate_fwd applies; cells out of range are skipped and
 * reported as there (or refused up front with opts->checked).
 */
moc_status_t moc_attenuate_fwd_compact(moc_handle_t handle, const moc_problem_t *problem,
                                       const moc_compact_segments_t *segments,
                                       const moc_fwd_opts_t *opts, void *stream);

/*
 * Same sweep, with every pointer of `problem` in HOST memory; returns when the host
 * arrays hold the results. This is the drop-in for a host program that calls
 * run_kernel(I, S, table) on host arrays (src/cpu/main.c:46). Page-locked arrays mapped
 * into the device's address space (cudaHostAlloc, cudaHostRegister, pinned torch tensors)
 * are used in place: the sweep reads the offsets, descriptors and psi over the host link
 * and writes psi back there; sigT and source are copied up first; the tallies are
 * reduced on the device and added into fine_flux in place (a fine_flux that is not
 * mapped is copied up before the sweep and back after it). Other host arrays, and every
 * array in checked mode, are copied to device memory held by the handle (large problems
 * in a pipeline of parts) and the results copied back. Page-locked memory is not
 * required.
 */
moc_status_t moc_attenuate_fwd_host(moc_handle_t handle, const moc_problem_t *problem,
                                    const moc_fwd_opts_t *opts);

/*
 * Batching form: sweep several problems (different group counts, tracks of very uneven
 * length) in ONE persistent kernel launch. No single counterpart in the reference (its
 * run_kernel, src/cpu/kernel.c:3-73, sweeps one problem); each problem is swept as
 * moc_attenuate_fwd sweeps it (plain form, either exp mode; opts is shared). Long tracks
 * are cut into chunks as opts.track_chunk says, with one chunk length for the whole
 * batch (opts.track_chunk = 0: from the batch's total work; -1: never cut), so a problem's
 * psi equals moc_attenuate_fwd's with that chunk length. Tracks (or chunk records) are
 * bucket-sorted by length on the device and consumed longest first from one work queue;
 * problems whose G does not fill a warp are swept by sub-warps carrying several tracks
 * each. The first call for a given set of problems (pointers and sizes)
 * and options captures the whole sequence into a CUDA graph on the handle; later calls
 * with the same set replay it with one cudaGraphLaunch on `stream`. At most
 * MOC_BATCH_MAX_PROBLEMS problems, and at most 16 group ranges in total (a problem needs
 * ceil(G / (32 * groups-per-lane)) of them). Groups per lane and warps per block come
 * from opts->vec / opts->warps_per_block, else from moc_autotune_batch's result for this
 * set, else 2 and 8.
 */
#define MOC_BATCH_MAX_PROBLEMS 8
moc_status_t moc_attenuate_fwd_batch(moc_handle_t handle, const moc_problem_t *problems,
                                     int32_t n_problems, const moc_fwd_opts_t *opts,
                                     void *stream);

/* Result of moc_autotune_batch. */
#define MOC_TUNE_MAX_CANDIDATES 48
typedef struct {
    int32_t vec;                  /* chosen groups per lane (1, 2 or 4)                  */
    int32_t warps_per_block;      /* chosen warps per block (1..16)                      */
    int32_t tracks_per_block;     /* tracks a block carries at once in a full-warp chunk
                                     (one track per warp): warps_per_block                */
    float best_ms;                /* device time of one batched sweep with that choice   */
    int32_t n_candidates;
    int32_t candidate_vec[MOC_TUNE_MAX_CANDIDATES];
    int32_t candidate_warps[MOC_TUNE_MAX_CANDIDATES];
    float candidate_ms[MOC_TUNE_MAX_CANDIDATES];
} moc_tune_result_t;

/*
 * Autotuner of the batching form: times every (groups per lane in {1, 2, 4}) x
 * (tracks per block in {1, ..., 16}) on the given problems - a block of W warps carries W
 * tracks at once in every full-warp group chunk (and 32/L times more in a remainder chunk
 * swept by sub-warps of L lanes) - keeps the fastest for this set of problems in the
 * handle (used by later moc_attenuate_fwd_batch calls whose opts leave vec /
 * warps_per_block at 0), and reports all candidates. psi and fine_flux of the problems
 * are saved before the trials and restored after them, so the call leaves them
 * unchanged. Synchronous.
 */
moc_status_t moc_autotune_batch(moc_handle_t handle, const moc_problem_t *problems,
                                int32_t n_problems, const moc_fwd_opts_t *opts, void *stream,
                                moc_tune_result_t *result);

/*
 * Reverse-mode derivative of the sweep. No counterpart in the reference (which has no
 * derivative): for
 *     L = sum_{cells, g} w[c][g] * fine_flux_out[c][g] + sum_{tracks, g} v[t][g] * psi_out[t][g]
 * with w = dL_dfine_flux ([R][I][group_stride]) and v = dL_dpsi_out ([T][group_stride]),
 * writes dL/dsigT ([R][group_stride]), dL/dsource ([R][I][group_stride]) and dL/dpsi_in
 * ([T][group_stride]) for the inputs in `problem` (problem->psi is the INCOMING psi and is
 * only read; problem->fine_flux is not used). Padding entries of the outputs are not
 * written. The derivative is that of the exact attenuation formula; exponentials are
 * recomputed in the reverse sweep, and psi entering each segment is recorded by a first
 * forward pass in handle workspace (4 * n_segments * group_stride bytes). opts->exp_mode
 * must be MOC_EXP_FULL (the table is not differentiable); precision and tally options
 * are ignored. Asynchronous on `stream`.
 */
moc_status_t moc_attenuate_adj(moc_handle_t handle, const moc_problem_t *problem,
                               const moc_fwd_opts_t *opts, const float *dL_dfine_flux,
                               const float *dL_dpsi_out, float *dL_dsigT, float *dL_dsource,
                               float *dL_dpsi_in, void *stream);

/*
 * moc_attenuate_fwd without allocating. No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc — a transport code whose own pool allocator holds
 * the GPU's memory and forbids further allocations, a sweep loop that cannot take the
 * device-wide synchronisation cudaMalloc/cudaFree may cause while other streams run,
 * or a stateless call site with nowhere to keep a handle.
 *
 * Same sweep, same kernels and same results as moc_attenuate_fwd (plain form,
 * opts->precision = MOC_PREC_FP32, either exp mode, opts->prefetch 0 or 1; other
 * precisions and the bulk-copy ring return MOC_ERR_UNSUPPORTED), on the current CUDA
 * device, asynchronous on `stream`. Its scratch is one fixed array in the library's
 * device image (every GPU that loads the library holds it, about 10.2 MiB, until the
 * process exits); nothing is allocated per call: no cudaMalloc, cudaFree or allocating
 * library routine. Limits: n_regions * n_intervals * group_stride <=
 * MOC_NOALLOC_MAX_CELL_GROUPS (16 bytes of scratch each) and, in table mode,
 * table_points <= MOC_NOALLOC_MAX_TABLE_POINTS; larger problems return
 * MOC_ERR_TOO_LARGE.
 *
 * The first call on each device looks up the array's device address (once, with that
 * device current) and keeps it for the life of the process: after cudaDeviceReset of a device (which unloads the
 * library's device image there) this entry point must not be called on that device
 * again. Every call shares the one array, and it keeps the last call's contents: calls
 * whose kernels overlap on the GPU race on it, so order them on one stream. Every array
 * of `problem` must be memory of the current device (or managed memory), else
 * MOC_ERR_INVALID_ARG.
 *
 * Bad input: with opts->checked = 1 the call validates every offset and index first,
 * waits for that check on `stream` (cudaStreamSynchronize), and returns
 * MOC_ERR_BAD_INDEX without touching psi or fine_flux. With opts->checked = 0 the
 * kernels skip out-of-range segments and tracks whose offsets leave [0, S] without
 * reporting them: this entry point has no handle whose error word a later call could
 * read, so callers that need the report pass checked = 1. In table mode the table is
 * built in a static host buffer and copied from it on `stream`; the next call rewrites
 * that buffer.
 */
#define MOC_NOALLOC_MAX_CELL_GROUPS 655360 /* 10 MiB of cell blocks */
#define MOC_NOALLOC_MAX_TABLE_POINTS 24000
moc_status_t moc_attenuate_fwd_noalloc(const moc_problem_t *problem,
                                       const moc_fwd_opts_t *opts, void *stream);

/*
 * Wait for `stream`, then report and clear the device-side error word of the handle:
 * MOC_ERR_BAD_INDEX if any sweep since the last call met a segment whose region or
 * interval was out of range, or a track whose offsets were not inside [0, S]. Such a
 * segment or track is skipped by the sweep (nothing is read or written through its
 * indices); the rest of the sweep completes. MOC_ERR_BAD_TRACK (first) if a
 * moc_trace_segments call since then met an invalid track record or one whose segment
 * count disagreed with the offsets (include/moc_tracks.h). MOC_ERR_DEVICE_TIMEOUT (next)
 * if a sweep with a bulk-copy ring (opts.prefetch > 1) gave up waiting for a copy (each
 * warp waits about a second at most): its results are incomplete.
 */
moc_status_t moc_synchronize(moc_handle_t handle, void *stream);

/*
 * Build the reference's exponential table on the host (src/cpu/init.c:81-117) for a
 * given point count N: dx = maxVal / N, values[2n] = -exp(-n dx),
 * values[2n+1] = 1 + (n dx - 1) exp(-n dx), and the lookup bound maxVal - dx.
 * values has room for 2N floats. The reference picks N from a precision
 * (N = (int)(maxVal * sqrt(1 / (8 * precision * 0.01))), 353 for 0.01 / 10.0).
 */
moc_status_t moc_build_exp_table(int32_t n_points, float max_val, float *values,
                                 float *dx, float *lookup_max);

/* Wait for the events of the last profiled call and report its kernel times. Returns
 * MOC_ERR_INVALID_ARG if no profiled call was made on this handle. */
moc_status_t moc_last_timings(moc_handle_t handle, moc_timings_t *timings);

/* Static description of a status code. */
const char *moc_status_string(moc_status_t status);
/* Text of the last CUDA error recorded by this handle ("" if none). */
const char *moc_last_error(moc_handle_t handle);
/* MOC_ABI_VERSION of the loaded library. */
int32_t moc_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MOC_ATTENUATE_H */
