// moc_internal.h — kernels and launchers behind the C ABI (not part of the ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "moc_attenuate.h"
#include "moc_tracks.h"
#include "moc_transport.h"

// Two groups' FP32 arithmetic per packed .f32x2 instruction where a lane of the sweep holds
// an even number of groups (bit-identical to the one-group form; -DMOC_PAIRED_FP32=0
// builds the one-group form everywhere).
#ifndef MOC_PAIRED_FP32
#define MOC_PAIRED_FP32 1
#endif

namespace moc {

constexpr bool PAIRED_FP32 = MOC_PAIRED_FP32 != 0;
// The sweep with `vec` groups per lane reads FP32 cell blocks in the pair layout (below).
constexpr bool f32_pairs(int vec) { return PAIRED_FP32 && vec % 2 == 0; }

// The size / enum / alignment checks of moc_attenuate_fwd, and its check that every
// problem pointer is memory of device `dev` (or managed memory).
moc_status_t check_args(const moc_problem_t *p, const moc_fwd_opts_t *o);
bool all_device_accessible(const moc_problem_t *p, int dev);

// Streaming multiprocessors of the current device (queried once per device), for the
// grid sizes of the grid-stride kernels: at most sm_count * per_sm blocks.
int current_sm_count();
inline int64_t grid_cap(int per_sm) { return (int64_t)current_sm_count() * per_sm; }

// Device error bits, OR-ed into the handle's error word by the kernels.
enum : int32_t {
    DEVERR_OFFSETS = 1,  // a track's [begin, end) is not inside [0, S]
    DEVERR_INDEX = 2,    // a segment's region or interval is out of range
    DEVERR_TRACK = 4,    // track generation: a track record is invalid
    DEVERR_TIMEOUT = 8,  // a bounded wait on a bulk copy gave up (the sweep stopped)
};

// SM clocks a warp waits for one bulk copy before it reports DEVERR_TIMEOUT and stops:
// about a second at GB300 clocks, far beyond any copy's latency.
constexpr long long BULK_WAIT_LIMIT = 2000000000LL;

// How 1 - exp(-tau) and the cancelling terms are evaluated.
enum ExpKind : int {
    EXPK_PLAIN = 0,   // 1 - ex2(-tau log2 e); the reference's expressions (drop-in)
    EXPK_TABLE = 1,   // the reference's table, bit-exact lookup
    EXPK_STABLE = 2,  // Taylor branches for small tau, range-reduced ex2 elsewhere
};

// Storage of the cell blocks (sigT, q0, q1*mu, q2*mu2).
enum StoreKind : int {
    STORE_F32 = 0,   // float4 per (cell, group)
    STORE_BF16 = 1,  // four bf16 per (cell, group), widened to FP32 on load
    STORE_F16 = 2,   // four fp16 per (cell, group)
};

// Accumulation of the fine_flux tallies.
enum TallyKind : int {
    TALLY_F32 = 0,   // red.global.add.v4.f32 into fine_flux
    TALLY_COMP = 1,  // atomics into fine_flux + error-free-transform remainders into lo
    TALLY_F64 = 2,   // red.global.add.f64 into a double accumulator
};

// Long tracks are cut into chunks that sweep in parallel (moc_split.cu). A chunk record
// is an int4 {beg (low 32 bits), beg (high 32 bits), len | flags, track}.
enum : int32_t {
    CHUNK_LEN_MASK = 0x0fffffff,
    CHUNK_SINGLE = 1 << 30,  // the whole track: psi read and written in place
    CHUNK_LAST = 1 << 29,    // a split track's last chunk: writes the track's psi
    CHUNK_FIRST = 1 << 28,   // a split track's first chunk
};
constexpr int SPLIT_MIN_FACTOR = 4;       // tracks longer than 4 chunks are split
constexpr int SPLIT_CHUNK_MAX = 1 << 24;

// Everything a sweep launch reads. Device pointers.
struct SweepParams {
    int32_t R, I, G, Gs, T, n_chunks;
    int32_t group_major;          // item order: 1 group chunk by group chunk, 0 track by track
    int32_t null_cell;            // R*I when blk has the null-cell row after the cells, else -1
    int32_t ring_d;               // bulk-copy ring: slots per warp (RD_BULK loop)
    int64_t S, n_items;
    const int64_t *off;
    const int32_t *reg;
    const uint8_t *itv;
    const float *ds;
    // compact descriptors (moc_attenuate_fwd_compact), in place of reg / itv / ds when
    // cell is set: cell = region * I + interval, ds as IEEE half bits
    const uint32_t *cell;
    const uint16_t *ds16;
    const void *blk;     // [R*I][Gs]: (sigT, q0, q1*mu, q2*mu2) per cell and group,
                         // float4 or four 16-bit values (StoreKind)
    float *ff;           // [R*I][Gs]
    float *lo;           // [R*I][Gs] compensation remainders (TALLY_COMP)
    double *ff64;        // [R*I][Gs] double accumulator (TALLY_F64)
    float *psi;          // [T][Gs]
    float weight;
    const float *table;  // [2*tab_n] (slope, intercept) pairs, EXPK_TABLE only
    int32_t tab_n;
    float tab_dx, tab_max;
    int32_t *err;
    unsigned long long *counter;  // work-queue head, zeroed before each launch
    // split mode (rec != null): work items are (chunk record, group chunk)
    const int4 *rec;              // chunk records, in track order
    const int64_t *n_rec;         // number of records (device)
    const int64_t *map_list;      // record ids of the non-last chunks (map items)
    const int64_t *n_map;         // their number (device)
    int64_t rec_cap;              // records the buffers hold (items beyond are not run)
    float *start;                 // [records][Gs] psi entering each chunk of a split track
    float *map_a, *map_b;         // [records][Gs] psi_out = a psi_in + b of non-last chunks
};

// Split workspace (device) and the chunk length.
struct SplitWork {
    int64_t *base;    // [T + 1] first record of each track; base[T] = records
    int64_t *bsum;    // [2 * ceil(T / 1024)] scan block sums (records, maps)
    int4 *rec;        // [cap]
    int64_t *map_list;  // [cap] record ids of non-last chunks
    int64_t *n_map;     // number of map items
    int64_t cap;      // split_max_records(); offsets that are not a partition of [0, S]
                      // can ask for more: those records are dropped and reported
    int32_t chunk;
    int32_t map_all;  // 0: the map list holds the non-last chunks (forward); 1: every
                      // chunk of a split track (adjoint)
};
// Upper bound on the records of a problem (tracks + S / chunk).
int64_t split_max_records(int64_t T, int64_t S, int chunk);
// Records of every track (scan of the chunk counts, then the records; 3 launches).
cudaError_t launch_split_records(const SweepParams &P, const SplitWork &W, cudaStream_t st);
// psi entering every chunk of the split tracks from the maps: start_0 = psi_in,
// start_{k+1} = a_k start_k + b_k.
cudaError_t launch_split_start(const SweepParams &P, const SplitWork &W, int sm_count,
                               cudaStream_t st);

// Cell blocks of every (region, interval) and group: blk[c][g] = (sigT of the region,
// q0, q1*mu, q2*mu2), the coefficients rounded exactly as src/cpu/kernel.c:111-191 and
// the first product of kernel.c:250-251 / 311-322 round them.
// null_row: also write the null cell (1, 0, 0, 0) per group after the last cell (blk
// then holds R*I + 1 rows).
// pairs: the pair layout, in which groups 2h and 2h+1 of a cell share two float4,
// (sigT_2h, sigT_2h+1, q0_2h, q0_2h+1) and (q1mu_2h, q1mu_2h+1, q2mu2_2h, q2mu2_2h+1), so
// that a lane's loads land every pair of operands of the packed arithmetic in adjacent
// registers (Gs is a multiple of 4, so pairs never straddle cells).
// strided = VEC > 1 (with pairs): the lane-strided layout of the bulk-copy ring, in which
// each 32*VEC-group chunk of a row (n float4, n/VEC lanes) holds lane l's k-th float4 of
// the pair layout at k*(n/VEC) + l, so that a warp's lanes read a slot copied from it
// with conflict-free 16-byte shared loads.
cudaError_t launch_prep_block(const float *sigT, const float *source, float4 *blk, int R,
                              int I, int Gs, float dz, float zin, float mu, float mu2,
                              cudaStream_t st, bool null_row = false, bool pairs = false,
                              int strided = 0);
// The same blocks rounded to bf16 (store = STORE_BF16) or fp16 (STORE_F16), to nearest.
cudaError_t launch_prep_block16(const float *sigT, const float *source, void *blk, int store,
                                int R, int I, int Gs, float dz, float zin, float mu,
                                float mu2, cudaStream_t st, bool null_row = false);
// fine_flux[k] = (float)((double)fine_flux[k] + lo[k]) (or + ff64[k]) over n entries.
cudaError_t launch_finish(float *ff, const float *lo, const double *ff64, int64_t n,
                          cudaStream_t st);

// The forward sweep (persistent, one warp per (track, group chunk) work item).
constexpr int RING_MAX = 16;      // most slots of a warp's bulk-copy ring
constexpr int DESC_RING_F4 = 32;  // a warp's 64 (cell, ds) descriptor pairs
struct FwdConfig {
    int vec;              // groups per lane: 1, 2, 4
    int warps_per_block;  // 1..16
    int exp_kind;         // ExpKind
    int blocks;           // grid size (0 = fill the GPU)
    int store = STORE_F32;
    int tally = TALLY_F32;
    int prefetch = 1;     // 1: registers, one segment ahead; 2..RING_MAX: a ring of that
                          // many slots in shared memory per warp, filled by bulk copies
                          // (FP32 blocks in the lane-strided layout, FP32 tallies)
    int mode = 0;         // 0: the sweep; 1: affine maps of split chunks (split mode)
    bool branch_free = false;  // the null-cell row exists and G is a multiple of vec
};
// The bulk-copy ring reads FP32 cell blocks in the lane-strided layout (launch_prep_block
// with strided = vec).
inline bool fwd_bulk(const FwdConfig &c) { return c.prefetch > 1; }
cudaError_t launch_fwd(const SweepParams &p, const FwdConfig &cfg, cudaStream_t st);
// Dynamic shared memory of a configuration (table of tab_n pairs in table mode + rings).
size_t fwd_smem_bytes(const FwdConfig &cfg, int tab_n);
// Default groups per lane for G groups (measured fastest at G = 64 and 128 on GB300:
// two groups per lane keeps registers low enough for 32 resident warps per SM).
inline int auto_vec(int G) { return G > 32 ? 2 : 1; }
// Default warps per block: 8, or 16 in table mode, where each block stages the table in
// shared memory (80 KB at 10,000 points): two blocks of 16 warps keep 32 warps per SM.
inline int auto_warps_per_block(int exp_kind) { return exp_kind == EXPK_TABLE ? 16 : 8; }
// Resident blocks per SM for a configuration (0 if the configuration is invalid).
int fwd_blocks_per_sm(const FwdConfig &cfg, int tab_n);

// Checked mode: scan offsets and segment indices, OR errors into p.err. No writes
// to psi or fine_flux.
cudaError_t launch_check(const SweepParams &p, cudaStream_t st);

// ------------------------------------------------------------------------------------
// Batching form (moc_batch.cu).
// ------------------------------------------------------------------------------------
constexpr int BATCH_BUCKETS = 128;   // log-scale track-length buckets, longest first
constexpr int BATCH_MAX_PROB = 8;
constexpr int BATCH_MAX_SUB = 16;

struct BatchProb {                   // one problem (device pointers)
    const int64_t *off;
    const int32_t *reg;
    const uint8_t *itv;
    const float *ds;
    const float4 *blk;               // its cell blocks (FP32)
    float *ff;
    float *psi;
    int32_t R, I, G, Gs, T, perm_off;  // perm_off: start of its sorted unit list
    int64_t S;
    // long tracks cut into chunks (rec != null): the units are chunk records (as in the
    // single-problem sweep), rec_cap of them at most, n_rec on the device; a chunk of a
    // cut track starts from start[record] and only a track's last chunk writes its psi
    const int4 *rec;
    const int64_t *n_rec;
    const float *start;
    int64_t rec_cap;
};
struct BatchSub {                    // one group range of one problem
    int32_t prob, g_begin, g_count, lpt;  // lpt: lanes per track (power of two <= 32)
    int64_t item_base;               // first global item id; items = ceil(T / (32/lpt))
};
struct BatchParams {
    BatchProb prob[BATCH_MAX_PROB];
    BatchSub sub[BATCH_MAX_SUB];
    int32_t n_prob, n_sub;
    int64_t n_items;
    float weight;
    const float *table;
    int32_t tab_n;
    float tab_dx, tab_max;
    int32_t *err;
    unsigned long long *counter;
};
struct BatchWork {                   // device workspace of the queue construction
    int *hist;                       // [(n_prob + 1) * BATCH_BUCKETS]
    int *perm;                       // [sum T] sorted track ids
    int2 *queue;                     // [n_items] (sub-problem, first sorted position)
};
// Queue construction + the persistent sweep (vec in {1, 2, 4}; ek EXPK_PLAIN/TABLE).
cudaError_t launch_batch(const BatchParams &B, const BatchWork &W, int vec, int ek,
                         int warps_per_block, int blocks, cudaStream_t st);
int batch_blocks_per_sm(int vec, int ek, int warps_per_block, size_t smem);

// ------------------------------------------------------------------------------------
// Adjoint (moc_adjoint.cu).
// ------------------------------------------------------------------------------------
struct AdjParams {
    SweepParams fw;          // geometry, descriptors, cell blocks (FP32), psi = psi_in,
                             // weight, err, counter; ff unused
    float *hist;             // [S][Gs] psi entering each segment (workspace)
    const float *w;          // [R*I][Gs] dL/dfine_flux
    const float *v;          // [T][Gs]   dL/dpsi_out
    float4 *gblk;            // [R*I][Gs] (dL/dsigT, dL/da0, dL/da1, dL/da2) per cell
    float *dpsi_in;          // [T][Gs]   dL/dpsi_in (out)
    // split tracks (fw.rec != null): fw.start / fw.map_a / fw.map_b as the forward's, and
    float *map_c;            // [records][Gs] lambda_in = a lambda_out + c of each chunk
    float *lam_end;          // [records][Gs] lambda leaving each chunk
    const int64_t *base;     // [T + 1] first record of each track
};
// Forward pass that records psi entering every segment, then the reverse sweep that
// scatters the cell-block gradients; vec in {1, 2, 4}.
cudaError_t launch_adj_forward(const AdjParams &p, int vec, int blocks, cudaStream_t st);
cudaError_t launch_adj_reverse(const AdjParams &p, int vec, int blocks, cudaStream_t st);
int adj_blocks_per_sm(int vec, bool reverse);
// Split tracks: (a, b, c) of every chunk of a split track (the map list, fw.counter is the
// queue head), then psi entering and lambda leaving every chunk.
cudaError_t launch_adj_maps(const AdjParams &p, int vec, int blocks, cudaStream_t st);
cudaError_t launch_adj_starts(const AdjParams &p, cudaStream_t st);
int adj_map_blocks_per_sm(int vec);
// dL/dsigT[r][g] = sum over intervals of the sigT gradients; dL/dsource through the
// transpose of the axial fit (jac[type][k][m]: d q_k / d y_{i+m-1}, type 0 = first
// interval, 1 = interior, 2 = last), q1 = a1 / mu and q2 = a2 / mu2.
// vec: the reverse pass's groups per lane, which sets the gradient blocks' slots.
cudaError_t launch_adj_finish(const float4 *gblk, float *d_sigT, float *d_source, int R, int I,
                              int G, int Gs, const float *jac27, float mu, float mu2, int vec,
                              cudaStream_t st);

// Track generation (moc_trace.cu). Scratch of a scan over T entries:
// trace_scan_scratch(T) int64. Bound: per-track upper bounds of the segment counts,
// scanned into bnd[0 .. T] (the scratch layout). Walk: every track once into its scratch
// slot, counts scanned into off[0 .. T]. Compact: scratch to the caller's arrays. Emit: a
// second walk straight into the caller's arrays at off. Bad records set DEVERR_TRACK.
bool trace_geometry_ok(const moc_geometry_t *g);
int64_t trace_scan_scratch(int64_t n_tracks);
cudaError_t launch_trace_bound(const moc_geometry_t *g, const moc_track_t *tr, int64_t T,
                               int64_t *bnd, int64_t *scratch, int32_t *err, cudaStream_t st);
// Tables of the walk (grid lines, pin centres, fine planes): trace_table_len(g) doubles.
int64_t trace_table_len(const moc_geometry_t *g);
cudaError_t launch_trace_tables(const moc_geometry_t *g, double *tab, cudaStream_t st);
cudaError_t launch_trace_walk(const moc_geometry_t *g, const double *tab, const moc_track_t *tr,
                              int64_t T, const int64_t *bnd, int64_t *off, int64_t *scratch,
                              int32_t *sreg, uint8_t *sitv, float *sds, int32_t *err,
                              cudaStream_t st);
cudaError_t launch_trace_compact(const moc_track_t *tr, int64_t T, const int64_t *bnd,
                                 const int64_t *off, const int32_t *sreg, const uint8_t *sitv,
                                 const float *sds, int32_t *reg, uint8_t *itv, float *ds,
                                 cudaStream_t st);
cudaError_t launch_trace_emit(const moc_geometry_t *g, const double *tab, const moc_track_t *tr,
                              int64_t T, const int64_t *off, int32_t *reg, uint8_t *itv,
                              float *ds, int32_t *err, cudaStream_t st);

// Source update (moc_transport.cu). rk = (float)(1 / k), rpi = (float)(1 / (4 pi)).
struct TransportParams {
    int64_t ncell;  // R * I fine cells
    int M, G, Gs, I;
    const float *scatter, *nu_fission, *chi;
    float rk, rpi;
};
cudaError_t launch_region_sigT(const moc_xs_t *xs, const int32_t *material, int64_t R,
                               float *sigT, int32_t *err, cudaStream_t st);
cudaError_t launch_source_update(const TransportParams &P, const int32_t *material,
                                 const double *volume, const float *tally, float *source,
                                 double *fission, int32_t *err, cudaStream_t st);

}  // namespace moc
