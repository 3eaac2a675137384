// moc_api.cu — the C ABI (include/moc_attenuate.h): handles, argument checks, workspace,
// and the launch sequence of one forward sweep.
#include "moc_attenuate.h"
#include "moc_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

struct moc_handle_s {
    int device = 0;
    int sm_count = 0;
    size_t l2_bytes = 0;
    // workspace (device)
    float4 *blk = nullptr;     // cell blocks (sigT, q0, q1*mu, q2*mu2), FP32 or 16-bit
    size_t blk_cap = 0;        // bytes
    float *lo = nullptr;       // compensated-tally remainders
    size_t lo_cap = 0;
    double *ff64 = nullptr;    // FP64 tally accumulator
    size_t ff64_cap = 0;
    float4 *gblk = nullptr;    // adjoint: cell-block gradients
    size_t gblk_cap = 0;
    float *hist = nullptr;     // adjoint: psi entering every segment
    size_t hist_cap = 0;
    // long-track split: per-track record base, scan sums, records, starts and maps
    int64_t *sbase = nullptr, *sbsum = nullptr;
    size_t sbase_cap = 0, sbsum_cap = 0;
    int4 *srec = nullptr;
    size_t srec_cap = 0;
    int64_t *smlist = nullptr;   // map list; smlist[cap] holds the map count
    size_t smlist_cap = 0;
    float *sstart = nullptr, *smap = nullptr;
    size_t sstart_cap = 0, smap_cap = 0;
    float *sadj = nullptr;       // adjoint: lambda maps and lambda leaving each chunk
    size_t sadj_cap = 0;
    // batching form
    float4 *bblk = nullptr;    // cell blocks of all problems of a batch
    size_t bblk_cap = 0;
    int *bhist = nullptr, *bperm = nullptr;
    size_t bhist_cap = 0, bperm_cap = 0;
    int2 *bqueue = nullptr;
    size_t bqueue_cap = 0;
    float *bsave = nullptr;    // autotuner: saved psi and fine_flux
    unsigned char *bsplit = nullptr;  // batch: split workspace of every problem
    size_t bsplit_cap = 0;
    // batch: one side stream per problem for its cell-block and split passes, forked from
    // and joined back into the batch's stream (parallel branches of the captured graph)
    cudaStream_t bside[MOC_BATCH_MAX_PROBLEMS] = {};
    cudaEvent_t bfork = nullptr, bjoin[MOC_BATCH_MAX_PROBLEMS] = {};
    size_t bsave_cap = 0;
    cudaStream_t gstream = nullptr;        // capture stream of the batch graph
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey;       // what the captured graph was built for
    std::vector<unsigned char> tune_key;   // problem set the tuned choice belongs to
    int tune_vec = 0, tune_wpb = 0;
    float *table = nullptr;
    int32_t table_n = 0;
    float table_maxval = 0.0f, table_dx = 0.0f, table_lookup = 0.0f;
    // track generation: scan tile sums, per-track bound offsets, and the scratch that
    // moc_trace_count walks into (with the arguments of that call, for
    // moc_trace_segments to recognise it)
    int64_t *tscan = nullptr, *tbnd = nullptr;
    size_t tscan_cap = 0, tbnd_cap = 0;
    double *ttab = nullptr;              // the walk's tables of the geometry
    size_t ttab_cap = 0;
    double *fis = nullptr;               // power iteration: the fission total
    size_t fis_cap = 0;
    int32_t *treg = nullptr;
    uint8_t *titv = nullptr;
    float *tds = nullptr;
    size_t treg_cap = 0, titv_cap = 0, tds_cap = 0;
    bool tvalid = false;
    const void *ttracks = nullptr;
    const int64_t *toff = nullptr;
    int64_t tT = 0;
    moc_geometry_t tgeo{};
    int32_t *err = nullptr;              // device error word
    unsigned long long *counter = nullptr;
    int32_t *err_host = nullptr;         // pinned mirror
    // device copies for the host-buffer entry point
    void *hbuf[9] = {};        // [8]: the caller's fine_flux, added after the pipelined sweep
    size_t hcap[9] = {};
    cudaStream_t hstream = nullptr;
    // its pipeline: copies in, sweeps (hstream) and copies out overlap part by part
    cudaStream_t hin = nullptr, hout = nullptr, hcomp2 = nullptr;
    cudaEvent_t hev_tab = nullptr, hev_prep = nullptr, hev_in[8] = {}, hev_done[8] = {};
    // kernel timing of the last profiled call
    cudaEvent_t ev[5] = {};   // start, after prep, after sweep, after finish, after split
    int timed_launches = 0;   // 0: no profiled call yet
    bool timed_finish = false;
    bool timed_split = false;
    std::string last_error;
};

namespace {

moc_status_t cuda_fail(moc_handle_t h, cudaError_t e, const char *what)
{
    if (h) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        h->last_error = buf;
    }
    return e == cudaErrorMemoryAllocation ? MOC_ERR_OUT_OF_MEMORY : MOC_ERR_CUDA;
}

#define MOC_CUDA(h, call)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
    } while (0)

bool aligned(const void *p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

// Size, enum and alignment checks shared by the device and host entry points.
moc_status_t check_problem(const moc_problem_t *p, const moc_fwd_opts_t *o)
{
    if (!p || !o) return MOC_ERR_INVALID_ARG;
    if (p->n_regions < 1 || p->n_intervals < 2 || p->n_intervals > 255 || p->n_groups < 1 ||
        p->group_stride < p->n_groups || p->n_tracks < 0 || p->n_segments < 0)
        return MOC_ERR_INVALID_ARG;
    if (p->group_stride % 4 != 0) return MOC_ERR_UNSUPPORTED;
    // cell * group_stride + group is formed in 32-bit arithmetic by the sweep, for every
    // cell and the null cell after them
    if (((int64_t)p->n_regions * p->n_intervals + 1) * p->group_stride > INT32_MAX)
        return MOC_ERR_UNSUPPORTED;
    if (!p->track_offsets || !p->sigT || !p->source || !p->fine_flux) return MOC_ERR_INVALID_ARG;
    if (p->n_tracks > 0 && !p->psi) return MOC_ERR_INVALID_ARG;
    if (p->n_segments > 0 && (!p->seg_region || !p->seg_interval || !p->seg_ds))
        return MOC_ERR_INVALID_ARG;
    if (!aligned(p->sigT, 16) || !aligned(p->source, 16) || !aligned(p->fine_flux, 16) ||
        (p->psi && !aligned(p->psi, 16)) || !aligned(p->track_offsets, 8) ||
        (p->seg_region && !aligned(p->seg_region, 4)) || (p->seg_ds && !aligned(p->seg_ds, 4)))
        return MOC_ERR_MISALIGNED;
    if (o->exp_mode != MOC_EXP_FULL && o->exp_mode != MOC_EXP_TABLE) return MOC_ERR_INVALID_ARG;
    if (o->precision != MOC_PREC_FP32 && o->precision != MOC_PREC_BF16 &&
        o->precision != MOC_PREC_FP16 && o->precision != MOC_PREC_FP32_STABLE)
        return MOC_ERR_INVALID_ARG;
    if (o->tally != MOC_TALLY_ATOMIC_FP32 && o->tally != MOC_TALLY_COMPENSATED &&
        o->tally != MOC_TALLY_FP64)
        return MOC_ERR_INVALID_ARG;
    if (o->exp_mode == MOC_EXP_TABLE &&
        (o->table_points < 2 || o->table_points > 24000 || !(o->table_max > 0.0f)))
        return MOC_ERR_INVALID_ARG;
    if (o->vec != 0 && o->vec != 1 && o->vec != 2 && o->vec != 4) return MOC_ERR_INVALID_ARG;
    if (o->warps_per_block < 0 || o->warps_per_block > 16) return MOC_ERR_INVALID_ARG;
    if (o->prefetch < 0 || o->prefetch > moc::RING_MAX) return MOC_ERR_INVALID_ARG;
    if (o->track_chunk != 0 && o->track_chunk != -1 &&
        (o->track_chunk < 32 || o->track_chunk > moc::SPLIT_CHUNK_MAX))
        return MOC_ERR_INVALID_ARG;
    // the bulk-copy ring: FP32 cell blocks and FP32 tallies
    if (o->prefetch > 1 &&
        (o->precision == MOC_PREC_BF16 || o->precision == MOC_PREC_FP16 ||
         o->tally != MOC_TALLY_ATOMIC_FP32))
        return MOC_ERR_UNSUPPORTED;
    if (!std::isfinite(o->dz) || o->dz == 0.0f) return MOC_ERR_INVALID_ARG;
    // The precision forms use the accurate exponential; the table is the plain form's.
    if (o->exp_mode == MOC_EXP_TABLE && o->precision != MOC_PREC_FP32)
        return MOC_ERR_UNSUPPORTED;
    if (o->precision == MOC_PREC_FP32 && o->tally != MOC_TALLY_ATOMIC_FP32)
        return MOC_ERR_UNSUPPORTED;
    return MOC_OK;
}

// Device pointers must be memory of device `dev` or managed memory: a sweep on one device
// does not read or write another device's memory (it may have no peer access to it).
bool device_accessible(const void *p, int dev)
{
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

moc_status_t ensure(moc_handle_t h, void **buf, size_t *cap, size_t bytes)
{
    if (bytes <= *cap) return MOC_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    MOC_CUDA(h, cudaMalloc(buf, bytes));
    *cap = bytes;
    return MOC_OK;
}

moc_status_t ensure_table(moc_handle_t h, const moc_fwd_opts_t *o, cudaStream_t st)
{
    if (h->table && h->table_n == o->table_points && h->table_maxval == o->table_max)
        return MOC_OK;
    const size_t n = 2 * (size_t)o->table_points;
    float *host = new (std::nothrow) float[n];
    if (!host) return MOC_ERR_OUT_OF_MEMORY;
    float dx = 0, lk = 0;
    moc_build_exp_table(o->table_points, o->table_max, host, &dx, &lk);
    if (h->table) cudaFree(h->table);
    h->table = nullptr;
    h->table_n = 0;
    cudaError_t e = cudaMalloc(&h->table, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->table, host, n * sizeof(float),
                                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    delete[] host;
    if (e != cudaSuccess) return cuda_fail(h, e, "exp table upload");
    h->table_n = o->table_points;
    h->table_maxval = o->table_max;
    h->table_dx = dx;
    h->table_lookup = lk;
    return MOC_OK;
}

// Automatic chunk length. A lone warp takes about 260 ns per segment of its item, and the
// whole GPU runs about 9e9 warp-segment steps per second (GB300, 32 resident warps per
// SM): the sweep of S segments x n_gch group chunks takes S n_gch / 9e9 s. Tracks whose
// lone time would exceed a quarter of that, L* = S n_gch / 9360 segments, are cut into
// chunks of L* / 4 (rounded to a power of two, at least 32).
int auto_chunk_steps(double warp_steps)
{
    const double target = warp_steps / 9360.0 / moc::SPLIT_MIN_FACTOR;
    int c = 32;
    while (c < moc::SPLIT_CHUNK_MAX && c * 1.41421356 < target) c *= 2;
    return c;
}

// A problem's chunk length is also raised towards a sixteenth of its mean track length (in
// powers of two) while the chunks still number at least 8192 work items, about the resident
// warps of the GPU: cutting tracks of about the mean length into more pieces adds records,
// maps and start-scan steps and balances nothing (1M segments in 1,000 equal tracks:
// 32-segment chunks 0.218 ms per step, 64-segment 0.200), while a problem of a few long
// tracks keeps the short chunks that spread it over the GPU.
int auto_chunk(int64_t S, int64_t n_gch, int64_t T)
{
    int c = auto_chunk_steps((double)S * (double)n_gch);
    const double mean16 = T > 0 ? (double)S / (double)T / 16.0 : 0.0;
    const double most = (double)S * (double)n_gch / 8192.0;
    while (c < moc::SPLIT_CHUNK_MAX && c < mean16 && 2.0 * c <= most) c *= 2;
    return c;
}

// Whether long tracks are split (opts.track_chunk, and S long enough for any track to be
// cut), and if so the split workspace, wired into *sp. The workspace holds at most
// split_max_records records (below 2^31, record ids are stored in 32-bit fields); offsets
// that ask for more have the excess dropped and reported. n_gch: group chunks per track.
moc_status_t split_setup(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                         int map_all, int64_t n_gch, moc::SweepParams *sp, moc::SplitWork *sw,
                         bool *split)
{
    const int chunk =
        o->track_chunk == 0 ? auto_chunk(p->n_segments, n_gch, p->n_tracks) : o->track_chunk;
    *split = o->track_chunk != -1 && p->n_tracks > 0 &&
             p->n_segments > (int64_t)moc::SPLIT_MIN_FACTOR * chunk &&
             moc::split_max_records(p->n_tracks, p->n_segments, chunk) < INT32_MAX;
    if (!*split) return MOC_OK;
    moc_status_t s;
    const int64_t T = p->n_tracks, Gs = p->group_stride;
    const int64_t cap = moc::split_max_records(T, p->n_segments, chunk);
    const int64_t nb = (T + 1023) / 1024;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->sbase), &h->sbase_cap,
                    (size_t)(T + 1) * sizeof(int64_t))) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->sbsum), &h->sbsum_cap,
                    2 * (size_t)nb * sizeof(int64_t))) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->srec), &h->srec_cap,
                    (size_t)cap * sizeof(int4))) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->smlist), &h->smlist_cap,
                    (size_t)(cap + 1) * sizeof(int64_t))) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->sstart), &h->sstart_cap,
                    (size_t)cap * Gs * sizeof(float))) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->smap), &h->smap_cap,
                    2 * (size_t)cap * Gs * sizeof(float))))
        return s;
    sw->base = h->sbase;
    sw->bsum = h->sbsum;
    sw->rec = h->srec;
    sw->map_list = h->smlist;
    sw->n_map = h->smlist + cap;
    sw->cap = cap;
    sw->chunk = chunk;
    sw->map_all = map_all;
    sp->rec = h->srec;
    sp->n_rec = h->sbase + T;
    sp->map_list = sw->map_list;
    sp->n_map = sw->n_map;
    sp->rec_cap = cap;
    sp->start = h->sstart;
    sp->map_a = h->smap;
    sp->map_b = h->smap + cap * Gs;
    return MOC_OK;
}

// Launch configuration: groups per lane from G unless given, grid filling the GPU.
moc_status_t pick_config(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                         moc::FwdConfig *c)
{
    int vec = o->vec;
    if (vec == 0) vec = moc::auto_vec(p->n_groups);
    c->vec = vec;
    c->exp_kind = o->exp_mode == MOC_EXP_TABLE ? moc::EXPK_TABLE : moc::EXPK_PLAIN;
    c->warps_per_block =
        o->warps_per_block ? o->warps_per_block : moc::auto_warps_per_block(c->exp_kind);
    c->store = moc::STORE_F32;
    c->tally = moc::TALLY_F32;
    if (o->precision != MOC_PREC_FP32) {
        c->exp_kind = moc::EXPK_STABLE;
        c->store = o->precision == MOC_PREC_BF16   ? moc::STORE_BF16
                   : o->precision == MOC_PREC_FP16 ? moc::STORE_F16
                                                   : moc::STORE_F32;
        c->tally = o->tally == MOC_TALLY_COMPENSATED ? moc::TALLY_COMP
                   : o->tally == MOC_TALLY_FP64      ? moc::TALLY_F64
                                                     : moc::TALLY_F32;
    }
    c->prefetch = o->prefetch > 1 ? o->prefetch : 1;
    // the bulk-copy ring reads the lane-strided layout of the pair layout (or of one
    // group per lane)
    if (moc::fwd_bulk(*c) && vec > 1 && !moc::f32_pairs(vec)) return MOC_ERR_UNSUPPORTED;
    // the branch-free segment loop needs whole rows per lane (and the null-cell row,
    // which fwd_device writes after the cell blocks)
    c->branch_free = p->n_groups % vec == 0;
    const int per_sm = moc::fwd_blocks_per_sm(*c, o->table_points);
    if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
    c->blocks = per_sm * h->sm_count;
    return MOC_OK;
}

// The forward sweep of one problem on device buffers. prep = false: the cell blocks of
// this problem's tables are already in h->blk (a later part of a pipelined call).
// compact: the segments as 32-bit cells and half lengths (moc_attenuate_fwd_compact) in
// place of the problem's three descriptor arrays.
moc_status_t fwd_device(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                        cudaStream_t st, bool prep = true,
                        unsigned long long *counter = nullptr,
                        const moc_compact_segments_t *compact = nullptr)
{
    // queue heads: [0] the sweep's, [1] the map pass's (a pipelined call gives every other
    // part its own pair so that parts on two streams can overlap)
    unsigned long long *ctr = counter ? counter : h->counter;
    moc_status_t s;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    // cell blocks and the null-cell row after them
    const size_t blk_bytes = (size_t)(ncell + 1) * p->group_stride * sizeof(float4);
    if ((s = ensure(h, reinterpret_cast<void **>(&h->blk), &h->blk_cap, blk_bytes))) return s;
    if (o->exp_mode == MOC_EXP_TABLE && (s = ensure_table(h, o, st))) return s;

    moc::SweepParams sp{};
    sp.R = p->n_regions;
    sp.I = p->n_intervals;
    sp.G = p->n_groups;
    sp.Gs = p->group_stride;
    sp.T = p->n_tracks;
    sp.S = p->n_segments;
    sp.off = p->track_offsets;
    sp.reg = p->seg_region;
    sp.itv = p->seg_interval;
    sp.ds = p->seg_ds;
    if (compact) {
        sp.cell = compact->seg_cell;
        sp.ds16 = compact->seg_ds_half;
    }
    sp.blk = h->blk;
    sp.ff = p->fine_flux;
    sp.psi = p->psi;
    sp.weight = o->weight;
    sp.table = h->table;
    sp.tab_n = h->table_n;
    sp.tab_dx = h->table_dx;
    sp.tab_max = h->table_lookup;
    sp.err = h->err;
    sp.counter = ctr;

    if (o->checked) {
        MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));
        MOC_CUDA(h, moc::launch_check(sp, st));
        MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, st));
        MOC_CUDA(h, cudaStreamSynchronize(st));
        if (*h->err_host) {
            MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));  // reported here
            return MOC_ERR_BAD_INDEX;
        }
    }
    if (p->n_tracks == 0) return MOC_OK;

    moc::FwdConfig cfg;
    if ((s = pick_config(h, p, o, &cfg))) return s;
    sp.n_chunks = (p->n_groups + 32 * cfg.vec - 1) / (32 * cfg.vec);
    sp.group_major = 1;
    sp.null_cell = (int32_t)ncell;
    sp.n_items = (int64_t)p->n_tracks * sp.n_chunks;

    const size_t nff = (size_t)ncell * p->group_stride;
    if (cfg.tally == moc::TALLY_COMP) {
        if ((s = ensure(h, reinterpret_cast<void **>(&h->lo), &h->lo_cap, nff * sizeof(float))))
            return s;
        sp.lo = h->lo;
    } else if (cfg.tally == moc::TALLY_F64) {
        if ((s = ensure(h, reinterpret_cast<void **>(&h->ff64), &h->ff64_cap,
                        nff * sizeof(double))))
            return s;
        sp.ff64 = h->ff64;
    }

    // Long tracks: chunk records, the maps of non-last chunks, the chunk starts.
    moc::SplitWork sw{};
    bool split = false;
    if ((s = split_setup(h, p, o, 0, sp.n_chunks, &sp, &sw, &split))) return s;
    moc::FwdConfig mcfg = cfg;
    if (split) {
        mcfg.mode = 1;  // the same loop and block layout as the sweep
        mcfg.tally = moc::TALLY_F32;
        const int per_sm = moc::fwd_blocks_per_sm(mcfg, o->table_points);
        if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
        mcfg.blocks = per_sm * h->sm_count;
    }

    const bool prof = o->profile != 0;
    if (prof && !h->ev[0])
        for (auto &e : h->ev) MOC_CUDA(h, cudaEventCreate(&e));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[0], st));
    if (prep && cfg.store == moc::STORE_F32)
        MOC_CUDA(h, moc::launch_prep_block(p->sigT, p->source, h->blk, p->n_regions,
                                           p->n_intervals, p->group_stride, o->dz, o->zin,
                                           o->mu, o->mu2, st, true, moc::f32_pairs(cfg.vec),
                                           moc::fwd_bulk(cfg) ? cfg.vec : 0));
    else if (prep)
        MOC_CUDA(h, moc::launch_prep_block16(p->sigT, p->source, h->blk, cfg.store,
                                             p->n_regions, p->n_intervals, p->group_stride,
                                             o->dz, o->zin, o->mu, o->mu2, st, true));
    if (sp.lo) MOC_CUDA(h, cudaMemsetAsync(sp.lo, 0, nff * sizeof(float), st));
    if (sp.ff64) MOC_CUDA(h, cudaMemsetAsync(sp.ff64, 0, nff * sizeof(double), st));
    // counter[0]: the sweep's queue head, counter[1]: the map pass's
    MOC_CUDA(h, cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned long long), st));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[1], st));
    if (split) {
        MOC_CUDA(h, moc::launch_split_records(sp, sw, st));
        moc::SweepParams mp = sp;
        mp.counter = ctr + 1;
        MOC_CUDA(h, moc::launch_fwd(mp, mcfg, st));
        MOC_CUDA(h, moc::launch_split_start(sp, sw, h->sm_count, st));
    }
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[4], st));
    MOC_CUDA(h, moc::launch_fwd(sp, cfg, st));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[2], st));
    const bool finish = sp.lo || sp.ff64;
    if (finish) MOC_CUDA(h, moc::launch_finish(p->fine_flux, sp.lo, sp.ff64, (int64_t)nff, st));
    if (prof) {
        if (finish) MOC_CUDA(h, cudaEventRecord(h->ev[3], st));
        h->timed_launches = (finish ? 3 : 2) + (split ? 5 : 0) - (prep ? 0 : 1);
        h->timed_finish = finish;
        h->timed_split = split;
    }
    return MOC_OK;
}

// ------------------------------------------------------------------------------------
// Batching form
// ------------------------------------------------------------------------------------
moc_status_t check_batch(moc_handle_t h, const moc_problem_t *probs, int32_t n,
                         const moc_fwd_opts_t *o)
{
    if (!h || !probs || !o || n < 1 || n > MOC_BATCH_MAX_PROBLEMS) return MOC_ERR_INVALID_ARG;
    if (o->precision != MOC_PREC_FP32) return MOC_ERR_UNSUPPORTED;  // the plain form
    for (int32_t k = 0; k < n; k++) {
        moc_status_t s = check_problem(&probs[k], o);
        if (s) return s;
        if (!moc::all_device_accessible(&probs[k], h->device)) return MOC_ERR_INVALID_ARG;
    }
    return MOC_OK;
}

void append(std::vector<unsigned char> &key, const void *p, size_t n)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    key.insert(key.end(), b, b + n);
}

// The problem set and the options that shape the computation.
std::vector<unsigned char> set_key(const moc_problem_t *probs, int32_t n, const moc_fwd_opts_t *o)
{
    std::vector<unsigned char> key;
    append(key, probs, sizeof(moc_problem_t) * (size_t)n);
    const float f[7] = {o->table_max, o->dz, o->zin, o->weight, o->mu, o->mu2, 0.0f};
    const int32_t i[3] = {(int32_t)o->exp_mode, o->table_points, o->track_chunk};
    append(key, f, sizeof(f));
    append(key, i, sizeof(i));
    return key;
}

// Long-track split of each problem of a batch: its records, maps and starts are made by
// the single-problem passes before the batched sweep, which then takes chunk records as
// its units.
struct BatchSplit {
    bool on[MOC_BATCH_MAX_PROBLEMS] = {};
    moc::SweepParams sp[MOC_BATCH_MAX_PROBLEMS];
    moc::SplitWork sw[MOC_BATCH_MAX_PROBLEMS];
    moc::FwdConfig mcfg[MOC_BATCH_MAX_PROBLEMS];
};

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Lay out sub-problems, workspace and launch parameters for one (vec, wpb) choice.
moc_status_t build_batch(moc_handle_t h, const moc_problem_t *probs, int32_t n,
                         const moc_fwd_opts_t *o, int vec, int wpb, moc::BatchParams &B,
                         moc::BatchWork &W, BatchSplit &X, int &blocks)
{
    moc_status_t s;
    std::memset(&B, 0, sizeof(B));
    X = BatchSplit{};
    // chunk length: from the whole batch's warp-segment steps (a problem's group range
    // runs as ceil(G / 32 vec) warp-wide parts, or one sub-warp part for small G)
    const int gw = 32 * vec;
    double steps = 0.0;
    for (int32_t k = 0; k < n; k++) {
        const int full = probs[k].n_groups / gw, rest = probs[k].n_groups % gw;
        double per_track = full;
        if (rest) {
            int lpt = 1;
            while (lpt < (rest + vec - 1) / vec) lpt *= 2;
            per_track += (double)lpt / 32.0;
        }
        steps += (double)probs[k].n_segments * per_track;
    }
    const int chunk_len = o->track_chunk == 0 ? auto_chunk_steps(steps) : o->track_chunk;
    size_t blk_total = 0, perm_total = 0, split_bytes = 0;
    int64_t cap[MOC_BATCH_MAX_PROBLEMS] = {};
    for (int32_t k = 0; k < n; k++) {
        const moc_problem_t &p = probs[k];
        // each problem's cell blocks and its null-cell row
        blk_total += ((size_t)p.n_regions * p.n_intervals + 1) * p.group_stride;
        X.on[k] = o->track_chunk != -1 && p.n_tracks > 0 &&
                  p.n_segments > (int64_t)moc::SPLIT_MIN_FACTOR * chunk_len &&
                  moc::split_max_records(p.n_tracks, p.n_segments, chunk_len) < INT32_MAX;
        cap[k] = X.on[k] ? moc::split_max_records(p.n_tracks, p.n_segments, chunk_len) : 0;
        perm_total += X.on[k] ? (size_t)cap[k] : (size_t)p.n_tracks;
        if (X.on[k]) {
            const size_t T = p.n_tracks, Gs = p.group_stride, c = cap[k];
            split_bytes += align_up((T + 1) * 8) + align_up((T + 1023) / 1024 * 16) +
                           align_up(c * 16) + align_up((c + 1) * 8) + 3 * align_up(c * Gs * 4);
        }
    }
    if ((s = ensure(h, reinterpret_cast<void **>(&h->bblk), &h->bblk_cap,
                    (blk_total ? blk_total : 1) * sizeof(float4))))
        return s;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->bperm), &h->bperm_cap,
                    (perm_total ? perm_total : 1) * sizeof(int))))
        return s;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->bhist), &h->bhist_cap,
                    sizeof(int) * moc::BATCH_BUCKETS * (MOC_BATCH_MAX_PROBLEMS + 1))))
        return s;
    if (split_bytes && (s = ensure(h, reinterpret_cast<void **>(&h->bsplit), &h->bsplit_cap,
                                   split_bytes)))
        return s;
    if (o->exp_mode == MOC_EXP_TABLE) {
        if ((s = ensure_table(h, o, h->hstream))) return s;
        B.table = h->table;
        B.tab_n = h->table_n;
        B.tab_dx = h->table_dx;
        B.tab_max = h->table_lookup;
    }
    size_t boff = 0, soff = 0;
    int perm_off = 0, nsub = 0;
    int64_t items = 0;
    for (int32_t k = 0; k < n; k++) {
        const moc_problem_t &p = probs[k];
        moc::BatchProb &bp = B.prob[k];
        bp.off = p.track_offsets;
        bp.reg = p.seg_region;
        bp.itv = p.seg_interval;
        bp.ds = p.seg_ds;
        bp.blk = h->bblk + boff;
        bp.ff = p.fine_flux;
        bp.psi = p.psi;
        bp.R = p.n_regions;
        bp.I = p.n_intervals;
        bp.G = p.n_groups;
        bp.Gs = p.group_stride;
        bp.T = p.n_tracks;
        bp.S = p.n_segments;
        bp.perm_off = perm_off;
        const int64_t ncell = (int64_t)p.n_regions * p.n_intervals;
        boff += (size_t)(ncell + 1) * p.group_stride;
        int64_t units = p.n_tracks;
        if (X.on[k]) {
            // the problem's split workspace and the parameters of its split passes
            const size_t T = p.n_tracks, Gs = p.group_stride, c = cap[k];
            unsigned char *base = h->bsplit + soff;
            moc::SplitWork &sw = X.sw[k];
            sw.base = reinterpret_cast<int64_t *>(base);
            base += align_up((T + 1) * 8);
            sw.bsum = reinterpret_cast<int64_t *>(base);
            base += align_up((T + 1023) / 1024 * 16);
            sw.rec = reinterpret_cast<int4 *>(base);
            base += align_up(c * 16);
            sw.map_list = reinterpret_cast<int64_t *>(base);
            sw.n_map = sw.map_list + c;
            base += align_up((c + 1) * 8);
            float *start = reinterpret_cast<float *>(base);
            base += align_up(c * Gs * 4);
            float *map_a = reinterpret_cast<float *>(base);
            base += align_up(c * Gs * 4);
            float *map_b = reinterpret_cast<float *>(base);
            base += align_up(c * Gs * 4);
            soff = (size_t)(base - h->bsplit);
            sw.cap = (int64_t)c;
            sw.chunk = chunk_len;
            sw.map_all = 0;
            moc::SweepParams &sp = X.sp[k];
            sp = moc::SweepParams{};
            sp.R = p.n_regions;
            sp.I = p.n_intervals;
            sp.G = p.n_groups;
            sp.Gs = p.group_stride;
            sp.T = p.n_tracks;
            sp.S = p.n_segments;
            sp.off = p.track_offsets;
            sp.reg = p.seg_region;
            sp.itv = p.seg_interval;
            sp.ds = p.seg_ds;
            sp.blk = bp.blk;
            sp.null_cell = (int32_t)ncell;
            sp.group_major = 1;
            sp.psi = p.psi;
            sp.weight = o->weight;
            sp.table = B.table;
            sp.tab_n = B.tab_n;
            sp.tab_dx = B.tab_dx;
            sp.tab_max = B.tab_max;
            sp.err = h->err;
            sp.counter = h->counter + 1;  // unused by the map pass (static assignment)
            sp.rec = sw.rec;
            sp.n_rec = sw.base + T;
            sp.map_list = sw.map_list;
            sp.n_map = sw.n_map;
            sp.rec_cap = (int64_t)c;
            sp.start = start;
            sp.map_a = map_a;
            sp.map_b = map_b;
            moc::FwdConfig &mc = X.mcfg[k];
            mc.vec = vec;  // the batch's groups per lane: its cell-block layout
            mc.warps_per_block = 8;
            mc.exp_kind = o->exp_mode == MOC_EXP_TABLE ? moc::EXPK_TABLE : moc::EXPK_PLAIN;
            mc.mode = 1;
            mc.prefetch = 1;
            mc.branch_free = p.n_groups % mc.vec == 0;
            sp.n_chunks = (p.n_groups + 32 * mc.vec - 1) / (32 * mc.vec);
            const int per_sm = moc::fwd_blocks_per_sm(mc, o->table_points);
            if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
            mc.blocks = per_sm * h->sm_count;
            bp.rec = sw.rec;
            bp.n_rec = sw.base + T;
            bp.start = start;
            bp.rec_cap = (int64_t)c;
            units = (int64_t)c;
        }
        perm_off += (int)units;
        // full chunks of 32*vec groups, then the remainder on narrower sub-warps
        for (int g = 0; g < p.n_groups; g += gw) {
            const int count = p.n_groups - g < gw ? p.n_groups - g : gw;
            const int lanes = (count + vec - 1) / vec;
            int lpt = 1;
            while (lpt < lanes) lpt *= 2;
            if (nsub >= moc::BATCH_MAX_SUB) return MOC_ERR_UNSUPPORTED;
            moc::BatchSub &sb = B.sub[nsub++];
            sb.prob = k;
            sb.g_begin = g;
            sb.g_count = count;
            sb.lpt = lpt;
            sb.item_base = items;
            const int per_warp = 32 / lpt;
            items += (units + per_warp - 1) / per_warp;
        }
    }
    B.n_prob = n;
    B.n_sub = nsub;
    B.n_items = items;
    B.weight = o->weight;
    B.err = h->err;
    B.counter = h->counter;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->bqueue), &h->bqueue_cap,
                    (size_t)(items ? items : 1) * sizeof(int2))))
        return s;
    W.hist = h->bhist;
    W.perm = h->bperm;
    W.queue = h->bqueue;
    const int ek = o->exp_mode == MOC_EXP_TABLE ? moc::EXPK_TABLE : moc::EXPK_PLAIN;
    const size_t smem = ek == moc::EXPK_TABLE ? (size_t)o->table_points * 8 : 0;
    const int per_sm = moc::batch_blocks_per_sm(vec, ek, wpb, smem);
    if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
    blocks = per_sm * h->sm_count;
    return MOC_OK;
}

// Enqueue one batched sweep: the coefficient pass of every problem, then the queue and
// the sweep.
moc_status_t enqueue_batch(moc_handle_t h, const moc_problem_t *probs, int32_t n,
                           const moc_fwd_opts_t *o, const moc::BatchParams &B,
                           const moc::BatchWork &W, const BatchSplit &X, int vec, int wpb,
                           int blocks, cudaStream_t st)
{
    // Per problem, on its own side stream: the cell blocks, then (long tracks) its
    // records, chunk maps and chunk starts. The problems' passes are independent, and a
    // map pass over a few long chunks is latency-bound, so they run side by side.
    if (!h->bfork) MOC_CUDA(h, cudaEventCreateWithFlags(&h->bfork, cudaEventDisableTiming));
    for (int32_t k = 0; k < n; k++) {
        if (!h->bside[k])
            MOC_CUDA(h, cudaStreamCreateWithFlags(&h->bside[k], cudaStreamNonBlocking));
        if (!h->bjoin[k])
            MOC_CUDA(h, cudaEventCreateWithFlags(&h->bjoin[k], cudaEventDisableTiming));
    }
    MOC_CUDA(h, cudaEventRecord(h->bfork, st));
    for (int32_t k = 0; k < n; k++) {
        cudaStream_t sk = h->bside[k];
        MOC_CUDA(h, cudaStreamWaitEvent(sk, h->bfork, 0));
        MOC_CUDA(h, moc::launch_prep_block(probs[k].sigT, probs[k].source,
                                           const_cast<float4 *>(B.prob[k].blk),
                                           probs[k].n_regions, probs[k].n_intervals,
                                           probs[k].group_stride, o->dz, o->zin, o->mu, o->mu2,
                                           sk, true, moc::f32_pairs(vec)));
        if (X.on[k]) {
            MOC_CUDA(h, moc::launch_split_records(X.sp[k], X.sw[k], sk));
            MOC_CUDA(h, moc::launch_fwd(X.sp[k], X.mcfg[k], sk));
            MOC_CUDA(h, moc::launch_split_start(X.sp[k], X.sw[k], h->sm_count, sk));
        }
        MOC_CUDA(h, cudaEventRecord(h->bjoin[k], sk));
        MOC_CUDA(h, cudaStreamWaitEvent(st, h->bjoin[k], 0));
    }
    if (B.n_items == 0) return MOC_OK;
    const int ek = o->exp_mode == MOC_EXP_TABLE ? moc::EXPK_TABLE : moc::EXPK_PLAIN;
    MOC_CUDA(h, moc::launch_batch(B, W, vec, ek, wpb, blocks, st));
    return MOC_OK;
}

// The cell blocks (and the null-cell row) of a problem's tables, in the storage of its
// precision form.
moc_status_t prep_blocks(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                         cudaStream_t st)
{
    moc_status_t s;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    const size_t blk_bytes = (size_t)(ncell + 1) * p->group_stride * sizeof(float4);
    if ((s = ensure(h, reinterpret_cast<void **>(&h->blk), &h->blk_cap, blk_bytes))) return s;
    if (o->exp_mode == MOC_EXP_TABLE && (s = ensure_table(h, o, st))) return s;
    // the layout the sweep's lanes read (its groups per lane and loop)
    moc::FwdConfig cfg;
    if ((s = pick_config(h, p, o, &cfg))) return s;
    if (cfg.store == moc::STORE_F32)
        MOC_CUDA(h, moc::launch_prep_block(p->sigT, p->source, h->blk, p->n_regions,
                                           p->n_intervals, p->group_stride, o->dz, o->zin,
                                           o->mu, o->mu2, st, true, moc::f32_pairs(cfg.vec),
                                           moc::fwd_bulk(cfg) ? cfg.vec : 0));
    else
        MOC_CUDA(h, moc::launch_prep_block16(p->sigT, p->source, h->blk, cfg.store,
                                             p->n_regions, p->n_intervals, p->group_stride,
                                             o->dz, o->zin, o->mu, o->mu2, st, true));
    return MOC_OK;
}

// Pipelined host-buffer sweep: the tables go up first; the tracks are then cut into
// `parts` contiguous ranges of about equal segment counts, and while part k sweeps on
// hstream, part k+1's descriptors and psi go up on hin and part k-1's psi comes back on
// hout. Parts share the cell blocks and add into the same fine_flux; the chunk length of
// long tracks is fixed from the whole problem, so psi is the one-call result bit for bit.
moc_status_t fwd_host_pipelined(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                                int parts, const int64_t *cut, int64_t longest)
{
    moc_status_t s;
    const int64_t T = p->n_tracks, S = p->n_segments, Gs = p->group_stride;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    if (!h->hin) MOC_CUDA(h, cudaStreamCreateWithFlags(&h->hin, cudaStreamNonBlocking));
    if (!h->hout) MOC_CUDA(h, cudaStreamCreateWithFlags(&h->hout, cudaStreamNonBlocking));
    if (!h->hcomp2) MOC_CUDA(h, cudaStreamCreateWithFlags(&h->hcomp2, cudaStreamNonBlocking));
    if (!h->hev_tab) MOC_CUDA(h, cudaEventCreateWithFlags(&h->hev_tab, cudaEventDisableTiming));
    if (!h->hev_prep)
        MOC_CUDA(h, cudaEventCreateWithFlags(&h->hev_prep, cudaEventDisableTiming));
    for (int k = 0; k < parts; k++) {
        if (!h->hev_in[k])
            MOC_CUDA(h, cudaEventCreateWithFlags(&h->hev_in[k], cudaEventDisableTiming));
        if (!h->hev_done[k])
            MOC_CUDA(h, cudaEventCreateWithFlags(&h->hev_done[k], cudaEventDisableTiming));
    }
    int64_t *d_off = static_cast<int64_t *>(h->hbuf[0]);
    int32_t *d_reg = static_cast<int32_t *>(h->hbuf[1]);
    uint8_t *d_itv = static_cast<uint8_t *>(h->hbuf[2]);
    float *d_ds = static_cast<float *>(h->hbuf[3]);
    float *d_sig = static_cast<float *>(h->hbuf[4]);
    float *d_src = static_cast<float *>(h->hbuf[5]);
    float *d_ff = static_cast<float *>(h->hbuf[6]);
    float *d_psi = static_cast<float *>(h->hbuf[7]);
    cudaStream_t cin = h->hin, comp = h->hstream, cout = h->hout;
    // tables, offsets and the tallies first
    MOC_CUDA(h, cudaMemcpyAsync(d_off, p->track_offsets, (size_t)(T + 1) * 8,
                                cudaMemcpyHostToDevice, cin));
    MOC_CUDA(h, cudaMemcpyAsync(d_sig, p->sigT, (size_t)p->n_regions * Gs * 4,
                                cudaMemcpyHostToDevice, cin));
    MOC_CUDA(h, cudaMemcpyAsync(d_src, p->source, (size_t)ncell * Gs * 4,
                                cudaMemcpyHostToDevice, cin));
    MOC_CUDA(h, cudaEventRecord(h->hev_tab, cin));
    // the parts add their tallies into zeros; the caller's fine_flux goes up last and is
    // added on the device before the copy back
    MOC_CUDA(h, cudaMemsetAsync(d_ff, 0, (size_t)ncell * Gs * 4, comp));
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), comp));
    MOC_CUDA(h, cudaStreamWaitEvent(comp, h->hev_tab, 0));
    moc_problem_t d = *p;
    d.track_offsets = d_off;
    d.seg_region = d_reg;
    d.seg_interval = d_itv;
    d.seg_ds = d_ds;
    d.sigT = d_sig;
    d.source = d_src;
    d.fine_flux = d_ff;
    d.psi = d_psi;
    moc_fwd_opts_t oo = *o;
    if (oo.track_chunk == 0) {
        const int vec = o->vec ? o->vec : moc::auto_vec(p->n_groups);
        oo.track_chunk = auto_chunk(S, (p->n_groups + 32 * vec - 1) / (32 * vec), T);
    }
    // no track long enough to be cut (the host has the offsets): the parts skip the split
    // passes, with the same result
    if (oo.track_chunk > 0 && longest <= (int64_t)moc::SPLIT_MIN_FACTOR * oo.track_chunk)
        oo.track_chunk = -1;
    // Without split passes the parts share only read-only cell blocks and atomic tallies:
    // consecutive parts alternate between two compute streams with their own queue heads,
    // so a part's blocks fill the SMs its predecessor's tail leaves idle. With split passes
    // (one split workspace) every part runs on one stream.
    const bool two = oo.track_chunk == -1;
    cudaStream_t cs[2] = {comp, two ? h->hcomp2 : comp};
    if ((s = prep_blocks(h, &d, &oo, comp))) return s;
    MOC_CUDA(h, cudaEventRecord(h->hev_prep, comp));
    if (two) MOC_CUDA(h, cudaStreamWaitEvent(cs[1], h->hev_prep, 0));
    for (int k = 0; k < parts; k++) {
        const int64_t t0 = cut[k], t1 = cut[k + 1];
        const int64_t s0 = p->track_offsets[t0], s1 = p->track_offsets[t1];
        if (s1 > s0) {
            MOC_CUDA(h, cudaMemcpyAsync(d_reg + s0, p->seg_region + s0, (size_t)(s1 - s0) * 4,
                                        cudaMemcpyHostToDevice, cin));
            MOC_CUDA(h, cudaMemcpyAsync(d_itv + s0, p->seg_interval + s0, (size_t)(s1 - s0),
                                        cudaMemcpyHostToDevice, cin));
            MOC_CUDA(h, cudaMemcpyAsync(d_ds + s0, p->seg_ds + s0, (size_t)(s1 - s0) * 4,
                                        cudaMemcpyHostToDevice, cin));
        }
        MOC_CUDA(h, cudaMemcpyAsync(d_psi + t0 * Gs, p->psi + t0 * Gs,
                                    (size_t)(t1 - t0) * Gs * 4, cudaMemcpyHostToDevice, cin));
        MOC_CUDA(h, cudaEventRecord(h->hev_in[k], cin));
        cudaStream_t ck = cs[k & 1];
        MOC_CUDA(h, cudaStreamWaitEvent(ck, h->hev_in[k], 0));
        // part k: its tracks, absolute segment offsets into the full descriptor arrays
        moc_problem_t part = d;
        part.track_offsets = d_off + t0;
        part.n_tracks = (int32_t)(t1 - t0);
        part.psi = d_psi + t0 * Gs;
        if ((s = fwd_device(h, &part, &oo, ck, false, h->counter + 2 * (k & 1)))) return s;
        MOC_CUDA(h, cudaEventRecord(h->hev_done[k], ck));
        MOC_CUDA(h, cudaStreamWaitEvent(cout, h->hev_done[k], 0));
        MOC_CUDA(h, cudaMemcpyAsync(p->psi + t0 * Gs, d_psi + t0 * Gs,
                                    (size_t)(t1 - t0) * Gs * 4, cudaMemcpyDeviceToHost, cout));
    }
    float *d_ff0 = static_cast<float *>(h->hbuf[8]);
    MOC_CUDA(h, cudaMemcpyAsync(d_ff0, p->fine_flux, (size_t)ncell * Gs * 4,
                                cudaMemcpyHostToDevice, cin));
    MOC_CUDA(h, cudaEventRecord(h->hev_tab, cin));
    MOC_CUDA(h, cudaStreamWaitEvent(comp, h->hev_tab, 0));
    if (two && parts > 1) {
        // the second stream's last part (the odd one nearest the end)
        const int last_odd = (parts - 1) % 2 == 1 ? parts - 1 : parts - 2;
        MOC_CUDA(h, cudaStreamWaitEvent(comp, h->hev_done[last_odd], 0));
    }
    MOC_CUDA(h, moc::launch_finish(d_ff, d_ff0, nullptr, ncell * Gs, comp));
    MOC_CUDA(h, cudaEventRecord(h->hev_done[0], comp));
    MOC_CUDA(h, cudaStreamWaitEvent(cout, h->hev_done[0], 0));
    MOC_CUDA(h, cudaMemcpyAsync(p->fine_flux, d_ff, (size_t)ncell * Gs * 4,
                                cudaMemcpyDeviceToHost, cout));
    MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                cout));
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), cout));  // reported here
    MOC_CUDA(h, cudaStreamSynchronize(cout));
    return *h->err_host ? MOC_ERR_BAD_INDEX : MOC_OK;
}

}  // namespace

// Argument checks shared with the other entry points (declared in moc_internal.h).
moc_status_t moc::check_args(const moc_problem_t *p, const moc_fwd_opts_t *o)
{
    return check_problem(p, o);
}

bool moc::all_device_accessible(const moc_problem_t *p, int dev)
{
    const void *ptrs[] = {p->track_offsets, p->seg_region, p->seg_interval, p->seg_ds,
                          p->sigT, p->source, p->fine_flux, p->psi};
    for (const void *q : ptrs)
        if (!device_accessible(q, dev)) return false;
    return true;
}

extern "C" {

void moc_fwd_opts_default(moc_fwd_opts_t *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->exp_mode = MOC_EXP_FULL;
    o->table_points = 353;
    o->table_max = 10.0f;
    o->precision = MOC_PREC_FP32;
    o->tally = MOC_TALLY_ATOMIC_FP32;
    o->dz = 0.1f;
    o->zin = 0.3f;
    o->weight = 0.5f;
    o->mu = 0.9f;
    o->mu2 = 0.3f;
}

moc_status_t moc_create(moc_handle_t *out, int device)
{
    if (!out) return MOC_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return MOC_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return MOC_ERR_NO_DEVICE;
    moc_handle_t h = new (std::nothrow) moc_handle_s;
    if (!h) return MOC_ERR_OUT_OF_MEMORY;
    h->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
    int l2 = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device);
    h->l2_bytes = (size_t)l2;
    if (e == cudaSuccess) e = cudaMalloc(&h->err, 64);
    if (e == cudaSuccess) e = cudaMemset(h->err, 0, 64);
    if (e == cudaSuccess) h->counter = reinterpret_cast<unsigned long long *>(
                              reinterpret_cast<char *>(h->err) + 8);
    if (e == cudaSuccess) e = cudaMallocHost(&h->err_host, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->hstream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        moc_destroy(h);
        return e == cudaErrorMemoryAllocation ? MOC_ERR_OUT_OF_MEMORY : MOC_ERR_CUDA;
    }
    *out = h;
    return MOC_OK;
}

moc_status_t moc_destroy(moc_handle_t h)
{
    if (!h) return MOC_OK;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    if (h->blk) cudaFree(h->blk);
    if (h->tscan) cudaFree(h->tscan);
    if (h->tbnd) cudaFree(h->tbnd);
    if (h->ttab) cudaFree(h->ttab);
    if (h->fis) cudaFree(h->fis);
    if (h->treg) cudaFree(h->treg);
    if (h->titv) cudaFree(h->titv);
    if (h->tds) cudaFree(h->tds);
    if (h->lo) cudaFree(h->lo);
    if (h->ff64) cudaFree(h->ff64);
    if (h->gblk) cudaFree(h->gblk);
    if (h->hist) cudaFree(h->hist);
    if (h->sbase) cudaFree(h->sbase);
    if (h->sbsum) cudaFree(h->sbsum);
    if (h->srec) cudaFree(h->srec);
    if (h->smlist) cudaFree(h->smlist);
    if (h->sadj) cudaFree(h->sadj);
    if (h->sstart) cudaFree(h->sstart);
    if (h->smap) cudaFree(h->smap);
    if (h->bblk) cudaFree(h->bblk);
    if (h->bhist) cudaFree(h->bhist);
    if (h->bperm) cudaFree(h->bperm);
    if (h->bqueue) cudaFree(h->bqueue);
    if (h->bsave) cudaFree(h->bsave);
    if (h->bsplit) cudaFree(h->bsplit);
    for (int k = 0; k < MOC_BATCH_MAX_PROBLEMS; k++) {
        if (h->bside[k]) cudaStreamDestroy(h->bside[k]);
        if (h->bjoin[k]) cudaEventDestroy(h->bjoin[k]);
    }
    if (h->bfork) cudaEventDestroy(h->bfork);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->gstream) cudaStreamDestroy(h->gstream);
    if (h->table) cudaFree(h->table);
    if (h->err) cudaFree(h->err);
    if (h->err_host) cudaFreeHost(h->err_host);
    for (int k = 0; k < 9; k++)
        if (h->hbuf[k]) cudaFree(h->hbuf[k]);
    if (h->hstream) cudaStreamDestroy(h->hstream);
    if (h->hin) cudaStreamDestroy(h->hin);
    if (h->hout) cudaStreamDestroy(h->hout);
    if (h->hcomp2) cudaStreamDestroy(h->hcomp2);
    if (h->hev_tab) cudaEventDestroy(h->hev_tab);
    if (h->hev_prep) cudaEventDestroy(h->hev_prep);
    for (int k = 0; k < 8; k++) {
        if (h->hev_in[k]) cudaEventDestroy(h->hev_in[k]);
        if (h->hev_done[k]) cudaEventDestroy(h->hev_done[k]);
    }
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    delete h;
    return MOC_OK;
}

moc_status_t moc_attenuate_fwd(moc_handle_t h, const moc_problem_t *p,
                               const moc_fwd_opts_t *o, void *stream)
{
    if (!h) return MOC_ERR_INVALID_ARG;
    moc_status_t s = check_problem(p, o);
    if (s) return s;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    const void *ptrs[] = {p->track_offsets, p->seg_region, p->seg_interval, p->seg_ds,
                          p->sigT, p->source, p->fine_flux, p->psi};
    for (const void *q : ptrs)
        if (!device_accessible(q, h->device)) return MOC_ERR_INVALID_ARG;
    return fwd_device(h, p, o, static_cast<cudaStream_t>(stream));
}

moc_status_t moc_attenuate_fwd_compact(moc_handle_t h, const moc_problem_t *p,
                                       const moc_compact_segments_t *c,
                                       const moc_fwd_opts_t *o, void *stream)
{
    if (!h || !p || !c) return MOC_ERR_INVALID_ARG;
    if (p->n_segments > 0 && (!c->seg_cell || !c->seg_ds_half)) return MOC_ERR_INVALID_ARG;
    if (!aligned(c->seg_cell, 4) || !aligned(c->seg_ds_half, 2)) return MOC_ERR_MISALIGNED;
    if ((int64_t)p->n_regions * p->n_intervals > (int64_t)UINT32_MAX) return MOC_ERR_INVALID_ARG;
    // the problem's own descriptor arrays are not used: check the rest with them standing
    // for the compact ones
    moc_problem_t q = *p;
    q.seg_region = reinterpret_cast<const int32_t *>(c->seg_cell);
    q.seg_interval = reinterpret_cast<const uint8_t *>(c->seg_cell);
    q.seg_ds = reinterpret_cast<const float *>(c->seg_cell);
    moc_status_t s = check_problem(&q, o);
    if (s) return s;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    const void *ptrs[] = {p->track_offsets, c->seg_cell, c->seg_ds_half, p->sigT, p->source,
                          p->fine_flux, p->psi};
    for (const void *x : ptrs)
        if (!device_accessible(x, h->device)) return MOC_ERR_INVALID_ARG;
    return fwd_device(h, &q, o, static_cast<cudaStream_t>(stream), true, nullptr, c);
}

moc_status_t moc_attenuate_fwd_batch(moc_handle_t h, const moc_problem_t *probs, int32_t n,
                                     const moc_fwd_opts_t *o, void *stream)
{
    moc_status_t s = check_batch(h, probs, n, o);
    if (s) return s;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<unsigned char> key = set_key(probs, n, o);
    int vec = o->vec, wpb = o->warps_per_block;
    if (!vec) vec = (h->tune_vec && key == h->tune_key) ? h->tune_vec : 2;
    if (!wpb) wpb = (h->tune_wpb && key == h->tune_key) ? h->tune_wpb : 8;
    moc::BatchParams B;
    moc::BatchWork W;
    BatchSplit X;
    int blocks = 0;
    if ((s = build_batch(h, probs, n, o, vec, wpb, B, W, X, blocks))) return s;
    // the graph is valid for this set, this workspace and this launch shape
    append(key, &B, sizeof(B));
    append(key, &W, sizeof(W));
    const int shape[3] = {vec, wpb, blocks};
    append(key, shape, sizeof(shape));
    if (!h->gexec || key != h->gkey) {
        if (h->gexec) cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
        h->gkey.clear();
        if (!h->gstream)
            MOC_CUDA(h, cudaStreamCreateWithFlags(&h->gstream, cudaStreamNonBlocking));
        MOC_CUDA(h, cudaStreamBeginCapture(h->gstream, cudaStreamCaptureModeRelaxed));
        s = enqueue_batch(h, probs, n, o, B, W, X, vec, wpb, blocks, h->gstream);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->gstream, &graph);
        if (s) {
            if (graph) cudaGraphDestroy(graph);
            return s;
        }
        if (e != cudaSuccess) return cuda_fail(h, e, "batch graph capture");
        const cudaError_t e2 = cudaGraphInstantiate(&h->gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (e2 != cudaSuccess) {
            h->gexec = nullptr;
            return cuda_fail(h, e2, "batch graph instantiate");
        }
        h->gkey = key;
    }
    const bool prof = o->profile != 0;
    if (prof && !h->ev[0])
        for (auto &e : h->ev) MOC_CUDA(h, cudaEventCreate(&e));
    if (prof) {
        MOC_CUDA(h, cudaEventRecord(h->ev[0], st));
        MOC_CUDA(h, cudaEventRecord(h->ev[1], st));
    }
    MOC_CUDA(h, cudaGraphLaunch(h->gexec, st));
    if (prof) {
        MOC_CUDA(h, cudaEventRecord(h->ev[2], st));
        int cut = 0;
        for (int32_t k = 0; k < n; k++) cut += X.on[k] ? 5 : 0;
        h->timed_launches = n + cut + (B.n_items ? 7 : 0);
        h->timed_finish = false;
        h->timed_split = false;
    }
    return MOC_OK;
}

moc_status_t moc_autotune_batch(moc_handle_t h, const moc_problem_t *probs, int32_t n,
                                const moc_fwd_opts_t *o, void *stream, moc_tune_result_t *res)
{
    moc_status_t s = check_batch(h, probs, n, o);
    if (s) return s;
    if (!res) return MOC_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // save psi and fine_flux of every problem; trials run on the real buffers
    size_t save = 0;
    for (int32_t k = 0; k < n; k++)
        save += (size_t)probs[k].group_stride *
                ((size_t)probs[k].n_tracks + (size_t)probs[k].n_regions * probs[k].n_intervals);
    if ((s = ensure(h, reinterpret_cast<void **>(&h->bsave), &h->bsave_cap,
                    (save ? save : 1) * sizeof(float))))
        return s;
    auto copy_all = [&](bool to_save) -> moc_status_t {
        size_t at = 0;
        for (int32_t k = 0; k < n; k++) {
            const size_t np = (size_t)probs[k].group_stride * probs[k].n_tracks;
            const size_t nf = (size_t)probs[k].group_stride * probs[k].n_regions *
                              probs[k].n_intervals;
            float *sp = h->bsave + at, *sf = h->bsave + at + np;
            if (np)
                MOC_CUDA(h, cudaMemcpyAsync(to_save ? sp : probs[k].psi,
                                            to_save ? probs[k].psi : sp, np * 4,
                                            cudaMemcpyDeviceToDevice, st));
            MOC_CUDA(h, cudaMemcpyAsync(to_save ? sf : probs[k].fine_flux,
                                        to_save ? probs[k].fine_flux : sf, nf * 4,
                                        cudaMemcpyDeviceToDevice, st));
            at += np + nf;
        }
        return MOC_OK;
    };
    if ((s = copy_all(true))) return s;
    cudaEvent_t a = nullptr, b = nullptr;
    MOC_CUDA(h, cudaEventCreate(&a));
    MOC_CUDA(h, cudaEventCreate(&b));
    std::memset(res, 0, sizeof(*res));
    res->best_ms = -1.0f;
    const int vecs[3] = {1, 2, 4};
    for (int vi = 0; vi < 3 && s == MOC_OK; vi++)
        for (int w = 1; w <= 16 && s == MOC_OK; w++) {
            moc::BatchParams B;
            moc::BatchWork W;
            BatchSplit X;
            int blocks = 0;
            if (build_batch(h, probs, n, o, vecs[vi], w, B, W, X, blocks)) continue;
            float best = 1e30f;
            for (int rep = 0; rep < 3 && s == MOC_OK; rep++) {
                if ((s = copy_all(false))) break;
                cudaEventRecord(a, st);
                s = enqueue_batch(h, probs, n, o, B, W, X, vecs[vi], w, blocks, st);
                cudaEventRecord(b, st);
                if (cudaEventSynchronize(b) != cudaSuccess) s = MOC_ERR_CUDA;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, b);
                if (rep > 0 && ms < best) best = ms;  // the first repeat warms up
            }
            const int c = res->n_candidates++;
            res->candidate_vec[c] = vecs[vi];
            res->candidate_warps[c] = w;
            res->candidate_ms[c] = best;
            if (res->best_ms < 0.0f || best < res->best_ms) {
                res->best_ms = best;
                res->vec = vecs[vi];
                res->warps_per_block = w;
                res->tracks_per_block = w;
            }
        }
    const moc_status_t rs = copy_all(false);
    cudaStreamSynchronize(st);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (s) return s;
    if (rs) return rs;
    if (res->n_candidates == 0) return MOC_ERR_UNSUPPORTED;
    h->tune_key = set_key(probs, n, o);
    h->tune_vec = res->vec;
    h->tune_wpb = res->warps_per_block;
    return MOC_OK;
}

moc_status_t moc_attenuate_adj(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                               const float *w, const float *v, float *d_sigT, float *d_source,
                               float *d_psi_in, void *stream)
{
    if (!h || !p || !o) return MOC_ERR_INVALID_ARG;
    // fine_flux is not used by the adjoint; validate the rest of the problem as the
    // forward does
    moc_problem_t q = *p;
    if (!q.fine_flux) q.fine_flux = const_cast<float *>(p->sigT);
    moc_fwd_opts_t oo = *o;
    oo.precision = MOC_PREC_FP32;
    oo.tally = MOC_TALLY_ATOMIC_FP32;
    moc_status_t s = check_problem(&q, &oo);
    if (s) return s;
    if (o->exp_mode != MOC_EXP_FULL) return MOC_ERR_UNSUPPORTED;
    if (!w || !d_sigT || !d_source || (p->n_tracks > 0 && (!v || !d_psi_in)))
        return MOC_ERR_INVALID_ARG;
    if (!aligned(w, 16) || !aligned(d_sigT, 16) || !aligned(d_source, 16) ||
        (v && !aligned(v, 16)) || (d_psi_in && !aligned(d_psi_in, 16)))
        return MOC_ERR_MISALIGNED;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    const void *ptrs[] = {p->track_offsets, p->seg_region, p->seg_interval, p->seg_ds,
                          p->sigT, p->source, p->psi, w, v, d_sigT, d_source, d_psi_in};
    for (const void *ptr : ptrs)
        if (!device_accessible(ptr, h->device)) return MOC_ERR_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    const size_t nff = (size_t)ncell * p->group_stride;
    // cell blocks and the null-cell row after them
    if ((s = ensure(h, reinterpret_cast<void **>(&h->blk), &h->blk_cap,
                    (nff + p->group_stride) * sizeof(float4))))
        return s;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->gblk), &h->gblk_cap, nff * sizeof(float4))))
        return s;
    const size_t nhist = (size_t)(p->n_segments > 0 ? p->n_segments : 1) * p->group_stride;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->hist), &h->hist_cap, nhist * sizeof(float))))
        return s;

    moc::AdjParams ap{};
    moc::SweepParams &sp = ap.fw;
    sp.R = p->n_regions;
    sp.I = p->n_intervals;
    sp.G = p->n_groups;
    sp.Gs = p->group_stride;
    sp.T = p->n_tracks;
    sp.S = p->n_segments;
    sp.off = p->track_offsets;
    sp.reg = p->seg_region;
    sp.itv = p->seg_interval;
    sp.ds = p->seg_ds;
    sp.blk = h->blk;
    sp.null_cell = (int32_t)ncell;
    sp.psi = p->psi;
    sp.weight = o->weight;
    sp.err = h->err;
    sp.counter = h->counter;
    // Long tracks: every chunk of a split track gets its maps, then psi entering and
    // lambda leaving it.
    moc::SplitWork sw{};
    bool split = false;
    {
        const int v0 = o->vec ? o->vec : moc::auto_vec(p->n_groups);
        const int64_t n_gch = (p->n_groups + 32 * v0 - 1) / (32 * v0);
        if ((s = split_setup(h, p, o, 1, n_gch, &sp, &sw, &split))) return s;
    }
    if (split) {
        const size_t n = 2 * (size_t)sw.cap * p->group_stride;
        if ((s = ensure(h, reinterpret_cast<void **>(&h->sadj), &h->sadj_cap,
                        n * sizeof(float))))
            return s;
        ap.map_c = h->sadj;
        ap.lam_end = h->sadj + (size_t)sw.cap * p->group_stride;
        ap.base = sw.base;
    }
    // The reverse sweep carries more work per segment than the forward: with few work
    // items (fewer warps than about two per SM slot) split the groups finer.
    const int64_t units = split ? sw.cap : p->n_tracks;
    int vec = o->vec ? o->vec : moc::auto_vec(p->n_groups);
    while (!o->vec && vec > 1 &&
           units * ((p->n_groups + 32 * vec - 1) / (32 * vec)) < (int64_t)h->sm_count * 64)
        vec /= 2;
    sp.n_chunks = (p->n_groups + 32 * vec - 1) / (32 * vec);
    sp.n_items = (int64_t)p->n_tracks * sp.n_chunks;
    ap.hist = h->hist;
    ap.w = w;
    ap.v = v;
    ap.gblk = h->gblk;
    ap.dpsi_in = d_psi_in;

    // d q_k / d y_{i+m-1} of the axial fit, for the first / interior / last interval
    // (src/cpu/kernel.c:111-191)
    float jac[27] = {};
    {
        const double dz = o->dz, zin = o->zin, h1 = 1.0 / (2.0 * dz), h2 = 1.0 / (2.0 * dz * dz);
        const double t0[9] = {0, 1.0 - zin / dz, zin / dz, 0, -1.0 / dz, 1.0 / dz, 0, 0, 0};
        const double t1[9] = {h1 * zin + h2 * zin * zin, 1.0 - 2.0 * h2 * zin * zin,
                              -h1 * zin + h2 * zin * zin, h1 + 2.0 * h2 * zin, -4.0 * h2 * zin,
                              -h1 + 2.0 * h2 * zin, h2, -2.0 * h2, h2};
        const double t2[9] = {-zin / dz, 1.0 + zin / dz, 0, -1.0 / dz, 1.0 / dz, 0, 0, 0, 0};
        for (int k = 0; k < 9; k++) {
            jac[k] = (float)t0[k];
            jac[9 + k] = (float)t1[k];
            jac[18 + k] = (float)t2[k];
        }
    }

    const bool prof = o->profile != 0;
    if (prof && !h->ev[0])
        for (auto &e : h->ev) MOC_CUDA(h, cudaEventCreate(&e));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[0], st));
    MOC_CUDA(h, moc::launch_prep_block(p->sigT, p->source, h->blk, p->n_regions,
                                       p->n_intervals, p->group_stride, o->dz, o->zin, o->mu,
                                       o->mu2, st, true, moc::f32_pairs(vec)));
    MOC_CUDA(h, cudaMemsetAsync(h->gblk, 0, nff * sizeof(float4), st));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[1], st));
    int launches = 1;
    if (split) {
        const int bm = moc::adj_map_blocks_per_sm(vec);
        if (bm < 1) return MOC_ERR_UNSUPPORTED;
        MOC_CUDA(h, cudaMemsetAsync(h->counter, 0, 2 * sizeof(unsigned long long), st));
        MOC_CUDA(h, moc::launch_split_records(sp, sw, st));
        moc::AdjParams mp = ap;
        mp.fw.counter = h->counter + 1;
        MOC_CUDA(h, moc::launch_adj_maps(mp, vec, bm * h->sm_count, st));
        MOC_CUDA(h, moc::launch_adj_starts(ap, st));
        launches += 5;
    }
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[4], st));
    if (p->n_tracks > 0) {
        const int bf = moc::adj_blocks_per_sm(vec, false), br = moc::adj_blocks_per_sm(vec, true);
        if (bf < 1 || br < 1) return MOC_ERR_UNSUPPORTED;
        MOC_CUDA(h, cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), st));
        MOC_CUDA(h, moc::launch_adj_forward(ap, vec, bf * h->sm_count, st));
        MOC_CUDA(h, cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), st));
        MOC_CUDA(h, moc::launch_adj_reverse(ap, vec, br * h->sm_count, st));
        launches += 2;
    }
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[2], st));
    MOC_CUDA(h, moc::launch_adj_finish(h->gblk, d_sigT, d_source, p->n_regions, p->n_intervals,
                                       p->n_groups, p->group_stride, jac, o->mu, o->mu2, vec,
                                       st));
    if (prof) {
        MOC_CUDA(h, cudaEventRecord(h->ev[3], st));
        h->timed_launches = launches + 1;
        h->timed_finish = true;
        h->timed_split = split;
    }
    return MOC_OK;
}

// The device address of `bytes` bytes of page-locked host memory at p mapped into the
// current device's address space (pinned memory under unified addressing), or null for any
// other array. Its first and its last byte must both map, at the same offset, so an array
// whose allocation is shorter than its stated size is never read in place.
const void *mapped_on_device(const void *p, size_t bytes)
{
    if (!p || bytes == 0) return nullptr;
    const void *ends[2] = {p, static_cast<const char *>(p) + (bytes - 1)};
    const char *dev[2] = {nullptr, nullptr};
    for (int k = 0; k < 2; k++) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, ends[k]) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
        dev[k] = static_cast<const char *>(a.devicePointer);
    }
    return dev[1] - dev[0] == (ptrdiff_t)(bytes - 1) ? dev[0] : nullptr;
}

// The host-buffer sweep on arrays the GPU reads in place (NVLink-C2C on Grace-Blackwell,
// PCIe elsewhere): descriptors, offsets and psi stay in the caller's pinned memory and psi
// is updated there. The tables (read a few times each by the cell-block pass) are copied
// up first. The tallies live on the device, since reductions into host memory would cross
// the link once per segment and group: they start at zero, and a last pass adds them to
// the caller's fine_flux in place when that is mapped too (else fine_flux is copied up
// before the sweep and back after it).
moc_status_t fwd_host_mapped(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                             const moc_problem_t &mp)
{
    moc_status_t s;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    const size_t ff_bytes = (size_t)ncell * p->group_stride * 4;
    const size_t sig_bytes = (size_t)p->n_regions * p->group_stride * 4;
    if ((s = ensure(h, &h->hbuf[4], &h->hcap[4], sig_bytes)) ||
        (s = ensure(h, &h->hbuf[5], &h->hcap[5], ff_bytes)) ||
        (s = ensure(h, &h->hbuf[6], &h->hcap[6], ff_bytes)))
        return s;
    cudaStream_t st = h->hstream;
    moc_problem_t d = mp;
    d.sigT = static_cast<const float *>(h->hbuf[4]);
    d.source = static_cast<const float *>(h->hbuf[5]);
    d.fine_flux = static_cast<float *>(h->hbuf[6]);
    float *ff_mapped = static_cast<float *>(const_cast<void *>(mapped_on_device(p->fine_flux, ff_bytes)));
    MOC_CUDA(h, cudaMemcpyAsync(h->hbuf[4], p->sigT, sig_bytes, cudaMemcpyHostToDevice, st));
    MOC_CUDA(h, cudaMemcpyAsync(h->hbuf[5], p->source, ff_bytes, cudaMemcpyHostToDevice, st));
    if (ff_mapped)
        MOC_CUDA(h, cudaMemsetAsync(d.fine_flux, 0, ff_bytes, st));
    else
        MOC_CUDA(h, cudaMemcpyAsync(d.fine_flux, p->fine_flux, ff_bytes, cudaMemcpyHostToDevice, st));
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));
    if ((s = fwd_device(h, &d, o, st))) return s;
    if (ff_mapped)  // fine_flux += tallies, in the caller's memory
        MOC_CUDA(h, moc::launch_finish(ff_mapped, d.fine_flux, nullptr,
                                       ncell * p->group_stride, st));
    else
        MOC_CUDA(h, cudaMemcpyAsync(p->fine_flux, d.fine_flux, ff_bytes, cudaMemcpyDeviceToHost, st));
    MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));  // reported here
    MOC_CUDA(h, cudaStreamSynchronize(st));
    return *h->err_host ? MOC_ERR_BAD_INDEX : MOC_OK;
}

// Pipelined host-buffer sweeps: the segments per part and the parts' relative sizes
// (measured on GB300 at 50M x 128, 558 MB in and 77 MB out per call).
constexpr int64_t PART_SEGMENTS = 8 << 20;
constexpr double PART_WEIGHT[8] = {0.5, 1, 1, 1, 1, 1, 1, 1};

moc_status_t moc_attenuate_fwd_host(moc_handle_t h, const moc_problem_t *p,
                                    const moc_fwd_opts_t *o)
{
    if (!h) return MOC_ERR_INVALID_ARG;
    moc_status_t s = check_problem(p, o);
    if (s) return s;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    const int64_t T = p->n_tracks, S = p->n_segments, Gs = p->group_stride;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    // Page-locked, mapped descriptors, offsets and psi (cudaHostAlloc / cudaHostRegister,
    // e.g. torch's pin_memory): the sweep reads them in place (fwd_host_mapped). Checked
    // mode, empty problems and arrays that are not mapped take the copies below.
    if (!o->checked && S > 0 && T > 0) {
        moc_problem_t mp = *p;
        bool all = true;
        auto map = [&](const void *q, size_t n, auto *&out) {
            const void *dq = mapped_on_device(q, n);
            all = all && dq;
            out = static_cast<std::remove_reference_t<decltype(out)>>(const_cast<void *>(dq));
        };
        map(p->track_offsets, (size_t)(T + 1) * 8, mp.track_offsets);
        map(p->seg_region, (size_t)S * 4, mp.seg_region);
        map(p->seg_interval, (size_t)S, mp.seg_interval);
        map(p->seg_ds, (size_t)S * 4, mp.seg_ds);
        map(p->psi, (size_t)T * Gs * 4, mp.psi);
        if (all) return fwd_host_mapped(h, p, o, mp);
    }
    const size_t bytes[8] = {
        (size_t)(T + 1) * 8, (size_t)S * 4, (size_t)S, (size_t)S * 4,
        (size_t)p->n_regions * Gs * 4, (size_t)ncell * Gs * 4, (size_t)ncell * Gs * 4,
        (size_t)T * Gs * 4};
    const void *src[8] = {p->track_offsets, p->seg_region, p->seg_interval, p->seg_ds,
                          p->sigT, p->source, p->fine_flux, p->psi};
    for (int k = 0; k < 8; k++)
        if ((s = ensure(h, &h->hbuf[k], &h->hcap[k], bytes[k] ? bytes[k] : 16))) return s;
    // Large problems whose offsets partition [0, S] take the pipelined path: parts of
    // about PART_SEGMENTS segments (at most 8), sized by PART_WEIGHT (the first parts
    // smaller, so the first sweep starts sooner, the last smaller, so less of the sweep
    // remains when its copies start); checked mode and smaller problems copy everything
    // first.
    const int parts = (int)std::min<int64_t>(8, std::max<int64_t>(1, S / PART_SEGMENTS));
    if (!o->checked && parts > 1 && T >= parts) {
        bool csr = p->track_offsets[0] == 0 && p->track_offsets[T] == S;
        int64_t longest = 0;
        for (int64_t t = 0; csr && t < T; t++) {
            const int64_t len = p->track_offsets[t + 1] - p->track_offsets[t];
            csr = len >= 0;
            longest = len > longest ? len : longest;
        }
        if (csr && (s = ensure(h, &h->hbuf[8], &h->hcap[8], bytes[6] ? bytes[6] : 16)))
            return s;
        if (csr) {
            int64_t cut[9];
            cut[0] = 0;
            double wsum = 0.0;
            for (int k = 0; k < parts; k++) wsum += PART_WEIGHT[k];
            double acc = 0.0;
            for (int k = 1; k < parts; k++) {
                // first track whose start reaches the k-th cumulative share of the segments
                acc += PART_WEIGHT[k - 1];
                const int64_t target = (int64_t)((double)S * acc / wsum);
                int64_t lo = cut[k - 1], hi = T;
                while (lo < hi) {
                    const int64_t mid = (lo + hi) / 2;
                    if (p->track_offsets[mid] < target) lo = mid + 1;
                    else hi = mid;
                }
                cut[k] = lo;
            }
            cut[parts] = T;
            return fwd_host_pipelined(h, p, o, parts, cut, longest);
        }
    }
    cudaStream_t st = h->hstream;
    for (int k = 0; k < 8; k++)
        if (bytes[k])
            MOC_CUDA(h, cudaMemcpyAsync(h->hbuf[k], src[k], bytes[k], cudaMemcpyHostToDevice, st));
    moc_problem_t d = *p;
    d.track_offsets = static_cast<const int64_t *>(h->hbuf[0]);
    d.seg_region = static_cast<const int32_t *>(h->hbuf[1]);
    d.seg_interval = static_cast<const uint8_t *>(h->hbuf[2]);
    d.seg_ds = static_cast<const float *>(h->hbuf[3]);
    d.sigT = static_cast<const float *>(h->hbuf[4]);
    d.source = static_cast<const float *>(h->hbuf[5]);
    d.fine_flux = static_cast<float *>(h->hbuf[6]);
    d.psi = static_cast<float *>(h->hbuf[7]);
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));
    if ((s = fwd_device(h, &d, o, st))) return s;
    if (bytes[6])
        MOC_CUDA(h, cudaMemcpyAsync(p->fine_flux, d.fine_flux, bytes[6], cudaMemcpyDeviceToHost, st));
    if (bytes[7])
        MOC_CUDA(h, cudaMemcpyAsync(p->psi, d.psi, bytes[7], cudaMemcpyDeviceToHost, st));
    MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));  // reported here
    MOC_CUDA(h, cudaStreamSynchronize(st));
    return *h->err_host ? MOC_ERR_BAD_INDEX : MOC_OK;
}



moc_status_t moc_synchronize(moc_handle_t h, void *stream)
{
    if (!h) return MOC_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    MOC_CUDA(h, cudaStreamSynchronize(st));
    MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));
    MOC_CUDA(h, cudaStreamSynchronize(st));
    if (*h->err_host & moc::DEVERR_TRACK) return MOC_ERR_BAD_TRACK;
    if (*h->err_host & moc::DEVERR_TIMEOUT) return MOC_ERR_DEVICE_TIMEOUT;
    return *h->err_host ? MOC_ERR_BAD_INDEX : MOC_OK;
}

// ---- track generation (include/moc_tracks.h; kernels in moc_trace.cu) -----------------

// The walk's tables of geometry g in h->ttab.
moc_status_t trace_tables(moc_handle_t h, const moc_geometry_t *g, cudaStream_t st)
{
    moc_status_t s;
    const size_t n = (size_t)moc::trace_table_len(g);
    if ((s = ensure(h, reinterpret_cast<void **>(&h->ttab), &h->ttab_cap, n * sizeof(double))))
        return s;
    MOC_CUDA(h, moc::launch_trace_tables(g, h->ttab, st));
    return MOC_OK;
}

// Reads the error word; a track error is cleared (other bits stay for moc_synchronize).
moc_status_t take_track_error(moc_handle_t h, cudaStream_t st, bool *bad)
{
    MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                st));
    MOC_CUDA(h, cudaStreamSynchronize(st));
    *bad = (*h->err_host & moc::DEVERR_TRACK) != 0;
    if (*bad) {
        const int32_t rest = *h->err_host & ~moc::DEVERR_TRACK;
        MOC_CUDA(h, cudaMemcpyAsync(h->err, &rest, sizeof(int32_t), cudaMemcpyHostToDevice,
                                    st));
        MOC_CUDA(h, cudaStreamSynchronize(st));
    }
    return MOC_OK;
}

moc_status_t moc_trace_count(moc_handle_t h, const moc_geometry_t *g,
                             const moc_track_t *d_tracks, int64_t n_tracks,
                             int64_t *d_track_offsets, int64_t *n_segments, void *stream)
{
    if (!h || !moc::trace_geometry_ok(g) || n_tracks < 0 || !d_track_offsets || !n_segments ||
        (n_tracks > 0 && !d_tracks))
        return MOC_ERR_INVALID_ARG;
    if (!aligned(d_tracks, 8) || !aligned(d_track_offsets, 8)) return MOC_ERR_MISALIGNED;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    moc_status_t s;
    h->tvalid = false;
    const int64_t T = n_tracks;
    const size_t scratch = (size_t)moc::trace_scan_scratch(T) * sizeof(int64_t);
    if ((s = ensure(h, reinterpret_cast<void **>(&h->tscan), &h->tscan_cap, scratch))) return s;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->tbnd), &h->tbnd_cap,
                    (size_t)(T + 1) * sizeof(int64_t))))
        return s;
    // the scratch layout: one slot per track, sized by an upper bound of its count
    MOC_CUDA(h, moc::launch_trace_bound(g, d_tracks, T, h->tbnd, h->tscan, h->err, st));
    int64_t B = 0;
    MOC_CUDA(h, cudaMemcpyAsync(&B, h->tbnd + T, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    MOC_CUDA(h, cudaStreamSynchronize(st));
    const size_t nb = (size_t)(B > 0 ? B : 1);
    if ((s = ensure(h, reinterpret_cast<void **>(&h->treg), &h->treg_cap, nb * 4)) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->titv), &h->titv_cap, nb)) ||
        (s = ensure(h, reinterpret_cast<void **>(&h->tds), &h->tds_cap, nb * 4)))
        return s;
    if ((s = trace_tables(h, g, st))) return s;
    // one walk per track into the scratch, the counts scanned into the offsets
    MOC_CUDA(h, moc::launch_trace_walk(g, h->ttab, d_tracks, T, h->tbnd, d_track_offsets,
                                       h->tscan, h->treg, h->titv, h->tds, h->err, st));
    int64_t total = 0;
    MOC_CUDA(h, cudaMemcpyAsync(&total, d_track_offsets + T, sizeof(int64_t),
                                cudaMemcpyDeviceToHost, st));
    bool bad = false;
    if ((s = take_track_error(h, st, &bad))) return s;
    *n_segments = total;
    if (bad) return MOC_ERR_BAD_TRACK;
    h->tvalid = true;
    h->ttracks = d_tracks;
    h->toff = d_track_offsets;
    h->tT = T;
    h->tgeo = *g;
    return MOC_OK;
}

moc_status_t moc_trace_segments(moc_handle_t h, const moc_geometry_t *g,
                                const moc_track_t *d_tracks, int64_t n_tracks,
                                const int64_t *d_track_offsets, int32_t *d_seg_region,
                                uint8_t *d_seg_interval, float *d_seg_ds, void *stream)
{
    if (!h || !moc::trace_geometry_ok(g) || n_tracks < 0 || !d_track_offsets ||
        (n_tracks > 0 && (!d_tracks || !d_seg_region || !d_seg_interval || !d_seg_ds)))
        return MOC_ERR_INVALID_ARG;
    if (!aligned(d_tracks, 8) || !aligned(d_track_offsets, 8) || !aligned(d_seg_region, 4) ||
        !aligned(d_seg_ds, 4))
        return MOC_ERR_MISALIGNED;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // after moc_trace_count on the same arguments: copy its walk out of the scratch
    if (h->tvalid && h->ttracks == d_tracks && h->toff == d_track_offsets &&
        h->tT == n_tracks && std::memcmp(&h->tgeo, g, sizeof(*g)) == 0) {
        MOC_CUDA(h, moc::launch_trace_compact(d_tracks, n_tracks, h->tbnd, d_track_offsets,
                                              h->treg, h->titv, h->tds, d_seg_region,
                                              d_seg_interval, d_seg_ds, st));
        return MOC_OK;
    }
    moc_status_t s;
    if ((s = trace_tables(h, g, st))) return s;
    MOC_CUDA(h, moc::launch_trace_emit(g, h->ttab, d_tracks, n_tracks, d_track_offsets,
                                       d_seg_region, d_seg_interval, d_seg_ds, h->err, st));
    return MOC_OK;
}

// ---- source update and power iteration (include/moc_transport.h; moc_transport.cu) ----

bool xs_ok(const moc_xs_t *xs)
{
    return xs && xs->n_materials >= 1 && xs->n_groups >= 1 && xs->n_groups <= 256 &&
           xs->group_stride >= xs->n_groups && xs->group_stride % 4 == 0 && xs->sigT &&
           xs->scatter && xs->nu_fission && xs->chi && aligned(xs->sigT, 16) &&
           aligned(xs->scatter, 16) && aligned(xs->nu_fission, 16) && aligned(xs->chi, 16);
}

moc_status_t moc_region_sigT(moc_handle_t h, const moc_xs_t *xs, const int32_t *material,
                             int32_t n_regions, float *sigT, void *stream)
{
    if (!h || !xs_ok(xs) || n_regions < 0 || (n_regions > 0 && (!material || !sigT)))
        return MOC_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    MOC_CUDA(h, moc::launch_region_sigT(xs, material, n_regions, sigT, h->err,
                                        static_cast<cudaStream_t>(stream)));
    return MOC_OK;
}

moc_status_t source_update(moc_handle_t h, const moc_xs_t *xs, const int32_t *material,
                           int32_t R, int32_t I, const double *volume, const float *fine_flux,
                           double k, float *source, double *fission, cudaStream_t st)
{
    moc::TransportParams P;
    P.ncell = (int64_t)R * I;
    P.M = xs->n_materials;
    P.G = xs->n_groups;
    P.Gs = xs->group_stride;
    P.I = I;
    P.scatter = xs->scatter;
    P.nu_fission = xs->nu_fission;
    P.chi = xs->chi;
    P.rk = (float)(1.0 / k);
    P.rpi = (float)(1.0 / (4.0 * 3.14159265358979323846));
    MOC_CUDA(h, moc::launch_source_update(P, material, volume, fine_flux, source, fission,
                                          h->err, st));
    return MOC_OK;
}

moc_status_t moc_source_update(moc_handle_t h, const moc_xs_t *xs, const int32_t *material,
                               int32_t n_regions, int32_t n_intervals, const double *volume,
                               const float *fine_flux, double k, float *source,
                               double *fission, void *stream)
{
    if (!h || !xs_ok(xs) || n_regions < 0 || n_intervals < 1 || !(k > 0.0) ||
        (n_regions > 0 && (!material || !volume || !fine_flux || !source || !fission)))
        return MOC_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    return source_update(h, xs, material, n_regions, n_intervals, volume, fine_flux, k, source,
                         fission, static_cast<cudaStream_t>(stream));
}

moc_status_t moc_power_iteration(moc_handle_t h, const moc_problem_t *p,
                                 const moc_fwd_opts_t *opts, const moc_xs_t *xs,
                                 const int32_t *material, const double *volume,
                                 const moc_eigen_opts_t *eo, double *k, int32_t *iterations,
                                 void *stream)
{
    if (!h || !p || !opts || !xs_ok(xs) || !material || !volume || !eo || !k || !iterations ||
        !(*k > 0.0) || eo->max_iterations < 1 || !(eo->tolerance >= 0.0) ||
        xs->n_groups != p->n_groups || xs->group_stride != p->group_stride)
        return MOC_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    moc_status_t s;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->fis), &h->fis_cap, sizeof(double))))
        return s;
    const int32_t R = p->n_regions, I = p->n_intervals;
    const size_t nff = (size_t)R * I * p->group_stride;
    const size_t npsi = (size_t)p->n_tracks * p->group_stride;
    auto update = [&](double kk, double *F) -> moc_status_t {
        MOC_CUDA(h, cudaMemsetAsync(h->fis, 0, sizeof(double), st));
        // the problem's source is this call's workspace (see the header)
        moc_status_t s2 = source_update(h, xs, material, R, I, volume, p->fine_flux, kk,
                                        const_cast<float *>(p->source), h->fis, st);
        if (s2) return s2;
        MOC_CUDA(h, cudaMemcpyAsync(F, h->fis, sizeof(double), cudaMemcpyDeviceToHost, st));
        MOC_CUDA(h, cudaStreamSynchronize(st));
        return MOC_OK;
    };
    double kk = *k, F_prev = 0.0;
    if ((s = update(kk, &F_prev))) return s;
    int32_t it = 0;
    while (it < eo->max_iterations) {
        MOC_CUDA(h, cudaMemsetAsync(p->psi, 0, npsi * sizeof(float), st));
        MOC_CUDA(h, cudaMemsetAsync(p->fine_flux, 0, nff * sizeof(float), st));
        if ((s = moc_attenuate_fwd(h, p, opts, stream))) return s;
        double F = 0.0;
        if ((s = update(kk, &F))) return s;
        it++;
        if (!(F_prev > 0.0) || !(F >= 0.0)) {  // no fission source: nothing to normalise
            *k = kk;
            *iterations = it;
            return MOC_ERR_INVALID_ARG;
        }
        const double kn = kk * F / F_prev;
        const bool done = std::fabs(kn - kk) <= eo->tolerance * kn;
        kk = kn;
        F_prev = F;
        if (done) break;
    }
    *k = kk;
    *iterations = it;
    return moc_synchronize(h, stream);
}

moc_status_t moc_build_exp_table(int32_t n_points, float max_val, float *values, float *dx,
                                 float *lookup_max)
{
    if (n_points < 2 || !(max_val > 0.0f) || !values || !dx || !lookup_max)
        return MOC_ERR_INVALID_ARG;
    // src/cpu/init.c:88-114, rounded as the reference's float code rounds it (this file's
    // host code is compiled with -ffp-contract=off, so nothing here is fused).
    const float d = max_val / (float)n_points;
    for (int n = 0; n < n_points; n++) {
        const float nd = (float)n * d;
        const float ex = (float)std::exp((double)(-nd));
        values[2 * n] = -ex;
        const float a = nd - 1.0f;
        const float b = a * ex;
        values[2 * n + 1] = 1.0f + b;
    }
    *dx = d;
    *lookup_max = max_val - d;
    return MOC_OK;
}

moc_status_t moc_last_timings(moc_handle_t h, moc_timings_t *t)
{
    if (!h || !t || h->timed_launches == 0) return MOC_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    const cudaEvent_t last = h->timed_finish ? h->ev[3] : h->ev[2];
    MOC_CUDA(h, cudaEventSynchronize(last));
    float a = 0, b = 0, c = 0, d = 0;
    MOC_CUDA(h, cudaEventElapsedTime(&a, h->ev[0], h->ev[1]));
    if (h->timed_split) {
        MOC_CUDA(h, cudaEventElapsedTime(&d, h->ev[1], h->ev[4]));
        MOC_CUDA(h, cudaEventElapsedTime(&b, h->ev[4], h->ev[2]));
    } else {
        MOC_CUDA(h, cudaEventElapsedTime(&b, h->ev[1], h->ev[2]));
    }
    if (h->timed_finish) MOC_CUDA(h, cudaEventElapsedTime(&c, h->ev[2], h->ev[3]));
    t->prep_ms = a;
    t->sweep_ms = b;
    t->finish_ms = c;
    t->launches = h->timed_launches;
    t->split_ms = d;
    return MOC_OK;
}

const char *moc_status_string(moc_status_t s)
{
    switch (s) {
    case MOC_OK: return "ok";
    case MOC_ERR_INVALID_ARG: return "invalid argument";
    case MOC_ERR_MISALIGNED: return "misaligned buffer";
    case MOC_ERR_UNSUPPORTED: return "unsupported configuration";
    case MOC_ERR_CUDA: return "CUDA error";
    case MOC_ERR_NO_DEVICE: return "no CUDA device";
    case MOC_ERR_OUT_OF_MEMORY: return "out of device memory";
    case MOC_ERR_BAD_INDEX: return "segment index or track offset out of range";
    case MOC_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case MOC_ERR_TOO_LARGE: return "problem exceeds the fixed scratch of the no-allocation entry point";
    case MOC_ERR_BAD_TRACK: return "track record invalid or inconsistent with the offsets";
    case MOC_ERR_IO: return "track file unwritable, unreadable, short, corrupt or inconsistent";
    }
    return "unknown status";
}

const char *moc_last_error(moc_handle_t h) { return h ? h->last_error.c_str() : ""; }

int32_t moc_abi_version(void) { return MOC_ABI_VERSION; }

}  // extern "C"
