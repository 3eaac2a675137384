// moc_static.cu — moc_attenuate_fwd_noalloc: the forward sweep with no allocation.
//
// Some callers cannot call cudaMalloc: a transport code whose own pool allocator takes
// the GPU's memory at start-up and forbids later allocations, a sweep loop that cannot
// afford the device-wide synchronisation cudaMalloc/cudaFree may cause while other
// streams run, or a stateless call site with nowhere to keep a handle. For them this
// entry point sweeps with the same kernels as moc_attenuate_fwd, but its scratch (the
// per-cell blocks of sigT and axial coefficients, the exponential table, the work-queue
// head and the error word) lives in one file-scope __device__ array of fixed size,
// which every GPU that loads the library holds until the process exits.
//
// That array's name, used in host code, is only a host-side stand-in for the symbol,
// not a device address: a kernel given it would fault or, where the GPU can reach host
// memory, silently use the wrong memory. So the first call on each device (with that
// device current) asks the runtime for the array's device address with
// cudaGetSymbolAddress, checks the result, and caches it; later calls pass the cached
// address to the kernels.
//
// Every call shares the one array and it keeps the last call's contents: each call
// clears the work-queue head and error word before its kernels run and rewrites the cell
// coefficients (and the table in table mode). Calls whose kernels overlap on the GPU —
// on different streams, or from different host threads — race on the array and give
// wrong results; order them on one stream.
#include "moc_attenuate.h"
#include "moc_internal.h"

#include <mutex>

namespace {

// Layout of the scratch array (bytes):
//   [0, 256)                    work-queue head (u64 at 0) and error word (i32 at 8)
//   [256, 256 + TABLE_BYTES)    exponential table, MOC_NOALLOC_MAX_TABLE_POINTS pairs
//   [BLK_OFF, end)              cell blocks (sigT, q0, q1*mu, q2*mu2), 16 bytes for each
//                               of MOC_NOALLOC_MAX_CELL_GROUPS (region, interval, group)
constexpr size_t CTRL_BYTES = 256;
constexpr size_t TABLE_BYTES = ((size_t)MOC_NOALLOC_MAX_TABLE_POINTS * 8 + 255) / 256 * 256;
constexpr size_t BLK_OFF = CTRL_BYTES + TABLE_BYTES;
constexpr size_t SCRATCH_BYTES = BLK_OFF + (size_t)MOC_NOALLOC_MAX_CELL_GROUPS * 16;

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
unsigned char *g_scratch_ptr[MAX_DEVICES] = {};  // device address, per device
int g_sm_count[MAX_DEVICES] = {};
float g_table_host[2 * MOC_NOALLOC_MAX_TABLE_POINTS];  // static host staging, no malloc
int32_t g_err_host = 0;

// Once per device, with the device current: the array's device address.
moc_status_t setup_device(int dev, unsigned char **ptr, int *sms)
{
    if (dev < 0 || dev >= MAX_DEVICES) return MOC_ERR_NO_DEVICE;
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return MOC_ERR_CUDA;
        }
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return MOC_ERR_CUDA;
        }
        g_sm_count[dev] = n;
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *ptr = g_scratch_ptr[dev];
    *sms = g_sm_count[dev];
    return MOC_OK;
}

#define NA_CUDA(call)                                    \
    do {                                                 \
        if ((call) != cudaSuccess) {                     \
            cudaGetLastError();                          \
            return MOC_ERR_CUDA;                         \
        }                                                \
    } while (0)

}  // namespace

extern "C" moc_status_t moc_attenuate_fwd_noalloc(const moc_problem_t *p,
                                                   const moc_fwd_opts_t *o, void *stream)
{
    moc_status_t s = moc::check_args(p, o);
    if (s) return s;
    if (o->precision != MOC_PREC_FP32) return MOC_ERR_UNSUPPORTED;  // the plain form only
    // the register loops only: the bulk-copy ring's bounded waits report a timeout through
    // an error word, which this entry point has no handle to return to the caller
    if (o->prefetch > 1) return MOC_ERR_UNSUPPORTED;
    const int64_t cell_groups = (int64_t)p->n_regions * p->n_intervals * p->group_stride;
    if (cell_groups > MOC_NOALLOC_MAX_CELL_GROUPS) return MOC_ERR_TOO_LARGE;
    if (o->exp_mode == MOC_EXP_TABLE && o->table_points > MOC_NOALLOC_MAX_TABLE_POINTS)
        return MOC_ERR_TOO_LARGE;
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    // every array must be memory of the current device (or managed memory)
    if (!moc::all_device_accessible(p, dev)) return MOC_ERR_INVALID_ARG;

    std::lock_guard<std::mutex> lock(g_mutex);
    unsigned char *base = nullptr;
    int sms = 0;
    if ((s = setup_device(dev, &base, &sms))) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto *counter = reinterpret_cast<unsigned long long *>(base);
    auto *err = reinterpret_cast<int32_t *>(base + 8);
    auto *table = reinterpret_cast<float *>(base + CTRL_BYTES);
    auto *blk = reinterpret_cast<float4 *>(base + BLK_OFF);

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
    sp.blk = blk;
    sp.ff = p->fine_flux;
    sp.psi = p->psi;
    sp.weight = o->weight;
    sp.err = err;
    sp.counter = counter;
    if (o->exp_mode == MOC_EXP_TABLE) {
        float dx = 0.0f, lk = 0.0f;
        moc_build_exp_table(o->table_points, o->table_max, g_table_host, &dx, &lk);
        // From pageable memory the copy is staged before the call returns, so the
        // static host buffer may be rewritten by the next call.
        NA_CUDA(cudaMemcpyAsync(table, g_table_host, 2 * (size_t)o->table_points * 4,
                                cudaMemcpyHostToDevice, st));
        sp.table = table;
        sp.tab_n = o->table_points;
        sp.tab_dx = dx;
        sp.tab_max = lk;
    }
    NA_CUDA(cudaMemsetAsync(base, 0, 16, st));  // work-queue head and error word
    if (o->checked) {
        NA_CUDA(moc::launch_check(sp, st));
        NA_CUDA(cudaMemcpyAsync(&g_err_host, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        NA_CUDA(cudaStreamSynchronize(st));
        if (g_err_host) return MOC_ERR_BAD_INDEX;
    }
    if (p->n_tracks == 0) return MOC_OK;

    moc::FwdConfig cfg;
    cfg.vec = o->vec ? o->vec : moc::auto_vec(p->n_groups);
    cfg.exp_kind = o->exp_mode == MOC_EXP_TABLE ? moc::EXPK_TABLE : moc::EXPK_PLAIN;
    cfg.warps_per_block =
        o->warps_per_block ? o->warps_per_block : moc::auto_warps_per_block(cfg.exp_kind);
    cfg.prefetch = 1;
    const int per_sm = moc::fwd_blocks_per_sm(cfg, o->table_points);
    if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
    cfg.blocks = per_sm * sms;
    sp.n_chunks = (p->n_groups + 32 * cfg.vec - 1) / (32 * cfg.vec);
    sp.n_items = (int64_t)p->n_tracks * sp.n_chunks;
    sp.group_major = 1;
    sp.null_cell = -1;  // no null-cell row in the fixed scratch: the checked segment loop

    NA_CUDA(moc::launch_prep_block(p->sigT, p->source, blk, p->n_regions, p->n_intervals,
                                   p->group_stride, o->dz, o->zin, o->mu, o->mu2, st, false,
                                   moc::f32_pairs(cfg.vec)));
    NA_CUDA(moc::launch_fwd(sp, cfg, st));
    return MOC_OK;
}
