// moc_api.cu — the C ABI (include/moc_attenuate.h): handles, argument checks, workspace,
// and the launch sequence of one forward sweep.
#include "moc_attenuate.h"
#include "moc_internal.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

struct moc_handle_s {
    int device = 0;
    int sm_count = 0;
    size_t l2_bytes = 0;
    // workspace (device)
    float *coef = nullptr;
    size_t coef_cap = 0;  // floats
    float *table = nullptr;
    int32_t table_n = 0;
    float table_maxval = 0.0f, table_dx = 0.0f, table_lookup = 0.0f;
    int32_t *err = nullptr;              // device error word
    unsigned long long *counter = nullptr;
    int32_t *err_host = nullptr;         // pinned mirror
    // device copies for the host-buffer entry point
    void *hbuf[8] = {};
    size_t hcap[8] = {};
    cudaStream_t hstream = nullptr;
    // kernel timing of the last profiled call
    cudaEvent_t ev[4] = {};
    int timed_launches = 0;   // 0: no profiled call yet
    bool timed_finish = false;
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
        o->precision != MOC_PREC_FP16)
        return MOC_ERR_INVALID_ARG;
    if (o->tally != MOC_TALLY_ATOMIC_FP32 && o->tally != MOC_TALLY_COMPENSATED &&
        o->tally != MOC_TALLY_FP64)
        return MOC_ERR_INVALID_ARG;
    if (o->exp_mode == MOC_EXP_TABLE &&
        (o->table_points < 2 || o->table_points > 24000 || !(o->table_max > 0.0f)))
        return MOC_ERR_INVALID_ARG;
    if (o->vec != 0 && o->vec != 1 && o->vec != 2 && o->vec != 4) return MOC_ERR_INVALID_ARG;
    if (o->warps_per_block < 0 || o->warps_per_block > 8) return MOC_ERR_INVALID_ARG;
    if (!std::isfinite(o->dz) || o->dz == 0.0f) return MOC_ERR_INVALID_ARG;
    // Forms not built yet in this library version.
    if (o->precision != MOC_PREC_FP32 || o->tally != MOC_TALLY_ATOMIC_FP32)
        return MOC_ERR_UNSUPPORTED;
    return MOC_OK;
}

// Device pointers must be device or managed memory.
bool device_accessible(const void *p)
{
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
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

// Launch configuration: groups per lane from G unless given, grid filling the GPU.
moc_status_t pick_config(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                         moc::FwdConfig *c)
{
    int vec = o->vec;
    if (vec == 0) vec = p->n_groups > 64 ? 4 : (p->n_groups > 32 ? 2 : 1);
    c->vec = vec;
    c->warps_per_block = o->warps_per_block ? o->warps_per_block : 8;
    c->exp_kind = o->exp_mode == MOC_EXP_TABLE ? moc::EXPK_TABLE : moc::EXPK_PLAIN;
    const size_t smem = c->exp_kind == moc::EXPK_TABLE ? (size_t)o->table_points * 8 : 0;
    const int per_sm = moc::fwd_blocks_per_sm(*c, smem);
    if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
    c->blocks = per_sm * h->sm_count;
    return MOC_OK;
}

moc_status_t fwd_device(moc_handle_t h, const moc_problem_t *p, const moc_fwd_opts_t *o,
                        cudaStream_t st)
{
    moc_status_t s;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    const size_t coef_floats = (size_t)ncell * 3 * p->group_stride;
    if ((s = ensure(h, reinterpret_cast<void **>(&h->coef), &h->coef_cap, coef_floats * 4)))
        return s;
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
    sp.sigT = p->sigT;
    sp.coef = h->coef;
    sp.ff = p->fine_flux;
    sp.psi = p->psi;
    sp.weight = o->weight;
    sp.table = h->table;
    sp.tab_n = h->table_n;
    sp.tab_dx = h->table_dx;
    sp.tab_max = h->table_lookup;
    sp.err = h->err;
    sp.counter = h->counter;

    if (o->checked) {
        MOC_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), st));
        MOC_CUDA(h, moc::launch_check(sp, st));
        MOC_CUDA(h, cudaMemcpyAsync(h->err_host, h->err, sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, st));
        MOC_CUDA(h, cudaStreamSynchronize(st));
        if (*h->err_host) return MOC_ERR_BAD_INDEX;
    }
    if (p->n_tracks == 0) return MOC_OK;

    moc::FwdConfig cfg;
    if ((s = pick_config(h, p, o, &cfg))) return s;
    sp.n_chunks = (p->n_groups + 32 * cfg.vec - 1) / (32 * cfg.vec);
    sp.n_items = (int64_t)p->n_tracks * sp.n_chunks;

    const bool prof = o->profile != 0;
    if (prof && !h->ev[0])
        for (auto &e : h->ev) MOC_CUDA(h, cudaEventCreate(&e));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[0], st));
    MOC_CUDA(h, moc::launch_prep_coef(p->source, h->coef, p->n_regions, p->n_intervals,
                                      p->group_stride, o->dz, o->zin, o->mu, o->mu2, st));
    MOC_CUDA(h, cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), st));
    if (prof) MOC_CUDA(h, cudaEventRecord(h->ev[1], st));
    MOC_CUDA(h, moc::launch_fwd(sp, cfg, st));
    if (prof) {
        MOC_CUDA(h, cudaEventRecord(h->ev[2], st));
        h->timed_launches = 2;
        h->timed_finish = false;
    }
    return MOC_OK;
}

}  // namespace

// Argument checks shared with the other entry points (declared in moc_internal.h).
moc_status_t moc::check_args(const moc_problem_t *p, const moc_fwd_opts_t *o)
{
    return check_problem(p, o);
}

bool moc::all_device_accessible(const moc_problem_t *p)
{
    const void *ptrs[] = {p->track_offsets, p->seg_region, p->seg_interval, p->seg_ds,
                          p->sigT, p->source, p->fine_flux, p->psi};
    for (const void *q : ptrs)
        if (!device_accessible(q)) return false;
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
    if (h->coef) cudaFree(h->coef);
    if (h->table) cudaFree(h->table);
    if (h->err) cudaFree(h->err);
    if (h->err_host) cudaFreeHost(h->err_host);
    for (int k = 0; k < 8; k++)
        if (h->hbuf[k]) cudaFree(h->hbuf[k]);
    if (h->hstream) cudaStreamDestroy(h->hstream);
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
        if (!device_accessible(q)) return MOC_ERR_INVALID_ARG;
    return fwd_device(h, p, o, static_cast<cudaStream_t>(stream));
}

moc_status_t moc_attenuate_fwd_host(moc_handle_t h, const moc_problem_t *p,
                                    const moc_fwd_opts_t *o)
{
    if (!h) return MOC_ERR_INVALID_ARG;
    moc_status_t s = check_problem(p, o);
    if (s) return s;
    if (cudaSetDevice(h->device) != cudaSuccess) return MOC_ERR_NO_DEVICE;
    const int64_t T = p->n_tracks, S = p->n_segments, Gs = p->group_stride;
    const int64_t ncell = (int64_t)p->n_regions * p->n_intervals;
    const size_t bytes[8] = {
        (size_t)(T + 1) * 8, (size_t)S * 4, (size_t)S, (size_t)S * 4,
        (size_t)p->n_regions * Gs * 4, (size_t)ncell * Gs * 4, (size_t)ncell * Gs * 4,
        (size_t)T * Gs * 4};
    const void *src[8] = {p->track_offsets, p->seg_region, p->seg_interval, p->seg_ds,
                          p->sigT, p->source, p->fine_flux, p->psi};
    for (int k = 0; k < 8; k++)
        if ((s = ensure(h, &h->hbuf[k], &h->hcap[k], bytes[k] ? bytes[k] : 16))) return s;
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
    return *h->err_host ? MOC_ERR_BAD_INDEX : MOC_OK;
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
    float a = 0, b = 0, c = 0;
    MOC_CUDA(h, cudaEventElapsedTime(&a, h->ev[0], h->ev[1]));
    MOC_CUDA(h, cudaEventElapsedTime(&b, h->ev[1], h->ev[2]));
    if (h->timed_finish) MOC_CUDA(h, cudaEventElapsedTime(&c, h->ev[2], h->ev[3]));
    t->prep_ms = a;
    t->sweep_ms = b;
    t->finish_ms = c;
    t->launches = h->timed_launches;
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
    }
    return "unknown status";
}

const char *moc_last_error(moc_handle_t h) { return h ? h->last_error.c_str() : ""; }

int32_t moc_abi_version(void) { return MOC_ABI_VERSION; }

}  // extern "C"
