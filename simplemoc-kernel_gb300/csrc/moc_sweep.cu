// moc_sweep.cu — forward segment-attenuation sweep kernels for sm_103a.
//
// Work decomposition: a work item is (track, chunk of 32*VEC groups). One warp owns an
// item from start to end: lanes hold VEC consecutive groups each, psi stays in registers
// for the whole track, and the warp walks the track's segments in CSR order (psi is
// carried from one segment to the next, src/cpu/kernel.c:53). Energy groups are
// independent, so a track's chunks are independent items. Warps take items from a
// global queue head (one atomicAdd per item), so tracks of uneven length balance.
//
// Per segment a warp reads: the segment descriptor (region, interval, ds; one coalesced
// load per 32 segments, broadcast by shuffles and fetched one window ahead), the sigT
// row of the region and the 2 or 3 axial-coefficient rows of the cell (128-bit loads),
// and adds the tally row into fine_flux with vector reductions. The rows of the next
// segment are loaded before the current one is computed, so their L2 latency overlaps
// the arithmetic.
#include "moc_device.cuh"
#include "moc_internal.h"

namespace moc {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------------------------------
// Axial fit, src/cpu/kernel.c:111-191, rounded as the reference's C rounds it (no
// contraction), then the first product of q1 * mu * ... and q2 * mu2 * ....
// ------------------------------------------------------------------------------------
__global__ void prep_coef_kernel(const float *__restrict__ source, float *__restrict__ coef,
                                 int R, int I, int Gs, float dz, float zin, float mu, float mu2)
{
    const int64_t n = (int64_t)R * I * Gs;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t cell = k / Gs;
        const int g = (int)(k - cell * Gs);
        const int i = (int)(cell % I);
        const float *row = source + cell * Gs + g;
        float q0, q1, q2;
        if (i == 0) {
            const float y2 = row[0], y3 = row[Gs];
            const float c1 = __fdiv_rn(__fsub_rn(y3, y2), dz);
            q0 = __fadd_rn(y2, __fmul_rn(c1, zin));
            q1 = c1;
            q2 = 0.0f;
        } else if (i == I - 1) {
            const float y1 = row[-Gs], y2 = row[0];
            const float c1 = __fdiv_rn(__fsub_rn(y2, y1), dz);
            q0 = __fadd_rn(y2, __fmul_rn(c1, zin));
            q1 = c1;
            q2 = 0.0f;
        } else {
            const float y1 = row[-Gs], y2 = row[0], y3 = row[Gs];
            const float c1 = __fdiv_rn(__fsub_rn(y1, y3), __fmul_rn(2.0f, dz));
            const float c2 = __fdiv_rn(__fadd_rn(__fsub_rn(y1, __fmul_rn(2.0f, y2)), y3),
                                       __fmul_rn(__fmul_rn(2.0f, dz), dz));
            q0 = __fadd_rn(__fadd_rn(y2, __fmul_rn(c1, zin)),
                           __fmul_rn(__fmul_rn(c2, zin), zin));
            q1 = __fadd_rn(c1, __fmul_rn(__fmul_rn(2.0f, c2), zin));
            q2 = c2;
        }
        float *out = coef + cell * 3 * Gs + g;
        out[0] = q0;
        out[Gs] = __fmul_rn(q1, mu);
        out[2 * Gs] = __fmul_rn(q2, mu2);
    }
}

// ------------------------------------------------------------------------------------
// The per-(segment, group) arithmetic.
// ------------------------------------------------------------------------------------
template <int VEC>
struct Rows {
    Vec<VEC> s, a0, a1, a2;
};

struct TableRef {
    const float2 *tab;
    int n;
    float dx, max;
};

// src/cpu/kernel.c:200-332 for VEC groups. a1 = q1*mu and a2 = q2*mu2 come from the
// prep pass. Divisions by sigT powers become products with one reciprocal.
template <int VEC, int EK>
__device__ __forceinline__ void attenuate(const Rows<VEC> &x, float ds, float weight,
                                          const TableRef &tr, Vec<VEC> &psi,
                                          Vec<VEC> &tally)
{
#pragma unroll
    for (int k = 0; k < VEC; k++) {
        const float s = x.s.v[k], a0 = x.a0.v[k], a1 = x.a1.v[k], a2 = x.a2.v[k];
        const float ps = psi.v[k];
        const float tau = __fmul_rn(s, ds);  // kept exact: the table index depends on it
        float e, p, tme, cub;
        if constexpr (EK == EXPK_TABLE) {
            e = table_lookup(tr.tab, tr.n, tr.dx, tr.max, tau);
            p = 1.0f - e;
            tme = tau - e;
            cub = tau * (tau * (tau - 3.0f) + 6.0f) - 6.0f * e;
        } else if constexpr (EK == EXPK_PLAIN) {
            p = ex2_approx(tau * -1.44269504088896341f);
            e = 1.0f - p;
            tme = tau - e;
            cub = tau * (tau * (tau - 3.0f) + 6.0f) - 6.0f * e;
        } else {
            if (tau < 0.25f) {
                e = one_minus_exp_series(tau);
                tme = tau_minus_e_series(tau);
                p = 1.0f - e;
            } else {
                p = exp_neg_rr(tau);
                e = 1.0f - p;
                tme = tau - e;
            }
            cub = tau < 1.0f ? cubic_series(tau) : tau * (tau * (tau - 3.0f)) + 6.0f * tme;
        }
        const float rs = rcp_approx(s);
        const float rs2 = rs * rs;
        const float reuse = fmaf(tau, tau - 2.0f, 2.0f * e * (rs * rs2));
        float fi;
        if constexpr (EK == EXPK_STABLE) {
            // (q0 tau + (s psi - q0) e)/s^2 == q0 (tau - e)/s^2 + psi e/s, exactly
            fi = fmaf(a0 * tme, rs2, ps * e * rs);
        } else {
            fi = (fmaf(s, ps, -a0) * e + a0 * tau) * rs2;
        }
        fi = fmaf(a1, reuse, fi);
        fi = fmaf(a2 * cub, rs2 * rs2 * (1.0f / 3.0f), fi);
        tally.v[k] = weight * fi;
        float pn = a0 * e * rs;
        pn = fmaf(a1 * tme, rs2, pn);
        pn = fmaf(a2, reuse, pn);
        psi.v[k] = fmaf(ps, p, pn);
    }
}

template <int VEC>
__device__ __forceinline__ void load_rows(const SweepParams &P, int r, int iv, int g0,
                                          Rows<VEC> &x)
{
    x.s = ld_row<VEC>(P.sigT + (int64_t)r * P.Gs + g0);
    const float *c = P.coef + ((int64_t)r * P.I + iv) * 3 * P.Gs + g0;
    x.a0 = ld_row<VEC>(c);
    x.a1 = ld_row<VEC>(c + P.Gs);
    if (iv > 0 && iv < P.I - 1) {
        x.a2 = ld_row<VEC>(c + 2 * P.Gs);
    } else {
#pragma unroll
        for (int k = 0; k < VEC; k++) x.a2.v[k] = 0.0f;
    }
}

__device__ __forceinline__ void load_desc(const SweepParams &P, int64_t j, int64_t end,
                                          int &r, int &iv, float &d)
{
    if (j < end) {
        r = ld_stream(P.reg + j);
        iv = ld_stream(P.itv + j);
        d = ld_stream(P.ds + j);
    } else {
        r = 0;
        iv = 0;
        d = 0.0f;
    }
}

template <int VEC, int EK>
__device__ __forceinline__ void sweep_item(const SweepParams &P, int64_t item, int lane,
                                           const TableRef &tr)
{
    const int t = (int)(item / P.n_chunks);
    const int ch = (int)(item - (int64_t)t * P.n_chunks);
    const int g0 = (ch * 32 + lane) * VEC;
    const int nvalid = P.G - g0;
    const bool act = nvalid > 0;
    const int64_t beg = P.off[t], end = P.off[t + 1];
    if (!(beg >= 0 && beg <= end && end <= P.S)) {
        if (lane == 0) atomicOr(P.err, DEVERR_OFFSETS);
        return;
    }
    float *psi_row = P.psi + (int64_t)t * P.Gs + g0;
    Vec<VEC> psi;
    if (act) psi = ld_psi<VEC>(psi_row, nvalid);

    // Descriptor windows: A = segments [wb, wb+32), B = the next 32.
    int64_t wb = beg;
    int rA, iA, rB, iB;
    float dA, dB;
    load_desc(P, wb + lane, end, rA, iA, dA);
    load_desc(P, wb + 32 + lane, end, rB, iB, dB);

    Rows<VEC> cur;
    int rc = __shfl_sync(FULL, rA, 0), ic = __shfl_sync(FULL, iA, 0);
    float dc = __shfl_sync(FULL, dA, 0);
    bool okc = (unsigned)rc < (unsigned)P.R && (unsigned)ic < (unsigned)P.I;
    if (beg < end && okc && act) load_rows<VEC>(P, rc, ic, g0, cur);

    for (int64_t j = beg; j < end; ++j) {
        Rows<VEC> nxt;
        int rn = 0, in_ = 0;
        float dn = 0.0f;
        bool okn = false;
        const int64_t jn = j + 1;
        if (jn < end) {
            int k = (int)(jn - wb);
            if (k == 32) {
                rA = rB; iA = iB; dA = dB;
                wb += 32;
                k = 0;
                load_desc(P, wb + 32 + lane, end, rB, iB, dB);
            }
            rn = __shfl_sync(FULL, rA, k);
            in_ = __shfl_sync(FULL, iA, k);
            dn = __shfl_sync(FULL, dA, k);
            okn = (unsigned)rn < (unsigned)P.R && (unsigned)in_ < (unsigned)P.I;
            if (okn && act) load_rows<VEC>(P, rn, in_, g0, nxt);
        }
        if (okc) {
            if (act) {
                Vec<VEC> tally;
                attenuate<VEC, EK>(cur, dc, P.weight, tr, psi, tally);
                red_row<VEC>(P.ff + ((int64_t)rc * P.I + ic) * P.Gs + g0, tally, nvalid);
            }
        } else if (lane == 0) {
            atomicOr(P.err, DEVERR_INDEX);
        }
        cur = nxt;
        rc = rn;
        ic = in_;
        dc = dn;
        okc = okn;
    }
    if (act) st_psi<VEC>(psi_row, psi, nvalid);
}

template <int VEC, int EK>
__global__ void __launch_bounds__(256) fwd_kernel(const SweepParams P)
{
    extern __shared__ float2 s_tab[];
    TableRef tr{nullptr, 0, 0.0f, 0.0f};
    if constexpr (EK == EXPK_TABLE) {
        const float2 *src = reinterpret_cast<const float2 *>(P.table);
        for (int k = threadIdx.x; k < P.tab_n; k += blockDim.x) s_tab[k] = src[k];
        __syncthreads();
        tr = TableRef{s_tab, P.tab_n, P.tab_dx, P.tab_max};
    }
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(P.counter, 1ULL);
        item = __shfl_sync(FULL, item, 0);
        if (item >= (unsigned long long)P.n_items) break;
        sweep_item<VEC, EK>(P, (int64_t)item, lane, tr);
    }
}

// Checked mode: offsets monotone inside [0, S], indices in range.
__global__ void check_kernel(const SweepParams P)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int bad = 0;
    for (int64_t t = tid; t < P.T; t += stride) {
        const int64_t b = P.off[t], e = P.off[t + 1];
        if (!(b >= 0 && b <= e && e <= P.S)) bad |= DEVERR_OFFSETS;
    }
    if (tid == 0 && (P.off[0] != 0 || P.off[P.T] != P.S)) bad |= DEVERR_OFFSETS;
    for (int64_t j = tid; j < P.S; j += stride) {
        if ((unsigned)P.reg[j] >= (unsigned)P.R || (unsigned)P.itv[j] >= (unsigned)P.I)
            bad |= DEVERR_INDEX;
    }
    if (bad) atomicOr(P.err, bad);
}

template <int VEC, int EK>
const void *fwd_fn()
{
    return reinterpret_cast<const void *>(&fwd_kernel<VEC, EK>);
}

const void *pick(const FwdConfig &c)
{
#define MOC_PICK(V)                                                 \
    if (c.vec == V) {                                               \
        if (c.exp_kind == EXPK_PLAIN) return fwd_fn<V, EXPK_PLAIN>();   \
        if (c.exp_kind == EXPK_TABLE) return fwd_fn<V, EXPK_TABLE>();   \
        if (c.exp_kind == EXPK_STABLE) return fwd_fn<V, EXPK_STABLE>(); \
    }
    MOC_PICK(1)
    MOC_PICK(2)
    MOC_PICK(4)
#undef MOC_PICK
    return nullptr;
}

}  // namespace

cudaError_t launch_prep_coef(const float *source, float *coef, int R, int I, int Gs,
                             float dz, float zin, float mu, float mu2, cudaStream_t st)
{
    const int64_t n = (int64_t)R * I * Gs;
    if (n == 0) return cudaSuccess;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    prep_coef_kernel<<<blocks, 256, 0, st>>>(source, coef, R, I, Gs, dz, zin, mu, mu2);
    return cudaGetLastError();
}

int fwd_blocks_per_sm(const FwdConfig &c, size_t smem)
{
    const void *fn = pick(c);
    if (!fn || c.warps_per_block < 1 || c.warps_per_block > 8) return 0;
    int n = 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, c.warps_per_block * 32, smem) !=
        cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_fwd(const SweepParams &p, const FwdConfig &c, cudaStream_t st)
{
    const void *fn = pick(c);
    if (!fn || c.warps_per_block < 1 || c.warps_per_block > 8 || c.blocks < 1)
        return cudaErrorInvalidValue;
    const size_t smem = c.exp_kind == EXPK_TABLE ? (size_t)p.tab_n * sizeof(float2) : 0;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    SweepParams copy = p;
    void *args[] = {&copy};
    return cudaLaunchKernel(fn, dim3(c.blocks), dim3(c.warps_per_block * 32), args, smem, st);
}

cudaError_t launch_check(const SweepParams &p, cudaStream_t st)
{
    int64_t work = p.S > p.T ? p.S : p.T;
    int blocks = (int)((work + 255) / 256);
    if (blocks < 1) blocks = 1;
    if (blocks > 152 * 8) blocks = 152 * 8;
    check_kernel<<<blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace moc
