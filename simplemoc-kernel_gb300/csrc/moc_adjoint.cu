// moc_adjoint.cu — reverse-mode derivative of the sweep (moc_attenuate_adj).
//
// For L = sum w . fine_flux_out + sum v . psi_out the gradients with respect to sigT,
// the fine source and the incoming psi are accumulated by one reverse sweep per track.
// Per segment and group (tau = s ds, e = 1 - exp(-tau), p = exp(-tau), tme = tau - e,
// cub = tau(tau(tau-3)+6) - 6e, reuse = tau(tau-2) + 2e/s^3, a1 = q1 mu, a2 = q2 mu2):
//   FI   = a0 tme/s^2 + psi e/s + a1 reuse + a2 cub/(3 s^4)         (tally / weight)
//   psi' = a0 e/s + a1 tme/s^2 + a2 reuse + psi p
// (src/cpu/kernel.c:233-331 with (q0 tau + (s psi - q0) e)/s^2 = q0 tme/s^2 + psi e/s).
// With lambda = dL/dpsi' and W = weight * w[cell]:
//   dL/ds   += lambda dpsi'/ds + W dFI/ds
//   dL/da_k += lambda dpsi'/da_k + W dFI/da_k
//   lambda  <- lambda p + W e/s                                       (dL/dpsi)
// where, with D1 = tau e - 2 tme, D2 = tau p - e, D3 = tau dcub/dtau - 4 cub,
//   dFI/ds   = a0 D1/s^3 + psi D2/s^2 + a1 dreuse/ds + a2 D3/(3 s^5)
//   dpsi'/ds = a0 D2/s^2 + a1 D1/s^3 + a2 dreuse/ds - psi p ds
//   dreuse/ds = (2 tau - 2) tau/s + (2 tau p - 6 e)/s^4.
// D1, D2 and D3 cancel for small tau (D3 ~ -tau^5/20 from tau^4 terms); below tau = 2
// they come from a fitted polynomial of their series, like the forward's stable terms. The exponentials
// are recomputed from tau in the reverse sweep instead of being stored; psi entering
// each segment is recorded by a first forward pass (one float per segment and group).
//
// Long tracks are split into chunks as in the forward (moc_split.cu): lambda obeys
// lambda_in = p lambda_out + W e/s, affine backwards with the same factor a = prod p as
// psi forwards, so one map pass gives (a, b, c) per chunk, a scan over each track's
// chunks gives psi entering and lambda leaving every chunk, and the recording and
// reverse passes then run all chunks in parallel.
#include "moc_device.cuh"
#include "moc_internal.h"

namespace moc {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// Every term the reverse sweep needs, accurate for all tau >= 0 (cub3 = cub / 3,
// d33 = D3 / 3).
struct AdjTerms {
    float e, p, tme, cub3, d1, d2, d33;
};

__device__ __forceinline__ AdjTerms adj_terms(float tau)
{
    AdjTerms r;
    if (tau < 2.0f) {
        // s4 = sum_{k>=4} (-1)^k tau^k / k! = tau^4 h, h = 1/24 - tau h5, with
        // h5 = sum_{j>=0} (-tau)^j / (j+5)!: a degree-5 polynomial fitted to the series on
        // [0, 2] for least maximum relative error (weighted least squares on Chebyshev
        // points, reweighted until the error equioscillates), within 1.3e-7 of h5 with FP32
        // Horner steps, as the Taylor sum through tau^16 is. The threshold 2 keeps warps
        // whose groups have tau up to 2 on this branch.
        float h5 = fmaf(-1.626123236e-07f, tau, 2.524867341e-06f);
        h5 = fmaf(h5, tau, -2.457161099e-05f);
        h5 = fmaf(h5, tau, 1.983064285e-04f);
        h5 = fmaf(h5, tau, -1.388870645e-03f);
        h5 = fmaf(h5, tau, 8.333332837e-03f);
        const float h = fmaf(h5, -tau, 1.0f / 24.0f);
        const float t2 = tau * tau, t3 = t2 * tau, t4 = t2 * t2;
        const float s4 = h * t4;
        r.cub3 = 2.0f * s4;
        r.tme = fmaf(t2, fmaf(tau, -1.0f / 6.0f, 0.5f), s4);
        r.e = tau - r.tme;
        r.p = 1.0f - r.e;
        // D1 = tau e - 2 tme = -tau^3/6 + tau^4/6 - (tau + 2) s4
        r.d1 = fmaf(-(tau + 2.0f), s4, t3 * fmaf(tau, 1.0f / 6.0f, -1.0f / 6.0f));
        // D2 = tau p - e = -tau^2/2 + tau^3/3 - tau^4/6 + (1 + tau) s4
        r.d2 = fmaf(1.0f + tau, s4, t2 * fmaf(tau, fmaf(tau, -1.0f / 6.0f, 1.0f / 3.0f), -0.5f));
        // D3 = tau dcub/dtau - 4 cub with dcub/dtau = tau^3 - 6 s4:
        //    = tau^4 - (6 tau + 24) s4 = tau^5 ((6 tau + 24) h5 - 1/4)
        // (-1/4 against ~1/5: the leading terms cancel 5-fold at small tau, 9-fold at 2)
        r.d33 = t4 * tau * fmaf(fmaf(2.0f, tau, 8.0f), h5, -1.0f / 12.0f);
    } else {
        // little cancellation from tau = 2 on: one ex2.approx
        r.p = ex2_approx(tau * -1.44269504088896341f);
        r.e = 1.0f - r.p;
        r.tme = tau - r.e;
        // cub / 3 = tau^2 (tau/3 - 1) + 2 tme; dcub/dtau / 3 = tau (tau - 2) + 2 e
        r.cub3 = fmaf(tau * tau, fmaf(tau, 1.0f / 3.0f, -1.0f), r.tme + r.tme);
        r.d1 = fmaf(tau, r.e, -2.0f * r.tme);
        r.d2 = fmaf(tau, r.p, -r.e);
        r.d33 = fmaf(tau, fmaf(tau, tau - 2.0f, r.e + r.e), -4.0f * r.cub3);
    }
    return r;
}

// The pair layout of the cell blocks for lanes holding pairs of groups (f32_pairs(VEC)):
// groups 2j and 2j + 1 of the lane in two float4, (s_a, s_b, a0_a, a0_b) and
// (a1_a, a1_b, a2_a, a2_b). blk_group reads group k of a lane's blocks in either layout.
template <int VEC>
__device__ __forceinline__ float4 blk_group(const float4 (&b)[VEC], int k)
{
    if constexpr (f32_pairs(VEC)) {
        const float4 u = b[k & ~1], v = b[k | 1];
        return (k & 1) ? make_float4(u.y, u.w, v.y, v.w) : make_float4(u.x, u.z, v.x, v.z);
    } else {
        return b[k];
    }
}

__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

// psi' of one segment, for the recording pass and the chunk maps: the forward sweep's
// arithmetic (one ex2.approx for p, e = 1 - p). psi only needs the forward's FP32
// accuracy, which the plain exponential meets; the cancelling derivative terms of the
// reverse pass come from their series (adj_terms). Also returns p and e/s. With pairs of
// groups (f32_pairs(VEC)) b holds them in the pair layout and the packed FP32 form runs
// (fma/mul/add .rn.f32x2: one instruction, two groups): every packed operation stands
// for the same scalar operation, with 1 - x and a - b written fma(x, -1, 1) and
// fma(b, -1, a), which round once to the same value, so both forms give identical bits.
template <int VEC>
__device__ __forceinline__ void advance(const float4 (&b)[VEC], float ds, Vec<VEC> &psi,
                                        Vec<VEC> &pv, Vec<VEC> &e1v)
{
    if constexpr (f32_pairs(VEC)) {
#pragma unroll
        for (int k = 0; k < VEC; k += 2) {
            const float2 s = make_float2(b[k].x, b[k].y), a0 = make_float2(b[k].z, b[k].w);
            const float2 a1 = make_float2(b[k + 1].x, b[k + 1].y);
            const float2 a2 = make_float2(b[k + 1].z, b[k + 1].w);
            const float2 tau = __fmul2_rn(s, dup2(ds));
            const float2 m = __fmul2_rn(tau, dup2(-1.44269504088896341f));
            const float2 p = make_float2(ex2_approx(m.x), ex2_approx(m.y));
            const float2 e = __ffma2_rn(p, dup2(-1.0f), dup2(1.0f));
            const float2 tme = __ffma2_rn(e, dup2(-1.0f), tau);
            const float2 rs = make_float2(rcp_approx(s.x), rcp_approx(s.y));
            const float2 rs2 = __fmul2_rn(rs, rs);
            const float2 e1 = __fmul2_rn(e, rs), t2 = __fmul2_rn(tme, rs2);
            const float2 reuse = __ffma2_rn(__fadd2_rn(e1, e1), rs2,
                                            __fmul2_rn(tau, __fadd2_rn(tau, dup2(-2.0f))));
            float2 pn = __ffma2_rn(a1, t2, __fmul2_rn(a0, e1));
            pn = __ffma2_rn(a2, reuse, pn);
            const float2 np = __ffma2_rn(make_float2(psi.v[k], psi.v[k + 1]), p, pn);
            psi.v[k] = np.x;
            psi.v[k + 1] = np.y;
            pv.v[k] = p.x;
            pv.v[k + 1] = p.y;
            e1v.v[k] = e1.x;
            e1v.v[k + 1] = e1.y;
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < VEC; k++) {
        const float s = b[k].x, a0 = b[k].y, a1 = b[k].z, a2 = b[k].w;
        const float tau = s * ds;
        const float p = ex2_approx(tau * -1.44269504088896341f);
        const float e = 1.0f - p;
        const float tme = tau - e;
        const float rs = rcp_approx(s), rs2 = rs * rs;
        const float e1 = e * rs, t2 = tme * rs2;
        const float reuse = fmaf(e1 + e1, rs2, tau * (tau - 2.0f));
        float pn = fmaf(a1, t2, a0 * e1);
        pn = fmaf(a2, reuse, pn);
        psi.v[k] = fmaf(psi.v[k], p, pn);
        pv.v[k] = p;
        e1v.v[k] = e1;
    }
}

// Segment j of [lo, hi): its cell and ds; outside the range or with a bad index, cell
// `none` and ds = 0 (-1 to be skipped, or the null cell R*I: an exact no-op).
__device__ __forceinline__ void decode(const SweepParams &P, int64_t j, int64_t lo, int64_t hi,
                                       int none, int &cell, float &ds)
{
    cell = none;
    ds = 0.0f;
    if (j >= lo && j < hi) {
        const int r = ld_stream(P.reg + j);
        const int iv = ld_stream(P.itv + j);
        const float d = ld_stream(P.ds + j);
        if ((unsigned)r < (unsigned)P.R && (unsigned)iv < (unsigned)P.I) {
            cell = r * P.I + iv;
            ds = d;
        } else {
            atomicOr(P.err, DEVERR_INDEX);
        }
    }
}

template <int VEC>
__device__ __forceinline__ void load4(const float4 *p, float4 (&b)[VEC])
{
#pragma unroll
    for (int k = 0; k < VEC; k++) b[k] = __ldg(p + k);
}

// Work item of an adjoint pass: (track, group chunk), or (chunk record, group chunk)
// when long tracks are split; a record's chunk starts from its precomputed psi (forward)
// or lambda (reverse).
struct AdjItem {
    int64_t beg, end, q;  // q: the record (split tracks) or -1
    int t, g0, flags;
};

// Items are numbered group chunk by group chunk (see the forward sweep): item =
// chunk * n_units + unit, n_units the tracks or records.
__device__ __forceinline__ bool adj_item(const SweepParams &P, int64_t item, int64_t n_units,
                                         int lane, int vec, AdjItem &it)
{
    const int ch = (int)(item / n_units);
    const int64_t u = item - (int64_t)ch * n_units;
    it.g0 = (ch * 32 + lane) * vec;
    if (P.rec) {
        const int4 r = __ldg(P.rec + u);
        it.q = u;
        it.t = r.w;
        it.flags = r.z;
        it.beg = (int64_t)(uint32_t)r.x | ((int64_t)r.y << 32);
        it.end = it.beg + (r.z & CHUNK_LEN_MASK);
        if (!(it.beg >= 0 && it.end <= P.S && (unsigned)r.w < (unsigned)P.T)) {
            if (lane == 0) atomicOr(P.err, DEVERR_OFFSETS);
            return false;
        }
        return true;
    }
    it.q = -1;
    it.t = (int)u;
    it.flags = CHUNK_SINGLE;
    it.beg = P.off[u];
    it.end = P.off[u + 1];
    if (!(it.beg >= 0 && it.beg <= it.end && it.end <= P.S)) {
        if (lane == 0) atomicOr(P.err, DEVERR_OFFSETS);
        return false;
    }
    return true;
}

// Units of a pass: tracks, or records of split tracks.
__device__ __forceinline__ int64_t adj_units(const SweepParams &P)
{
    if (!P.rec) return P.T;
    const int64_t n = *P.n_rec;
    return n < P.rec_cap ? n : P.rec_cap;
}

// One segment's inputs for the reverse sweep, fetched one segment ahead.
template <int VEC>
struct RevSeg {
    int c;
    float d;
    float4 b[VEC];
    Vec<VEC> psi, w;
};

// Full-row gradient reduction of one group, sent only where (unsigned) cell < lim (lim is
// R*I on active lanes and 0 on idle ones; the null cell R*I sends nothing). Padding groups
// of an active lane land in the workspace's padding, which the finish pass ignores.
//
// Slots of the gradient blocks: within each chunk of 32 VEC groups starting at group b,
// the q-th group of lane l (group b + VEC l + q) is kept at slot b + L q + l, L the lanes
// the chunk's storage spans (min(32, (Gs - b) / VEC)). A warp's q-th reduction then covers
// L consecutive 16-byte slots, whole 32-byte sectors, where slots in group order would
// leave every sector half-covered by each of two reductions (twice the L2 reduction
// traffic, which bounds the reverse pass).
// grad_of returns group g's (dL/ds, dL/da0, dL/da1, dL/da2) from a cell's row of slots.
__device__ __forceinline__ float4 grad_of(const float4 *row, int g, int vec, int Gs)
{
    const int b = g / (32 * vec) * (32 * vec), w = g - b;
    const int L = (Gs - b) / vec < 32 ? (Gs - b) / vec : 32;
    return row[b + L * (w % vec) + w / vec];
}
__device__ __forceinline__ void red4_if(float4 *p, const float4 &g, int cell, int lim)
{
    asm volatile("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %5, %6;\n\t"
                 "@q red.global.add.v4.f32 [%0], {%1, %2, %3, %4};\n\t}"
                 ::"l"(p), "f"(g.x), "f"(g.y), "f"(g.z), "f"(g.w), "r"(cell), "r"(lim)
                 : "memory");
}

// The reverse sweep of one segment for VEC groups: gradient block scattered, lambda
// carried back. The forward is built from four functions of (s, tau):
//   f1 = e/s, f2 = tme/s^2, f3 = reuse, f4 = cub/(3 s^4);
//   FI = a0 f2 + psi f1 + a1 f3 + a2 f4,   psi' = a0 f1 + a1 f2 + a2 f3 + psi p,
// and their s-derivatives are f1' = D2/s^2, f2' = D1/s^3, f3' = dreuse/ds,
// f4' = D3/(3 s^5). So, with lambda = dL/dpsi' and W = weight w[cell]:
//   dL/da_k  = lambda f_{k+1} + W f_{k+2}                     (k = 0, 1, 2)
//   dL/ds    = sum_k a_k (lambda f'_{k+1} + W f'_{k+2}) + psi (W f1' - lambda ds p)
//   lambda  <- lambda p + W f1.
template <int VEC>
__device__ __forceinline__ void reverse_segment(const AdjParams &A, const RevSeg<VEC> &sg,
                                                Vec<VEC> &lam, float4 *gb, int gstride,
                                                int lim)
{
#pragma unroll
    for (int q = 0; q < VEC; q++) {
        const float4 bq = blk_group<VEC>(sg.b, q);
        const float s = bq.x, a0 = bq.y, a1 = bq.z, a2 = bq.w;
        const float d = sg.d;
        const float ps = sg.psi.v[q], la = lam.v[q], W = A.fw.weight * sg.w.v[q];
        const float tau = s * d;
        const AdjTerms x = adj_terms(tau);
        const float rs = rcp_approx(s), rs2 = rs * rs, rs3 = rs2 * rs;
        const float rs4 = rs2 * rs2;
        const float f1 = x.e * rs, f2 = x.tme * rs2;
        const float f3 = fmaf(tau, tau - 2.0f, (x.e + x.e) * rs3);
        const float f4 = x.cub3 * rs4;
        const float g1 = x.d2 * rs2, g2 = x.d1 * rs3;
        const float g3 = fmaf((tau + tau - 2.0f) * tau, rs, fmaf(tau + tau, x.p, -6.0f * x.e) * rs4);
        const float g4 = x.d33 * rs4 * rs;
        float4 gr;
        gr.y = fmaf(la, f1, W * f2);
        gr.z = fmaf(la, f2, W * f3);
        gr.w = fmaf(la, f3, W * f4);
        float gs = ps * fmaf(W, g1, -la * d * x.p);
        gs = fmaf(a0, fmaf(la, g1, W * g2), gs);
        gs = fmaf(a1, fmaf(la, g2, W * g3), gs);
        gs = fmaf(a2, fmaf(la, g3, W * g4), gs);
        gr.x = gs;
        lam.v[q] = fmaf(la, x.p, W * f1);
        red4_if(gb + sg.c * A.fw.Gs + q * gstride, gr, sg.c, lim);
    }
}

template <int VEC>
__global__ void __launch_bounds__(256) adj_forward_kernel(const AdjParams A)
{
    const SweepParams &P = A.fw;
    const int lane = threadIdx.x & 31;
    const int64_t n_units = adj_units(P), n_items = n_units * P.n_chunks;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(P.counter, 1ULL);
        item = __shfl_sync(FULL, item, 0);
        if (item >= (unsigned long long)n_items) break;
        AdjItem it;
        if (!adj_item(P, (int64_t)item, n_units, lane, VEC, it)) continue;
        const int g0 = it.g0;
        const int64_t beg = it.beg, end = it.end;
        const int nvalid = P.G - g0;
        const bool act = nvalid > 0;
        const int Gs = P.Gs;
        // idle lanes (groups past G) read group 0 and store nothing
        const float4 *bb = static_cast<const float4 *>(P.blk) + (act ? g0 : 0);
        const float *psi_src = (it.flags & CHUNK_SINGLE) ? P.psi + (int64_t)it.t * Gs
                                                         : P.start + it.q * Gs;
        Vec<VEC> psi;
#pragma unroll
        for (int k = 0; k < VEC; k++) psi.v[k] = 0.0f;
        if (act) psi = ld_psi<VEC>(psi_src + g0, nvalid);
        float *hist = A.hist + g0;
        // Branch-free, as the forward sweep: descriptor windows A = [wb, wb+32) and B = the
        // next 32; segments past the end or with bad indices decode to the null cell (an
        // exact no-op of advance: tau = 0, p = 1, every term 0) and store no history; the
        // pair loop keeps the blocks of segments k and k+1 in two buffers in turn.
        const int nullc = P.null_cell;
        int64_t wb = beg;
        int cA, cB;
        float dA, dB;
        decode(P, wb + lane, beg, end, nullc, cA, dA);
        decode(P, wb + 32 + lane, beg, end, nullc, cB, dB);
        float4 b0[VEC], b1[VEC];
        int c0 = __shfl_sync(FULL, cA, 0), c1;
        float d0 = __shfl_sync(FULL, dA, 0), d1;
        load4<VEC>(bb + c0 * Gs, b0);
        Vec<VEC> pv, e1v;
        for (; wb < end; wb += 32) {
            const int nk = end - wb < 32 ? (int)(end - wb) : 32;
            for (int k = 0; k < nk; k += 2) {
                c1 = __shfl_sync(FULL, cA, k + 1);
                d1 = __shfl_sync(FULL, dA, k + 1);
                load4<VEC>(bb + c1 * Gs, b1);
                if (act) st_psi<VEC>(hist + (wb + k) * Gs, psi, nvalid);
                advance<VEC>(b0, d0, psi, pv, e1v);
                const int kn = k + 2;
                const int cs = kn < 32 ? cA : cB;
                const float dsn = kn < 32 ? dA : dB;
                c0 = __shfl_sync(FULL, cs, kn & 31);
                d0 = __shfl_sync(FULL, dsn, kn & 31);
                load4<VEC>(bb + c0 * Gs, b0);
                if (act && k + 1 < nk) st_psi<VEC>(hist + (wb + k + 1) * Gs, psi, nvalid);
                advance<VEC>(b1, d1, psi, pv, e1v);
            }
            cA = cB;
            dA = dB;
            decode(P, wb + 64 + lane, beg, end, nullc, cB, dB);
        }
    }
}

template <int VEC>
__global__ void __launch_bounds__(256) adj_reverse_kernel(const AdjParams A)
{
    const SweepParams &P = A.fw;
    const int lane = threadIdx.x & 31;
    const int64_t n_units = adj_units(P), n_items = n_units * P.n_chunks;
    const int nullc = P.null_cell;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(P.counter, 1ULL);
        item = __shfl_sync(FULL, item, 0);
        if (item >= (unsigned long long)n_items) break;
        AdjItem it;
        if (!adj_item(P, (int64_t)item, n_units, lane, VEC, it)) continue;
        const int g0 = it.g0;
        const int64_t beg = it.beg, end = it.end;
        const int nvalid = P.G - g0;
        const bool act = nvalid > 0;
        const int Gs = P.Gs;
        // idle lanes (groups past G) read group 0 and send nothing
        const int gl = act ? g0 : 0;
        const int lim = act ? nullc : 0;
        const float4 *bb = static_cast<const float4 *>(P.blk) + gl;
        // this lane's gradient slots: chunk base + lane, then every L slots (grad_of)
        const int cb0 = g0 - lane * VEC;
        const int gstride = (Gs - cb0) / VEC < 32 ? (Gs - cb0) / VEC : 32;
        float4 *gb = A.gblk + cb0 + lane;
        const bool single = (it.flags & CHUNK_SINGLE) != 0;
        const float *lam_src = single ? A.v + (int64_t)it.t * Gs : A.lam_end + it.q * Gs;
        Vec<VEC> lam;
        if (act) lam = ld_psi<VEC>(lam_src + g0, nvalid);
        // Descriptor windows aligned to the item's end: A = [wa, wa+32), B = the 32 before
        // it; segments below beg decode to the null cell (no-ops). The pair loop walks k =
        // 31, 30, ... of window A with two fetch slots in turn (no copies); only the pair at
        // a window's start reaches into window B.
        int64_t wa = end - 32;
        int cA, cB;
        float dA, dB;
        decode(P, wa + lane, beg, end, nullc, cA, dA);
        decode(P, wa - 32 + lane, beg, end, nullc, cB, dB);
        auto fetch = [&](int c, float d, int64_t j, RevSeg<VEC> &sg) {
            sg.c = c;
            sg.d = d;
            const int64_t jl = j < beg ? beg : j;  // a null segment below beg reads row beg
            const int cw = c < nullc ? c : 0;      // the null cell has no w row
            load4<VEC>(bb + c * Gs, sg.b);
            sg.psi = ld_psi<VEC>(A.hist + jl * Gs + gl, VEC);
            sg.w = ld_psi<VEC>(A.w + cw * Gs + gl, VEC);
        };
        RevSeg<VEC> s0, s1;
        if (end > beg) {
            fetch(__shfl_sync(FULL, cA, 31), __shfl_sync(FULL, dA, 31), wa + 31, s0);
            for (; wa + 31 >= beg; wa -= 32) {
                const int klo = beg > wa ? (int)(beg - wa) : 0;
                for (int k = 31; k >= klo; k -= 2) {
                    fetch(__shfl_sync(FULL, cA, k - 1), __shfl_sync(FULL, dA, k - 1),
                          wa + k - 1, s1);
                    reverse_segment<VEC>(A, s0, lam, gb, gstride, lim);
                    const int kn = k - 2;
                    const int cs = kn >= 0 ? cA : cB;
                    const float dsn = kn >= 0 ? dA : dB;
                    fetch(__shfl_sync(FULL, cs, kn & 31), __shfl_sync(FULL, dsn, kn & 31),
                          wa + kn, s0);
                    reverse_segment<VEC>(A, s1, lam, gb, gstride, lim);
                }
                cA = cB;
                dA = dB;
                decode(P, wa - 64 + lane, beg, end, nullc, cB, dB);
            }
        }
        if (act && (single || (it.flags & CHUNK_FIRST)))
            st_psi<VEC>(A.dpsi_in + (int64_t)it.t * Gs + g0, lam, nvalid);
    }
}

// Maps of every chunk of a split track, per group: psi_out = a psi_in + b (forward) and
// lambda_in = a lambda_out + c (reverse), with a the product of the chunk's p and
// c = sum_j (product of p before segment j) W_j e_j / s_j, the chunk's lambda sources
// carried to its start. The arithmetic is the recording pass's (advance); the segment loop
// is the recording pass's branch-free windowed pair loop (segments past the chunk's end
// decode to the null cell, an exact no-op with W = 0). Map items are full chunks of equal
// length, so a static warp-strided assignment balances them without a queue atomic.
template <int VEC>
__global__ void __launch_bounds__(256) adj_map_kernel(const AdjParams A)
{
    const SweepParams &P = A.fw;
    const int lane = threadIdx.x & 31;
    int64_t n_maps = *P.n_map;
    n_maps = n_maps < P.rec_cap ? n_maps : P.rec_cap;
    const int64_t n_items = n_maps * P.n_chunks;
    const int64_t n_units = adj_units(P);
    const int nullc = P.null_cell;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t item = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
         item < n_items; item += nw) {
        const int ch = (int)(item / n_maps);
        const int64_t m = item - (int64_t)ch * n_maps;
        const int64_t q = P.map_list[m];
        if ((uint64_t)q >= (uint64_t)n_units) continue;
        AdjItem it;
        if (!adj_item(P, (int64_t)ch * n_units + q, n_units, lane, VEC, it)) continue;
        const int g0 = it.g0;
        const int64_t beg = it.beg, end = it.end;
        const int nvalid = P.G - g0;
        const bool act = nvalid > 0;
        const int Gs = P.Gs;
        // idle lanes (groups past G) read group 0 and store nothing
        const int gl = act ? g0 : 0;
        const float4 *bb = static_cast<const float4 *>(P.blk) + gl;
        Vec<VEC> ma, mb, mc;
#pragma unroll
        for (int k = 0; k < VEC; k++) {
            ma.v[k] = 1.0f;
            mb.v[k] = 0.0f;
            mc.v[k] = 0.0f;
        }
        // a segment's blocks and loss weights (none for the null cell)
        auto fetch = [&](int c, float4 (&b)[VEC], Vec<VEC> &wv) {
            load4<VEC>(bb + c * Gs, b);
            wv = ld_psi<VEC>(A.w + (c < nullc ? c : 0) * Gs + gl, VEC);
            if (c >= nullc) {
#pragma unroll
                for (int k = 0; k < VEC; k++) wv.v[k] = 0.0f;
            }
        };
        auto step = [&](const float4 (&b)[VEC], float d, const Vec<VEC> &wv) {
            Vec<VEC> pv, e1v;
            advance<VEC>(b, d, mb, pv, e1v);
#pragma unroll
            for (int k = 0; k < VEC; k++) {
                mc.v[k] = fmaf(ma.v[k], P.weight * wv.v[k] * e1v.v[k], mc.v[k]);
                ma.v[k] *= pv.v[k];
            }
        };
        int64_t wb = beg;
        int cA, cB;
        float dA, dB;
        decode(P, wb + lane, beg, end, nullc, cA, dA);
        decode(P, wb + 32 + lane, beg, end, nullc, cB, dB);
        float4 b0[VEC], b1[VEC];
        Vec<VEC> w0, w1;
        int c0 = __shfl_sync(FULL, cA, 0), c1;
        float d0 = __shfl_sync(FULL, dA, 0), d1;
        fetch(c0, b0, w0);
        for (; wb < end; wb += 32) {
            const int nk = end - wb < 32 ? (int)(end - wb) : 32;
            for (int k = 0; k < nk; k += 2) {
                c1 = __shfl_sync(FULL, cA, k + 1);
                d1 = __shfl_sync(FULL, dA, k + 1);
                fetch(c1, b1, w1);
                step(b0, d0, w0);
                const int kn = k + 2;
                const int cs = kn < 32 ? cA : cB;
                const float dsn = kn < 32 ? dA : dB;
                c0 = __shfl_sync(FULL, cs, kn & 31);
                d0 = __shfl_sync(FULL, dsn, kn & 31);
                fetch(c0, b0, w0);
                step(b1, d1, w1);
            }
            cA = cB;
            dA = dB;
            decode(P, wb + 64 + lane, beg, end, nullc, cB, dB);
        }
        if (act) {
            st_psi<VEC>(P.map_a + q * Gs + g0, ma, nvalid);
            st_psi<VEC>(P.map_b + q * Gs + g0, mb, nvalid);
            st_psi<VEC>(A.map_c + q * Gs + g0, mc, nvalid);
        }
    }
}

// psi entering and lambda leaving every chunk of the split tracks: one warp per (split
// track, 32-group slice, direction), its lanes over the slice's groups: psi_0 = psi_in,
// psi_{k+1} = a_k psi_k + b_k forwards; lambda leaving the last chunk = dL/dpsi_out,
// lambda leaving chunk k-1 = a_k lambda_k + c_k backwards. The maps of 8 chunks are
// loaded ahead of their 8 dependent FMAs. The split tracks are found from whichever list
// is shorter: the tracks (by_track), or the map items, which hold every chunk of a split
// track and so its first chunk once.
__global__ void adj_start_kernel(const AdjParams A)
{
    const SweepParams &P = A.fw;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float *__restrict__ ma = P.map_a;
    const float *__restrict__ mb = P.map_b;
    const float *__restrict__ mc = A.map_c;
    float *__restrict__ start = P.start;
    float *__restrict__ lam_end = A.lam_end;
    constexpr int NB = 8;
    const int nsl = (P.G + 31) / 32;
    int64_t n_map = *P.n_map;
    n_map = n_map < P.rec_cap ? n_map : P.rec_cap;
    const bool by_track = n_map > P.T;
    const int64_t units = (by_track ? (int64_t)P.T : n_map) * nsl * 2;
    for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < units;
         u += nwarps) {
        const int64_t m = u / (2 * nsl);
        const int rest = (int)(u - m * 2 * nsl);
        const int sl = rest >> 1, dir = rest & 1;
        int64_t t, b;
        if (by_track) {
            t = m;
            b = A.base[t];
            if (b >= P.rec_cap) continue;
        } else {
            const int64_t q = P.map_list[m];
            if ((uint64_t)q >= (uint64_t)P.rec_cap) continue;
            const int4 r = P.rec[q];
            if (!(r.z & CHUNK_FIRST) || (unsigned)r.w >= (unsigned)P.T) continue;
            t = r.w;
            b = q;
        }
        const int64_t e = A.base[t + 1] < P.rec_cap ? A.base[t + 1] : P.rec_cap;
        const int64_t nq = e - b;
        const int g = sl * 32 + lane;
        if (nq < 2 || g >= P.G) continue;
        if (dir == 0) {
            float psi = P.psi[t * P.Gs + g];
            for (int64_t k0 = 0; k0 < nq; k0 += NB) {
                float av[NB], bv[NB];
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    const int64_t row = (b + k0 + k) * P.Gs + g;
                    av[k] = k0 + k < nq ? ma[row] : 0.0f;
                    bv[k] = k0 + k < nq ? mb[row] : 0.0f;
                }
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    if (k0 + k < nq) start[(b + k0 + k) * P.Gs + g] = psi;
                    psi = fmaf(av[k], psi, bv[k]);
                }
            }
        } else {
            float lam = A.v[t * P.Gs + g];
            for (int64_t k0 = nq - 1; k0 >= 0; k0 -= NB) {
                float av[NB], cv[NB];
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    const int64_t row = (b + k0 - k) * P.Gs + g;
                    av[k] = k0 - k >= 0 ? ma[row] : 0.0f;
                    cv[k] = k0 - k >= 0 ? mc[row] : 0.0f;
                }
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    if (k0 - k >= 0) lam_end[(b + k0 - k) * P.Gs + g] = lam;
                    lam = fmaf(av[k], lam, cv[k]);
                }
            }
        }
    }
}

struct Jac {
    float a[27];
};

__global__ void adj_finish_kernel(const float4 *__restrict__ gblk, float *__restrict__ d_sigT,
                                  float *__restrict__ d_source, int R, int I, int G, int Gs,
                                  Jac jac, float mu, float mu2, int vec)
{
    const int64_t n = (int64_t)R * Gs;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k / Gs;
        const int g = (int)(k - r * Gs);
        if (g >= G) continue;
        const float4 *cb = gblk + r * I * Gs;
        float ds = 0.0f;
        for (int i = 0; i < I; i++) ds += grad_of(cb + (int64_t)i * Gs, g, vec, Gs).x;
        d_sigT[r * Gs + g] = ds;
        // source interval y of region r: every cell i with |i - y| <= 1 whose fit uses it
        for (int y = 0; y < I; y++) {
            float acc = 0.0f;
            for (int i = y - 1; i <= y + 1; i++) {
                if (i < 0 || i >= I) continue;
                const int type = i == 0 ? 0 : (i == I - 1 ? 2 : 1);
                const int m = y - i + 1;
                const float4 gq = grad_of(cb + (int64_t)i * Gs, g, vec, Gs);
                const float dq[3] = {gq.y, gq.z * mu, gq.w * mu2};
#pragma unroll
                for (int kk = 0; kk < 3; kk++) acc = fmaf(jac.a[(type * 3 + kk) * 3 + m], dq[kk], acc);
            }
            d_source[(r * I + y) * Gs + g] = acc;
        }
    }
}

template <int VEC>
const void *fwd_fn() { return reinterpret_cast<const void *>(&adj_forward_kernel<VEC>); }
template <int VEC>
const void *rev_fn() { return reinterpret_cast<const void *>(&adj_reverse_kernel<VEC>); }

const void *pick(int vec, bool reverse)
{
    if (vec == 1) return reverse ? rev_fn<1>() : fwd_fn<1>();
    if (vec == 2) return reverse ? rev_fn<2>() : fwd_fn<2>();
    if (vec == 4) return reverse ? rev_fn<4>() : fwd_fn<4>();
    return nullptr;
}

cudaError_t launch(const AdjParams &p, int vec, int blocks, bool reverse, cudaStream_t st)
{
    const void *fn = pick(vec, reverse);
    if (!fn || blocks < 1) return cudaErrorInvalidValue;
    AdjParams copy = p;
    void *args[] = {&copy};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(256), args, 0, st);
}

}  // namespace

int adj_blocks_per_sm(int vec, bool reverse)
{
    const void *fn = pick(vec, reverse);
    int n = 0;
    if (!fn || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, 256, 0) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_adj_forward(const AdjParams &p, int vec, int blocks, cudaStream_t st)
{
    return launch(p, vec, blocks, false, st);
}

cudaError_t launch_adj_reverse(const AdjParams &p, int vec, int blocks, cudaStream_t st)
{
    return launch(p, vec, blocks, true, st);
}

int adj_map_blocks_per_sm(int vec)
{
    const void *fn = vec == 1   ? reinterpret_cast<const void *>(&adj_map_kernel<1>)
                     : vec == 2 ? reinterpret_cast<const void *>(&adj_map_kernel<2>)
                     : vec == 4 ? reinterpret_cast<const void *>(&adj_map_kernel<4>)
                                : nullptr;
    int n = 0;
    if (!fn || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, 256, 0) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_adj_maps(const AdjParams &p, int vec, int blocks, cudaStream_t st)
{
    if (blocks < 1) return cudaErrorInvalidValue;
    if (vec == 1) adj_map_kernel<1><<<blocks, 256, 0, st>>>(p);
    else if (vec == 2) adj_map_kernel<2><<<blocks, 256, 0, st>>>(p);
    else if (vec == 4) adj_map_kernel<4><<<blocks, 256, 0, st>>>(p);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_adj_starts(const AdjParams &p, cudaStream_t st)
{
    const int64_t warps = (int64_t)p.fw.T * ((p.fw.G + 31) / 32) * 2;
    int64_t blocks = (warps * 32 + 255) / 256;
    if (blocks > grid_cap(16)) blocks = grid_cap(16);
    if (blocks < 1) blocks = 1;
    adj_start_kernel<<<(int)blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_adj_finish(const float4 *gblk, float *d_sigT, float *d_source, int R, int I,
                              int G, int Gs, const float *jac27, float mu, float mu2, int vec,
                              cudaStream_t st)
{
    Jac j;
    for (int k = 0; k < 27; k++) j.a[k] = jac27[k];
    const int64_t n = (int64_t)R * Gs;
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > grid_cap(16)) blocks = grid_cap(16);
    adj_finish_kernel<<<(int)blocks, 256, 0, st>>>(gblk, d_sigT, d_source, R, I, G, Gs, j, mu,
                                                   mu2, vec);
    return cudaGetLastError();
}

}  // namespace moc
