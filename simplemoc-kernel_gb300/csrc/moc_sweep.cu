// moc_sweep.cu — forward segment-attenuation sweep kernels for sm_103a.
//
// Work decomposition: a work item is (track, chunk of 32*VEC groups), or (chunk of a
// long track, group chunk) when long tracks are split (moc_split.cu). One warp owns an
// item from start to end: lanes hold VEC consecutive groups each, psi stays in registers
// for the whole item, and the warp walks its segments in CSR order (psi is carried from
// one segment to the next, src/cpu/kernel.c:53). Energy groups are independent, so a
// track's group chunks are independent items. Items are numbered group chunk by group
// chunk, so the warps in flight share one slice of the cell blocks and tally rows in L2.
// Warps take items from a global queue head (one atomicAdd per item), so tracks of
// uneven length balance.
//
// The sweep is bound by instruction issue, so everything that is not arithmetic is cut
// down:
//  * a prep pass writes one block per (region, interval) cell, interleaved by group:
//    blk[cell][g] = (sigT, q0, q1*mu, q2*mu2), so a segment needs one address and a lane
//    reads its VEC groups' four values with VEC 128-bit loads at immediate offsets;
//    q2*mu2 is 0 at the first and last interval, so no branch on the interval;
//  * segment descriptors are decoded lane-parallel: lane l validates segment wb+l of a
//    32-segment window and forms its cell index once; the warp then only shuffles
//    (cell, ds) per segment; the next window is loaded 32 segments ahead;
//  * the segment loop is unrolled by two with ping-pong registers: the block of segment
//    j+1 is loaded before segment j is computed, without register moves; the pairs run
//    inside each 32-segment window with 32-bit indices;
//  * segments are branch-free: past the item's end or with a bad index a segment is a
//    null-cell no-op, idle lanes read group 0, the tally is one predicated reduction.
// Tallies go out as red.global.add.v4.f32 (one L2 request per lane, 16 bytes).
#include "moc_arith.cuh"
#include "moc_device.cuh"
#include "moc_internal.h"

namespace moc {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------------------------------
// Axial fit, src/cpu/kernel.c:111-191, rounded as the reference's C rounds it (no
// contraction), then the first product of q1 * mu * ... and q2 * mu2 * ...
// (kernel.c:250-251, 311-322), packed with the region's sigT into the cell block.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float4 cell_block(const float *__restrict__ sigT,
                                             const float *__restrict__ source, int64_t k, int I,
                                             int Gs, float dz, float zin, float mu, float mu2)
{
    const int64_t cell = k / Gs;
    const int g = (int)(k - cell * Gs);
    const int64_t r = cell / I;
    const int i = (int)(cell - r * I);
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
        q0 = __fadd_rn(__fadd_rn(y2, __fmul_rn(c1, zin)), __fmul_rn(__fmul_rn(c2, zin), zin));
        q1 = __fadd_rn(c1, __fmul_rn(__fmul_rn(2.0f, c2), zin));
        q2 = c2;
    }
    return make_float4(sigT[r * Gs + g], q0, __fmul_rn(q1, mu), __fmul_rn(q2, mu2));
}

// ST = STORE_F32 writes float4 blocks; STORE_BF16 / STORE_F16 round them to 16 bits (to
// nearest even) and write four 16-bit values per (cell, group).
// With null_row, the row after the last cell is the null cell: (1, 0, 0, 0) per group.
template <int ST>
__global__ void prep_block_kernel(const float *__restrict__ sigT,
                                  const float *__restrict__ source, void *__restrict__ blk,
                                  int R, int I, int Gs, float dz, float zin, float mu, float mu2,
                                  int null_row)
{
    const int64_t n = (int64_t)R * I * Gs;
    const int64_t n_all = n + (null_row ? Gs : 0);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_all;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = k < n ? cell_block(sigT, source, k, I, Gs, dz, zin, mu, mu2)
                               : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        if constexpr (ST == STORE_F32) {
            static_cast<float4 *>(blk)[k] = v;
        } else {
            uint32_t w0, w1;
            if constexpr (ST == STORE_BF16) {
                const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
                const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
                w0 = *reinterpret_cast<const uint32_t *>(&a);
                w1 = *reinterpret_cast<const uint32_t *>(&b);
            } else {
                const __half2 a = __floats2half2_rn(v.x, v.y);
                const __half2 b = __floats2half2_rn(v.z, v.w);
                w0 = *reinterpret_cast<const uint32_t *>(&a);
                w1 = *reinterpret_cast<const uint32_t *>(&b);
            }
            static_cast<uint2 *>(blk)[k] = make_uint2(w0, w1);
        }
    }
}

// The FP32 blocks in the pair layout: one thread per pair of groups (k, k + 1), k even.
// svec > 1: in the lane-strided layout of the bulk-copy ring (float4 w of a 32*svec-group
// chunk of n float4 goes to (w % svec) * (n / svec) + w / svec of the chunk).
__global__ void prep_pairs_kernel(const float *__restrict__ sigT,
                                  const float *__restrict__ source, float4 *__restrict__ blk,
                                  int R, int I, int Gs, float dz, float zin, float mu,
                                  float mu2, int null_row, int svec)
{
    const int64_t n = (int64_t)R * I * Gs;
    const int64_t n_all = n + (null_row ? Gs : 0);
    for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; 2 * h < n_all;
         h += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = 2 * h;
        const float4 nul = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        const float4 u = k < n ? cell_block(sigT, source, k, I, Gs, dz, zin, mu, mu2) : nul;
        const float4 w =
            k < n ? cell_block(sigT, source, k + 1, I, Gs, dz, zin, mu, mu2) : nul;
        int64_t d0 = k, d1 = k + 1;
        if (svec > 1) {
            const int64_t row = k / Gs;
            const int g = (int)(k - row * Gs);
            const int cw = 32 * svec;
            const int cb = g / cw * cw;                   // the chunk's first group
            const int nl = min(Gs - cb, cw) / svec;       // lanes the chunk covers
            const int w0 = g - cb, w1 = w0 + 1;
            d0 = row * Gs + cb + (w0 % svec) * nl + w0 / svec;
            d1 = row * Gs + cb + (w1 % svec) * nl + w1 / svec;
        }
        blk[d0] = make_float4(u.x, w.x, u.y, w.y);
        blk[d1] = make_float4(u.z, w.z, u.w, w.w);
    }
}

// ------------------------------------------------------------------------------------
// The per-(segment, group) arithmetic.
// ------------------------------------------------------------------------------------
template <int VEC>
struct Blk {
    float4 v[VEC];  // per group: (sigT, q0, q1*mu, q2*mu2)
};

// Block of VEC groups at element index idx (= cell * Gs + g0). FP32 blocks are 16 bytes
// per group; BF16/FP16 blocks 8 bytes (four 16-bit values), widened to FP32 on load.
// One 16-bit block (four bf16 or fp16 values) widened to FP32.
template <int ST>
__device__ __forceinline__ float4 widen(uint2 w)
{
    if constexpr (ST == STORE_BF16) {
        return make_float4(__uint_as_float(w.x << 16), __uint_as_float(w.x & 0xffff0000u),
                           __uint_as_float(w.y << 16), __uint_as_float(w.y & 0xffff0000u));
    } else {
        const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&w.x));
        const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&w.y));
        return make_float4(lo.x, lo.y, hi.x, hi.y);
    }
}

// PAIRS: the lane's groups are consumed two at a time by the packed arithmetic, with each
// pair's two float4 in the pair layout (sigT_a, sigT_b, q0_a, q0_b), (q1mu_a, q1mu_b,
// q2mu2_a, q2mu2_b): FP32 blocks are stored that way; 16-bit blocks, stored per group, are
// widened straight into that order.
template <int VEC, int ST, bool PAIRS = f32_pairs(VEC)>
__device__ __forceinline__ void load_blk(const void *base, int idx, Blk<VEC> &b)
{
    if constexpr (ST == STORE_F32) {
        const float4 *p = static_cast<const float4 *>(base) + idx;
        if constexpr (VEC % 2 == 0) {
            // idx is even (a lane's first group) and rows are multiples of 4 groups, so
            // each pair of blocks is 32-byte aligned: one 256-bit load per pair
#pragma unroll
            for (int k = 0; k < VEC; k += 2) ldg_2x4(p + k, b.v[k], b.v[k + 1]);
        } else {
#pragma unroll
            for (int k = 0; k < VEC; k++) b.v[k] = __ldg(p + k);
        }
    } else {
        const uint2 *p = static_cast<const uint2 *>(base) + idx;
        uint2 w[VEC];
        if constexpr (VEC == 4) {
            const uint4 a = __ldg(reinterpret_cast<const uint4 *>(p));
            const uint4 c = __ldg(reinterpret_cast<const uint4 *>(p) + 1);
            w[0] = make_uint2(a.x, a.y); w[1] = make_uint2(a.z, a.w);
            w[2] = make_uint2(c.x, c.y); w[3] = make_uint2(c.z, c.w);
        } else if constexpr (VEC == 2) {
            const uint4 a = __ldg(reinterpret_cast<const uint4 *>(p));
            w[0] = make_uint2(a.x, a.y); w[1] = make_uint2(a.z, a.w);
        } else {
            w[0] = __ldg(p);
        }
        float4 f[VEC];
#pragma unroll
        for (int k = 0; k < VEC; k++) f[k] = widen<ST>(w[k]);
        if constexpr (PAIRS) {
#pragma unroll
            for (int k = 0; k < VEC; k += 2) {
                b.v[k] = make_float4(f[k].x, f[k + 1].x, f[k].y, f[k + 1].y);
                b.v[k + 1] = make_float4(f[k].z, f[k + 1].z, f[k].w, f[k + 1].w);
            }
        } else {
#pragma unroll
            for (int k = 0; k < VEC; k++) b.v[k] = f[k];
        }
    }
}

// src/cpu/kernel.c:200-332 for VEC groups (moc_arith.cuh).
// pmul gets p = exp(-tau) per group (the map mode's product; unused otherwise).
template <int VEC, int EK>
__device__ __forceinline__ void attenuate(const Blk<VEC> &x, float ds, float weight,
                                          const TableRef &tr, Vec<VEC> &psi,
                                          Vec<VEC> &tally, Vec<VEC> &pmul)
{
    attenuate_row<VEC, EK, f32_pairs(VEC)>(x.v, ds, weight, tr, psi, tally, pmul);
}

// Lane-parallel descriptor decode of segment j: its cell index and its ds, from the three
// arrays or from the compact pair (a 32-bit cell index and a half length; the branch is
// the same for every lane and taken once per 32-segment window). Out-of-range regions,
// intervals or cells are reported through the error word. A segment past the item's end
// or with an out-of-range index decodes to cell `none` with ds = 0: -1 (skipped by the
// loops that test it), or the null cell R*I, whose block (sigT 1, coefficients 0) makes
// the segment an exact no-op (p = 1, every term 0).
__device__ __forceinline__ void decode(const SweepParams &P, int64_t j, int64_t end, int none,
                                       int &cell, float &ds)
{
    cell = none;
    ds = 0.0f;
    if (j < end) {
        if (P.cell) {
            const uint32_t c = ld_stream(P.cell + j);
            const unsigned short hb = ld_stream(reinterpret_cast<const unsigned short *>(P.ds16) + j);
            if (c < (uint32_t)P.R * (uint32_t)P.I) {
                cell = (int)c;
                ds = __half2float(__ushort_as_half(hb));
            } else {
                atomicOr(P.err, DEVERR_INDEX);
            }
            return;
        }
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

enum : int { MODE_SWEEP = 0, MODE_MAP = 1 };

// Segment loops of sweep_item (template parameter RD):
enum : int {
    RD_REG = 0,       // one segment ahead in registers, checks per segment
    RD_FREE = -1,     // branch-free windowed pair loop, one segment ahead in registers
    RD_FREE_LB = -2,  // RD_FREE compiled for blocks of at most 8 warps, 5 blocks per SM
                      // (at most 48 registers: 40 resident warps per SM instead of 32)
    RD_BULK = -3,     // a ring of P.ring_d slots per warp filled by bulk copies
};

// A warp's position in its bulk-copy ring, kept across its work items: the slot the next
// copy goes to (lane 0), the slot and phase parity the next wait is on, and the copies in
// flight (lane 0).
struct RingState {
    int is, cs, inflight;
    uint32_t ph;
};

// One work item. Without chunk records an item is (track, group chunk). With records
// (split mode) it is (record, group chunk): a whole track (psi in place), or a chunk of
// a split track, which starts from its precomputed psi and, if it is the track's last,
// writes the track's psi. MODE_MAP runs the non-last chunks of split tracks from psi = 0
// without tallies and writes (a, b) = (product of p, outgoing psi) per group.
// Items are numbered group chunk by group chunk (all tracks or records of groups
// [0, 32 VEC) first, ...) when P.group_major is set, so the warps in flight read one
// group chunk's slice of every cell block and tally row, a smaller working set in L2;
// else track by track. n_units: tracks, records or map items.
// Returns false when a bounded wait of the bulk-copy ring gave up (the warp stops).
template <int VEC, int EK, int ST, int TL, int RD, int MODE>
__device__ __forceinline__ bool sweep_item(const SweepParams &P, int64_t item, int64_t n_units,
                                           int lane, const TableRef &tr, float4 *ring,
                                           RingState &rs)
{
    const int Gs = P.Gs;
    int64_t beg, end, row_q = 0, unit;
    int ch;
    if (P.group_major) {
        ch = (int)(item / n_units);
        unit = item - (int64_t)ch * n_units;
    } else {
        unit = item / P.n_chunks;
        ch = (int)(item - unit * P.n_chunks);
    }
    const float *psi_in;
    float *psi_out;  // null: the chunk's outgoing psi is not kept
    if (P.rec) {
        int64_t q = unit;
        if constexpr (MODE == MODE_MAP) {
            q = P.map_list[q];
            if ((uint64_t)q >= (uint64_t)P.rec_cap) return true;
        }
        const int4 r = __ldg(P.rec + q);
        const int flags = r.z;
        if constexpr (MODE == MODE_MAP)
            if (flags & (CHUNK_SINGLE | CHUNK_LAST)) return true;
        beg = (int64_t)(uint32_t)r.x | ((int64_t)r.y << 32);
        end = beg + (flags & CHUNK_LEN_MASK);
        // records come from offsets that may not be a partition of [0, S]: check them
        if (!(beg >= 0 && end <= P.S && (unsigned)r.w < (unsigned)P.T)) {
            if (lane == 0) atomicOr(P.err, DEVERR_OFFSETS);
            return true;
        }
        float *track_psi = P.psi + (int64_t)r.w * Gs;
        if (flags & CHUNK_SINGLE) {
            psi_in = psi_out = track_psi;
        } else {
            psi_in = P.start + q * Gs;
            psi_out = (flags & CHUNK_LAST) ? track_psi : nullptr;
        }
        row_q = q * Gs;
    } else {
        const int t = (int)unit;
        beg = P.off[t];
        end = P.off[t + 1];
        if (!(beg >= 0 && beg <= end && end <= P.S)) {
            if (lane == 0) atomicOr(P.err, DEVERR_OFFSETS);
            return true;
        }
        psi_in = psi_out = P.psi + (int64_t)t * Gs;
    }
    const int g0 = (ch * 32 + lane) * VEC;
    const int nvalid = P.G - g0;
    const bool act = nvalid > 0;
    Vec<VEC> psi, amul;
#pragma unroll
    for (int k = 0; k < VEC; k++) {
        psi.v[k] = 0.0f;
        amul.v[k] = 1.0f;
    }
    if (MODE == MODE_SWEEP && act) psi = ld_psi<VEC>(psi_in + g0, nvalid);

    // Descriptor windows: A = segments [wb, wb+32), B = the next 32 (the branch-free and
    // bulk loops keep them in shared memory instead).
    const int none = RD < 0 ? P.null_cell : -1;
    int64_t wb = beg;
    int cA = none, cB = none;
    float dA = 0.0f, dB = 0.0f;
    if constexpr (RD == RD_REG) {
        decode(P, wb + lane, end, none, cA, dA);
        decode(P, wb + 32 + lane, end, none, cB, dB);
    }
    auto desc = [&](int64_t j, int &c, float &d) {
        int k = (int)(j - wb);
        if (k >= 32) {
            cA = cB;
            dA = dB;
            wb += 32;
            k -= 32;
            decode(P, wb + 32 + lane, end, none, cB, dB);
        }
        c = __shfl_sync(FULL, cA, k);
        d = __shfl_sync(FULL, dA, k);
    };
    auto step = [&](const Blk<VEC> &b, int c, float d) {
        if (c >= 0 && act) {
            Vec<VEC> tally, p;
            attenuate<VEC, EK>(b, d, P.weight, tr, psi, tally, p);
            const int idx = c * Gs + g0;
            if constexpr (MODE == MODE_MAP) {
#pragma unroll
                for (int k = 0; k < VEC; k++) amul.v[k] *= p.v[k];
            } else if constexpr (TL == TALLY_F32)
                red_row<VEC>(P.ff + idx, tally, nvalid);
            else if constexpr (TL == TALLY_COMP)
                comp_row<VEC>(P.ff + idx, P.lo + idx, tally, nvalid);
            else
                red_row_f64<VEC>(P.ff64 + idx, tally, nvalid);
        }
    };

    if constexpr (RD == RD_FREE || RD == RD_FREE_LB) {
        // Branch-free segments, one ahead (ping-pong registers), 32-bit indexing inside
        // 32-segment descriptor windows: the pair loop shuffles lanes k and k+1 of window
        // A; only the pair at a full window's end reaches into window B. Segments past the
        // end or with bad indices are null-cell no-ops (decode), lanes past G read group
        // 0's block, and the tally is one predicated reduction (red_row_if) sent only for
        // real cells on lanes whose groups are all real (G is a multiple of VEC here).
        const int gl = act ? g0 : 0;
        const int lim = act ? P.null_cell : 0;
        auto load = [&](int c, Blk<VEC> &b) { load_blk<VEC, ST>(P.blk, c * Gs + gl, b); };
        auto step_nb = [&](const Blk<VEC> &b, int c, float d) {
            Vec<VEC> tally, p;
            attenuate<VEC, EK>(b, d, P.weight, tr, psi, tally, p);
            if constexpr (MODE == MODE_MAP) {
#pragma unroll
                for (int k = 0; k < VEC; k++) amul.v[k] *= p.v[k];
            } else {
                // the load's index: it differs from c * Gs + g0 only on lanes past G,
                // whose reductions lim = 0 turns off
                const int idx = c * Gs + gl;
                if constexpr (TL == TALLY_F32) {
                    red_row_if<VEC>(P.ff + idx, tally, c, lim);
                } else if ((unsigned)c < (unsigned)lim) {
                    if constexpr (TL == TALLY_COMP)
                        comp_row<VEC>(P.ff + idx, P.lo + idx, tally, VEC);
                    else
                        red_row_f64<VEC>(P.ff64 + idx, tally, VEC);
                }
            }
        };
        // The warp's 64-entry descriptor ring in shared memory (`ring`, 512 bytes): segment
        // j's (cell, ds bits) at slot (j - beg) & 63, written lane-parallel a 32-segment
        // window at a time and read two segments at a time by one broadcast 16-byte load
        // (one L1 wavefront per pair of segments, where two shuffles per segment took two).
        int2 *win = reinterpret_cast<int2 *>(ring);
        auto put = [&](int64_t w0, int slot0) {
            int c;
            float d;
            decode(P, w0 + lane, end, none, c, d);
            win[slot0 + lane] = make_int2(c, __float_as_int(d));
        };
        auto get2 = [&](int slot) {  // slot even: segments slot, slot + 1
            return reinterpret_cast<const int4 *>(win)[slot >> 1];
        };
        put(beg, 0);
        put(beg + 32, 32);
        __syncwarp();
        Blk<VEC> b0, b1;
        int4 q = get2(0);
        load(q.x, b0);
        int slot = 0;  // slot of segment wb
        for (; wb < end; wb += 32) {
            const int nk = end - wb < 32 ? (int)(end - wb) : 32;
            for (int k = 0; k < nk; k += 2) {
                load(q.z, b1);
                step_nb(b0, q.x, __int_as_float(q.y));
                const int4 qn = get2((slot + k + 2) & 63);
                load(qn.x, b0);
                step_nb(b1, q.z, __int_as_float(q.w));
                q = qn;
            }
            __syncwarp();  // every lane is past its reads of this window's slots
            put(wb + 64, slot);
            __syncwarp();
            slot ^= 32;
        }
    } else if constexpr (RD == 0) {
        // one segment ahead, in registers (ping-pong, no moves)
        Blk<VEC> b0, b1;
        int c0 = -1, c1 = -1;
        float d0 = 0.0f, d1 = 0.0f;
        if (beg < end) {
            desc(beg, c0, d0);
            if (c0 >= 0 && act) load_blk<VEC, ST>(P.blk, c0 * Gs + g0, b0);
        }
        for (int64_t j = beg; j < end; j += 2) {
            const bool has1 = j + 1 < end;
            if (has1) {
                desc(j + 1, c1, d1);
                if (c1 >= 0 && act) load_blk<VEC, ST>(P.blk, c1 * Gs + g0, b1);
            }
            step(b0, c0, d0);
            if (!has1) break;
            if (j + 2 < end) {
                desc(j + 2, c0, d0);
                if (c0 >= 0 && act) load_blk<VEC, ST>(P.blk, c0 * Gs + g0, b0);
            }
            step(b1, c1, d1);
        }
    } else if constexpr (RD == RD_BULK) {
        // P.ring_d slots per warp in shared memory after the descriptor ring, each holding
        // one segment's cell blocks for the warp's group chunk (nrow float4, copied from
        // the lane-strided layout with one bulk copy), and one mbarrier per slot. Lane 0
        // starts the copy of segment j + ring_d - 1 before the warp waits on segment j, so
        // ring_d - 1 copies are in flight behind the arithmetic. Copies are made only for
        // segments that name a cell (the null cell included), and each is waited on and
        // read exactly once, in order, so the copy and wait sides step through the slots
        // alike; a slot is refilled only after every lane has read it (__syncwarp).
        static_assert(ST == STORE_F32 && TL == TALLY_F32, "bulk ring: FP32 blocks and tallies");
        const int D = P.ring_d;
        float4 *slots = ring + DESC_RING_F4;
        const uint32_t bar0 = smem_addr(slots + D * 32 * VEC);
        const int gw = g0 - lane * VEC;                            // the chunk's first group
        const int nrow = Gs - gw < 32 * VEC ? Gs - gw : 32 * VEC;  // its float4 in a row
        const uint32_t bytes = (uint32_t)nrow * 16u;
        const int nl = nrow / VEC;                                 // lanes it covers
        const int li = lane < nl ? lane : 0;
        const float4 *src = static_cast<const float4 *>(P.blk) + gw;
        const int ncell = P.R * P.I;
        const int lim = act ? ncell : 0;
        const int gl = act ? g0 : 0;
        int2 *win = reinterpret_cast<int2 *>(ring);
        auto put = [&](int64_t w0, int slot0) {
            int c;
            float d;
            decode(P, w0 + lane, end, none, c, d);
            win[slot0 + lane] = make_int2(c, __float_as_int(d));
        };
        auto issue = [&](int pos) {  // lane 0: the copy of the segment at ring position pos
            const int c = win[pos].x;
            if (c >= 0) {
                const uint32_t bar = bar0 + 8u * (uint32_t)rs.is;
                mbar_expect_tx(bar, bytes);
                bulk_g2s(smem_addr(slots + rs.is * 32 * VEC), src + (int64_t)c * Gs, bytes, bar);
                rs.is = rs.is + 1 == D ? 0 : rs.is + 1;
                rs.inflight++;
            }
        };
        put(beg, 0);
        put(beg + 32, 32);
        __syncwarp();
        if (lane == 0) {
            const int64_t n0 = end - beg < D - 1 ? end - beg : D - 1;
            for (int s0 = 0; s0 < (int)n0; s0++) issue(s0);
        }
        int slot = 0;  // ring position of segment wb
        for (; wb < end; wb += 32) {
            const int nk = end - wb < 32 ? (int)(end - wb) : 32;
            for (int k = 0; k < nk; k++) {
                if (lane == 0 && wb + k + D - 1 < end) issue((slot + k + D - 1) & 63);
                const int2 q = win[(slot + k) & 63];
                const int c = q.x;
                if (c >= 0) {
                    const bool ok = mbar_wait_bounded(bar0 + 8u * (uint32_t)rs.cs, rs.ph,
                                                      BULK_WAIT_LIMIT);
                    if (!__all_sync(FULL, ok)) {
                        // give up: report, let the copies in flight land (bounded), stop
                        if (lane == 0) {
                            atomicOr(P.err, DEVERR_TIMEOUT);
                            int cs = rs.cs;
                            uint32_t ph = rs.ph;
                            for (int m = 0; m < rs.inflight; m++) {
                                mbar_wait_bounded(bar0 + 8u * (uint32_t)cs, ph, BULK_WAIT_LIMIT);
                                if (++cs == D) {
                                    cs = 0;
                                    ph ^= 1u;
                                }
                            }
                        }
                        __syncwarp();
                        return false;
                    }
                    const float4 *sl = slots + rs.cs * 32 * VEC;
                    Blk<VEC> b;
#pragma unroll
                    for (int v = 0; v < VEC; v++) b.v[v] = sl[v * nl + li];
                    if (++rs.cs == D) {
                        rs.cs = 0;
                        rs.ph ^= 1u;
                    }
                    if (lane == 0) rs.inflight--;
                    Vec<VEC> tally, p;
                    attenuate<VEC, EK>(b, __int_as_float(q.y), P.weight, tr, psi, tally, p);
                    if constexpr (MODE == MODE_MAP) {
#pragma unroll
                        for (int v = 0; v < VEC; v++) amul.v[v] *= p.v[v];
                    } else {
                        if (nvalid >= VEC || !act)
                            red_row_if<VEC>(P.ff + c * Gs + gl, tally, c, lim);
                        else if ((unsigned)c < (unsigned)ncell)
                            red_row<VEC>(P.ff + c * Gs + g0, tally, nvalid);
                    }
                }
                __syncwarp();  // every lane has read the slot before it is refilled
            }
            put(wb + 64, slot);
            __syncwarp();
            slot ^= 32;
        }
    }
    if (!act) return true;
    if constexpr (MODE == MODE_MAP) {
        st_psi<VEC>(P.map_a + row_q + g0, amul, nvalid);
        st_psi<VEC>(P.map_b + row_q + g0, psi, nvalid);
    } else {
        if (psi_out) st_psi<VEC>(psi_out + g0, psi, nvalid);
    }
    return true;
}

// Per-warp shared memory of the bulk-copy ring (float4): the descriptor ring, d slots of
// 32*vec float4, and d 8-byte mbarriers.
__host__ __device__ inline int bulk_warp_f4(int d, int vec)
{
    return DESC_RING_F4 + d * 32 * vec + (8 * d + 15) / 16;
}

// Dynamic shared memory: the exponential table (table mode), then per warp its 64-segment
// descriptor ring (RD < 0), followed by its bulk-copy slots and barriers (RD_BULK).
// Launch bounds: RD_FREE_LB asks for five 256-thread blocks per SM (48 registers); the
// other loops name only the 512-thread limit (a minimum of 0 blocks leaves the register
// choice to the compiler, which then aims at occupancy; asking for 1 block would let it
// take up to 128 registers, and it takes 76-86, halving the resident warps).
constexpr int lb_threads(int rd) { return rd == RD_FREE_LB ? 256 : 512; }
constexpr int lb_blocks(int rd) { return rd == RD_FREE_LB ? 5 : 0; }

template <int VEC, int EK, int ST, int TL, int RD, int MODE>
__global__ void __launch_bounds__(lb_threads(RD), lb_blocks(RD)) fwd_kernel(const SweepParams P)
{
    extern __shared__ float4 s_dyn[];
    TableRef tr{nullptr, 0, 0.0f, 0.0f};
    float2 *s_tab = reinterpret_cast<float2 *>(s_dyn);
    if constexpr (EK == EXPK_TABLE) {
        const float2 *src = reinterpret_cast<const float2 *>(P.table);
        for (int k = threadIdx.x; k < P.tab_n; k += blockDim.x) s_tab[k] = src[k];
        __syncthreads();
        tr = TableRef{s_tab, P.tab_n, P.tab_dx, P.tab_max};
    }
    const int lane = threadIdx.x & 31;
    float4 *ring = nullptr;  // the warp's descriptor ring (and bulk-copy slots)
    RingState rs{0, 0, 0, 0u};
    if constexpr (RD != RD_REG) {
        const int tab_f4 = EK == EXPK_TABLE ? (P.tab_n + 1) / 2 : 0;
        const int per_warp = RD == RD_BULK ? bulk_warp_f4(P.ring_d, VEC) : DESC_RING_F4;
        ring = s_dyn + tab_f4 + (threadIdx.x >> 5) * per_warp;
    }
    if constexpr (RD == RD_BULK) {
        if (lane == 0) {
            const uint32_t bar0 = smem_addr(ring + DESC_RING_F4 + P.ring_d * 32 * VEC);
            for (int d = 0; d < P.ring_d; d++) mbar_init(bar0 + 8u * (uint32_t)d, 1);
            mbar_init_fence();
        }
        __syncwarp();
    }
    int64_t n_items = P.n_items, n_units = P.T;
    if (P.rec) {
        const int64_t n = MODE == MODE_MAP ? *P.n_map : *P.n_rec;
        n_units = n < P.rec_cap ? n : P.rec_cap;
        n_items = n_units * P.n_chunks;
    }
    if constexpr (MODE == MODE_MAP) {
        // Map items (the non-last chunks, listed by the record pass) are full chunks of
        // equal length: a static warp-strided assignment balances without a queue atomic.
        const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
        for (int64_t item = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
             item < n_items; item += nw)
            if (!sweep_item<VEC, EK, ST, TL, RD, MODE>(P, item, n_units, lane, tr, ring, rs))
                break;
    } else {
        for (;;) {
            unsigned long long item = 0;
            if (lane == 0) item = atomicAdd(P.counter, 1ULL);
            item = __shfl_sync(FULL, item, 0);
            if (item >= (unsigned long long)n_items) break;
            if (!sweep_item<VEC, EK, ST, TL, RD, MODE>(P, (int64_t)item, n_units, lane, tr,
                                                       ring, rs))
                break;
        }
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
        if (P.cell ? P.cell[j] >= (uint32_t)P.R * (uint32_t)P.I
                   : ((unsigned)P.reg[j] >= (unsigned)P.R || (unsigned)P.itv[j] >= (unsigned)P.I))
            bad |= DEVERR_INDEX;
    }
    if (bad) atomicOr(P.err, bad);
}

__global__ void finish_kernel(float *__restrict__ ff, const float *__restrict__ lo,
                              const double *__restrict__ ff64, int64_t n)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double add = lo ? (double)lo[k] : ff64[k];
        ff[k] = (float)((double)ff[k] + add);
    }
}

template <int VEC, int EK, int ST, int TL, int RD = RD_REG, int MODE = MODE_SWEEP>
const void *fwd_fn()
{
    return reinterpret_cast<const void *>(&fwd_kernel<VEC, EK, ST, TL, RD, MODE>);
}

// The register-prefetch loop: the branch-free windowed pair loop (RD_FREE) where the
// configuration allows it (a null-cell row, G a multiple of VEC), else the ping-pong loop
// with per-segment checks (RD_REG).
template <int VEC, int EK, int ST, int TL, int MODE = MODE_SWEEP>
const void *reg_fn(bool branch_free)
{
    return branch_free ? fwd_fn<VEC, EK, ST, TL, RD_FREE, MODE>()
                       : fwd_fn<VEC, EK, ST, TL, RD_REG, MODE>();
}

// FP32 cell blocks with FP32 tallies: the register loops, or the bulk-copy ring
// (c.prefetch > 1). The plain exponential with one or two groups per lane in blocks of at
// most 8 warps takes the 48-register build of the branch-free loop (measured 3 % faster at
// 50M x 128 than 58 registers with 32 resident warps).
template <int V, int EK, int MODE>
const void *f32_fn(const FwdConfig &c)
{
    if (fwd_bulk(c)) return fwd_fn<V, EK, STORE_F32, TALLY_F32, RD_BULK, MODE>();
    if constexpr (EK == EXPK_PLAIN && V <= 2)
        if (c.branch_free && c.warps_per_block <= 8)
            return fwd_fn<V, EK, STORE_F32, TALLY_F32, RD_FREE_LB, MODE>();
    return reg_fn<V, EK, STORE_F32, TALLY_F32, MODE>(c.branch_free);
}

// The instantiated (exp, storage, tally, loop) combinations, for every VEC:
//   plain FP32 / table FP32 / stable FP32 with FP32 atomics: every loop (f32_fn);
//   stable math with FP32 storage and compensated or FP64 tallies, and stable math with
//   BF16 / FP16 storage and all three tally kinds: the register loops.
template <int V>
const void *pick_vec(const FwdConfig &c)
{
    const bool plain_loops = !fwd_bulk(c);
    if (c.mode == MODE_MAP) {  // maps: no tallies
        if (c.store == STORE_F32) {
            if (c.exp_kind == EXPK_PLAIN) return f32_fn<V, EXPK_PLAIN, MODE_MAP>(c);
            if (c.exp_kind == EXPK_TABLE) return f32_fn<V, EXPK_TABLE, MODE_MAP>(c);
            return f32_fn<V, EXPK_STABLE, MODE_MAP>(c);
        }
        if (c.exp_kind != EXPK_STABLE || !plain_loops) return nullptr;
        if (c.store == STORE_BF16)
            return reg_fn<V, EXPK_STABLE, STORE_BF16, TALLY_F32, MODE_MAP>(c.branch_free);
        if (c.store == STORE_F16)
            return reg_fn<V, EXPK_STABLE, STORE_F16, TALLY_F32, MODE_MAP>(c.branch_free);
        return nullptr;
    }
    if (c.mode != MODE_SWEEP) return nullptr;
    if (c.store == STORE_F32 && c.tally == TALLY_F32) {
        if (c.exp_kind == EXPK_PLAIN) return f32_fn<V, EXPK_PLAIN, MODE_SWEEP>(c);
        if (c.exp_kind == EXPK_TABLE) return f32_fn<V, EXPK_TABLE, MODE_SWEEP>(c);
        return f32_fn<V, EXPK_STABLE, MODE_SWEEP>(c);
    }
    if (c.exp_kind != EXPK_STABLE || !plain_loops) return nullptr;
    if (c.store == STORE_F32) {
        if (c.tally == TALLY_COMP) return reg_fn<V, EXPK_STABLE, STORE_F32, TALLY_COMP>(c.branch_free);
        if (c.tally == TALLY_F64) return reg_fn<V, EXPK_STABLE, STORE_F32, TALLY_F64>(c.branch_free);
        return nullptr;
    }
    if (c.store == STORE_BF16) {
        if (c.tally == TALLY_F32) return reg_fn<V, EXPK_STABLE, STORE_BF16, TALLY_F32>(c.branch_free);
        if (c.tally == TALLY_COMP) return reg_fn<V, EXPK_STABLE, STORE_BF16, TALLY_COMP>(c.branch_free);
        if (c.tally == TALLY_F64) return reg_fn<V, EXPK_STABLE, STORE_BF16, TALLY_F64>(c.branch_free);
    }
    if (c.store == STORE_F16) {
        if (c.tally == TALLY_F32) return reg_fn<V, EXPK_STABLE, STORE_F16, TALLY_F32>(c.branch_free);
        if (c.tally == TALLY_COMP) return reg_fn<V, EXPK_STABLE, STORE_F16, TALLY_COMP>(c.branch_free);
        if (c.tally == TALLY_F64) return reg_fn<V, EXPK_STABLE, STORE_F16, TALLY_F64>(c.branch_free);
    }
    return nullptr;
}

const void *pick(const FwdConfig &c)
{
    if (c.vec == 1) return pick_vec<1>(c);
    if (c.vec == 2) return pick_vec<2>(c);
    if (c.vec == 4) return pick_vec<4>(c);
    return nullptr;
}

}  // namespace

int current_sm_count()
{
    constexpr int MAX_DEV = 64;
    static int cached[MAX_DEV] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) {
        cudaGetLastError();
        return 1;
    }
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            n < 1) {
            cudaGetLastError();
            return 1;
        }
        cached[dev] = n;
    }
    return cached[dev];
}

static int grid_for(int64_t n)
{
    int64_t blocks = (n + 255) / 256;
    if (blocks > grid_cap(16)) blocks = grid_cap(16);
    return (int)(blocks < 1 ? 1 : blocks);
}

cudaError_t launch_prep_block(const float *sigT, const float *source, float4 *blk, int R,
                              int I, int Gs, float dz, float zin, float mu, float mu2,
                              cudaStream_t st, bool null_row, bool pairs, int strided)
{
    const int64_t n = (int64_t)R * I * Gs + (null_row ? Gs : 0);
    if (n == 0) return cudaSuccess;
    if (strided > 1 && !pairs) return cudaErrorInvalidValue;
    if (pairs)  // n is a multiple of Gs, itself a multiple of 4: whole pairs
        prep_pairs_kernel<<<grid_for(n / 2), 256, 0, st>>>(sigT, source, blk, R, I, Gs, dz,
                                                            zin, mu, mu2, null_row, strided);
    else
        prep_block_kernel<STORE_F32><<<grid_for(n), 256, 0, st>>>(sigT, source, blk, R, I, Gs,
                                                                   dz, zin, mu, mu2, null_row);
    return cudaGetLastError();
}

cudaError_t launch_prep_block16(const float *sigT, const float *source, void *blk, int store,
                                int R, int I, int Gs, float dz, float zin, float mu,
                                float mu2, cudaStream_t st, bool null_row)
{
    const int64_t n = (int64_t)R * I * Gs + (null_row ? Gs : 0);
    if (n == 0) return cudaSuccess;
    if (store == STORE_BF16)
        prep_block_kernel<STORE_BF16><<<grid_for(n), 256, 0, st>>>(sigT, source, blk, R, I, Gs,
                                                                    dz, zin, mu, mu2, null_row);
    else if (store == STORE_F16)
        prep_block_kernel<STORE_F16><<<grid_for(n), 256, 0, st>>>(sigT, source, blk, R, I, Gs,
                                                                   dz, zin, mu, mu2, null_row);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_finish(float *ff, const float *lo, const double *ff64, int64_t n,
                          cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    finish_kernel<<<grid_for(n), 256, 0, st>>>(ff, lo, ff64, n);
    return cudaGetLastError();
}

size_t fwd_smem_bytes(const FwdConfig &c, int tab_n)
{
    size_t b = c.exp_kind == EXPK_TABLE ? (size_t)(tab_n + 1) / 2 * sizeof(float4) : 0;
    if (fwd_bulk(c))
        b += (size_t)c.warps_per_block * bulk_warp_f4(c.prefetch, c.vec) * sizeof(float4);
    else if (c.branch_free)
        b += (size_t)c.warps_per_block * DESC_RING_F4 * sizeof(float4);
    return b;
}

int fwd_blocks_per_sm(const FwdConfig &c, int tab_n)
{
    const void *fn = pick(c);
    if (!fn || c.warps_per_block < 1 || c.warps_per_block > 16) return 0;
    if (c.prefetch < 1 || c.prefetch > RING_MAX) return 0;
    const size_t smem = fwd_smem_bytes(c, tab_n);
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
    if (!fn || c.warps_per_block < 1 || c.warps_per_block > 16 || c.blocks < 1 ||
        c.prefetch < 1 || c.prefetch > RING_MAX)
        return cudaErrorInvalidValue;
    const size_t smem = fwd_smem_bytes(c, p.tab_n);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    SweepParams copy = p;
    copy.ring_d = fwd_bulk(c) ? c.prefetch : 0;
    void *args[] = {&copy};
    return cudaLaunchKernel(fn, dim3(c.blocks), dim3(c.warps_per_block * 32), args, smem, st);
}

cudaError_t launch_check(const SweepParams &p, cudaStream_t st)
{
    int64_t work = p.S > p.T ? p.S : p.T;
    int blocks = (int)((work + 255) / 256);
    if (blocks < 1) blocks = 1;
    if (blocks > grid_cap(8)) blocks = (int)grid_cap(8);
    check_kernel<<<blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace moc
