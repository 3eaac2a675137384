// moc_batch.cu — the batching form: several problems (any group counts) swept by ONE
// persistent kernel launch from a length-sorted work queue (moc_attenuate_fwd_batch).
//
// Each problem's group range is cut into sub-problems: full chunks of 32*VEC groups,
// swept by whole warps, and a remainder chunk swept by sub-warps of LPT lanes (LPT the
// smallest power of two covering the remainder), so a warp carries 32/LPT tracks of a
// small-G problem at once instead of leaving lanes idle. Tracks are sorted by length
// (a log-scale bucket sort on the device), consecutive tracks of equal bucket form one
// warp item, and the items of all sub-problems are ordered longest first in one queue
// that the warps of the persistent kernel consume with one atomicAdd per item. The whole
// sequence (coefficient passes, queue construction, sweep) is a handful of kernels that
// the host side captures into a CUDA graph and replays.
#include "moc_arith.cuh"
#include "moc_device.cuh"
#include "moc_internal.h"

namespace moc {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NB = BATCH_BUCKETS;

// Longest tracks first: bucket 0 holds the longest. Log-scale, 8 buckets per octave.
__device__ __forceinline__ int len_bucket(int64_t len)
{
    const float lg = __log2f((float)len + 1.0f) * 8.0f;
    int k = (int)lg;
    k = k < 0 ? 0 : (k > NB - 1 ? NB - 1 : k);
    return NB - 1 - k;
}

// Units of problem p: its tracks, or the chunk records of its tracks when long tracks are
// cut (counted on the device; at most rec_cap).
__device__ __forceinline__ int64_t units_of(const BatchProb &P)
{
    if (!P.rec) return P.T;
    const int64_t n = *P.n_rec;
    return n < P.rec_cap ? n : P.rec_cap;
}

// Host-side upper bound on the units (grid sizes and item counts).
__host__ __device__ __forceinline__ int64_t units_bound(const BatchProb &P)
{
    return P.rec ? P.rec_cap : P.T;
}

__device__ __forceinline__ int64_t track_len(const BatchParams &B, int p, int64_t u)
{
    const BatchProb &P = B.prob[p];
    if (P.rec) return __ldg(P.rec + u).z & CHUNK_LEN_MASK;
    const int64_t a = P.off[u], b = P.off[u + 1];
    return (b >= a) ? b - a : 0;
}

// 1. histogram of unit-length buckets per problem
__global__ void track_hist_kernel(const BatchParams B, int *hist)
{
    for (int p = 0; p < B.n_prob; p++) {
        const int64_t n = units_of(B.prob[p]);
        for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n;
             u += (int64_t)gridDim.x * blockDim.x)
            atomicAdd(&hist[p * NB + len_bucket(track_len(B, p, u))], 1);
    }
}

// 2. exclusive scans of a [rows][NB] histogram, one row per thread (rows are few)
__global__ void scan_rows_kernel(int *hist, int rows)
{
    const int r = threadIdx.x;
    if (r >= rows) return;
    int acc = 0;
    for (int b = 0; b < NB; b++) {
        const int c = hist[r * NB + b];
        hist[r * NB + b] = acc;
        acc += c;
    }
}

// 3. scatter every unit into its problem's sorted list
__global__ void track_scatter_kernel(const BatchParams B, int *cursor, int *perm)
{
    for (int p = 0; p < B.n_prob; p++) {
        const int64_t n = units_of(B.prob[p]);
        for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n;
             u += (int64_t)gridDim.x * blockDim.x) {
            const int pos = atomicAdd(&cursor[p * NB + len_bucket(track_len(B, p, u))], 1);
            perm[B.prob[p].perm_off + pos] = (int)u;
        }
    }
}

// Sub-problem and local index of a global item id.
__device__ __forceinline__ int sub_of(const BatchParams &B, int64_t item, int64_t &local)
{
    int s = 0;
    while (s + 1 < B.n_sub && item >= B.sub[s + 1].item_base) s++;
    local = item - B.sub[s].item_base;
    return s;
}

// 4./6. histogram and scatter of warp items (one row: all sub-problems together)
__global__ void item_hist_kernel(const BatchParams B, const int *perm, int *hist)
{
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < B.n_items;
         it += (int64_t)gridDim.x * blockDim.x) {
        int64_t local;
        const int s = sub_of(B, it, local);
        const BatchSub &S = B.sub[s];
        const int first = (int)(local * (32 / S.lpt));
        // items past the units counted on the device are empty: last bucket
        const int bucket = first < units_of(B.prob[S.prob])
                               ? len_bucket(track_len(B, S.prob,
                                                      perm[B.prob[S.prob].perm_off + first]))
                               : NB - 1;
        atomicAdd(&hist[bucket], 1);
    }
}

__global__ void item_scatter_kernel(const BatchParams B, const int *perm, int *cursor,
                                    int2 *queue)
{
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < B.n_items;
         it += (int64_t)gridDim.x * blockDim.x) {
        int64_t local;
        const int s = sub_of(B, it, local);
        const BatchSub &S = B.sub[s];
        const int first = (int)(local * (32 / S.lpt));
        const int bucket = first < units_of(B.prob[S.prob])
                               ? len_bucket(track_len(B, S.prob,
                                                      perm[B.prob[S.prob].perm_off + first]))
                               : NB - 1;
        const int pos = atomicAdd(&cursor[bucket], 1);
        queue[pos] = make_int2(s, first);
    }
}

template <int VEC, int EK>
__device__ __forceinline__ void attenuate_b(const float4 (&x)[VEC], float ds, float weight,
                                            const float2 *tab, const BatchParams &B,
                                            Vec<VEC> &psi, Vec<VEC> &tally)
{
    // the same arithmetic as the single-problem sweep, on blocks in the same layout
    const TableRef tr{tab, B.tab_n, B.tab_dx, B.tab_max};
    Vec<VEC> pmul;
    attenuate_row<VEC, EK, f32_pairs(VEC)>(x, ds, weight, tr, psi, tally, pmul);
}

// 7. the persistent sweep over the queue
template <int VEC, int EK>
__global__ void __launch_bounds__(512) batch_kernel(const BatchParams B, const int *perm,
                                                    const int2 *queue)
{
    extern __shared__ float2 s_tab[];
    if constexpr (EK == EXPK_TABLE) {
        const float2 *src = reinterpret_cast<const float2 *>(B.table);
        for (int k = threadIdx.x; k < B.tab_n; k += blockDim.x) s_tab[k] = src[k];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long q = 0;
        if (lane == 0) q = atomicAdd(B.counter, 1ULL);
        q = __shfl_sync(FULL, q, 0);
        if (q >= (unsigned long long)B.n_items) break;
        const int2 item = queue[q];
        const BatchSub &S = B.sub[item.x];
        const BatchProb &P = B.prob[S.prob];
        const int lpt = S.lpt;
        const int sw = lane / lpt, sl = lane - sw * lpt;
        const int pos = item.y + sw;
        int t = -1;  // this sub-warp's unit: a track, or a chunk record
        if (pos < units_of(P) && sw < 32 / lpt) t = perm[P.perm_off + pos];
        const int g0 = S.g_begin + sl * VEC;
        const int nvalid = S.g_begin + S.g_count - g0;
        int64_t beg = 0, len = 0;
        const float *psi_src = nullptr;
        float *psi_dst = nullptr;  // null: a non-last chunk's outgoing psi is not kept
        if (t >= 0) {
            int64_t end;
            int trk = t;
            if (P.rec) {
                const int4 r = __ldg(P.rec + t);
                beg = (int64_t)(uint32_t)r.x | ((int64_t)r.y << 32);
                end = beg + (r.z & CHUNK_LEN_MASK);
                trk = r.w;
                if ((unsigned)trk >= (unsigned)P.T) end = -1;  // reported below
                const bool single = (r.z & CHUNK_SINGLE) != 0;
                psi_src = single ? P.psi + (int64_t)trk * P.Gs : P.start + (int64_t)t * P.Gs;
                psi_dst = (single || (r.z & CHUNK_LAST)) ? P.psi + (int64_t)trk * P.Gs
                                                         : nullptr;
            } else {
                beg = P.off[t];
                end = P.off[t + 1];
                psi_src = psi_dst = P.psi + (int64_t)t * P.Gs;
            }
            if (beg >= 0 && beg <= end && end <= P.S) {
                len = end - beg;
            } else {
                if (sl == 0) atomicOr(B.err, DEVERR_OFFSETS);
                t = -1;
            }
        }
        const bool act = t >= 0 && nvalid > 0;
        int64_t maxlen = len;
        for (int o = 16; o > 0; o >>= 1) {
            const int64_t other = __shfl_xor_sync(FULL, maxlen, o);
            maxlen = other > maxlen ? other : maxlen;
        }
        Vec<VEC> psi;
        if (act) psi = ld_psi<VEC>(psi_src + g0, nvalid);
        const float4 *bb = P.blk + g0;
        int cw = -1;
        float dw = 0.0f;
        for (int64_t j = 0; j < maxlen; j++) {
            const int k = (int)(j & (lpt - 1));
            if (k == 0) {
                cw = -1;
                dw = 0.0f;
                const int64_t jj = j + sl;
                if (t >= 0 && jj < len) {
                    const int r = ld_stream(P.reg + beg + jj);
                    const int iv = ld_stream(P.itv + beg + jj);
                    dw = ld_stream(P.ds + beg + jj);
                    if ((unsigned)r < (unsigned)P.R && (unsigned)iv < (unsigned)P.I)
                        cw = r * P.I + iv;
                    else
                        atomicOr(B.err, DEVERR_INDEX);
                }
            }
            const int c = __shfl_sync(FULL, cw, k, lpt);
            const float d = __shfl_sync(FULL, dw, k, lpt);
            if (act && j < len && c >= 0) {
                float4 x[VEC];
#pragma unroll
                for (int v = 0; v < VEC; v++) x[v] = __ldg(bb + c * P.Gs + v);
                Vec<VEC> tally;
                attenuate_b<VEC, EK>(x, d, B.weight, s_tab, B, psi, tally);
                red_row<VEC>(P.ff + c * P.Gs + g0, tally, nvalid);
            }
        }
        if (act && psi_dst) st_psi<VEC>(psi_dst + g0, psi, nvalid);
    }
}

template <int VEC, int EK>
const void *bfn() { return reinterpret_cast<const void *>(&batch_kernel<VEC, EK>); }

const void *pick(int vec, int ek)
{
    const bool tab = ek == EXPK_TABLE;
    if (vec == 1) return tab ? bfn<1, EXPK_TABLE>() : bfn<1, EXPK_PLAIN>();
    if (vec == 2) return tab ? bfn<2, EXPK_TABLE>() : bfn<2, EXPK_PLAIN>();
    if (vec == 4) return tab ? bfn<4, EXPK_TABLE>() : bfn<4, EXPK_PLAIN>();
    return nullptr;
}

int grid_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > grid_cap(8)) b = grid_cap(8);
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

int batch_blocks_per_sm(int vec, int ek, int warps_per_block, size_t smem)
{
    const void *fn = pick(vec, ek);
    int n = 0;
    if (!fn || warps_per_block < 1 || warps_per_block > 16) return 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, warps_per_block * 32, smem) !=
        cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_batch(const BatchParams &B, const BatchWork &W, int vec, int ek,
                         int warps_per_block, int blocks, cudaStream_t st)
{
    const void *fn = pick(vec, ek);
    if (!fn || blocks < 1 || warps_per_block < 1 || warps_per_block > 16)
        return cudaErrorInvalidValue;
    cudaError_t e;
    int64_t max_t = 0;
    for (int p = 0; p < B.n_prob; p++) {
        const int64_t u = units_bound(B.prob[p]);
        max_t = u > max_t ? u : max_t;
    }
    // length-sorted track lists
    if ((e = cudaMemsetAsync(W.hist, 0, sizeof(int) * NB * (B.n_prob + 1), st))) return e;
    track_hist_kernel<<<grid_for(max_t), 256, 0, st>>>(B, W.hist);
    scan_rows_kernel<<<1, 32, 0, st>>>(W.hist, B.n_prob);
    track_scatter_kernel<<<grid_for(max_t), 256, 0, st>>>(B, W.hist, W.perm);
    // longest-first queue of warp items
    int *ih = W.hist + NB * B.n_prob;
    item_hist_kernel<<<grid_for(B.n_items), 256, 0, st>>>(B, W.perm, ih);
    scan_rows_kernel<<<1, 32, 0, st>>>(ih, 1);
    item_scatter_kernel<<<grid_for(B.n_items), 256, 0, st>>>(B, W.perm, ih, W.queue);
    if ((e = cudaGetLastError())) return e;
    if ((e = cudaMemsetAsync(B.counter, 0, sizeof(unsigned long long), st))) return e;
    const size_t smem = ek == EXPK_TABLE ? (size_t)B.tab_n * sizeof(float2) : 0;
    if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
        return e;
    BatchParams copy = B;
    const int *perm = W.perm;
    const int2 *queue = W.queue;
    void *args[] = {&copy, &perm, &queue};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(warps_per_block * 32), args, smem, st);
}

}  // namespace moc
