// moc_split.cu — long tracks cut into chunks that sweep in parallel.
//
// psi is carried along a track segment by segment (src/cpu/kernel.c:53, 289-331): per
// group psi' = p psi + b, with p = exp(-tau) and b the source part of the attenuated
// flux, which does not depend on psi. A run of segments is therefore the affine map
// psi_out = a psi_in + b, with a the product of the p's and b the sweep of the run from
// psi = 0. A track of more than SPLIT_MIN_FACTOR * C segments is cut into chunks of C
// segments (the last one shorter):
//   1. records: an exclusive scan of the chunk counts of the tracks, one record per chunk;
//   2. maps: the sweep kernel in map mode composes (a, b) of every non-last chunk (the
//      records pass lists them; for the adjoint it lists every chunk of a split track);
//   3. starts: per track and group, psi entering each chunk, start_0 = psi_in,
//      start_{k+1} = a_k start_k + b_k;
//   4. the sweep runs every chunk from its start, with tallies, all chunks at once; a
//      split track's last chunk writes the track's outgoing psi.
// Whether and where a track is cut depends on its length only, so a track's psi is the
// same whatever the other tracks of the problem are. Shorter tracks are one record and
// sweep exactly as in one pass.
#include "moc_internal.h"

namespace moc {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_BATCH = 8;  // chunk maps loaded ahead of the start scan's FMA chain

__device__ __forceinline__ bool track_ok(int64_t a, int64_t b, int64_t S)
{
    return a >= 0 && a <= b && b <= S;
}

__device__ __forceinline__ int64_t chunks_of(int64_t len, int64_t C)
{
    return len > SPLIT_MIN_FACTOR * C ? (len + C - 1) / C : 1;
}

// Records of track t (1 for a track with bad offsets: it is reported and skipped).
__device__ __forceinline__ int64_t count_of(const SweepParams &P, const SplitWork &W, int64_t t)
{
    const int64_t a = P.off[t], b = P.off[t + 1];
    const int64_t n = track_ok(a, b, P.S) ? chunks_of(b - a, W.chunk) : 1;
    return n < W.cap ? n : W.cap;
}

// Map items of a track with n records: its non-last chunks (forward) or all its chunks
// (adjoint); none for a whole track.
__device__ __forceinline__ int64_t maps_of(int64_t n, int map_all)
{
    return n > 1 ? (map_all ? n : n - 1) : 0;
}

// Records and map items of a track, scanned together as a pair of 64-bit counts (offsets
// that are not a partition of [0, S] can make either total large; records beyond the
// workspace are dropped and reported, and neither count can spill into the other).
struct Counts {
    int64_t rec, map;
};
__device__ __forceinline__ Counts operator+(Counts a, Counts b)
{
    return Counts{a.rec + b.rec, a.map + b.map};
}
__device__ __forceinline__ Counts operator-(Counts a, Counts b)
{
    return Counts{a.rec - b.rec, a.map - b.map};
}
__device__ __forceinline__ Counts counts_of(int64_t n, int map_all)
{
    return Counts{n, maps_of(n, map_all)};
}
__device__ __forceinline__ Counts shfl_up(Counts v, int o)
{
    return Counts{(int64_t)__shfl_up_sync(FULL, (long long)v.rec, o),
                  (int64_t)__shfl_up_sync(FULL, (long long)v.map, o)};
}

// Inclusive scan of v over the block; *total = the block's sum. Called by every thread.
__device__ Counts block_incl_scan(Counts v, Counts *total)
{
    __shared__ Counts ws[SCAN_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const Counts u = shfl_up(v, o);
        if (lane >= o) v = v + u;
    }
    if (lane == 31) ws[w] = v;
    __syncthreads();
    if (w == 0) {
        Counts s = lane < nw ? ws[lane] : Counts{0, 0};
        for (int o = 1; o < 32; o <<= 1) {
            const Counts u = shfl_up(s, o);
            if (lane >= o) s = s + u;
        }
        if (lane < nw) ws[lane] = s;
    }
    __syncthreads();
    if (w > 0) v = v + ws[w - 1];
    *total = ws[nw - 1];
    __syncthreads();  // ws is reused by the next call
    return v;
}

// W.bsum holds one Counts (two int64) per scan block.
__global__ void __launch_bounds__(SCAN_BLOCK) scan_sums_kernel(const SweepParams P,
                                                               const SplitWork W)
{
    const int64_t t = blockIdx.x * (int64_t)SCAN_BLOCK + threadIdx.x;
    Counts total;
    block_incl_scan(t < P.T ? counts_of(count_of(P, W, t), W.map_all) : Counts{0, 0}, &total);
    if (threadIdx.x == 0) reinterpret_cast<Counts *>(W.bsum)[blockIdx.x] = total;
}

// One block: exclusive scan of the nb block sums, in place.
__global__ void __launch_bounds__(SCAN_BLOCK) scan_bsum_kernel(int64_t *bsum64, int64_t nb)
{
    Counts *bsum = reinterpret_cast<Counts *>(bsum64);
    Counts carry{0, 0};
    for (int64_t b0 = 0; b0 < nb; b0 += SCAN_BLOCK) {
        const int64_t i = b0 + threadIdx.x;
        const Counts v = i < nb ? bsum[i] : Counts{0, 0};
        Counts total;
        const Counts incl = block_incl_scan(v, &total);
        if (i < nb) bsum[i] = carry + incl - v;
        carry = carry + total;
    }
}

// base[t] = exclusive prefix of the record counts; thread t then writes track t's
// records and the ids of its non-last chunks into the map list.
__global__ void __launch_bounds__(SCAN_BLOCK) split_records_kernel(const SweepParams P,
                                                                   const SplitWork W)
{
    const int64_t t = blockIdx.x * (int64_t)SCAN_BLOCK + threadIdx.x;
    const int64_t n = t < P.T ? count_of(P, W, t) : 0;
    const Counts pk = counts_of(n, W.map_all);
    const int64_t nm = pk.map;
    Counts total;
    const Counts incl = block_incl_scan(pk, &total);
    if (t >= P.T) return;
    const Counts excl = reinterpret_cast<const Counts *>(W.bsum)[blockIdx.x] + incl - pk;
    const int64_t b = excl.rec, mb = excl.map;
    W.base[t] = b;
    if (t == P.T - 1) {
        W.base[P.T] = b + n;
        *W.n_map = mb + nm;
    }
    for (int64_t k = 0; k < nm; k++)
        if (b + k < W.cap && mb + k < W.cap) W.map_list[mb + k] = b + k;
    const int64_t a = P.off[t], e = P.off[t + 1];
    bool dropped = false;
    auto put = [&](int64_t q, int64_t beg, int64_t len, int32_t flags) {
        if (q >= W.cap) {  // overlapping offsets: more chunks than S allows
            dropped = true;
            return;
        }
        W.rec[q] = make_int4((int32_t)(uint32_t)(uint64_t)beg, (int32_t)(beg >> 32),
                             (int32_t)len | flags, (int32_t)t);
    };
    if (!track_ok(a, e, P.S)) {
        atomicOr(P.err, DEVERR_OFFSETS);
        put(b, 0, 0, CHUNK_SINGLE);  // psi passes through unchanged
        return;
    }
    if (n == 1) {
        put(b, a, e - a, CHUNK_SINGLE);
    } else {
        const int64_t C = W.chunk;
        for (int64_t k = 0; k < n; k++) {
            const int64_t beg = a + k * C;
            const int64_t len = k + 1 < n ? C : e - beg;
            put(b + k, beg, len, (k + 1 < n ? 0 : CHUNK_LAST) | (k == 0 ? CHUNK_FIRST : 0));
        }
    }
    if (dropped) atomicOr(P.err, DEVERR_OFFSETS);
}

// The split tracks, for the start passes: track u's first record, or -1 for a track that
// is not cut. They are found from whichever list is shorter, the tracks (by_track) or the
// map items (every split track's first chunk is one of them, once).
__device__ __forceinline__ int64_t split_track_of(const SweepParams &P, const SplitWork &W,
                                                  bool by_track, int64_t u, int64_t &t)
{
    if (by_track) {
        t = u;
        const int64_t b = W.base[t];
        return b < W.cap ? b : -1;
    }
    const int64_t q = W.map_list[u];
    if ((uint64_t)q >= (uint64_t)W.cap) return -1;
    const int4 r = W.rec[q];
    if (!(r.z & CHUNK_FIRST) || (unsigned)r.w >= (unsigned)P.T) return -1;
    t = r.w;
    return q;
}

// psi entering each chunk of every split track: one warp per (split track, 32-group
// slice), its lanes over the slice's groups (split_track_of finds the tracks).
__global__ void split_start_kernel(const SweepParams P, const SplitWork W)
{
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float *__restrict__ ma = P.map_a;
    const float *__restrict__ mb = P.map_b;
    float *__restrict__ start = P.start;
    int64_t n_map = *W.n_map;
    n_map = n_map < W.cap ? n_map : W.cap;
    const bool by_track = n_map > P.T;
    const int nsl = (P.G + 31) / 32;
    const int64_t units = (by_track ? (int64_t)P.T : n_map) * nsl;
    for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < units;
         u += nwarps) {
        const int64_t m = u / nsl;
        const int g = (int)(u - m * nsl) * 32 + lane;
        int64_t t = 0;
        const int64_t b = split_track_of(P, W, by_track, m, t);
        if (b < 0) continue;
        const int64_t e = W.base[t + 1] < W.cap ? W.base[t + 1] : W.cap;
        const int64_t nq = e - b;
        if (nq >= 2 && g < P.G) {
            float psi = P.psi[t * P.Gs + g];
            // the maps of SCAN_BATCH chunks are loaded before their dependent FMAs, so the
            // chain waits for memory once per batch, not once per chunk
            for (int64_t c0 = 0; c0 < nq; c0 += SCAN_BATCH) {
                float av[SCAN_BATCH], bv[SCAN_BATCH];
#pragma unroll
                for (int k = 0; k < SCAN_BATCH; k++) {
                    const int64_t row = (b + c0 + k) * P.Gs + g;
                    av[k] = c0 + k + 1 < nq ? ma[row] : 0.0f;
                    bv[k] = c0 + k + 1 < nq ? mb[row] : 0.0f;
                }
#pragma unroll
                for (int k = 0; k < SCAN_BATCH; k++) {
                    if (c0 + k < nq) start[(b + c0 + k) * P.Gs + g] = psi;
                    psi = fmaf(av[k], psi, bv[k]);
                }
            }
        }
    }
}

}  // namespace

int64_t split_max_records(int64_t T, int64_t S, int chunk)
{
    return T + S / chunk + 1;
}

cudaError_t launch_split_records(const SweepParams &P, const SplitWork &W, cudaStream_t st)
{
    if (P.T < 1 || W.chunk < 1) return cudaErrorInvalidValue;
    const int64_t nb = (P.T + SCAN_BLOCK - 1) / SCAN_BLOCK;
    scan_sums_kernel<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(P, W);
    scan_bsum_kernel<<<1, SCAN_BLOCK, 0, st>>>(W.bsum, nb);
    split_records_kernel<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(P, W);
    return cudaGetLastError();
}

cudaError_t launch_split_start(const SweepParams &P, const SplitWork &W, int sm_count,
                               cudaStream_t st)
{
    split_start_kernel<<<sm_count * 8, 256, 0, st>>>(P, W);
    return cudaGetLastError();
}

}  // namespace moc
