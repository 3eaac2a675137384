// moc_trace.cu — track generation: the plan of 3D tracks (host) and the GPU walk that
// turns them into the sweep's CSR segment descriptors (include/moc_tracks.h).
//
// The reference kernel draws every segment's region, interval and length at random
// (src/cpu/kernel.c:47-50, src/cuda/kernel.cu:52-60); this file produces them by ray
// tracing straight tracks through a pin-cell lattice with ringed fuel cylinders and fine
// axial intervals. The walk runs one thread per track in FP64 and this file is compiled
// without multiply-add contraction (-fmad=false), so every crossing, midpoint and length
// is the correctly rounded result of the same operations as the C oracle's
// (oracle/tracks.c), and the descriptors match it bit for bit.
//
// Crossings along a track, t being the distance along its 2D line:
//   grid line x = i P:         t = (i P - x0) rux
//   grid line y = j P:         t = (j P - y0) ruy
//   ring k of pin (i, j):      t = w -+ sqrt(r_k^2 - d^2), w = (c - p0).u,
//                              d = (c - p0) x u (signed distance of the centre c)
//   fine axial plane z = m dz: t = ta + (m dz - za) rcot
// A segment runs between consecutive distinct crossings strictly inside (ta, tb), plus
// ta and tb; its cell is that of its midpoint and its length (t1 - t0) rsin.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "moc_internal.h"
#include "moc_tracks.h"

namespace moc {

namespace {

constexpr double INF = __builtin_huge_val();

// Ordering key of a double: for values that are not NaN and a reference t >= +0, x <= t
// exactly when key(x) <= key(t) (non-negative doubles order as their bit patterns, and
// every negative one, -0 included, is below every non-negative one). The walk orders its
// crossings with these integer comparisons, off the FP64 pipe.
__host__ __device__ __forceinline__ int64_t key(double x)
{
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    int64_t r;
    std::memcpy(&r, &x, sizeof(r));
    return r;
#endif
}

// Geometry constants of the walk, derived from moc_geometry_t by trace_geo().
struct TraceGeo {
    int nx, ny, K, n_axial, n_int, NZ;
    double P, rP, dz, rdz;
    double r2[MOC_TRACKS_MAX_RINGS];  // ring radii squared, equal areas
    // device tables (trace_tables): grid lines i P (i = 0..nx, j = 0..ny), pin centres
    // (i + 1/2) P, fine planes m dz (m = 0..NZ); each entry the same rounded product the
    // oracle forms, so the walk needs no int-to-double conversion per crossing
    const double *lx, *ly, *cx, *cy, *pz;
};

// Entries of the tables of a geometry: (nx + 1) + (ny + 1) + nx + ny + (NZ + 1).
int64_t table_len(const moc_geometry_t *g)
{
    return 2 * ((int64_t)g->nx + g->ny) + 3 + (int64_t)g->n_axial * g->n_intervals;
}

// floor(x) clamped to [0, n - 1], from the bits of x (exact; integer pipe). Negative x
// (and -0) give 0, as floor's -1 (or 0) clamped does.
__host__ __device__ __forceinline__ int floor_clamp(double x, int n)
{
    const int64_t b = key(x);
    if (b < 0) return 0;
    const int e = (int)(b >> 52) - 1023;
    if (e < 0) return 0;
    if (e >= 31) return n - 1;
    const int64_t v = ((b & ((1ll << 52) - 1)) | (1ll << 52)) >> (52 - e);
    return v >= n ? n - 1 : (int)v;
}

bool geo_ok(const moc_geometry_t *g)
{
    return g && g->nx >= 1 && g->ny >= 1 && g->n_rings >= 1 &&
           g->n_rings <= MOC_TRACKS_MAX_RINGS && g->n_axial >= 1 && g->n_intervals >= 2 &&
           g->n_intervals <= 255 && g->pitch > 0.0 && g->fuel_radius > 0.0 &&
           g->fuel_radius < 0.45 * g->pitch && g->height > 0.0 && std::isfinite(g->pitch) &&
           std::isfinite(g->height) &&
           (int64_t)g->nx * g->ny * (g->n_rings + 1) * g->n_axial <= INT32_MAX &&
           (int64_t)g->n_axial * g->n_intervals <= (1 << 24);
}

bool quad_ok(const moc_quadrature_t *q)
{
    return q && q->n_azim >= 2 && q->n_azim % 2 == 0 && q->n_polar >= 2 &&
           q->n_polar % 2 == 0 && (q->both_directions == 0 || q->both_directions == 1) &&
           q->spacing > 0.0 && q->axial_spacing > 0.0 && std::isfinite(q->spacing) &&
           std::isfinite(q->axial_spacing);
}

TraceGeo trace_geo(const moc_geometry_t *g)
{
    TraceGeo G{};
    G.nx = g->nx;
    G.ny = g->ny;
    G.K = g->n_rings;
    G.n_axial = g->n_axial;
    G.n_int = g->n_intervals;
    G.NZ = g->n_axial * g->n_intervals;
    G.P = g->pitch;
    G.rP = 1.0 / g->pitch;
    G.dz = g->height / (double)G.NZ;
    G.rdz = (double)G.NZ / g->height;
    const double rf2 = g->fuel_radius * g->fuel_radius;
    for (int k = 0; k < G.K; k++) G.r2[k] = rf2 * ((double)(k + 1) / (double)G.K);
    return G;
}

TraceGeo trace_geo(const moc_geometry_t *g, const double *tab)
{
    TraceGeo G = trace_geo(g);
    G.lx = tab;
    G.ly = G.lx + (G.nx + 1);
    G.cx = G.ly + (G.ny + 1);
    G.cy = G.cx + G.nx;
    G.pz = G.cy + G.ny;
    return G;
}

__global__ void trace_tables_kernel(const TraceGeo G, double *tab)
{
    const int n = 2 * (G.nx + G.ny) + 3 + G.NZ;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int j = i;
        double v;
        if (j <= G.nx) {
            v = (double)j * G.P;
        } else if ((j -= G.nx + 1) <= G.ny) {
            v = (double)j * G.P;
        } else if ((j -= G.ny + 1) < G.nx) {
            v = ((double)j + 0.5) * G.P;
        } else if ((j -= G.nx) < G.ny) {
            v = ((double)j + 0.5) * G.P;
        } else {
            j -= G.ny;
            v = (double)j * G.dz;
        }
        tab[i] = v;
    }
}

// Region and interval of the point at t (the midpoint of a segment).
__host__ __device__ __forceinline__ void classify(const TraceGeo &G, const moc_track_t &tr,
                                                  double tm, int32_t &region, int &itv)
{
    const double xm = tr.x0 + tm * tr.ux, ym = tr.y0 + tm * tr.uy;
    const double zm = tr.za + (tm - tr.ta) * tr.cot;
    const int ix = floor_clamp(xm * G.rP, G.nx), iy = floor_clamp(ym * G.rP, G.ny);
    const double ddx = xm - G.cx[ix], ddy = ym - G.cy[iy];
    const double rr = ddx * ddx + ddy * ddy;  // >= +0: ordered by its key
    const int64_t kr = key(rr);
    int k = 0;
    while (k < G.K && !(kr < key(G.r2[k]))) k++;
    const int f = floor_clamp(zm * G.rdz, G.NZ);
    const int a = f / G.n_int;
    itv = f - a * G.n_int;
    region = ((iy * G.nx + ix) * (G.K + 1) + k) * G.n_axial + a;
}

// The walk of one track: visits its segments in order. EMIT = false counts them;
// EMIT = true writes segment k to base + k (base + n - 1 - k for a reversed track).
// Returns the count, or -1 if the record is invalid or the walk exceeds its bound.
template <bool EMIT>
__host__ __device__ int64_t walk(const TraceGeo &G, const moc_track_t &tr, int64_t base, int64_t n,
                        int32_t *reg, uint8_t *itv, float *dsv)
{
    if (!(tr.ta >= 0.0 && tr.tb >= tr.ta && tr.tb < INF && tr.rsin >= 1.0 && tr.rsin < INF &&
          tr.cot == tr.cot && tr.rcot == tr.rcot && tr.x0 == tr.x0 && tr.y0 == tr.y0 &&
          tr.za == tr.za && tr.rux == tr.rux && tr.ruy == tr.ruy))
        return -1;
    const int sx = tr.ux > 0.0 ? 1 : (tr.ux < 0.0 ? -1 : 0);
    const int sy = tr.uy > 0.0 ? 1 : (tr.uy < 0.0 ? -1 : 0);
    const int dm = tr.cot > 0.0 ? 1 : -1;
    if (tr.cot == 0.0) return -1;
    // every crossing is visited at most once; a bound on their number ends a walk on a
    // record whose fields disagree with one another
    const int64_t bound = 4 * ((int64_t)G.nx + G.ny + 4) * (G.K + 2) + 2 * (int64_t)G.NZ + 64;
    int64_t steps = 0;
    double t = tr.ta + 0.0;  // +0 for a record whose ta is -0
    int64_t kt = key(t);
    // start one cell behind the point at ta (never ahead of it); lines at or behind t
    // are passed below
    const double xa = tr.x0 + tr.ta * tr.ux, ya = tr.y0 + tr.ta * tr.uy;
    int ix = (int)fmax(fmin(floor(xa * G.rP), (double)G.nx + 1.0), -2.0) - sx;
    int iy = (int)fmax(fmin(floor(ya * G.rP), (double)G.ny + 1.0), -2.0) - sy;
    // the next grid line ahead must exist (index 0 .. nx): a start left of (below) the
    // lattice waits at the cell just outside it
    if (sx > 0 && ix < -1) ix = -1;
    if (sx < 0 && ix > G.nx) ix = G.nx;
    if (sy > 0 && iy < -1) iy = -1;
    if (sy < 0 && iy > G.ny) iy = G.ny;
    auto line_x = [&](int i) { return (i < 0 || i > G.nx) ? INF : (G.lx[i] - tr.x0) * tr.rux; };
    auto line_y = [&](int j) { return (j < 0 || j > G.ny) ? INF : (G.ly[j] - tr.y0) * tr.ruy; };
    int ixn = sx > 0 ? ix + 1 : ix, iyn = sy > 0 ? iy + 1 : iy;
    double txn = sx ? line_x(ixn) : INF, tyn = sy ? line_y(iyn) : INF;
    // ring crossings of the current cell: entering k = K-1 .. kmin, leaving kmin .. K-1
    double w = 0.0, dp2 = 0.0;
    int kmin = G.K, e = 0;
    auto setup_cell = [&]() {
        kmin = G.K;
        e = 0;
        if (ix < 0 || ix >= G.nx || iy < 0 || iy >= G.ny) return;
        const double dxc = G.cx[ix] - tr.x0;
        const double dyc = G.cy[iy] - tr.y0;
        w = dxc * tr.ux + dyc * tr.uy;
        const double dp = dxc * tr.uy - dyc * tr.ux;
        dp2 = dp * dp;
        // r2 - dp2 > 0 exactly when r2 > dp2 (both >= 0: ordered by their keys)
        const int64_t kd = key(dp2);
        while (kmin > 0 && kd < key(G.r2[kmin - 1])) kmin--;
    };
    // a ring's leaving crossing reuses the half-chord its entering one computed (every
    // entering event of the cell is evaluated, in order, before any leaving one)
    double hk[MOC_TRACKS_MAX_RINGS];
    auto ring_event = [&]() {
        const int nk = G.K - kmin;
        if (e >= 2 * nk) return INF;
        if (e < nk) {
            const int kk = G.K - 1 - e;
            const double h = sqrt(G.r2[kk] - dp2);
            hk[kk] = h;
            return w - h;
        }
        return w + hk[kmin + e - nk];
    };
    setup_cell();
    double tcn = ring_event();
    // fine axial planes, from one or two below (above) the start
    int m = (int)fmax(fmin(floor(tr.za * G.rdz), (double)G.NZ + 1.0), -1.0);
    m = dm > 0 ? (m - 1 < 0 ? 0 : m - 1) : (m + 2 > G.NZ ? G.NZ : m + 2);
    auto plane = [&](int mm) {
        return (mm < 0 || mm > G.NZ) ? INF : tr.ta + (G.pz[mm] - tr.za) * tr.rcot;
    };
    double tzn = plane(m);
    int64_t k = 0;
    const int64_t kb = key(tr.tb);
    while (kt < kb) {
        bool moved = false;
        while (key(txn) <= kt && steps++ < bound) {
            ix += sx;
            ixn += sx;
            txn = line_x(ixn);
            moved = true;
        }
        while (key(tyn) <= kt && steps++ < bound) {
            iy += sy;
            iyn += sy;
            tyn = line_y(iyn);
            moved = true;
        }
        if (moved) {
            setup_cell();
            tcn = ring_event();
        }
        while (key(tcn) <= kt && steps++ < bound) {
            e++;
            tcn = ring_event();
        }
        while (key(tzn) <= kt && steps++ < bound) {
            m += dm;
            tzn = plane(m);
        }
        if (steps >= bound) return -1;
        // every candidate is now above t >= 0, so their keys order them
        double tn = tr.tb;
        int64_t kn = kb;
        if (key(txn) < kn) { tn = txn; kn = key(txn); }
        if (key(tyn) < kn) { tn = tyn; kn = key(tyn); }
        if (key(tcn) < kn) { tn = tcn; kn = key(tcn); }
        if (key(tzn) < kn) { tn = tzn; kn = key(tzn); }
        if (!(kn > kt)) return -1;
        if constexpr (EMIT) {
            int32_t r;
            int iv;
            classify(G, tr, (t + tn) * 0.5, r, iv);
            const int64_t pos = tr.reversed ? base + n - 1 - k : base + k;
            if (k < n) {
                reg[pos] = r;
                itv[pos] = (uint8_t)iv;
                dsv[pos] = (float)((tn - t) * tr.rsin);
            }
        }
        k++;
        t = tn;
        kt = kn;
        if (++steps > bound) return -1;
    }
    return k;
}

// Upper bound of a track's segment count: the grid lines and fine planes its extent can
// cross, the ring crossings of every cell its 2D line can visit, plus one. -1 for a
// record the walk would reject.
__host__ __device__ __forceinline__ int64_t track_bound(const TraceGeo &G,
                                                       const moc_track_t &tr)
{
    const double L = tr.tb - tr.ta;
    if (!(L >= 0.0 && L < INF)) return -1;
    const double dx = L * fabs(tr.ux) * G.rP, dy = L * fabs(tr.uy) * G.rP;
    const double dz = L * fabs(tr.cot) * G.rdz;
    if (!(dx < 1e9 && dy < 1e9 && dz < 1e12)) return -1;
    const int64_t nx = (int64_t)dx + 2, ny = (int64_t)dy + 2, nz = (int64_t)dz + 2;
    return nx + ny + 2 * (int64_t)G.K * (nx + ny + 1) + nz + 1;
}

// bounds[t] -> bnd[t + 1] (0 and DEVERR_TRACK for a bad record)
__global__ void __launch_bounds__(256) trace_bound_kernel(const TraceGeo G,
                                                          const moc_track_t *__restrict__ tr,
                                                          int64_t T, int64_t *__restrict__ bnd,
                                                          int32_t *err)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t b = track_bound(G, tr[t]);
        if (b < 0) {
            atomicOr(err, DEVERR_TRACK);
            b = 0;
        }
        bnd[t + 1] = b;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) bnd[0] = 0;
}

// One walk per track into the scratch slot [bnd[t], bnd[t+1]), in walk order; its count
// to off[t + 1]. A bad record or a walk past its bound counts 0 and sets DEVERR_TRACK.
__global__ void __launch_bounds__(256) trace_walk_kernel(const TraceGeo G,
                                                         const moc_track_t *__restrict__ tr,
                                                         int64_t T,
                                                         const int64_t *__restrict__ bnd,
                                                         int64_t *__restrict__ off,
                                                         int32_t *__restrict__ reg,
                                                         uint8_t *__restrict__ itv,
                                                         float *__restrict__ dsv, int32_t *err)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T;
         t += (int64_t)gridDim.x * blockDim.x) {
        moc_track_t k = tr[t];
        k.reversed = 0;
        const int64_t b0 = bnd[t], cap = bnd[t + 1] - b0;
        int64_t n = walk<true>(G, k, b0, cap, reg, itv, dsv);
        if (n < 0 || n > cap) {
            atomicOr(err, DEVERR_TRACK);
            n = 0;
        }
        off[t + 1] = n;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) off[0] = 0;
}

// Scratch -> the caller's CSR arrays, one warp per track (reversed tracks last to first).
__global__ void __launch_bounds__(256) trace_compact_kernel(
    const moc_track_t *__restrict__ tr, int64_t T, const int64_t *__restrict__ bnd,
    const int64_t *__restrict__ off, const int32_t *__restrict__ sreg,
    const uint8_t *__restrict__ sitv, const float *__restrict__ sds, int32_t *__restrict__ reg,
    uint8_t *__restrict__ itv, float *__restrict__ dsv)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t t = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); t < T;
         t += nw) {
        const int64_t src = bnd[t], dst = off[t], n = off[t + 1] - dst;
        const bool rev = tr[t].reversed != 0;
        for (int64_t k = lane; k < n; k += 32) {
            const int64_t d = rev ? dst + n - 1 - k : dst + k;
            reg[d] = sreg[src + k];
            itv[d] = sitv[src + k];
            dsv[d] = sds[src + k];
        }
    }
}

__global__ void __launch_bounds__(256) trace_emit_kernel(const TraceGeo G,
                                                         const moc_track_t *__restrict__ tr,
                                                         int64_t T,
                                                         const int64_t *__restrict__ off,
                                                         int32_t *__restrict__ reg,
                                                         uint8_t *__restrict__ itv,
                                                         float *__restrict__ dsv, int32_t *err)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T;
         t += (int64_t)gridDim.x * blockDim.x) {
        const moc_track_t k = tr[t];
        const int64_t base = off[t], n = off[t + 1] - base;
        const int64_t got = walk<true>(G, k, base, n, reg, itv, dsv);
        if (got != n) atomicOr(err, DEVERR_TRACK);
    }
}

// In-place inclusive scan of x[0 .. n) (int64) in tiles of 1024: tile scans with tile
// sums, a scan of the tile sums by one block, then the tile offsets added.
constexpr int SCAN_TILE = 1024;

__device__ int64_t block_scan_incl(int64_t v, int64_t *sh)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int64_t s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t u = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += u;
        }
        sh[lane] = s;
    }
    __syncthreads();
    if (wid > 0) v += sh[wid - 1];
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(SCAN_TILE) scan_tiles_kernel(int64_t *x, int64_t n,
                                                               int64_t *tile_sum)
{
    __shared__ int64_t sh[32];
    const int64_t i = blockIdx.x * (int64_t)SCAN_TILE + threadIdx.x;
    int64_t v = i < n ? x[i] : 0;
    v = block_scan_incl(v, sh);
    if (i < n) x[i] = v;
    if (threadIdx.x == SCAN_TILE - 1) tile_sum[blockIdx.x] = v;
}

__global__ void __launch_bounds__(SCAN_TILE) scan_sums_kernel(int64_t *s, int64_t n)
{
    __shared__ int64_t sh[32];
    int64_t carry = 0;
    for (int64_t b = 0; b < n; b += SCAN_TILE) {
        const int64_t i = b + threadIdx.x;
        int64_t v = i < n ? s[i] : 0;
        v = block_scan_incl(v, sh) + carry;
        if (i < n) s[i] = v;
        if (threadIdx.x == SCAN_TILE - 1) sh[0] = v;
        __syncthreads();
        carry = sh[0];
        __syncthreads();
    }
}

__global__ void scan_add_kernel(int64_t *x, int64_t n, const int64_t *tile_sum)
{
    const int64_t tile = blockIdx.x + 1;  // tile 0 has nothing to add
    const int64_t i = tile * SCAN_TILE + threadIdx.x;
    if (i < n) x[i] += tile_sum[tile - 1];
}

int grid_tracks(int64_t T)
{
    int64_t b = (T + 255) / 256;
    if (b > grid_cap(64)) b = grid_cap(64);
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

int64_t trace_scan_scratch(int64_t n_tracks)
{
    return (n_tracks + SCAN_TILE - 1) / SCAN_TILE + 1;
}

namespace {

// inclusive scan of x[0 .. n) in place (tile sums in scratch)
cudaError_t scan_inclusive(int64_t *x, int64_t n, int64_t *scratch, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    scan_tiles_kernel<<<(unsigned)tiles, SCAN_TILE, 0, st>>>(x, n, scratch);
    if (tiles > 1) {
        scan_sums_kernel<<<1, SCAN_TILE, 0, st>>>(scratch, tiles);
        scan_add_kernel<<<(unsigned)(tiles - 1), SCAN_TILE, 0, st>>>(x, n, scratch);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace_bound(const moc_geometry_t *g, const moc_track_t *tr, int64_t T,
                               int64_t *bnd, int64_t *scratch, int32_t *err, cudaStream_t st)
{
    trace_bound_kernel<<<grid_tracks(T), 256, 0, st>>>(trace_geo(g), tr, T, bnd, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return scan_inclusive(bnd + 1, T, scratch, st);
}

int64_t trace_table_len(const moc_geometry_t *g) { return table_len(g); }

cudaError_t launch_trace_tables(const moc_geometry_t *g, double *tab, cudaStream_t st)
{
    const int64_t n = table_len(g);
    trace_tables_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(trace_geo(g), tab);
    return cudaGetLastError();
}

cudaError_t launch_trace_walk(const moc_geometry_t *g, const double *tab, const moc_track_t *tr,
                              int64_t T, const int64_t *bnd, int64_t *off, int64_t *scratch,
                              int32_t *sreg, uint8_t *sitv, float *sds, int32_t *err,
                              cudaStream_t st)
{
    trace_walk_kernel<<<grid_tracks(T), 256, 0, st>>>(trace_geo(g, tab), tr, T, bnd, off, sreg,
                                                       sitv, sds, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return scan_inclusive(off + 1, T, scratch, st);
}

cudaError_t launch_trace_compact(const moc_track_t *tr, int64_t T, const int64_t *bnd,
                                 const int64_t *off, const int32_t *sreg, const uint8_t *sitv,
                                 const float *sds, int32_t *reg, uint8_t *itv, float *ds,
                                 cudaStream_t st)
{
    if (T == 0) return cudaSuccess;
    int64_t blocks = (T + 7) / 8;
    if (blocks > grid_cap(16)) blocks = grid_cap(16);
    trace_compact_kernel<<<(unsigned)blocks, 256, 0, st>>>(tr, T, bnd, off, sreg, sitv, sds,
                                                           reg, itv, ds);
    return cudaGetLastError();
}

cudaError_t launch_trace_emit(const moc_geometry_t *g, const double *tab, const moc_track_t *tr,
                              int64_t T, const int64_t *off, int32_t *reg, uint8_t *itv,
                              float *ds, int32_t *err, cudaStream_t st)
{
    if (T == 0) return cudaSuccess;
    const TraceGeo G = trace_geo(g, tab);
    trace_emit_kernel<<<grid_tracks(T), 256, 0, st>>>(G, tr, T, off, reg, itv, ds, err);
    return cudaGetLastError();
}

bool trace_geometry_ok(const moc_geometry_t *g) { return geo_ok(g); }

}  // namespace moc

// ---------------------------------------------------------------------------------------
// Host-only entry points of include/moc_tracks.h.
// ---------------------------------------------------------------------------------------
extern "C" {

int32_t moc_geometry_regions(const moc_geometry_t *g)
{
    if (!moc::geo_ok(g)) return 0;
    return g->nx * g->ny * (g->n_rings + 1) * g->n_axial;
}

moc_status_t moc_geometry_volumes(const moc_geometry_t *g, double *vol)
{
    if (!moc::geo_ok(g) || !vol) return MOC_ERR_INVALID_ARG;
    const int K = g->n_rings, I = g->n_intervals;
    const double pi = 3.14159265358979323846;
    const double fuel = pi * g->fuel_radius * g->fuel_radius;
    const double h = g->height / ((double)g->n_axial * I);
    int64_t c = 0;
    for (int pin = 0; pin < g->nx * g->ny; pin++)
        for (int k = 0; k <= K; k++) {
            const double area = k < K ? fuel / K : g->pitch * g->pitch - fuel;
            for (int a = 0; a < g->n_axial; a++)
                for (int i = 0; i < I; i++) vol[c++] = area * h;
        }
    return MOC_OK;
}

double moc_tracks_weight(const moc_quadrature_t *q)
{
    if (!moc::quad_ok(q)) return 0.0;
    const double pi = 3.14159265358979323846;
    const double omega = (q->both_directions ? 2.0 : 4.0) * pi / ((double)q->n_azim * q->n_polar);
    return omega * q->spacing * q->axial_spacing;
}

// The plan. For azimuth a: direction u = (cos phi, sin phi), normal n = (-sin phi, cos phi);
// the lattice [0, W] x [0, Y] projects onto n as [cmin, cmax]; floor((cmax - cmin) / s)
// lines at spacing s, centred in that range; each clipped to the lattice (slab test) and
// re-based at its entry point, placed exactly on the entry face, with its length the
// walk's crossing of the exit face. The top of the box is the walk's top fine plane
// NZ (height / NZ). For polar bin p: mu = 1 - (2p + 1)/n_polar, sin = sqrt(1 -
// mu^2), cot = mu / sin; the 3D tracks over a 2D line of length L are z = z0 + t cot with
// z0 at vertical spacing axial_spacing / sin, centred in the range of z0 whose track meets
// the box ((-L cot, H) upwards, (0, H - L cot) downwards), clipped to 0 <= z <= H.
moc_status_t moc_tracks_plan(const moc_geometry_t *g, const moc_quadrature_t *q,
                             moc_track_t *tracks, int64_t cap, int64_t *n_tracks_out)
{
    if (!moc::geo_ok(g) || !moc::quad_ok(q) || !n_tracks_out || cap < 0 ||
        (cap > 0 && !tracks))
        return MOC_ERR_INVALID_ARG;
    const double pi = 3.14159265358979323846;
    const double W = (double)g->nx * g->pitch, Y = (double)g->ny * g->pitch;
    // the top as the walk's top fine plane, NZ (height / NZ)
    const int NZ = g->n_axial * g->n_intervals;
    const double H = (double)NZ * (g->height / (double)NZ);
    int64_t n = 0;
    auto put = [&](const moc_track_t &r) {
        if (n < cap) tracks[n] = r;
        n++;
    };
    for (int a = 0; a < q->n_azim; a++) {
        const double phi = pi * ((double)a + 0.5) / (double)q->n_azim;
        const double ux = cos(phi), uy = sin(phi);
        const double nxv = -uy, nyv = ux;
        const double c[4] = {0.0, W * nxv, Y * nyv, W * nxv + Y * nyv};
        double cmin = c[0], cmax = c[0];
        for (int i = 1; i < 4; i++) {
            cmin = c[i] < cmin ? c[i] : cmin;
            cmax = c[i] > cmax ? c[i] : cmax;
        }
        const int64_t nl = (int64_t)floor((cmax - cmin) / q->spacing);
        const double off = ((cmax - cmin) - (double)nl * q->spacing) * 0.5;
        for (int64_t l = 0; l < nl; l++) {
            const double cl = cmin + off + ((double)l + 0.5) * q->spacing;
            const double px = cl * nxv, py = cl * nyv;
            double tlo = -INFINITY, thi = INFINITY;
            if (ux != 0.0) {
                const double t1 = (0.0 - px) / ux, t2 = (W - px) / ux;
                tlo = fmax(tlo, fmin(t1, t2));
                thi = fmin(thi, fmax(t1, t2));
            } else if (!(px >= 0.0 && px <= W)) {
                continue;
            }
            if (uy != 0.0) {
                const double t1 = (0.0 - py) / uy, t2 = (Y - py) / uy;
                tlo = fmax(tlo, fmin(t1, t2));
                thi = fmin(thi, fmax(t1, t2));
            } else if (!(py >= 0.0 && py <= Y)) {
                continue;
            }
            if (!(thi > tlo)) continue;
            moc_track_t r;
            std::memset(&r, 0, sizeof(r));
            r.ux = ux;
            r.uy = uy;
            r.rux = 1.0 / ux;
            r.ruy = 1.0 / uy;
            r.azim = a;
            // entry on a face exactly, and the 2D length as the walk's crossing of the exit
            // face, so that the faces' grid lines coincide with the ends of the track
            const double xin = ux > 0.0 ? 0.0 : W, xout = ux > 0.0 ? W : 0.0;
            if (ux != 0.0 && tlo == fmin((0.0 - px) / ux, (W - px) / ux)) {
                r.x0 = xin;
                r.y0 = py + tlo * uy;
            } else {
                r.x0 = px + tlo * ux;
                r.y0 = 0.0;  // uy > 0: the y = 0 face
            }
            const double tyo = (Y - r.y0) * r.ruy;
            const double L = ux != 0.0 ? fmin((xout - r.x0) * r.rux, tyo) : tyo;
            if (!(L > 0.0)) continue;
            for (int p = 0; p < q->n_polar; p++) {
                const double mu = 1.0 - (2.0 * (double)p + 1.0) / (double)q->n_polar;
                const double s = sqrt(1.0 - mu * mu);
                const double cot = mu / s, rcot = s / mu;
                const double dz0 = q->axial_spacing / s;
                const double zlo = mu > 0.0 ? -L * cot : 0.0;
                const double zhi = mu > 0.0 ? H : H - L * cot;
                const int64_t nz = (int64_t)floor((zhi - zlo) / dz0);
                const double zoff = ((zhi - zlo) - (double)nz * dz0) * 0.5;
                r.polar = p;
                r.cot = cot;
                r.rcot = rcot;
                r.rsin = 1.0 / s;
                for (int64_t j = 0; j < nz; j++) {
                    const double z0 = zlo + zoff + ((double)j + 0.5) * dz0;
                    // the leaving plane's crossing exactly as the walk computes it
                    if (mu > 0.0) {
                        r.ta = z0 < 0.0 ? -z0 * rcot : 0.0;
                        r.za = z0 < 0.0 ? 0.0 : z0;
                        r.tb = fmin(L, r.ta + (H - r.za) * rcot);
                    } else {
                        r.ta = z0 > H ? (H - z0) * rcot : 0.0;
                        r.za = z0 > H ? H : z0;
                        r.tb = fmin(L, r.ta + (0.0 - r.za) * rcot);
                    }
                    if (!(r.tb > r.ta)) continue;
                    r.reversed = 0;
                    put(r);
                    if (q->both_directions) {
                        r.reversed = 1;
                        put(r);
                    }
                }
            }
        }
    }
    *n_tracks_out = n;
    return MOC_OK;
}

}  // extern "C"
