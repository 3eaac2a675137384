// moc_transport.cu — the source update after a sweep (include/moc_transport.h): tallies to
// scalar flux, scalar flux to the next fine source (scattering + fission), and the
// fission total for the eigenvalue; plus the gather of the regions' sigT from their
// materials.
//
// One warp per run of fine cells; lane l holds groups l, l + 32, ... (NJ of them), so
// every row scatter[m][g'][.] is read coalesced, and once for all the run's cells. The
// sum over g' runs in increasing g': phi[g'] is broadcast from the lane holding it and
// every lane extends its own chains with one fused multiply-add per group and cell, so
// each source value is the FP32 chain
//   acc = fma(scatter[m][g'][g], phi[g'], acc), g' = 0 .. G-1,
// and q = fma(chi[m][g], F * (1/k), acc) * (1 / 4 pi), which the oracle restates in C
// (oracle/transport.c) bit for bit. The file is compiled without contraction
// (-fmad=false) so that no other product is fused.
#include <cstdint>

#include "moc_internal.h"
#include "moc_transport.h"

namespace moc {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__global__ void region_sigT_kernel(const float *__restrict__ xs_sigT, int32_t M,
                                   const int32_t *__restrict__ material, int64_t R, int Gs,
                                   float *__restrict__ sigT, int32_t *err)
{
    const int64_t n = R * Gs;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / Gs;
        const int g = (int)(i - r * Gs);
        const int32_t m = material[r];
        if ((uint32_t)m >= (uint32_t)M) {
            if (g == 0) atomicOr(err, DEVERR_INDEX);
            sigT[i] = 0.0f;
            continue;
        }
        sigT[i] = xs_sigT[(int64_t)m * Gs + g];
    }
}

// Cells c0 .. c0 + NC - 1, all of material m: every row scatter[m][g'] loaded once
// serves the NC cells (each with its own chains, in the same order as one cell alone).
template <int NJ, int NC>
__device__ __forceinline__ void update_cells(const TransportParams &P, int64_t c0, int32_t m,
                                             const double *__restrict__ volume,
                                             const float *__restrict__ tally,
                                             float *__restrict__ source, double *fission,
                                             int lane)
{
    const int G = P.G, Gs = P.Gs;
    const float *S = P.scatter + (int64_t)m * G * Gs;
    const float *nuf = P.nu_fission + (int64_t)m * Gs;
    float phi[NC][NJ], acc[NC][NJ], F[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const float rv = (float)(1.0 / volume[c0 + c]);
        const float *row = tally + (c0 + c) * Gs;
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            const int g = lane + 32 * j;
            phi[c][j] = g < G ? row[g] * rv : 0.0f;
            acc[c][j] = 0.0f;
        }
        F[c] = 0.0f;
    }
#pragma unroll
    for (int jp = 0; jp < NJ; jp++) {
        const int nl = G - 32 * jp < 32 ? G - 32 * jp : 32;  // g' of this lane column
#pragma unroll 4
        for (int lp = 0; lp < nl; lp++) {
            const int gp = 32 * jp + lp;
            const float nf = __ldg(nuf + gp);
            const float *Srow = S + (int64_t)gp * Gs;
            float sv[NJ];
#pragma unroll
            for (int j = 0; j < NJ; j++) {
                const int g = lane + 32 * j;
                sv[j] = g < G ? __ldg(Srow + g) : 0.0f;
            }
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const float p = __shfl_sync(FULL, phi[c][jp], lp);
                F[c] = fmaf(nf, p, F[c]);
#pragma unroll
                for (int j = 0; j < NJ; j++) acc[c][j] = fmaf(sv[j], p, acc[c][j]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const float f = F[c] * P.rk;
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            const int g = lane + 32 * j;
            if (g < G) {
                const float chi = __ldg(P.chi + (int64_t)m * Gs + g);
                source[(c0 + c) * Gs + g] = fmaf(chi, f, acc[c][j]) * P.rpi;
            }
        }
        if (lane == 0) atomicAdd(fission, (double)F[c] * volume[c0 + c]);
    }
}

// One warp per run of 4 consecutive cells (a region's intervals share its material, and
// neighbouring regions often do too): the run at once when its 4 cells share a
// material, else cell by cell.
constexpr int CELLS_PER_WARP = 4;

template <int NJ>
__global__ void __launch_bounds__(256) source_update_kernel(
    TransportParams P, const int32_t *__restrict__ material, const double *__restrict__ volume,
    const float *__restrict__ tally, float *__restrict__ source, double *fission, int32_t *err)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t nrun = (P.ncell + CELLS_PER_WARP - 1) / CELLS_PER_WARP;
    for (int64_t run = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); run < nrun;
         run += nw) {
        const int64_t c0 = run * CELLS_PER_WARP;
        const int n = P.ncell - c0 < CELLS_PER_WARP ? (int)(P.ncell - c0) : CELLS_PER_WARP;
        int32_t m[CELLS_PER_WARP];
        bool same = n == CELLS_PER_WARP, bad = false;
#pragma unroll
        for (int c = 0; c < CELLS_PER_WARP; c++) {
            m[c] = c < n ? material[(c0 + c) / P.I] : -1;
            if (c < n && (uint32_t)m[c] >= (uint32_t)P.M) bad = true;
            if (c > 0 && m[c] != m[0]) same = false;
        }
        if (bad) {
            if (lane == 0) atomicOr(err, DEVERR_INDEX);
            same = false;
        }
        if (same) {
            update_cells<NJ, CELLS_PER_WARP>(P, c0, m[0], volume, tally, source, fission, lane);
        } else {
            for (int c = 0; c < n; c++)
                if ((uint32_t)m[c] < (uint32_t)P.M)
                    update_cells<NJ, 1>(P, c0 + c, m[c], volume, tally, source, fission, lane);
        }
    }
}

int grid_for(int64_t n, int per)
{
    int64_t b = (n + per - 1) / per;
    if (b > grid_cap(16)) b = grid_cap(16);
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_region_sigT(const moc_xs_t *xs, const int32_t *material, int64_t R,
                               float *sigT, int32_t *err, cudaStream_t st)
{
    if (R == 0) return cudaSuccess;
    region_sigT_kernel<<<grid_for(R * xs->group_stride, 256), 256, 0, st>>>(
        xs->sigT, xs->n_materials, material, R, xs->group_stride, sigT, err);
    return cudaGetLastError();
}

cudaError_t launch_source_update(const TransportParams &P, const int32_t *material,
                                 const double *volume, const float *tally, float *source,
                                 double *fission, int32_t *err, cudaStream_t st)
{
    if (P.ncell == 0) return cudaSuccess;
    const int blocks = grid_for((P.ncell + CELLS_PER_WARP - 1) / CELLS_PER_WARP, 8);
    const int nj = (P.G + 31) / 32;
    if (nj <= 1)
        source_update_kernel<1><<<blocks, 256, 0, st>>>(P, material, volume, tally, source,
                                                        fission, err);
    else if (nj <= 2)
        source_update_kernel<2><<<blocks, 256, 0, st>>>(P, material, volume, tally, source,
                                                        fission, err);
    else if (nj <= 4)
        source_update_kernel<4><<<blocks, 256, 0, st>>>(P, material, volume, tally, source,
                                                        fission, err);
    else if (nj <= 8)
        source_update_kernel<8><<<blocks, 256, 0, st>>>(P, material, volume, tally, source,
                                                        fission, err);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace moc
