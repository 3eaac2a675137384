// moc_internal.h — kernels and launchers behind the C ABI (not part of the ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "moc_attenuate.h"

namespace moc {

// The size / enum / alignment checks of moc_attenuate_fwd, and its check that every
// problem pointer is device (or managed) memory.
moc_status_t check_args(const moc_problem_t *p, const moc_fwd_opts_t *o);
bool all_device_accessible(const moc_problem_t *p);

// Device error bits, OR-ed into the handle's error word by the kernels.
enum : int32_t {
    DEVERR_OFFSETS = 1,  // a track's [begin, end) is not inside [0, S]
    DEVERR_INDEX = 2,    // a segment's region or interval is out of range
};

// How 1 - exp(-tau) and the cancelling terms are evaluated.
enum ExpKind : int {
    EXPK_PLAIN = 0,   // 1 - ex2(-tau log2 e); the reference's expressions (drop-in)
    EXPK_TABLE = 1,   // the reference's table, bit-exact lookup
    EXPK_STABLE = 2,  // Taylor branches for small tau, range-reduced ex2 elsewhere
};

// Everything a sweep launch reads. Device pointers.
struct SweepParams {
    int32_t R, I, G, Gs, T, n_chunks;
    int64_t S, n_items;
    const int64_t *off;
    const int32_t *reg;
    const uint8_t *itv;
    const float *ds;
    const float *sigT;   // [R][Gs]
    const float *coef;   // [R*I][3][Gs]: q0, q1*mu, q2*mu2
    float *ff;           // [R*I][Gs]
    float *psi;          // [T][Gs]
    float weight;
    const float *table;  // [2*tab_n] (slope, intercept) pairs, EXPK_TABLE only
    int32_t tab_n;
    float tab_dx, tab_max;
    int32_t *err;
    unsigned long long *counter;  // work-queue head, zeroed before each launch
};

// Axial coefficients of every (region, interval): coef[c][0] = q0, [1] = q1*mu,
// [2] = q2*mu2, rounded exactly as src/cpu/kernel.c:111-191 and the first product of
// kernel.c:250-251 / 311-322 round them.
cudaError_t launch_prep_coef(const float *source, float *coef, int R, int I, int Gs,
                             float dz, float zin, float mu, float mu2, cudaStream_t st);

// The forward sweep (persistent, one warp per (track, group chunk) work item).
struct FwdConfig {
    int vec;              // groups per lane: 1, 2, 4
    int warps_per_block;  // 1..32
    int exp_kind;         // ExpKind
    int blocks;           // grid size (0 = fill the GPU)
};
cudaError_t launch_fwd(const SweepParams &p, const FwdConfig &cfg, cudaStream_t st);
// Resident blocks per SM for a configuration (0 if the configuration is invalid).
int fwd_blocks_per_sm(const FwdConfig &cfg, size_t smem_bytes);

// Checked mode: scan offsets and segment indices, OR errors into p.err. No writes
// to psi or fine_flux.
cudaError_t launch_check(const SweepParams &p, cudaStream_t st);

}  // namespace moc
