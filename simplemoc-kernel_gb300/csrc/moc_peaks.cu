// moc_peaks.cu — microbenchmarks for the roofline of the sweep (libmocpeaks.so).
//
// The sweep is not bound by HBM or tensor cores but by L2 (row gathers and tally
// reductions into L2-resident tables) and by FP32/MUFU issue. None of those peaks is a
// plain HBM copy or a bf16 GEMM, so this file measures them on the GPU at hand:
//   [0] L2 streaming read GB/s   float4 __ldcg over a 64 MiB buffer, many passes
//   [1] L2 row-gather GB/s       one random 512-byte row per warp from a 96 MiB table
//                                (the sweep's sigT / coefficient row pattern)
//   [2] L2 vector-reduction GB/s red.global.add.v4.f32 of random 512-byte rows into a
//                                25.6 MB array (the sweep's tally pattern), 16 B/lane
//   [3] FP32 FMA TFLOP/s         independent FMA chains, 2 flops each
//   [4] MUFU ex2 Gop/s           ex2.approx chains
//   [5] HBM read GB/s            float4 __ldcs over a 2 GiB buffer
//   [6..8] row_mix: 512-byte rows, four streams per warp (gathers, reductions, 4:1 mix)
//   [9] FP64 FMA TFLOP/s
//   [10..12] row_mix_wide: the sweep's access shape at its most parallel: 1 KB rows read
//       with one 256-bit load per lane (ld.global.nc.v8.f32) and 256-byte tally rows
//       reduced with red.global.add.v2.f32, eight independent row streams per warp, the
//       best of 8, 16 and 24 warps of 256 threads per SM: gathers only, reductions only,
//       and the sweep's mix (a 1 KB gather per 256-byte reduction: per segment and group
//       16 B read, 4 B reduced)
//   [13] packed FP32 FMA TFLOP/s (fma.rn.f32x2 chains, 4 flops per instruction)
// Every index is taken modulo its buffer; no kernel waits on anything.
#include <cstdint>
#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__global__ void stream_read(const float4 *__restrict__ buf, int64_t n4, int passes, float *out,
                            int streaming)
{
    const int64_t T = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float acc = 0.0f;
    for (int p = 0; p < passes; p++)
        for (int64_t k = tid; k < n4; k += T) {
            const float4 v = streaming ? __ldcs(buf + k) : __ldcg(buf + k);
            acc += v.x + v.y + v.z + v.w;
        }
    if (acc == 1234.5f) out[tid] = acc;  // keeps the loads alive
}

__global__ void row_gather(const float4 *__restrict__ rows, uint32_t n_rows, int iters,
                           float *out)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    float acc = 0.0f;
    for (int i = 0; i < iters; i++) {
        const uint32_t r = hash32(warp * 7919u + (uint32_t)i) % n_rows;
        const float4 v = __ldg(rows + (int64_t)r * 32 + lane);
        acc += v.x + v.y + v.z + v.w;
    }
    if (acc == 1234.5f) out[warp] = acc;
}

__global__ void row_reduce(float *ff, uint32_t n_rows, int iters)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (int i = 0; i < iters; i++) {
        const uint32_t r = hash32(warp * 104729u + (uint32_t)i) % n_rows;
        float *p = ff + (int64_t)r * 128 + lane * 4;
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(1.0f),
                     "f"(1.0f), "f"(1.0f), "f"(1.0f)
                     : "memory");
    }
}

// Lean variants: rows drawn by a 32-bit LCG over a power-of-two row count (two integer
// operations per row), four independent streams per warp for memory-level parallelism,
// so the issue of the loop itself does not limit the L2.
//   mode 0: gathers only; 1: reductions only; 2: four gathers per reduction (the sweep's
//   byte mix: a 16-byte cell block per group read, a 4-byte tally per group reduced).
__global__ void row_mix(const float4 *__restrict__ rows, float *ff, int log2_rows,
                        int log2_ff_rows, int iters, int mode, float *out)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t s0 = hash32(warp * 4 + 1), s1 = hash32(warp * 4 + 2), s2 = hash32(warp * 4 + 3),
             s3 = hash32(warp * 4 + 4);
    const int sh = 32 - log2_rows, shf = 32 - log2_ff_rows;
    float acc = 0.0f;
    for (int i = 0; i < iters; i++) {
        s0 = s0 * 1664525u + 1013904223u;
        s1 = s1 * 1664525u + 1013904223u;
        s2 = s2 * 1664525u + 1013904223u;
        s3 = s3 * 1664525u + 1013904223u;
        if (mode != 1) {
            const float4 a = __ldg(rows + (size_t)(s0 >> sh) * 32 + lane);
            const float4 b = __ldg(rows + (size_t)(s1 >> sh) * 32 + lane);
            const float4 c = __ldg(rows + (size_t)(s2 >> sh) * 32 + lane);
            const float4 d = __ldg(rows + (size_t)(s3 >> sh) * 32 + lane);
            acc += (a.x + b.y) + (c.z + d.w);
        }
        if (mode != 0) {
            float *p = ff + (size_t)(s0 >> shf) * 128 + lane * 4;
            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(1.0f),
                         "f"(1.0f), "f"(1.0f), "f"(1.0f)
                         : "memory");
            if (mode == 1) {
                float *q = ff + (size_t)(s1 >> shf) * 128 + lane * 4;
                asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(q),
                             "f"(1.0f), "f"(1.0f), "f"(1.0f), "f"(1.0f)
                             : "memory");
            }
        }
    }
    if (acc == 1234.5f) out[warp] = acc;
}

// The sweep's shape, as parallel as it can be issued: eight independent streams per warp,
// each a random 1 KB row (64 float4; a lane reads float4 2l and 2l + 1 with one 256-bit
// load) and a random 256-byte tally row (a lane reduces two floats).
//   mode 0: gathers only; 1: reductions only; 2: one gather and one reduction per stream.
constexpr int WIDE_K = 8;
__global__ void row_mix_wide(const float4 *__restrict__ rows, float *ff, int log2_rows,
                             int log2_ff_rows, int iters, int mode, float *out)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t st[WIDE_K];
#pragma unroll
    for (int k = 0; k < WIDE_K; k++) st[k] = hash32(warp * WIDE_K + k + 1);
    const int sh = 32 - log2_rows, shf = 32 - log2_ff_rows;
    float acc = 0.0f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < WIDE_K; k++) st[k] = st[k] * 1664525u + 1013904223u;
        if (mode != 1) {
            float v[WIDE_K][2];
#pragma unroll
            for (int k = 0; k < WIDE_K; k++) {
                const float4 *p = rows + (size_t)(st[k] >> sh) * 64 + 2 * lane;
                float a0, a1, a2, a3, a4, a5, a6, a7;
                asm volatile("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                             : "=f"(a0), "=f"(a1), "=f"(a2), "=f"(a3), "=f"(a4), "=f"(a5),
                               "=f"(a6), "=f"(a7)
                             : "l"(p));
                v[k][0] = a0 + a5;
                v[k][1] = a2 + a7;
            }
#pragma unroll
            for (int k = 0; k < WIDE_K; k++) acc += v[k][0] * v[k][1];
        }
        if (mode != 0) {
#pragma unroll
            for (int k = 0; k < WIDE_K; k++) {
                float *p = ff + (size_t)(st[k] >> shf) * 64 + 2 * lane;
                asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(1.0f),
                             "f"(1.0f)
                             : "memory");
            }
        }
    }
    if (acc == 1234.5f) out[warp] = acc;
}

__global__ void fma2_chains(float *out, int iters, float a, float b)
{
    float2 x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = make_float2(threadIdx.x + k, threadIdx.x - k);
    const float2 aa = make_float2(a, a), bb = make_float2(b, b);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = __ffma2_rn(x[k], aa, bb);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k].x + x[k].y;
    if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void fma_chains(float *out, int iters, float a, float b)
{
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
        x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dfma_chains(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1234.5) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ex2_chains(float *out, int iters)
{
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 0.1f, x2 = x0 + 0.2f, x3 = x0 + 0.3f;
    for (int i = 0; i < iters; i++) {
        asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x0));
        asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x1));
        asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x2));
        asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x3));
    }
    const float s = x0 + x1 + x2 + x3;
    if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename F>
float time_ms(F launch, int reps)
{
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    launch();  // warm-up
    cudaEventRecord(a);
    for (int r = 0; r < reps; r++) launch();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
}

}  // namespace

extern "C" int mocpeak_run(double *res, int n_res)
{
    if (!res || n_res < 6) return -1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int blocks = sms * 8, threads = 256;
    float *out = nullptr, *l2buf = nullptr, *rows = nullptr, *ff = nullptr, *hbm = nullptr;
    const int64_t l2_bytes = 64ll << 20, row_bytes = 96ll << 20, ff_rows = 50000,
                  hbm_bytes = 2ll << 30;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return -2;
    if (cudaMalloc(&l2buf, l2_bytes) != cudaSuccess) return -2;
    if (cudaMalloc(&rows, row_bytes) != cudaSuccess) return -2;
    if (cudaMalloc(&ff, ff_rows * 128 * sizeof(float)) != cudaSuccess) return -2;
    if (cudaMalloc(&hbm, hbm_bytes) != cudaSuccess) return -2;
    cudaMemset(l2buf, 0, l2_bytes);
    cudaMemset(rows, 0, row_bytes);
    cudaMemset(ff, 0, ff_rows * 128 * sizeof(float));
    cudaMemset(hbm, 0, hbm_bytes);

    const int64_t n4 = l2_bytes / 16;
    const int passes = 20;
    float ms = time_ms([&] { stream_read<<<blocks, threads>>>((const float4 *)l2buf, n4, passes, out, 0); }, 5);
    res[0] = (double)l2_bytes * passes / (ms * 1e-3) / 1e9;

    const uint32_t n_rows = (uint32_t)(row_bytes / 512);
    const int giters = 2000;
    ms = time_ms([&] { row_gather<<<blocks, threads>>>((const float4 *)rows, n_rows, giters, out); }, 5);
    res[1] = (double)blocks * (threads / 32) * giters * 512.0 / (ms * 1e-3) / 1e9;

    const int riters = 1000;
    ms = time_ms([&] { row_reduce<<<blocks, threads>>>(ff, (uint32_t)ff_rows, riters); }, 5);
    res[2] = (double)blocks * (threads / 32) * riters * 512.0 / (ms * 1e-3) / 1e9;

    const int fiters = 20000;
    ms = time_ms([&] { fma_chains<<<blocks, threads>>>(out, fiters, 0.999f, 1e-3f); }, 5);
    res[3] = (double)blocks * threads * fiters * 8 * 2.0 / (ms * 1e-3) / 1e12;

    const int eiters = 5000;
    ms = time_ms([&] { ex2_chains<<<blocks, threads>>>(out, eiters); }, 5);
    res[4] = (double)blocks * threads * eiters * 4.0 / (ms * 1e-3) / 1e9;

    ms = time_ms([&] { stream_read<<<blocks, threads>>>((const float4 *)hbm, hbm_bytes / 16, 1, out, 1); }, 5);
    res[5] = (double)hbm_bytes / (ms * 1e-3) / 1e9;

    if (n_res >= 10) {
        double *dout = nullptr;
        if (cudaMalloc(&dout, (size_t)blocks * threads * sizeof(double)) == cudaSuccess) {
            const int diters = 2000;
            ms = time_ms([&] { dfma_chains<<<blocks, threads>>>(dout, diters, 0.999, 1e-3); }, 5);
            res[9] = (double)blocks * threads * diters * 8 * 2.0 / (ms * 1e-3) / 1e12;
            cudaFree(dout);
        }
    }

    if (n_res >= 9) {
        // 2^17 rows of 512 B (64 MiB) to gather from, 2^15 tally rows (16 MiB) to reduce into
        const int lr = 17, lf = 15, it = 2000;
        const double warps = (double)blocks * (threads / 32);
        ms = time_ms([&] { row_mix<<<blocks, threads>>>((const float4 *)rows, ff, lr, lf, it, 0, out); }, 5);
        res[6] = warps * it * 4 * 512.0 / (ms * 1e-3) / 1e9;
        ms = time_ms([&] { row_mix<<<blocks, threads>>>((const float4 *)rows, ff, lr, lf, it, 1, out); }, 5);
        res[7] = warps * it * 2 * 512.0 / (ms * 1e-3) / 1e9;
        ms = time_ms([&] { row_mix<<<blocks, threads>>>((const float4 *)rows, ff, lr, lf, it, 2, out); }, 5);
        res[8] = warps * it * 5 * 512.0 / (ms * 1e-3) / 1e9;
    }

    if (n_res >= 14) {
        // 2^16 rows of 1 KB (64 MiB: the sweep's half of its cell blocks) to gather from,
        // 2^16 tally rows of 256 B (16 MiB) to reduce into
        const int lr = 16, lf = 16, it = 400;
        double best[3] = {0.0, 0.0, 0.0};
        for (int per_sm : {8, 16, 24}) {
            int can = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&can, row_mix_wide, threads, 0);
            if (can * (threads / 32) < per_sm) continue;
            const int b = sms * per_sm / (threads / 32);
            const double warps = (double)b * (threads / 32);
            const double bytes[3] = {1024.0, 256.0, 1280.0};
            for (int mode = 0; mode < 3; mode++) {
                ms = time_ms([&] { row_mix_wide<<<b, threads>>>((const float4 *)rows, ff, lr, lf, it, mode, out); }, 5);
                const double gbs = warps * it * WIDE_K * bytes[mode] / (ms * 1e-3) / 1e9;
                if (gbs > best[mode]) best[mode] = gbs;
            }
        }
        res[10] = best[0];
        res[11] = best[1];
        res[12] = best[2];
        const int fiters = 10000;
        ms = time_ms([&] { fma2_chains<<<blocks, threads>>>(out, fiters, 0.999f, 1e-3f); }, 5);
        res[13] = (double)blocks * threads * fiters * 8 * 4.0 / (ms * 1e-3) / 1e12;
    }

    const cudaError_t e = cudaDeviceSynchronize();
    cudaFree(out);
    cudaFree(l2buf);
    cudaFree(rows);
    cudaFree(ff);
    cudaFree(hbm);
    return e == cudaSuccess ? 0 : -3;
}
