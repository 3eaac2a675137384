// bounded_wait_probe.cu — test-only probe of the sweep's bounded mbarrier wait
// (mbar_wait_bounded, simplemoc-kernel_gb300/csrc/moc_device.cuh), built by
// tests/test_bounded_wait_gpu.py.
//
// One warp initialises an mbarrier that expects one arrival and, in the "never" case,
// never arrives on it: the wait must give up after its limit and say so, and the kernel
// returns normally, leaving the context usable. In the "arrive" case lane 0 arrives
// first and the wait must succeed at once. Nothing faults, traps or spins without a limit.
#include <cstdint>

#include "moc_device.cuh"

namespace {

__global__ void probe_kernel(int arrive, long long limit, int *out)
{
    __shared__ __align__(8) unsigned long long bar;
    const uint32_t b = moc::smem_addr(&bar);
    if (threadIdx.x == 0) {
        moc::mbar_init(b, 1);
        moc::mbar_init_fence();
    }
    __syncwarp();
    if (arrive && threadIdx.x == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
    __syncwarp();
    const long long t0 = clock64();
    const bool ok = moc::mbar_wait_bounded(b, 0u, limit);
    const long long t1 = clock64();
    if (threadIdx.x == 0) {
        out[0] = ok ? 1 : 0;
        out[1] = (int)((t1 - t0) >> 10);  // clocks / 1024 spent waiting
    }
}

}  // namespace

// Returns 0 and fills out[2] = {completed, kiloclocks waited}, or a CUDA error code.
extern "C" int bounded_wait_probe(int arrive, long long limit_clocks, int *out)
{
    int *d = nullptr;
    cudaError_t e = cudaMalloc(&d, 2 * sizeof(int));
    if (e != cudaSuccess) return (int)e;
    cudaMemset(d, 0xff, 2 * sizeof(int));
    probe_kernel<<<1, 32>>>(arrive, limit_clocks, d);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, d, 2 * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return (int)e;
}
