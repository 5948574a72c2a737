// Random-gather ceiling of the current GPU (measurement only; no reference
// counterpart).
//
// A walk move is a dependent random gather into an array larger than L2, so
// the relevant peak is not the streaming copy bandwidth but the rate at which
// the memory system serves independent random 4-byte loads.  This kernel
// measures it: every thread runs `chains` independent chains of dependent
// loads whose next index is a hash of the loaded value, over an array of the
// given size filled with hashed values, with as many threads resident as fit.
#include <algorithm>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

__global__ void k_probe_fill(uint32_t *a, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = mix32((uint32_t)i * 2654435761u + 7u);
}

// n <= 2^32 - 1, so __umulhi(hash, n) < n indexes the array.
template <int CH>
__global__ void __launch_bounds__(256) k_probe_gather(const uint32_t *__restrict__ a, uint32_t n, int depth,
                                                      uint32_t seed, uint32_t *sink)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t v[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) v[c] = mix32(t * CH + c + seed);
    for (int d = 0; d < depth; ++d) {
#pragma unroll
        for (int c = 0; c < CH; ++c) v[c] = __ldg(&a[__umulhi(mix32(v[c] + (uint32_t)d), n)]);
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < CH; ++c) acc += v[c];
    if (acc == 0x9E3779B9u) *sink = acc;  // keeps the loads live
}

}  // namespace
}  // namespace ptw

using namespace ptw;

extern "C" int ptw_probe_gather(uint64_t array_bytes, uint32_t chains, double *loads_per_s)
try {
    if (!loads_per_s) return fail(PTW_EINVAL, "null output");
    *loads_per_s = 0.0;
    if (chains != 1 && chains != 2 && chains != 4 && chains != 8) return fail(PTW_EINVAL, "chains must be 1, 2, 4 or 8");
    const uint64_t n64 = array_bytes / 4;
    if (n64 < 1024 || n64 > 0xFFFFFFFFull) return fail(PTW_EINVAL, "array_bytes must be in [4 KiB, 16 GiB)");
    const uint32_t n = (uint32_t)n64;
    int dev = 0, sms = 0;
    PTW_CUDA(cudaGetDevice(&dev));
    PTW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = nullptr;
    PTW_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    uint32_t *a = nullptr, *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PTW_OK;
    cudaError_t e = device_malloc(&a, (size_t)n * 4);
    if (e == cudaSuccess) e = device_malloc(&sink, 4);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_probe_fill<<<(unsigned)sms * 16, 256, 0, st>>>(a, n);
        // eight 256-thread blocks per SM are resident; four waves of them
        const unsigned grid = (unsigned)sms * 8 * 4;
        const int depth = 32;
        auto launch = [&](uint32_t seed) {
            switch (chains) {
            case 1: k_probe_gather<1><<<grid, 256, 0, st>>>(a, n, depth, seed, sink); break;
            case 2: k_probe_gather<2><<<grid, 256, 0, st>>>(a, n, depth, seed, sink); break;
            case 4: k_probe_gather<4><<<grid, 256, 0, st>>>(a, n, depth, seed, sink); break;
            default: k_probe_gather<8><<<grid, 256, 0, st>>>(a, n, depth, seed, sink); break;
            }
        };
        launch(1);  // warm-up
        e = cudaEventRecord(e0, st);
        launch(2);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && ms > 0)
            *loads_per_s = (double)grid * 256 * chains * depth / (ms * 1e-3);
    }
    if (e != cudaSuccess) rc = cuda_fail(e, "gather probe");
    cudaStreamSynchronize(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(sink);
    cudaStreamDestroy(st);
    return rc;
} catch (...) {
    return host_exception();
}
