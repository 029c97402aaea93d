// dfpt_probe.cu - a bandwidth probe for rooflines: how fast this GPU streams reads of a buffer
// that stays resident in L2.
//
// The closest-hit traversal reads BVH node and triangle records that live in L2 (the scene's
// traversal records of the 1080p workloads take 57-130 MB), not in DRAM, so the HBM copy rate is
// not the roof it runs against. This kernel measures the roof that is: every thread streams 16-byte
// loads through L2 only (ld.global.cg: no L1 allocation, so repeats cannot hit in L1) over a
// caller's buffer smaller than L2, `repeats` times inside one launch, and the host times the launch
// with CUDA events on the caller's stream.
#include <cuda_runtime.h>

#include "dfpt.h"
#include "dfpt_internal.h"

namespace {

constexpr int kProbeThreads = 256;

// Keeps the loads alive: one atomic add per block of the block's checksum.
__device__ float g_probe_sink;

__global__ void __launch_bounds__(kProbeThreads) k_probe_read(const float4* __restrict__ buf, int64_t n4, int repeats) {
    float acc = 0.0f;
    const int64_t stride = (int64_t)gridDim.x * kProbeThreads;
    for (int r = 0; r < repeats; ++r) {
        // Each repeat shifts the blocks' starting points, so a block does not reread its own lines.
        const int64_t shift = ((int64_t)r * 7919 * kProbeThreads) % n4;
        for (int64_t i = (int64_t)blockIdx.x * kProbeThreads + threadIdx.x; i < n4; i += stride) {
            int64_t j = i + shift;
            if (j >= n4) j -= n4;
            const float4 v = __ldcg(buf + j);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    __shared__ float part[kProbeThreads / 32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < kProbeThreads / 32; ++w) s += part[w];
        atomicAdd(&g_probe_sink, s);
    }
}

}  // namespace

extern "C" int dfpt_probe_read_bandwidth(const void* device_buffer, int64_t bytes, int32_t repeats, void* stream, double* gbs) {
    if (!device_buffer || !gbs) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (((uintptr_t)device_buffer & 15u) != 0) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "buffer not 16-byte aligned");
    if (bytes < (1 << 20) || bytes % 16 != 0) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bytes %lld: at least 1 MiB, a multiple of 16", (long long)bytes);
    if (repeats < 1 || repeats > 100000) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "repeats %d outside [1, 100000]", repeats);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return dfpt_fail(DFPT_ERR_CUDA, "device query: %s", cudaGetErrorString(e));
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n4 = bytes / 16;
    const int blocks = sms * 8;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_probe_read<<<blocks, kProbeThreads, 0, s>>>((const float4*)device_buffer, n4, 1);  // brings the buffer into L2
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) {
        k_probe_read<<<blocks, kProbeThreads, 0, s>>>((const float4*)device_buffer, n4, repeats);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "read probe: %s", cudaGetErrorString(e));
    }
    *gbs = (double)bytes * (double)repeats / ((double)ms * 1.0e-3) / 1.0e9;
    return DFPT_OK;
}
