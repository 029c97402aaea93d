// dfpt_noalloc.cu - the allocation-free variant of the FP64 image-mean reduction.
//
// dfpt_read_film_mean reduces the film into a small device buffer that dfpt_create allocated.
// Some callers cannot allocate device memory at the point where they need the mean: a frame loop
// that must not call cudaMalloc/cudaFree once it is running (allocation can synchronise the device
// and stall the loop), or a host whose device memory is owned by another allocator (a JVM-side
// pool, an engine's frame allocator). dfpt_film_mean_noalloc serves them: the caller passes the
// film and the output in device memory, and the reduction's scratch is a fixed, file-scope device
// array that every GPU which loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "dfpt.h"
#include "dfpt_internal.h"

namespace {

constexpr int kThreads = 256;

// Per-block partial sums (r, g, b): DFPT_NOALLOC_MAX_BLOCKS * 3 doubles = 24 KiB. Every call writes
// all the partials it later reads, so nothing in it has to start at zero, and the contents of the
// last call simply stay behind. Calls that overlap on the GPU (two streams, or two threads) share
// this one array and race; callers serialise them.
static __device__ __align__(256) double g_mean_scratch[DFPT_NOALLOC_MAX_BLOCKS * 3];

__global__ void __launch_bounds__(kThreads) k_mean_partials(const float* __restrict__ rgb, int64_t n, double* __restrict__ partials) {
    __shared__ double sr[kThreads], sg[kThreads], sb[kThreads];
    double r = 0.0, g = 0.0, b = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        r += (double)rgb[3 * i];
        g += (double)rgb[3 * i + 1];
        b += (double)rgb[3 * i + 2];
    }
    sr[threadIdx.x] = r;
    sg[threadIdx.x] = g;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sr[threadIdx.x] += sr[threadIdx.x + s];
            sg[threadIdx.x] += sg[threadIdx.x + s];
            sb[threadIdx.x] += sb[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x] = sr[0];
        partials[3 * blockIdx.x + 1] = sg[0];
        partials[3 * blockIdx.x + 2] = sb[0];
    }
}

__global__ void __launch_bounds__(kThreads) k_mean_finish(const double* __restrict__ partials, int blocks, int64_t n, double* __restrict__ out3) {
    __shared__ double s[3][kThreads];
    for (int c = 0; c < 3; ++c) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < blocks; i += kThreads) acc += partials[3 * i + c];
        s[c][threadIdx.x] = acc;
    }
    __syncthreads();
    for (int st = kThreads / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int c = 0; c < 3; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 3) out3[threadIdx.x] = s[threadIdx.x][0] / (double)n;
}

// Device address of the scratch array, looked up once per device with that device current. In
// host code the array's name is only a host-side stand-in, never a device address.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {nullptr};

int scratch_for_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= kMaxDevices) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "device ordinal %d >= %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_mean_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            return dfpt_fail(DFPT_ERR_CUDA, "cudaGetSymbolAddress(g_mean_scratch): %s", cudaGetErrorString(e));
        }
        g_scratch_address[dev] = p;
    }
    *out = static_cast<double*>(g_scratch_address[dev]);
    return DFPT_OK;
}

}  // namespace

extern "C" int dfpt_film_mean_noalloc(const float* device_rgb, int64_t pixel_count, double* device_mean3, void* cuda_stream) {
    if (!device_rgb || !device_mean3) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "device_rgb and device_mean3 must not be NULL");
    if (pixel_count <= 0 || pixel_count > DFPT_NOALLOC_MAX_PIXELS)
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "pixel_count %lld is outside 1..%lld (the fixed scratch of dfpt_film_mean_noalloc)",
                         (long long)pixel_count, (long long)DFPT_NOALLOC_MAX_PIXELS);
    if (((uintptr_t)device_rgb & 3u) != 0 || ((uintptr_t)device_mean3 & 7u) != 0)
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "device_rgb must be 4-byte and device_mean3 8-byte aligned");
    double* scratch = nullptr;
    int r = scratch_for_current_device(&scratch);
    if (r) return r;
    const int64_t want = (pixel_count + kThreads - 1) / kThreads;
    const int blocks = (int)(want < DFPT_NOALLOC_MAX_BLOCKS ? want : DFPT_NOALLOC_MAX_BLOCKS);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    k_mean_partials<<<blocks, kThreads, 0, s>>>(device_rgb, pixel_count, scratch);
    k_mean_finish<<<1, kThreads, 0, s>>>(scratch, blocks, pixel_count, device_mean3);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return dfpt_fail(DFPT_ERR_CUDA, "dfpt_film_mean_noalloc launch: %s", cudaGetErrorString(e));
    return DFPT_OK;
}
