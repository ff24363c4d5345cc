// A host application's own kernel reading the brick cache through the device
// view (include/gc_cache_device.cuh), as a user of the reference reads it
// through K_CacheManager<T>::get_normalized.  Test input: compiled by
// tests/test_gpu_device_view.py with nvcc into a shared library.
#include <cuda_runtime.h>

#include "gc_cache_device.cuh"

__global__ void sample_kernel(const __grid_constant__ gc_cache_device_view v, const float4 *__restrict__ pos, int n,
                              float *__restrict__ value, int *__restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];  // x, y, z in [0, 1), level
    float out = -1.0f;
    status[i] = gc_sample_normalized(&v, static_cast<uint32_t>(p.w), p.x, p.y, p.z, &out);
    value[i] = out;
}

extern "C" int user_sample(const gc_cache_device_view *v, const float4 *pos, int n, float *value, int *status) {
    sample_kernel<<<(n + 255) / 256, 256>>>(*v, pos, n, value, status);
    const cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? static_cast<int>(e) : static_cast<int>(cudaDeviceSynchronize());
}
