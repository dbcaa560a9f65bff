// Host-buffer round trip of the vertex state: packed float3 arrays <-> the float4 SoA layout.
//
// These kernels serve the C ABI calls that move every body's state between host memory and HBM in
// one pair of copies (jsb_state_upload_all / jsb_state_download_all): the host hands over N x 3
// floats of positions and N x 3 floats of velocities; the kernels scatter them into x.xyz (keeping
// the inverse mass in x.w) and v.xyz, or gather them back.

#include <cuda_runtime.h>
#include <stdint.h>

namespace jsb {
namespace {

__global__ void unpack_kernel(const float *__restrict__ pos3, const float *__restrict__ vel3, float4 *__restrict__ x,
                              float4 *__restrict__ v, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
        float4 xi = x[i];
        x[i] = make_float4(pos3[3 * i + 0], pos3[3 * i + 1], pos3[3 * i + 2], xi.w);
        v[i] = make_float4(vel3[3 * i + 0], vel3[3 * i + 1], vel3[3 * i + 2], 0.0f);
    }
}

__global__ void pack_kernel(const float4 *__restrict__ x, const float4 *__restrict__ v, float *__restrict__ pos3,
                            float *__restrict__ vel3, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
        float4 xi = x[i], vi = v[i];
        pos3[3 * i + 0] = xi.x;
        pos3[3 * i + 1] = xi.y;
        pos3[3 * i + 2] = xi.z;
        vel3[3 * i + 0] = vi.x;
        vel3[3 * i + 1] = vi.y;
        vel3[3 * i + 2] = vi.z;
    }
}

}  // namespace

cudaError_t launch_unpack_state(const float *pos3, const float *vel3, float4 *x, float4 *v, uint64_t n, int num_sms,
                                cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    uint64_t blocks = (n + 255) / 256;
    uint64_t cap = uint64_t(num_sms) * 8;
    unpack_kernel<<<unsigned(blocks < cap ? blocks : cap), 256, 0, stream>>>(pos3, vel3, x, v, n);
    return cudaGetLastError();
}

cudaError_t launch_pack_state(const float4 *x, const float4 *v, float *pos3, float *vel3, uint64_t n, int num_sms,
                              cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    uint64_t blocks = (n + 255) / 256;
    uint64_t cap = uint64_t(num_sms) * 8;
    pack_kernel<<<unsigned(blocks < cap ? blocks : cap), 256, 0, stream>>>(x, v, pos3, vel3, n);
    return cudaGetLastError();
}

}  // namespace jsb
