// Sensor samples to complex64: the int16 I/Q pairs of the .wbd payload
// (common.cu:1096-1098 converts them on the host, static_cast<float> per
// component) converted on the GPU, so that callers move 4 bytes per sample
// to the device instead of 8.
#include <cuda_runtime.h>

#include "isar_kernels.h"

namespace isar {

// Two complex samples per thread and iteration: one 8-byte load of four
// int16, one 16-byte store of four floats (grid-stride).
__global__ void k_iq16_to_c64(const short4* __restrict__ in, float4* __restrict__ out, size_t pairs)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs; i += (size_t)gridDim.x * blockDim.x) {
        const short4 q = in[i];
        out[i] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
    }
}

__global__ void k_iq16_to_c64_tail(const short2* __restrict__ in, float2* __restrict__ out, size_t i)
{
    const short2 q = in[i];
    out[i] = make_float2((float)q.x, (float)q.y);
}

cudaError_t iq16_to_c64(const int16_t* in, float* out, size_t samples, cudaStream_t st)
{
    if (samples == 0) return cudaSuccess;
    const size_t pairs = samples / 2;
    if (pairs) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t want = (pairs + 255) / 256;
        const unsigned blocks = (unsigned)(want < (size_t)sms * 8 ? want : (size_t)sms * 8);
        k_iq16_to_c64<<<blocks, 256, 0, st>>>(reinterpret_cast<const short4*>(in), reinterpret_cast<float4*>(out),
                                               pairs);
        ISAR_COUNT(1);
    }
    if (samples & 1) {
        k_iq16_to_c64_tail<<<1, 1, 0, st>>>(reinterpret_cast<const short2*>(in), reinterpret_cast<float2*>(out),
                                            samples - 1);
        ISAR_COUNT(1);
    }
    return cudaGetLastError();
}

}  // namespace isar
