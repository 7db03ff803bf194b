// Common device helpers for the GB300 ISAR imaging kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace isar {

// Constants as the reference defines them (common.cuh:68-73).
constexpr float kPiF = 3.14159265358979f;
constexpr double kPiD = 3.14159265358979;
constexpr double kLightSpeed = 300000000.0;
constexpr int kRangeCut = 512;          // RANGE_NUM_CUT
constexpr int kRangeNumIfdsPc = 4096;   // RANGE_NUM_IFDS_PC (common.cuh:72)
constexpr int kEntropyIters = 120;      // FAST_ENTROPY_ITERATION_NUM
constexpr int kMaxN = 8192;            // largest supported range_num
constexpr int kMaxM = 1024;             // largest supported echo_num
constexpr int kTwN = 16384;             // twiddle table length

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ float2 cmulc(float2 a, float2 b)
{
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// Phase in cycles held as a 64-bit two's-complement fraction: value / 2^64.
// exp(j*2*pi*frac) from the top 32 bits.
__device__ __forceinline__ float2 cis_frac64(uint64_t ph)
{
    int32_t hi = (int32_t)(ph >> 32);
    float f = (float)hi * 4.656612873077392578125e-10f;   // 2^-31 : f in [-1, 1) half-cycles
    float s, c;
    sincospif(f, &s, &c);
    return make_float2(c, s);
}

__device__ __forceinline__ int bitrev8(int v)
{
    return (int)(__brev((unsigned)v) >> 24);
}

// Argmax key of maxRowsIdxABS (range_alignment.cu:134-168): larger |value|
// first; on equal values the class (index mod 256) with the smaller 8-bit
// reversed number wins (the shared-memory tree keeps its left operand on
// ties), and within a class the smaller index.
struct ArgKey {
    float a;   // |value|
    int i;     // index
};
__device__ __forceinline__ bool argkey_better(const ArgKey& x, const ArgKey& y)
{
    if (x.a != y.a) return x.a > y.a;
    int cx = x.i & 255, cy = y.i & 255;
    if (cx != cy) return bitrev8(cx) < bitrev8(cy);
    return x.i < y.i;
}

__device__ __forceinline__ unsigned float_as_ordered(float f)   // f >= 0
{
    return __float_as_uint(f);
}

}  // namespace isar
