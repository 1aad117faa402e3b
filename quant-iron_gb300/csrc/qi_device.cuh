// qi_device.cuh — device-side helpers shared by the engine's kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace qi {

// Complex arithmetic on the CUDA vector types (float2 / double2).
template <typename T> struct Cx;
template <> struct Cx<float> {
    using V2 = float2;
    __host__ __device__ static inline float2 make(float r, float i) { return make_float2(r, i); }
    __device__ static inline float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
    __device__ static inline float2 sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
    __device__ static inline float2 mul(float2 a, float2 b) {
        return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
    }
    // acc + a*b
    __device__ static inline float2 fma(float2 a, float2 b, float2 acc) {
        acc.x = fmaf(a.x, b.x, acc.x);
        acc.x = fmaf(-a.y, b.y, acc.x);
        acc.y = fmaf(a.x, b.y, acc.y);
        acc.y = fmaf(a.y, b.x, acc.y);
        return acc;
    }
};
template <> struct Cx<double> {
    using V2 = double2;
    __host__ __device__ static inline double2 make(double r, double i) { return make_double2(r, i); }
    __device__ static inline double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
    __device__ static inline double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
    __device__ static inline double2 mul(double2 a, double2 b) {
        return make_double2(::fma(a.x, b.x, -a.y * b.y), ::fma(a.x, b.y, a.y * b.x));
    }
    __device__ static inline double2 fma(double2 a, double2 b, double2 acc) {
        acc.x = ::fma(a.x, b.x, acc.x);
        acc.x = ::fma(-a.y, b.y, acc.x);
        acc.y = ::fma(a.x, b.y, acc.y);
        acc.y = ::fma(a.y, b.x, acc.y);
        return acc;
    }
};

// exp(2 pi i f / 2^32) for a phase in fixed-point turns: T1[f >> 22] (T1 = exp(2 pi i j / 1024))
// times exp(i x), x = the remaining 22 bits as an angle (< 2 pi / 1024), from the Taylor
// polynomials of sin and cos to x^5 and x^4 (remainder < 1e-16).
__device__ __forceinline__ float2 turn_phase(uint32_t f, const float2 *T1) {
    const float2 t = T1[f >> 22];
    const float x = (float)(f & 0x3FFFFFu) * 1.46291807926715968e-9f;   // 2 pi / 2^32
    const float x2 = x * x;
    const float s = x * (1.0f - x2 * (1.0f / 6.0f) * (1.0f - x2 * 0.05f));
    const float c = 1.0f - x2 * 0.5f * (1.0f - x2 * (1.0f / 12.0f));
    return make_float2(t.x * c - t.y * s, t.x * s + t.y * c);
}

// Streaming loads for data read exactly once (evict-first in L1/L2).
__device__ static inline float4 ldg_stream(const float4 *p) { return __ldcs(p); }
__device__ static inline double2 ldg_stream(const double2 *p) { return __ldcs(p); }
__device__ static inline float2 ldg_stream(const float2 *p) { return __ldcs(p); }

// Block-wide sum of one double (blockDim.x a multiple of 32, <= 1024).
__device__ static inline double block_sum(double v) {
    __shared__ double warp_part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();   // warp_part may still be read by a previous call
    if (lane == 0) warp_part[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double r = 0.0;
    if (wid == 0) {
        r = lane < nw ? warp_part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;   // valid in thread 0
}

// Insert a zero bit at each of the `np` ascending positions `pos[]` of w.
__device__ static inline uint64_t insert_zeros(uint64_t w, const int8_t *pos, int np) {
    for (int k = 0; k < np; ++k) {
        const int p = pos[k];
        const uint64_t lo = w & ((1ull << p) - 1);
        w = ((w >> p) << (p + 1)) | lo;
    }
    return w;
}

}  // namespace qi
