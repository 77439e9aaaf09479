// Storage types of the V-cycle levels: FP32, or FP16 for the mixed-precision
// preconditioner (values are converted to FP32 on load and all arithmetic is
// FP32; FP16 rounding happens only on store).
#pragma once

#include <cuda_fp16.h>

namespace flub {

template <typename T>
struct St;

template <>
struct St<float> {
    static __device__ __forceinline__ float ld(const float *p) { return *p; }
    static __device__ __forceinline__ float ld_ro(const float *p) { return __ldg(p); }
    static __device__ __forceinline__ void st(float *p, float v) { *p = v; }
    static __device__ __forceinline__ void ld8(const float *p, float o[8]) {
        const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
    }
    static __device__ __forceinline__ void ld8_ro(const float *p, float o[8]) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p)), b = __ldg(reinterpret_cast<const float4 *>(p) + 1);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
    }
    static __device__ __forceinline__ void ld4_ro(const float *p, float o[4]) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    }
    static __device__ __forceinline__ void ld4(const float *p, float o[4]) {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    }
    static __device__ __forceinline__ void ld2_ro(const float *p, float o[2]) {
        const float2 a = __ldg(reinterpret_cast<const float2 *>(p));
        o[0] = a.x; o[1] = a.y;
    }
    static __device__ __forceinline__ void ld2(const float *p, float o[2]) {
        const float2 a = *reinterpret_cast<const float2 *>(p);
        o[0] = a.x; o[1] = a.y;
    }
    // L2-only loads (ld.global.cg) of data other blocks wrote earlier in the
    // same launch (persistent and cluster kernels)
    static __device__ __forceinline__ float ld_cg(const float *p) { return __ldcg(p); }
    static __device__ __forceinline__ void ld2_cg(const float *p, float o[2]) {
        const float2 a = __ldcg(reinterpret_cast<const float2 *>(p));
        o[0] = a.x; o[1] = a.y;
    }
    static __device__ __forceinline__ void ld4_cg(const float *p, float o[4]) {
        const float4 a = __ldcg(reinterpret_cast<const float4 *>(p));
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    }
    static __device__ __forceinline__ void ld8_cg(const float *p, float o[8]) {
        const float4 a = __ldcg(reinterpret_cast<const float4 *>(p)), b = __ldcg(reinterpret_cast<const float4 *>(p) + 1);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
    }
    static __device__ __forceinline__ void st8(float *p, const float v[8]) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
        reinterpret_cast<float4 *>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
    }
    static __device__ __forceinline__ void st4(float *p, const float v[4]) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};

template <>
struct St<__half> {
    static __device__ __forceinline__ float ld(const __half *p) { return __half2float(*p); }
    static __device__ __forceinline__ float ld_ro(const __half *p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ void st(__half *p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ void unpack8(uint4 u, float o[8]) {
        const __half2 *h = reinterpret_cast<const __half2 *>(&u);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 f = __half22float2(h[q]);
            o[2 * q] = f.x;
            o[2 * q + 1] = f.y;
        }
    }
    static __device__ __forceinline__ void ld8(const __half *p, float o[8]) {
        unpack8(*reinterpret_cast<const uint4 *>(p), o);
    }
    static __device__ __forceinline__ void ld8_ro(const __half *p, float o[8]) {
        unpack8(__ldg(reinterpret_cast<const uint4 *>(p)), o);
    }
    static __device__ __forceinline__ void ld4_ro(const __half *p, float o[4]) {
        const uint2 u = __ldg(reinterpret_cast<const uint2 *>(p));
        const __half2 *h = reinterpret_cast<const __half2 *>(&u);
        const float2 a = __half22float2(h[0]), b = __half22float2(h[1]);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
    static __device__ __forceinline__ void ld4(const __half *p, float o[4]) {
        const uint2 u = *reinterpret_cast<const uint2 *>(p);
        const __half2 *h = reinterpret_cast<const __half2 *>(&u);
        const float2 a = __half22float2(h[0]), b = __half22float2(h[1]);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
    static __device__ __forceinline__ void ld2_ro(const __half *p, float o[2]) {
        const float2 a = __half22float2(__ldg(reinterpret_cast<const __half2 *>(p)));
        o[0] = a.x; o[1] = a.y;
    }
    static __device__ __forceinline__ void ld2(const __half *p, float o[2]) {
        const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(p));
        o[0] = a.x; o[1] = a.y;
    }
    static __device__ __forceinline__ float ld_cg(const __half *p) {
        const unsigned short u = __ldcg(reinterpret_cast<const unsigned short *>(p));
        return __half2float(__ushort_as_half(u));
    }
    static __device__ __forceinline__ void ld2_cg(const __half *p, float o[2]) {
        const unsigned int u = __ldcg(reinterpret_cast<const unsigned int *>(p));
        const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u));
        o[0] = a.x; o[1] = a.y;
    }
    static __device__ __forceinline__ void ld4_cg(const __half *p, float o[4]) {
        const uint2 u = __ldcg(reinterpret_cast<const uint2 *>(p));
        const __half2 *h = reinterpret_cast<const __half2 *>(&u);
        const float2 a = __half22float2(h[0]), b = __half22float2(h[1]);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
    static __device__ __forceinline__ void ld8_cg(const __half *p, float o[8]) {
        unpack8(__ldcg(reinterpret_cast<const uint4 *>(p)), o);
    }
    static __device__ __forceinline__ void st8(__half *p, const float v[8]) {
        uint4 u;
        __half2 *h = reinterpret_cast<__half2 *>(&u);
#pragma unroll
        for (int q = 0; q < 4; q++) h[q] = __floats2half2_rn(v[2 * q], v[2 * q + 1]);
        *reinterpret_cast<uint4 *>(p) = u;
    }
    static __device__ __forceinline__ void st4(__half *p, const float v[4]) {
        uint2 u;
        __half2 *h = reinterpret_cast<__half2 *>(&u);
        h[0] = __floats2half2_rn(v[0], v[1]);
        h[1] = __floats2half2_rn(v[2], v[3]);
        *reinterpret_cast<uint2 *>(p) = u;
    }
};

}  // namespace flub
