// Shared helpers of the flub_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <string>

#include "../../include/flub_gb300.h"

namespace flub {

// ------------------------------------------------------------------ errors
void set_last_error(const char *fmt, ...);
void count_launches(int64_t n);

#define FLUB_CHECK_CUDA(call)                                                                   \
    do {                                                                                        \
        cudaError_t _e = (call);                                                                \
        if (_e != cudaSuccess) {                                                                \
            ::flub::set_last_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
            return FLUB_ERR_CUDA;                                                               \
        }                                                                                       \
    } while (0)

#define FLUB_CHECK_LAUNCH()                                                                     \
    do {                                                                                        \
        cudaError_t _e = cudaGetLastError();                                                    \
        if (_e != cudaSuccess) {                                                                \
            ::flub::set_last_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
            return FLUB_ERR_CUDA;                                                               \
        }                                                                                       \
        ::flub::count_launches(1);                                                              \
    } while (0)

#define FLUB_REQUIRE(cond, ...)                                                                 \
    do {                                                                                        \
        if (!(cond)) {                                                                          \
            ::flub::set_last_error(__VA_ARGS__);                                                \
            return FLUB_ERR_INVALID_ARGUMENT;                                                   \
        }                                                                                       \
    } while (0)

static inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// ------------------------------------------------------------------ grid geometry
constexpr int kNumSMs = 152;

static inline unsigned blocks_for(int64_t n, int threads, int64_t cap = 152 * 32) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

// Row-wise launch for per-cell / per-face kernels: blockIdx.z = i, blockIdx.y
// = j, k along x; no integer division per cell.
constexpr int kRowThreads = 128;
static inline dim3 row_grid(int nx, int ny, int nz) {
    return dim3((unsigned)((nz + kRowThreads - 1) / kRowThreads), (unsigned)ny, (unsigned)nx);
}

// ------------------------------------------------------------------ cell codes
// The solver stores one byte per cell.  The byte is chosen so that "outside
// the domain" (a zero byte, e.g. a TMA out-of-bounds fill) behaves like a solid
// neighbour: it is excluded from the stencil, exactly as the reference's
// clamped-index neighbour contributes (x_c - x_c) = 0 and is not counted in the
// diagonal (multigrid/mgpcg.py:118-160).
//   reference tag 2 (solid) -> 0, tag 0 (air) -> 1, tag 1 (fluid) -> 2
constexpr uint8_t kCodeSolid = 0, kCodeAir = 1, kCodeFluid = 2;

__host__ __device__ __forceinline__ uint8_t encode_tag(int t) {
    return t == 2 ? kCodeSolid : (t == 0 ? kCodeAir : kCodeFluid);
}
__host__ __device__ __forceinline__ int decode_tag(uint8_t c) {
    return c == kCodeSolid ? 2 : (c == kCodeAir ? 0 : 1);
}

// One neighbour's contribution to L x at a fluid cell (mgpcg.py:131-137):
// excluded (solid / outside) -> 0, air -> (0 - xc), fluid -> (xn - xc).
__device__ __forceinline__ float nb_term(uint8_t cn, float xn, float xc) {
    return cn == kCodeSolid ? 0.0f : __fsub_rn(cn == kCodeAir ? 0.0f : xn, xc);
}

// ------------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum in a fixed tree order (deterministic).  `scratch` holds one
// double per warp.  Result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double *scratch) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (wid == 0) {
        t = lane < nw ? scratch[lane] : 0.0;
        t = warp_sum(t);
    }
    return t;
}

}  // namespace flub
