// The middle levels of the V-cycle in persistent cooperative kernels (opt-in,
// FLUB_PERSIST=1).
//
// Below level 0 a red-black half-sweep or a restriction has a few thousand
// to a few tens of thousands of 8-cell groups to visit: one short wave whose
// time is launch and dependent-load latency, not bandwidth.  Here every block
// of one cooperative launch (all co-resident) runs the same sequence of such
// passes over levels l0 .. l1-1, separated by grid barriers instead of kernel
// boundaries:
//   k_vcycle_down  pre-smoothing of each level (the first half-sweep from
//                  zero), then its residual + restriction into the next level
//                  (the restriction out of l1-1 writes the first coarse level,
//                  which the cluster / tail kernel takes over);
//   k_vcycle_up    from level l1-1 up to l0: the first post-smoothing half-sweep
//                  fused with the prolongation of the coarser correction, then
//                  the remaining half-sweeps.
// The passes are the functions of k_smooth8 / k_restrict8 (smooth8.cuh,
// restrict8.cuh) with the same operations in the same order, so results are
// bit-identical to the launch-per-pass path; only their loads of r and z use
// the coherent path, because other blocks wrote those earlier in the launch.
//
// The grid barrier is a generation counter: each block's thread 0 publishes
// its block's writes (fence), arrives on a counter, and the last arrival resets
// the counter and advances the generation that the others wait for.  Every wait
// is bounded: after kBarrierSpinLimit polls the block records FLUB_ERR_TIMEOUT
// in the solver state and goes on (the solve then reports the error instead of
// hanging).
#pragma once

#include "restrict8.cuh"
#include "smooth8.cuh"

namespace flub {

constexpr int kPersistThreads = 512;
constexpr unsigned kBarrierSpinLimit = 1u << 24;

struct LegLevel {
    Dims D;
    const uint8_t *code;
    const uint16_t *sw;
    const int *act, *act_n;
    void *r, *z, *z2;  // level storage (float, or __half in the mixed-precision V-cycle)
    int iters;         // red-black iterations per side
};

struct LegParams {
    int l0, l1;           // levels l0 .. l1-1 run here; l1 is the first coarse (cluster / tail) level
    LegLevel lv[12];      // indexed by level; l1 is filled for the restriction target and the prolongation source
    float rscale;         // restriction output scale (the schedule's, times 1/8 between FP16 levels)
    float zc_scale;       // prolongation input scale (1, or 8 between FP16 levels)
    MgState *st;          // barrier words and the status a timed-out wait reports
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void grid_barrier(MgState *st) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire_gpu(&st->bar_gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&st->bar_count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            unsigned spins = 0;
            while (ld_acquire_gpu(&st->bar_gen) == gen) {
                if (++spins > kBarrierSpinLimit) {
                    atomicExch(&st->status, FLUB_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

template <typename T>
__device__ __forceinline__ void leg_sweep(const LegLevel &L, int phase, int mode, const T *zin, T *zout,
                                          const T *zc, float zc_scale) {
    const T *r = static_cast<const T *>(L.r);
    if (mode == 1)
        smooth8_pass<true, false, false, T, T, T, T>(zout, zout, nullptr, 1.0f, r, L.code, L.sw, L.D, phase, L.act,
                                                     L.act_n, blockIdx.x, gridDim.x);
    else if (mode == 2)
        smooth8_pass<false, true, false, T, T, T, T>(zout, zin, zc, zc_scale, r, L.code, L.sw, L.D, phase, L.act,
                                                     L.act_n, blockIdx.x, gridDim.x);
    else
        smooth8_pass<false, false, false, T, T, T, T>(zout, zout, nullptr, 1.0f, r, L.code, L.sw, L.D, phase,
                                                      L.act, L.act_n, blockIdx.x, gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(kPersistThreads, 2) k_vcycle_down(const LegParams P, unsigned long long *kc) {
    if (kc && (blockIdx.x | threadIdx.x) == 0) atomicAdd(kc, 1ull);
    for (int l = P.l0; l < P.l1; l++) {
        const LegLevel &L = P.lv[l];
        T *z2 = static_cast<T *>(L.z2);
        for (int it = 0; it < L.iters; it++) {
            leg_sweep<T>(L, 0, it == 0 ? 1 : 0, z2, z2, nullptr, 1.0f);
            grid_barrier(P.st);
            leg_sweep<T>(L, 1, 0, z2, z2, nullptr, 1.0f);
            grid_barrier(P.st);
        }
        const LegLevel &C = P.lv[l + 1];
        if (l + 1 == P.l1) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        restrict8_pass<false, false>(static_cast<const T *>(L.r), (const T *)z2, L.code, L.sw, static_cast<T *>(C.r),
                                     C.code, C.D, P.rscale, C.act, C.act_n, blockIdx.x, gridDim.x);
        if (l + 1 < P.l1) grid_barrier(P.st);
    }
}

template <typename T>
__global__ void __launch_bounds__(kPersistThreads, 2) k_vcycle_up(const LegParams P, unsigned long long *kc) {
    if (kc && (blockIdx.x | threadIdx.x) == 0) atomicAdd(kc, 1ull);
    for (int l = P.l1 - 1; l >= P.l0; l--) {
        const LegLevel &L = P.lv[l];
        T *z = static_cast<T *>(L.z);
        const T *zc = static_cast<const T *>(P.lv[l + 1].z);
        for (int it = 0; it < L.iters; it++) {
            leg_sweep<T>(L, 1, it == 0 ? 2 : 0, static_cast<const T *>(L.z2), z, zc, P.zc_scale);
            grid_barrier(P.st);
            const bool last = l == P.l0 && it + 1 == L.iters;
            if (last) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
            leg_sweep<T>(L, 0, 0, z, z, nullptr, 1.0f);
            if (!last) grid_barrier(P.st);
        }
    }
}

}  // namespace flub
