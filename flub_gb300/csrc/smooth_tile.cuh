// TMA-staged red-black smoothing, two half-sweeps per launch.
//
// One CTA owns a tile of kTI x kTJ x kTK cells.  A single TMA transaction
// per array brings in the tile with its halo: z with two cells of halo in i
// and j (four in k, to keep the box start on a 16-byte boundary), the
// residual and the stencil words with one (k: four and eight).  The CTA then
// runs the first colour on the tile plus a one-cell halo and the second
// colour on the tile, in shared memory, and stores the tile.  The halo cells
// of the first colour are the values the neighbouring CTAs compute for their
// own tiles from the same inputs, so each CTA finishes a whole red-black
// iteration without hearing from the others.  The input and output z must be
// different buffers (other CTAs read this tile's cells as their halo).
//
// Per cell the arithmetic is k_smooth8's (multigrid/mgpcg.py:72-86, the
// reference's order), so the results are bit-identical to two k_smooth8
// half-sweeps; non-fluid cells of the tile are written 0.
//
// Measured on the 256^3 dam break (one GB300) it is slower than k_smooth8:
// 28 us per level-0 iteration against 2 x 11.5 us.  It executes several times
// the instructions of the row kernel (the halo cells of the first colour are
// computed twice, and the two colours diverge inside a warp), while the row
// kernel is bound by memory latency rather than by instructions.  So it runs
// only when FLUB_TILE=1 asks for it.
#pragma once

#include <cuda.h>

#include "mg_kernels.cuh"
#include "smooth8.cuh"

namespace flub {

constexpr int kTI = 8, kTJ = 8, kTK = 32;                                    // tile
constexpr int kZI = kTI + 4, kZJ = kTJ + 4, kZK = kTK + 8;                   // z box (halo 2, 2, 4)
constexpr int kRI = kTI + 2, kRJ = kTJ + 2, kRK = kTK + 8;                   // residual box (halo 1, 1, 4)
constexpr int kWI = kTI + 2, kWJ = kTJ + 2, kWK = kTK + 16;                  // stencil-word box (halo 1, 1, 8)
constexpr int kCI = kTI / 2 + 2, kCJ = kTJ / 2 + 2, kCK = kTK / 2 + 8;       // coarse z box (prolongation)
constexpr int kTileThreads = 256;
constexpr int kTileBlocksPerSM = 4;

constexpr int kZBytes = kZI * kZJ * kZK * 4;
constexpr int kRBytes = kRI * kRJ * kRK * 4;
constexpr int kWBytes = kWI * kWJ * kWK * 2;
constexpr int kCBytes = kCI * kCJ * kCK * 4;
constexpr int kTileOffR = kZBytes;
constexpr int kTileOffW = kTileOffR + kRBytes;
constexpr int kTileOffC = kTileOffW + kWBytes;
constexpr int kTileOffBar = kTileOffC + kCBytes;
constexpr int kTileSmem = kTileOffBar + 128;
static_assert(kZBytes % 128 == 0 && kRBytes % 128 == 0 && kWBytes % 128 == 0 && kCBytes % 128 == 0,
              "TMA destinations stay 128-byte aligned");
static_assert((kZK * 4) % 16 == 0 && (kRK * 4) % 16 == 0 && (kWK * 2) % 16 == 0 && (kCK * 4) % 16 == 0,
              "TMA boxes are whole 16-byte rows");

constexpr uint32_t kTileWaitLimit = 1u << 20;

enum TileMode { kTileInPlaceInput = 0, kTileFromZero = 1, kTileProlong = 2 };

__device__ __forceinline__ uint32_t tile_smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tile_tma_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ bool tile_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kTileWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One cell's update from the staged boxes: a, b, c are its z-box coordinates
// (cell (i0 - 2 + a, j0 - 2 + b, k0 - 4 + c)); it lies inside the residual and
// word boxes (1 <= a < kZI - 1, 1 <= b < kZJ - 1).  kFirstFromZero: z was 0
// before this half-sweep (k_smooth8's kFromZero formula).
template <bool kFirstFromZero>
__device__ __forceinline__ void tile_update(float *zs, const float *rs, const uint16_t *ws, int a, int b, int c) {
    const int zc = (a * kZJ + b) * kZK + c;
    const uint32_t w = ws[((a - 1) * kWJ + (b - 1)) * kWK + c + 4];
    if (sw_code(w, 0) != kCodeFluid) return;
    const float xc = zs[zc];
    int d = 0;
    float tp, tm, ret = 0.0f;
    uint32_t cn;
    tp = 0.0f; tm = 0.0f;
    cn = sw_code(w, 1); if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : zs[zc + kZJ * kZK], xc); d++; }
    cn = sw_code(w, 2); if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : zs[zc - kZJ * kZK], xc); d++; }
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    tp = 0.0f; tm = 0.0f;
    cn = sw_code(w, 3); if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : zs[zc + kZK], xc); d++; }
    cn = sw_code(w, 4); if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : zs[zc - kZK], xc); d++; }
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    tp = 0.0f; tm = 0.0f;
    cn = sw_code(w, 5); if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : zs[zc + 1], xc); d++; }
    cn = sw_code(w, 6); if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : zs[zc - 1], xc); d++; }
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    float zn = 0.0f;
    if (d != 0) {
        const float rv = rs[((a - 1) * kRJ + (b - 1)) * kRK + c];
        zn = kFirstFromZero ? __fdiv_rn(rv, (float)d) : __fadd_rn(xc, __fdiv_rn(__fadd_rn(rv, ret), (float)d));
    }
    zs[zc] = zn;
}

// The cells of one colour in the z-box region rows [lo, kZI - lo) x
// [lo, kZJ - lo), k-range [c_lo, c_lo + 2 * n): cell (i, j, k) is updated by
// phase p when (i + j + k) % 2 != p (k_smooth8's rule).
template <bool kFirstFromZero, int kLo, int kN>
__device__ __forceinline__ void tile_pass(float *zs, const float *rs, const uint16_t *ws, int i0, int j0, int k0,
                                          int phase, int c_lo) {
    constexpr int kRowsJ = kZJ - 2 * kLo, kRows = (kZI - 2 * kLo) * kRowsJ;
    for (int e = threadIdx.x; e < kRows * kN; e += kTileThreads) {
        const int row = e / kN, t = e - row * kN;
        const int a = kLo + row / kRowsJ, b = kLo + row % kRowsJ;
        // parity of k among the cells this phase updates in row (i, j)
        const int i = i0 - 2 + a, j = j0 - 2 + b;
        const int kpar = (i + j + phase + 1) & 1;  // (i + j + k) % 2 != phase  <=>  k % 2 == kpar
        const int kbase = k0 - 4 + c_lo;
        const int c = c_lo + 2 * t + ((kbase & 1) != kpar ? 1 : 0);
        tile_update<kFirstFromZero>(zs, rs, ws, a, b, c);
    }
}

// One red-black iteration (phase p, then 1 - p) over the listed tiles of a
// level, z_in -> z_out (different buffers).  Maps (3D, x = k innermost):
// mz over z_in, box kZK x kZJ x kZI; mr over r, box kRK x kRJ x kRI; mw over
// the stencil words, box kWK x kWJ x kWI; mc over the coarse z (kProlong
// only), box kCK x kCJ x kCI.  kMode: kTileFromZero (z_in is 0: not read),
// kTileProlong (z_in + zc[parent] first, multigrid/mgpcg.py:113-116), or
// plain.  A wait that gives up sets *status = FLUB_ERR_TIMEOUT and the CTA
// stops.  Grid: up to kTileBlocksPerSM CTAs per SM, over the tile list.
template <int kMode>
__global__ void __launch_bounds__(kTileThreads, kTileBlocksPerSM)
    k_smooth_tile(const __grid_constant__ CUtensorMap mz, const __grid_constant__ CUtensorMap mr,
                  const __grid_constant__ CUtensorMap mw, const __grid_constant__ CUtensorMap mc,
                  float *__restrict__ z_out, Dims D, int phase, const int *__restrict__ tiles,
                  const int *__restrict__ n_tiles, int *status, unsigned long long *kc) {
    count_kernel(kc);
    extern __shared__ __align__(128) unsigned char tsm[];
    float *zs = reinterpret_cast<float *>(tsm);
    const float *rs = reinterpret_cast<const float *>(tsm + kTileOffR);
    const uint16_t *ws = reinterpret_cast<const uint16_t *>(tsm + kTileOffW);
    const float *cs = reinterpret_cast<const float *>(tsm + kTileOffC);
    uint64_t *bar = reinterpret_cast<uint64_t *>(tsm + kTileOffBar);
    const uint32_t bar_a = tile_smem_u32(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int nt = *n_tiles;
    const int tnj = D.ny / kTJ, tnk = D.nz / kTK;
    uint32_t parity = 0;
    for (int q = blockIdx.x; q < nt; q += gridDim.x, parity ^= 1u) {
        const int t = tiles[q];
        const int i0 = (t / (tnj * tnk)) * kTI, j0 = ((t / tnk) % tnj) * kTJ, k0 = (t % tnk) * kTK;
        if (threadIdx.x == 0) {
            // the boxes were last read and written through the generic proxy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const uint32_t bytes = kRBytes + kWBytes + (kMode != kTileFromZero ? kZBytes : 0) +
                                   (kMode == kTileProlong ? kCBytes : 0);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(bytes) : "memory");
            if (kMode != kTileFromZero) tile_tma_3d(tile_smem_u32(zs), &mz, k0 - 4, j0 - 2, i0 - 2, bar_a);
            tile_tma_3d(tile_smem_u32(rs), &mr, k0 - 4, j0 - 1, i0 - 1, bar_a);
            tile_tma_3d(tile_smem_u32(ws), &mw, k0 - 8, j0 - 1, i0 - 1, bar_a);
            if (kMode == kTileProlong) tile_tma_3d(tile_smem_u32(cs), &mc, k0 / 2 - 4, j0 / 2 - 1, i0 / 2 - 1, bar_a);
        }
        if (kMode == kTileFromZero)
            for (int e = threadIdx.x; e < kZI * kZJ * kZK / 4; e += kTileThreads)
                reinterpret_cast<float4 *>(zs)[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const bool ok = tile_wait(bar_a, parity);
        if (!__syncthreads_and(ok ? 1 : 0)) {
            if (threadIdx.x == 0) atomicExch(status, FLUB_ERR_TIMEOUT);
            return;
        }
        if (kMode == kTileProlong) {
            // z_eff = z_in + zc[parent] over the whole z box; the parent of z-box
            // cell (a, b, c) is coarse-box cell (a / 2, b / 2, 2 + c / 2)
            for (int e = threadIdx.x; e < kZI * kZJ * kZK; e += kTileThreads) {
                const int c = e % kZK, bb = (e / kZK) % kZJ, a = e / (kZK * kZJ);
                zs[e] = __fadd_rn(zs[e], __fmul_rn(cs[((a >> 1) * kCJ + (bb >> 1)) * kCK + 2 + (c >> 1)], 1.0f));
            }
            __syncthreads();
        }
        // first colour on the tile and a one-cell halo (k from k0 - 1 to k0 + kTK + 1)
        tile_pass<kMode == kTileFromZero, 1, (kTK + 2) / 2>(zs, rs, ws, i0, j0, k0, phase, 3);
        __syncthreads();
        // second colour on the tile
        tile_pass<false, 2, kTK / 2>(zs, rs, ws, i0, j0, k0, 1 - phase, 4);
        __syncthreads();
        // store the tile: fluid cells their value, the others 0
        for (int e = threadIdx.x; e < kTI * kTJ * (kTK / 4); e += kTileThreads) {
            const int qd = e % (kTK / 4), row = e / (kTK / 4);
            const int a = 2 + row / kTJ, bb = 2 + row % kTJ;
            const float4 v = *reinterpret_cast<const float4 *>(zs + (a * kZJ + bb) * kZK + 4 + 4 * qd);
            const uint2 wv = *reinterpret_cast<const uint2 *>(ws + ((a - 1) * kWJ + (bb - 1)) * kWK + 8 + 4 * qd);
            float4 o;
            o.x = sw_code(wv.x & 0xffffu, 0) == kCodeFluid ? v.x : 0.0f;
            o.y = sw_code(wv.x >> 16, 0) == kCodeFluid ? v.y : 0.0f;
            o.z = sw_code(wv.y & 0xffffu, 0) == kCodeFluid ? v.z : 0.0f;
            o.w = sw_code(wv.y >> 16, 0) == kCodeFluid ? v.w : 0.0f;
            const int i = i0 + a - 2, j = j0 + bb - 2;
            *reinterpret_cast<float4 *>(z_out + ((int64_t)i * D.ny + j) * D.nz + k0 + 4 * qd) = o;
        }
        __syncthreads();  // the next tile's TMA overwrites the boxes
    }
}

// Tiles of a level that hold a fluid cell: flag the tile of every listed
// active 8-cell group, then list the flagged tiles.  Grid (flags): over the
// active groups; (list): over the tiles.
__global__ void __launch_bounds__(256) k_tile_flags(const int *__restrict__ act, const int *__restrict__ act_n, Dims D,
                                                    unsigned char *__restrict__ flags) {
    const int n = *act_n;
    const int tnj = D.ny / kTJ, tnk = D.nz / kTK;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        int i, j, kg;
        group_ijk(__ldg(act + q), D, i, j, kg);
        flags[((i / kTI) * tnj + j / kTJ) * tnk + (kg * 8) / kTK] = 1;
    }
}

__global__ void __launch_bounds__(256) k_tile_list(const unsigned char *__restrict__ flags, int n_tiles,
                                                   int *__restrict__ tiles, int *__restrict__ count) {
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n_tiles; base += gridDim.x * blockDim.x) {
        const int t = base + lane;
        const bool on = t < n_tiles && flags[t];
        const unsigned m = __ballot_sync(0xffffffffu, on);
        int first = 0;
        if (lane == 0 && m) first = atomicAdd(count, __popc(m));
        first = __shfl_sync(0xffffffffu, first, 0);
        if (on) tiles[first + __popc(m & ((1u << lane) - 1u))] = t;
    }
}

}  // namespace flub
