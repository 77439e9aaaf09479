// 3x3x3 convolution (stride 1, zero padding 1) as a tcgen05 implicit GEMM.
//
// Layout: activations channels-last [B][X][Y][Z][C] in BF16, weights
// [27][Cout][Cin] BF16 (tap = (dx+1)*9 + (dy+1)*3 + (dz+1)), FP32 accumulation.
// One CTA computes 128 consecutive output voxels (a box of nyb rows of nzb
// voxels at fixed b, x) for all Cout channels:
//   D[128 x Cout] (TMEM, FP32) = sum over taps t and sources s of
//                               A_t,s[128 x Cin_s] * W_t,s[Cout x Cin_s]^T
// where A_t,s is the input box shifted by the tap offset, loaded by TMA with
// zero fill outside the volume (= the convolution's zero padding).  A and W
// land in shared memory in the K-major swizzled layout whose swizzle width is
// one row (Cin * 2 bytes: 32, 64 or 128 B) and feed tcgen05.mma directly.
// A second source (the skip connection of a U-Net decoder) is accumulated
// into the same tile, so a concatenation is never materialised.
//
// Roles (128 threads): thread 0 issues TMA loads into a 4-stage ring, thread 32
// issues the MMAs (one per 16 input channels), all four warps run the
// epilogue (TMEM -> registers, bias, ReLU, BF16 store).  Every mbarrier wait
// is bounded; a timeout sets the error word and the CTA still frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace flub {

constexpr int kConvThreads = 128;
constexpr int kConvStages = 4;
constexpr int kConvATile = 128 * 64 * 2;  // bytes, Cin <= 64
constexpr int kConvBTile = 64 * 64 * 2;   // bytes, Cout, Cin <= 64
constexpr int kConvStage = kConvATile + kConvBTile;
constexpr int kConvSmem = kConvStages * kConvStage + 1024 /* alignment */ + 256 /* barriers */;
constexpr uint32_t kWaitLimit = 1u << 22;

static __device__ int g_conv_error;

struct ConvGeom {
    int B, NX, NY, NZ;
    int nzb, nyb;
    int cout;
    int cin0, cin1;  // cin1 = 0: one source
    int relu;
    // forward kernel's pipeline stage: activation tile (128 voxels x max cin)
    // then weight tile, rounded to 1 KB so that every tile stays 1 KB aligned
    int a_bytes, stage_bytes;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
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

// tcgen05 shared-memory matrix descriptor, K-major, swizzle width = row bytes.
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr, int row_bytes) {
    const uint64_t layout = row_bytes == 128 ? 2ull : (row_bytes == 64 ? 4ull : 6ull);  // 128B / 64B / 32B swizzle
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                          // leading byte offset (unused: K fits one swizzle row)
    d |= (uint64_t)((8u * row_bytes) >> 4) << 32;    // stride byte offset: 8 rows
    d |= (uint64_t)1 << 46;                          // descriptor version
    d |= layout << 61;
    return d;
}

// Instruction descriptor: kind::f16, A = B = BF16 K-major, D = FP32, M = 128.
__device__ __forceinline__ uint32_t mma_idesc(int n) {
    return (1u << 4)                       // D format FP32
           | (1u << 7) | (1u << 10)        // A, B format BF16
           | ((uint32_t)(n >> 3) << 17)    // N / 8
           | ((uint32_t)(128 >> 4) << 24); // M / 16
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
        "[%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

template <int COUT>
__global__ void __launch_bounds__(kConvThreads, 1)
    k_conv3d_tc(const __grid_constant__ CUtensorMap mx0, const __grid_constant__ CUtensorMap mw0,
                const __grid_constant__ CUtensorMap mx1, const __grid_constant__ CUtensorMap mw1, const ConvGeom g,
                const float *__restrict__ bias, __nv_bfloat16 *__restrict__ y) {
    extern __shared__ unsigned char conv_smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(conv_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kConvStages * g.stage_bytes);
    uint64_t *empty = full + kConvStages;
    uint64_t *done = empty + kConvStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // tile -> (b, x, y0, z0)
    int t = blockIdx.x;
    const int tz = g.NZ / g.nzb, ty = g.NY / g.nyb;
    const int z0 = (t % tz) * g.nzb;
    t /= tz;
    const int y0 = (t % ty) * g.nyb;
    t /= ty;
    const int x = t % g.NX, b = t / g.NX;

    if (threadIdx.x == 0) {
        fail = 0;
        for (int s = 0; s < kConvStages; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    constexpr uint32_t kCols = COUT < 32 ? 32 : COUT;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const int nsrc = g.cin1 > 0 ? 2 : 1;
    const int T = 27 * nsrc;
    if (threadIdx.x == 0) {
        // producer
        for (int it = 0; it < T; it++) {
            const int s = it % kConvStages, u = it / kConvStages;
            if (u > 0 && !mbar_wait(smem_u32(&empty[s]), (u - 1) & 1)) {
                fail = 1;
                break;
            }
            const int src = it / 27, tap = it % 27;
            const int dx = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dz = tap % 3 - 1;
            const int cin = src ? g.cin1 : g.cin0;
            const uint32_t bytes = (uint32_t)(128 * cin * 2 + COUT * cin * 2);
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(bytes) : "memory");
            const uint32_t a = smem_u32(smem + s * g.stage_bytes), w = a + g.a_bytes;
            tma_load_5d(a, src ? &mx1 : &mx0, 0, z0 + dz, y0 + dy, x + dx, b, fb);
            tma_load_2d(w, src ? &mw1 : &mw0, 0, tap * COUT, fb);
        }
    } else if (threadIdx.x == 32) {
        // MMA issuer
        const uint32_t idesc = mma_idesc(COUT);
        bool ok = true;
        for (int it = 0; it < T && ok; it++) {
            const int s = it % kConvStages, u = it / kConvStages;
            if (!mbar_wait(smem_u32(&full[s]), u & 1)) {
                ok = false;
                fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int cin = (it / 27) ? g.cin1 : g.cin0;
            const uint32_t a = smem_u32(smem + s * g.stage_bytes), w = a + g.a_bytes;
            for (int kk = 0; kk < cin / 16; kk++) {
                const uint64_t ad = sw_desc(a + kk * 32, cin * 2), bd = sw_desc(w + kk * 32, cin * 2);
                const uint32_t acc = (it > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&empty[s]))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(done))
                     : "memory");
    }
    __syncwarp();
    // epilogue: row m of the accumulator is TMEM lane m, owned by warp m / 32
    // warp-uniform outcome: tcgen05.ld below is a .sync.aligned warp instruction
    const bool got = __all_sync(0xffffffffu, mbar_wait(smem_u32(done), 0) ? 1 : 0) != 0;
    if (!got) fail = 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int m = warp * 32 + lane;
    const int yy = y0 + m / g.nzb, zz = z0 + m % g.nzb;
    const int64_t vox = (((int64_t)b * g.NX + x) * g.NY + yy) * g.NZ + zz;
    if (got) {
        float acc[COUT];
#pragma unroll
        for (int c = 0; c < COUT; c += 16) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c, acc + c);
        __align__(16) __nv_bfloat16 out[COUT];
#pragma unroll
        for (int c = 0; c < COUT; c++) {
            float v = acc[c] + (bias ? __ldg(bias + c) : 0.0f);
            if (g.relu) v = fmaxf(v, 0.0f);
            out[c] = __float2bfloat16_rn(v);
        }
        uint4 *dst = reinterpret_cast<uint4 *>(y + vox * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 8; q++) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (fail && threadIdx.x == 0) atomicExch(&g_conv_error, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// ---------------------------------------------------------------- weight gradient
//
//   dW[tap][co][ci] = sum over voxels v of X[v + off(tap)][ci] * dY[v][co]
// as a tcgen05 GEMM with the voxels as K:
//   D[m = (slot, ci)][co] += A[m][v] * B[co][v]
// A holds G = 128 / Cin tap-shifted input tiles side by side (a "tap group":
// M = 128 rows = G taps x Cin channels), B the output-gradient tile.  Both are
// the channels-last tiles TMA already writes for the forward pass, read as
// MN-major operands: the channel dimension is contiguous, one swizzle atom
// wide, and the tap tiles of a group are consecutive atoms along M (leading
// byte offset = one tile).  A persistent CTA walks its share of the
// 128-voxel tiles, keeps one FP32 accumulator per tap group in TMEM for its
// whole life, and adds it to dW with one atomic per entry at the end.
// Groups that do not fit in TMEM (512 columns) are split over blockIdx.y.

constexpr int kWgStages = 4;
constexpr int kWgA = 32768;  // G tap tiles of 128 voxels x Cin BF16
constexpr int kWgB = 16384;  // dY tile, 128 voxels x Cout <= 64
constexpr int kWgStage = kWgA + kWgB;
constexpr int kWgSmem = kWgStages * kWgStage + 1024 + 256;
constexpr uint32_t kDoneWaitLimit = 1u << 26;

// MN-major shared-memory descriptor: swizzle width = one row (the channel
// extent), lbo = stride between atoms along M/N, sbo = 8 rows along K.
__device__ __forceinline__ uint64_t sw_desc_mn(uint32_t saddr, int row_bytes, uint32_t lbo) {
    const uint64_t layout = row_bytes == 128 ? 2ull : (row_bytes == 64 ? 4ull : 6ull);
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)(((8u * row_bytes) >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= layout << 61;
    return d;
}

__device__ __forceinline__ bool mbar_wait_long(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kDoneWaitLimit; i++) {
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

template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads, 1)
    k_conv3d_wgrad_tc(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap mdy, const ConvGeom g,
                      int groups_per_slice, int tmem_cols, float *__restrict__ dw) {
    constexpr int G = 128 / CIN;                 // taps per group
    constexpr int NG = (27 + G - 1) / G;         // groups
    constexpr int TILE_A = 128 * CIN * 2;        // one tap tile
    constexpr int TILE_B = 128 * COUT * 2;
    extern __shared__ unsigned char conv_smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(conv_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kWgStages * kWgStage);
    uint64_t *empty = full + kWgStages;
    uint64_t *done = empty + kWgStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tz = g.NZ / g.nzb, ty = g.NY / g.nyb;
    const int ntiles = g.B * g.NX * ty * tz;
    const int my_tiles = blockIdx.x < (unsigned)ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int gbeg = blockIdx.y * groups_per_slice;
    const int gend = min(NG, gbeg + groups_per_slice);
    const int ng = gend - gbeg;
    const int T = my_tiles * ng;

    if (threadIdx.x == 0) {
        fail = 0;
        for (int s = 0; s < kWgStages; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 0) {
        for (int it = 0; it < T; it++) {
            const int s = it % kWgStages, u = it / kWgStages;
            if (u > 0 && !mbar_wait(smem_u32(&empty[s]), (u - 1) & 1)) {
                fail = 1;
                break;
            }
            int t = (int)blockIdx.x + (it / ng) * (int)gridDim.x;
            const int grp = gbeg + it % ng;
            const int z0 = (t % tz) * g.nzb;
            t /= tz;
            const int y0 = (t % ty) * g.nyb;
            t /= ty;
            const int x = t % g.NX, b = t / g.NX;
            const int taps = min(G, 27 - grp * G);
            const uint32_t bytes = (uint32_t)(taps * TILE_A + TILE_B);
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(bytes) : "memory");
            const uint32_t a = smem_u32(smem + s * kWgStage);
            for (int q = 0; q < taps; q++) {
                const int tap = grp * G + q;
                const int dx = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dz = tap % 3 - 1;
                tma_load_5d(a + q * TILE_A, &mx, 0, z0 + dz, y0 + dy, x + dx, b, fb);
            }
            tma_load_5d(a + kWgA, &mdy, 0, z0, y0, x, b, fb);
        }
    } else if (threadIdx.x == 32) {
        const uint32_t idesc = mma_idesc(COUT) | (1u << 15) | (1u << 16);  // A and B MN-major
        for (int it = 0; it < T; it++) {
            const int s = it % kWgStages, u = it / kWgStages;
            if (!mbar_wait(smem_u32(&full[s]), u & 1)) {
                fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int j = it % ng;
            const uint32_t a = smem_u32(smem + s * kWgStage), bb = a + kWgA;
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {  // 16 voxel rows per MMA
                const uint64_t ad = sw_desc_mn(a + kk * 16 * CIN * 2, CIN * 2, TILE_A);
                const uint64_t bd = sw_desc_mn(bb + kk * 16 * COUT * 2, COUT * 2, TILE_B);
                const uint32_t acc = (it >= ng || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem + (uint32_t)(j * COUT)),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&empty[s]))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(done))
                     : "memory");
    }
    __syncwarp();
    const bool got = __all_sync(0xffffffffu, mbar_wait_long(smem_u32(done), 0) ? 1 : 0) != 0;
    if (!got) fail = 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();  // every thread sees a failure of the producer or the MMA issuer
    if (got && !fail && my_tiles > 0) {
        const int m = warp * 32 + lane;
        const int slot = m / CIN, ci = m % CIN;
        for (int j = 0; j < ng; j++) {
            const int tap = (gbeg + j) * G + slot;
#pragma unroll
            for (int c = 0; c < COUT; c += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * COUT + c), v);
                if (tap < 27) {
#pragma unroll
                    for (int e = 0; e < 16; e++) atomicAdd(&dw[((int64_t)tap * COUT + c + e) * CIN + ci], v[e]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (fail && threadIdx.x == 0) atomicExch(&g_conv_error, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
}

// ---------------------------------------------------------------- host side

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_encode_mutex;

static int get_encode() {
    std::lock_guard<std::mutex> lock(g_encode_mutex);
    if (g_encode) return FLUB_OK;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
        set_last_error("cuTensorMapEncodeTiled not available: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return FLUB_ERR_CUDA;
    }
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return FLUB_OK;
}

static CUtensorMapSwizzle swizzle_for(int row_bytes) {
    return row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                            : (row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

// Activation map: dims (C, Z, Y, X, B), box (C, nzb, nyb, 1, 1).
static int make_act_map(CUtensorMap *m, const void *x, int C, const ConvGeom &g) {
    const cuuint64_t dims[5] = {(cuuint64_t)C, (cuuint64_t)g.NZ, (cuuint64_t)g.NY, (cuuint64_t)g.NX, (cuuint64_t)g.B};
    const cuuint64_t es = 2;
    const cuuint64_t strides[4] = {C * es, (cuuint64_t)g.NZ * C * es, (cuuint64_t)g.NY * g.NZ * C * es,
                                   (cuuint64_t)g.NX * g.NY * g.NZ * C * es};
    const cuuint32_t box[5] = {(cuuint32_t)C, (cuuint32_t)g.nzb, (cuuint32_t)g.nyb, 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(x), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(C * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_last_error("cuTensorMapEncodeTiled(activations, C=%d) failed: %d", C, (int)r);
        return FLUB_ERR_CUDA;
    }
    return FLUB_OK;
}

// Weight map: [27 * Cout rows][Cin], box (Cin, Cout).
static int make_w_map(CUtensorMap *m, const void *w, int cin, int cout) {
    const cuuint64_t dims[2] = {(cuuint64_t)cin, (cuuint64_t)27 * cout};
    const cuuint64_t strides[1] = {(cuuint64_t)cin * 2};
    const cuuint32_t box[2] = {(cuuint32_t)cin, (cuuint32_t)cout};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(w), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(cin * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_last_error("cuTensorMapEncodeTiled(weights, Cin=%d, Cout=%d) failed: %d", cin, cout, (int)r);
        return FLUB_ERR_CUDA;
    }
    return FLUB_OK;
}

template <int COUT>
static int launch_conv(const CUtensorMap &mx0, const CUtensorMap &mw0, const CUtensorMap &mx1, const CUtensorMap &mw1,
                       const ConvGeom &g, const float *bias, __nv_bfloat16 *y, cudaStream_t s) {
    static bool attr_set = false;
    if (!attr_set) {
        FLUB_CHECK_CUDA(cudaFuncSetAttribute(k_conv3d_tc<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem));
        attr_set = true;
    }
    const unsigned tiles = (unsigned)((int64_t)g.B * g.NX * (g.NY / g.nyb) * (g.NZ / g.nzb));
    // shared memory sized for this layer's channels: the 16- and 32-channel
    // layers fit several CTAs per SM, whose pipelines then overlap
    const size_t smem = (size_t)kConvStages * g.stage_bytes + 1024 + 256;
    k_conv3d_tc<COUT><<<tiles, kConvThreads, smem, s>>>(mx0, mw0, mx1, mw1, g, bias, y);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace flub

using namespace flub;

extern "C" int flub_conv3d_bf16(const void *x0, int cin0, const void *w0, const void *x1, int cin1, const void *w1,
                                const float *bias, void *y, int cout, int B, int NX, int NY, int NZ, int relu,
                                void *stream) {
    auto okc = [](int c) { return c == 16 || c == 32 || c == 64; };
    FLUB_REQUIRE(x0 && w0 && y, "flub_conv3d_bf16: NULL argument");
    FLUB_REQUIRE(okc(cin0) && okc(cout) && (x1 == nullptr ? cin1 == 0 : (okc(cin1) && w1 != nullptr)),
                 "flub_conv3d_bf16: channels must be 16, 32 or 64 (cin0=%d cin1=%d cout=%d)", cin0, cin1, cout);
    FLUB_REQUIRE(B > 0 && NX > 0 && NY > 0 && NZ > 0, "flub_conv3d_bf16: bad shape");
    FLUB_REQUIRE(aligned16(x0) && aligned16(w0) && aligned16(y) && (!x1 || (aligned16(x1) && aligned16(w1))),
                 "flub_conv3d_bf16: pointers must be 16-byte aligned");
    ConvGeom g;
    g.B = B; g.NX = NX; g.NY = NY; g.NZ = NZ;
    g.nzb = NZ < 128 ? NZ : 128;
    FLUB_REQUIRE(128 % g.nzb == 0 && NZ % g.nzb == 0, "flub_conv3d_bf16: NZ=%d must divide 128 or be a multiple of 128",
                 NZ);
    g.nyb = 128 / g.nzb;
    FLUB_REQUIRE(NY % g.nyb == 0, "flub_conv3d_bf16: NY=%d must be a multiple of %d", NY, g.nyb);
    g.cout = cout;
    g.cin0 = cin0;
    g.cin1 = x1 ? cin1 : 0;
    g.relu = relu ? 1 : 0;
    {
        const int cmax = g.cin1 > g.cin0 ? g.cin1 : g.cin0;
        g.a_bytes = 128 * cmax * 2;
        g.stage_bytes = (g.a_bytes + cout * cmax * 2 + 1023) & ~1023;
    }
    int st = get_encode();
    if (st) return st;
    CUtensorMap mx0, mw0, mx1, mw1;
    if ((st = make_act_map(&mx0, x0, cin0, g)) || (st = make_w_map(&mw0, w0, cin0, cout))) return st;
    if (x1) {
        if ((st = make_act_map(&mx1, x1, cin1, g)) || (st = make_w_map(&mw1, w1, cin1, cout))) return st;
    } else {
        mx1 = mx0;
        mw1 = mw0;
    }
    cudaStream_t s = as_stream(stream);
    __nv_bfloat16 *yo = static_cast<__nv_bfloat16 *>(y);
    switch (cout) {
    case 16: return launch_conv<16>(mx0, mw0, mx1, mw1, g, bias, yo, s);
    case 32: return launch_conv<32>(mx0, mw0, mx1, mw1, g, bias, yo, s);
    default: return launch_conv<64>(mx0, mw0, mx1, mw1, g, bias, yo, s);
    }
}

namespace flub {
int launch_bias_grad(const void *dy, int cout, int64_t nvox, float *db, cudaStream_t s);

template <int CIN, int COUT>
static int launch_wgrad(const CUtensorMap &mx, const CUtensorMap &mdy, const ConvGeom &g, float *dw, cudaStream_t s) {
    static bool attr_set = false;
    if (!attr_set) {
        FLUB_CHECK_CUDA(
            cudaFuncSetAttribute(k_conv3d_wgrad_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgSmem));
        attr_set = true;
    }
    constexpr int G = 128 / CIN, NG = (27 + G - 1) / G;
    const int per = NG * COUT <= 512 ? NG : 512 / COUT;
    const int slices = (NG + per - 1) / per;
    int cols = 32;
    while (cols < per * COUT) cols <<= 1;
    int dev = 0, sms = kNumSMs;
    FLUB_CHECK_CUDA(cudaGetDevice(&dev));
    FLUB_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t ntiles = (int64_t)g.B * g.NX * (g.NY / g.nyb) * (g.NZ / g.nzb);
    const unsigned gx = (unsigned)(ntiles < sms ? ntiles : sms);
    k_conv3d_wgrad_tc<CIN, COUT><<<dim3(gx, slices), kConvThreads, kWgSmem, s>>>(mx, mdy, g, per, cols, dw);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}
}  // namespace flub

extern "C" int flub_conv3d_wgrad(const void *x, int cin, const void *dy, int cout, float *dw, float *db, int B, int NX,
                                 int NY, int NZ, void *stream) {
    auto okc = [](int c) { return c == 16 || c == 32 || c == 64; };
    FLUB_REQUIRE(x && dy && dw, "flub_conv3d_wgrad: NULL argument");
    FLUB_REQUIRE(okc(cin) && okc(cout), "flub_conv3d_wgrad: channels must be 16, 32 or 64 (cin=%d cout=%d)", cin, cout);
    FLUB_REQUIRE(B > 0 && NX > 0 && NY > 0 && NZ > 0, "flub_conv3d_wgrad: bad shape");
    FLUB_REQUIRE(aligned16(x) && aligned16(dy), "flub_conv3d_wgrad: pointers must be 16-byte aligned");
    ConvGeom g;
    g.B = B; g.NX = NX; g.NY = NY; g.NZ = NZ;
    g.a_bytes = g.stage_bytes = 0;  // the forward kernel's stage layout; unused here
    g.nzb = NZ < 128 ? NZ : 128;
    FLUB_REQUIRE(128 % g.nzb == 0 && NZ % g.nzb == 0, "flub_conv3d_wgrad: NZ=%d must divide 128 or be a multiple of 128",
                 NZ);
    g.nyb = 128 / g.nzb;
    FLUB_REQUIRE(NY % g.nyb == 0, "flub_conv3d_wgrad: NY=%d must be a multiple of %d", NY, g.nyb);
    g.cout = cout;
    g.cin0 = cin;
    g.cin1 = 0;
    g.relu = 0;
    int st = get_encode();
    if (st) return st;
    CUtensorMap mx, mdy;
    if ((st = make_act_map(&mx, x, cin, g)) || (st = make_act_map(&mdy, dy, cout, g))) return st;
    cudaStream_t s = as_stream(stream);
#define FLUB_WG(CI, CO) \
    if (cin == CI && cout == CO) st = launch_wgrad<CI, CO>(mx, mdy, g, dw, s);
    FLUB_WG(16, 16) FLUB_WG(16, 32) FLUB_WG(16, 64)
    FLUB_WG(32, 16) FLUB_WG(32, 32) FLUB_WG(32, 64)
    FLUB_WG(64, 16) FLUB_WG(64, 32) FLUB_WG(64, 64)
#undef FLUB_WG
    if (st) return st;
    if (db) return launch_bias_grad(dy, cout, (int64_t)B * NX * NY * NZ, db, s);
    return FLUB_OK;
}

extern "C" int flub_conv_error(int *out, int reset) {
    FLUB_REQUIRE(out, "flub_conv_error: NULL argument");
    FLUB_CHECK_CUDA(cudaMemcpyFromSymbol(out, g_conv_error, sizeof(int)));
    if (reset) {
        const int z = 0;
        FLUB_CHECK_CUDA(cudaMemcpyToSymbol(g_conv_error, &z, sizeof(int)));
    }
    return FLUB_OK;
}
