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
//
// k_conv3d_halo (below) computes the same convolution from input planes
// staged once per CTA; halo_plan chooses between the two kernels per layer.
// The weight gradient (k_conv3d_wgrad_tc) is a third tcgen05 kernel.
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

// ---------------------------------------------------------------- halo-plane forward kernel
//
// The same convolution for NZ % 8 == 0 and NY % 16 == 0 when the layer's
// weights fit in shared memory, organised around input planes instead of
// tap-shifted tiles, with no TMA and no waits between MMAs.
//
// A CTA owns a 16 (y) x 8 (z) voxel tile at xr consecutive x planes x0 ..
// x0 + xr - 1; GEMM row m is voxel (y0 + m / 8, z0 + m % 8).  First all 128
// threads stage, with coalesced 16-byte loads:
//   - input plane p (x = x0 - 1 + p, p = 0 .. xr + 1) of each source as the
//     haloed 18 x 10 voxel region, zero outside the volume (the padding), in
//     the no-swizzle K-major layout
//         [chunk of 8 channels][y 0..17][z 0..9][8 channels]   (16-byte rows);
//   - every tap's weights, [tap][chunk][Cout][8 channels], the same layout
//     for the B operand (core matrix = 8 output channels x 16 bytes).
// A proxy fence publishes them to the tensor core.  The A operand of tap
// (dx, dy, dz) for output plane xi is plane xi + dx + 1 read from start
// offset ((dy + 1) * 10 + dz + 1) * 16 bytes: a core matrix is the 8 z-voxels
// of one y-row (128 contiguous bytes), core matrices adjacent in M are one
// padded row apart (SBO = 160 bytes) and adjacent chunks one chunk region apart
// (LBO = kHaloChunk).  So all 27 taps read one copy of the data, and one
// thread then issues every MMA of the CTA back to back into xr FP32
// accumulators side by side in TMEM (columns xi * Cout ...).
//
// Staging the weights with plain loads matters: per-tap TMA boxes of a few
// hundred bytes, requested by many CTAs per SM, arrived about 0.4 us apart
// and left the MMA thread waiting on every tap.
constexpr int kHaloZ = 10, kHaloY = 18;
constexpr int kHaloRows = kHaloZ * kHaloY;                      // 16-byte rows per chunk (180)
constexpr int kHaloChunk = (kHaloRows * 16 + 127) / 128 * 128;  // chunk region, 128-byte aligned (2944)

struct HaloGeom {
    int B, NX, NY, NZ;
    int xr;                 // output planes per CTA
    int cin0, cin1, relu;   // cin1 = 0: one source
    int plane0, plane1;     // bytes of one input plane per source (chunks x kHaloChunk)
    int planes1_off;        // offset of source 1's planes
    int w0_off, w1_off;     // weights of source 0 and 1 (27 taps each)
    int bar_off;            // completion mbarrier and TMEM slot
    uint32_t tmem_cols;
};

// tcgen05 shared-memory matrix descriptor, K-major without swizzle: core
// matrices of 8 rows x 16 bytes; lbo = bytes between core matrices adjacent
// in K, sbo = bytes between core matrices adjacent in M (or N).
__device__ __forceinline__ uint64_t ns_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version; layout type 0 (no swizzle) in bits 61-63
    return d;
}

// Stages the np haloed input planes of one source into dst (layout above).
// Item q = ((p * 18 + yh) * 10 + zh) * C8 + c, chunks fastest, so that a
// warp's loads cover whole voxel rows of the channels-last input.  Eight
// loads are in flight per thread before their stores.
__device__ __forceinline__ void halo_stage(const uint4 *__restrict__ x, unsigned char *dst, int c8_log2, int np,
                                           int plane_bytes, int b, int x0, int y0, int z0, const HaloGeom &g) {
    const int C8 = 1 << c8_log2;
    const int total = np * kHaloRows * C8;
    for (int base = 0; base < total; base += 8 * kConvThreads) {
        uint4 v[8];
        int off[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int q = base + u * kConvThreads + threadIdx.x;
            off[u] = -1;
            v[u] = make_uint4(0u, 0u, 0u, 0u);
            if (q < total) {
                const int c = q & (C8 - 1);
                int r = q >> c8_log2;
                const int zh = r % kHaloZ;
                r /= kHaloZ;
                const int yh = r % kHaloY, p = r / kHaloY;
                const int xx = x0 - 1 + p, yy = y0 - 1 + yh, zz = z0 - 1 + zh;
                off[u] = p * plane_bytes + c * kHaloChunk + (yh * kHaloZ + zh) * 16;
                if ((unsigned)xx < (unsigned)g.NX && (unsigned)yy < (unsigned)g.NY && (unsigned)zz < (unsigned)g.NZ)
                    v[u] = __ldg(x + ((((int64_t)b * g.NX + xx) * g.NY + yy) * g.NZ + zz) * C8 + c);
            }
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (off[u] >= 0) *reinterpret_cast<uint4 *>(dst + off[u]) = v[u];
    }
}

// Stages weights [27][COUT][Cin] (Cin = 8 << c8_log2) as [tap][chunk][COUT][8].
template <int COUT>
__device__ __forceinline__ void halo_stage_weights(const uint4 *__restrict__ w, unsigned char *dst, int c8_log2) {
    const int C8 = 1 << c8_log2;
    const int total = 27 * COUT * C8;
    for (int q = threadIdx.x; q < total; q += kConvThreads) {
        const int c = q & (C8 - 1);
        const int r = q >> c8_log2;  // tap * COUT + co
        const int tap = r / COUT, co = r - tap * COUT;
        *reinterpret_cast<uint4 *>(dst + (((tap << c8_log2) + c) * COUT + co) * 16) = __ldg(w + q);
    }
}

template <int COUT>
__global__ void __launch_bounds__(kConvThreads, 1)
    k_conv3d_halo(const __nv_bfloat16 *__restrict__ x0p, const __nv_bfloat16 *__restrict__ w0p,
                  const __nv_bfloat16 *__restrict__ x1p, const __nv_bfloat16 *__restrict__ w1p, const HaloGeom g,
                  const float *__restrict__ bias, __nv_bfloat16 *__restrict__ y) {
    extern __shared__ unsigned char conv_smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(conv_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char *planes1 = smem + g.planes1_off;
    uint64_t *done = reinterpret_cast<uint64_t *>(smem + g.bar_off);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int t = blockIdx.x;
    const int tz = g.NZ >> 3, ty = g.NY >> 4, tx = g.NX / g.xr;
    const int z0 = (t % tz) * 8;
    t /= tz;
    const int y0 = (t % ty) * 16;
    t /= ty;
    const int x0 = (t % tx) * g.xr, b = t / tx;
    const int nsrc = g.cin1 > 0 ? 2 : 1;
    const int lg0 = g.cin0 == 16 ? 1 : (g.cin0 == 32 ? 2 : 3), lg1 = g.cin1 == 16 ? 1 : (g.cin1 == 32 ? 2 : 3);

    if (threadIdx.x == 0) {
        fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(g.tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }

    // every input plane and every weight once, by all threads; then visible
    // to the tensor core
    halo_stage(reinterpret_cast<const uint4 *>(x0p), smem, lg0, g.xr + 2, g.plane0, b, x0, y0, z0, g);
    halo_stage_weights<COUT>(reinterpret_cast<const uint4 *>(w0p), smem + g.w0_off, lg0);
    if (nsrc > 1) {
        halo_stage(reinterpret_cast<const uint4 *>(x1p), planes1, lg1, g.xr + 2, g.plane1, b, x0, y0, z0, g);
        halo_stage_weights<COUT>(reinterpret_cast<const uint4 *>(w1p), smem + g.w1_off, lg1);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 32) {
        // MMA issuer: 27 taps x sources x planes x (Cin / 16), then one commit
        const uint32_t idesc = mma_idesc(COUT);
        for (int src = 0; src < nsrc; src++) {
            const int lg = src ? lg1 : lg0, ksteps = 1 << (lg - 1);
            const int pl = src ? g.plane1 : g.plane0;
            const uint32_t pbase = smem_u32(src ? planes1 : smem);
            const uint32_t wbase = smem_u32(smem + (src ? g.w1_off : g.w0_off));
            const uint64_t pstep = (uint64_t)(pl >> 4);
            for (int tap = 0; tap < 27; tap++) {
                const int dx = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dz = tap % 3 - 1;
                const uint32_t off = (uint32_t)(((dy + 1) * kHaloZ + dz + 1) * 16);
                // descriptors of (xi = 0, kk = 0); the start address field
                // (16-byte units) advances by one plane per xi and by two
                // chunks per kk
                const uint64_t a0 = ns_desc(pbase + (uint32_t)((dx + 1) * pl) + off, kHaloChunk, kHaloZ * 16);
                const uint64_t b0 = ns_desc(wbase + (uint32_t)(tap << lg) * (COUT * 16), COUT * 16, 128);
                const uint32_t acc = (tap > 0 || src > 0) ? 1u : 0u;
                uint64_t ax = a0;
                uint32_t d = tmem;
                for (int xi = 0; xi < g.xr; xi++, ax += pstep, d += COUT) {
#pragma unroll 1
                    for (int kk = 0; kk < ksteps; kk++) {
                        const uint64_t ad = ax + (uint64_t)(kk * (2 * kHaloChunk >> 4));
                        const uint64_t bd = b0 + (uint64_t)(kk * (2 * COUT * 16 >> 4));
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                            "l"(ad), "l"(bd), "r"(idesc), "r"(acc | (uint32_t)kk));
                    }
                }
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(done))
                     : "memory");
    }
    __syncwarp();
    // epilogue: row m of each accumulator is TMEM lane m, owned by warp m / 32
    const bool got = __all_sync(0xffffffffu, mbar_wait(smem_u32(done), 0) ? 1 : 0) != 0;
    if (!got) fail = 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int m = warp * 32 + lane;
    const int yy = y0 + (m >> 3), zz = z0 + (m & 7);
    if (got) {
        for (int xi = 0; xi < g.xr; xi++) {
            float acc[COUT];
#pragma unroll
            for (int c = 0; c < COUT; c += 16)
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(xi * COUT + c), acc + c);
            __align__(16) __nv_bfloat16 out[COUT];
#pragma unroll
            for (int c = 0; c < COUT; c++) {
                float v = acc[c] + (bias ? __ldg(bias + c) : 0.0f);
                if (g.relu) v = fmaxf(v, 0.0f);
                out[c] = __float2bfloat16_rn(v);
            }
            const int64_t vox = (((int64_t)b * g.NX + x0 + xi) * g.NY + yy) * g.NZ + zz;
            uint4 *dst = reinterpret_cast<uint4 *>(y + vox * COUT);
#pragma unroll
            for (int q = 0; q < COUT / 8; q++) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (fail && threadIdx.x == 0) atomicExch(&g_conv_error, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.tmem_cols));
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

// opt-in shared memory per block less an allowance for the kernel's static shared variables
constexpr int kHaloSmemMax = 227 * 1024 - 128;

static inline int align_up(int v, int a) { return (v + a - 1) / a * a; }

// Shared-memory layout of k_conv3d_halo for xr planes; returns the dynamic
// shared memory size (including the 1 KB alignment slack).
static size_t halo_layout(HaloGeom &h, int cout) {
    h.plane0 = (h.cin0 >> 3) * kHaloChunk;
    h.plane1 = (h.cin1 >> 3) * kHaloChunk;
    const int np = h.xr + 2;
    h.planes1_off = np * h.plane0;
    h.w0_off = h.planes1_off + np * h.plane1;
    h.w1_off = h.w0_off + 27 * cout * h.cin0 * 2;
    h.bar_off = align_up(h.w1_off + 27 * cout * h.cin1 * 2, 16);
    uint32_t cols = 32;
    while (cols < (uint32_t)(h.xr * cout)) cols <<= 1;
    h.tmem_cols = cols;
    return (size_t)h.bar_off + 16 /* mbarrier, TMEM slot */ + 1024;
}

static bool halo_enabled() {
    const char *e = getenv("FLUB_CONV_HALO");
    return !(e && e[0] == '0');
}

// FLUB_CONV_XR=n forces n planes per CTA (1, 2, 4 or 8) where it fits.
static int forced_xr() {
    const char *e = getenv("FLUB_CONV_XR");
    return e ? atoi(e) : 0;
}

// Chooses the planes per CTA for k_conv3d_halo: the largest xr in {8, 4, 2, 1}
// that divides NX, keeps the accumulators within 256 TMEM columns and the
// planes and weights within shared memory, and still gives at least three
// CTAs per SM (xr = 1 when none does).  Returns 0 when the layer goes to
// k_conv3d_tc instead: its weights do not fit beside three planes, or
// k_conv3d_tc takes its shape and it has two sources or fewer tiles than SMs.
// Both kernels run the same count of M = 128, N = Cout, K = 16 MMAs, which at
// N = 16 to 64 are bound by the SM reading their A operand (about 44 cycles
// for one 128 x 16 BF16 tile); the halo kernel saves the tap-shifted tile
// loads, and wins where its planes and weights leave room for several CTAs
// per SM.  For the two-source decoder layers they do not, and on grids of
// fewer tiles than SMs (16^3) its staging is not hidden: the tap-tile kernel
// measured faster in both cases.  FLUB_CONV_XR forces the halo kernel
// wherever it fits.
static size_t halo_plan(HaloGeom &h, int cout) {
    if (h.NZ % 8 || h.NY % 16 || !halo_enabled()) return 0;
    const int64_t tiles = (int64_t)h.B * (h.NY / 16) * (h.NZ / 8);
    const int fx = forced_xr();
    const int nzb = h.NZ < 128 ? h.NZ : 128;
    const bool tap_ok = 128 % nzb == 0 && h.NZ % nzb == 0 && h.NY % (128 / nzb) == 0;
    if (!fx && tap_ok && (h.cin1 > 0 || tiles * h.NX < kNumSMs)) return 0;
    for (int xr = 8; xr >= 1; xr >>= 1) {
        if (fx && xr != fx) continue;
        if (h.NX % xr || xr * cout > 256) continue;
        if (!fx && xr > 1 && tiles * (h.NX / xr) < 3 * kNumSMs) continue;
        h.xr = xr;
        const size_t smem = halo_layout(h, cout);
        if (smem <= (size_t)kHaloSmemMax) return smem;
    }
    return 0;
}

template <int COUT>
static int launch_halo(const void *x0, const void *w0, const void *x1, const void *w1, const HaloGeom &h, size_t smem,
                       const float *bias, __nv_bfloat16 *y, cudaStream_t s) {
    static size_t attr_smem = 0;  // largest dynamic shared memory enabled so far
    if (smem > attr_smem) {
        FLUB_CHECK_CUDA(
            cudaFuncSetAttribute(k_conv3d_halo<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_smem = smem;
    }
    const unsigned ctas = (unsigned)((int64_t)h.B * (h.NX / h.xr) * (h.NY / 16) * (h.NZ / 8));
    k_conv3d_halo<COUT><<<ctas, kConvThreads, smem, s>>>(
        static_cast<const __nv_bfloat16 *>(x0), static_cast<const __nv_bfloat16 *>(w0),
        static_cast<const __nv_bfloat16 *>(x1 ? x1 : x0), static_cast<const __nv_bfloat16 *>(w1 ? w1 : w0), h, bias,
        y);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

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
    int st = get_encode();
    if (st) return st;
    {
        HaloGeom h;
        memset(&h, 0, sizeof(h));
        h.B = B; h.NX = NX; h.NY = NY; h.NZ = NZ;
        h.cin0 = cin0;
        h.cin1 = x1 ? cin1 : 0;
        h.relu = relu ? 1 : 0;
        const size_t smem = halo_plan(h, cout);
        if (smem) {
            cudaStream_t s = as_stream(stream);
            __nv_bfloat16 *yo = static_cast<__nv_bfloat16 *>(y);
            switch (cout) {
            case 16: return launch_halo<16>(x0, w0, x1, w1, h, smem, bias, yo, s);
            case 32: return launch_halo<32>(x0, w0, x1, w1, h, smem, bias, yo, s);
            default: return launch_halo<64>(x0, w0, x1, w1, h, smem, bias, yo, s);
            }
        }
    }
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
