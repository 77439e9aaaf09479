// The coarse tail of the V-cycle in one thread block.
//
// Below a few thousand cells a level is pure launch latency: the reference
// schedule runs 6 << l red-black iterations per side at level l (384
// half-sweeps at 16^3 for a 256^3 grid).  This kernel keeps z, r and the cell
// codes of every tail level in shared memory and runs the whole sub-V-cycle
// (multigrid/mgpcg.py:296-349 from level lt down to the bottom and back) with
// __syncthreads between half-sweeps.  Arithmetic is the same as the global
// kernels, cell by cell, so the result is bit-identical.
#pragma once

#include <cuda_fp16.h>

#include "mg_kernels.cuh"

namespace flub {

constexpr int kTailThreads = 1024;
constexpr int kTailMaxLevels = 8;
constexpr int kTailMaxCells = 4096;  // the first tail level has at most this many cells

struct TailLevel {
    Dims D;
    const uint8_t *code;  // global cell codes of this level
    const uint32_t *pmask;  // the pairs' masks of tail_cache, built by set_tags (NULL: from the codes)
    int abs_level;        // level index in the full hierarchy (sets 6 << l)
    int off_z, off_r, off_c;  // byte offsets in shared memory
    int off_v;                // fine residual scratch for the restriction (-1 at the bottom level)
};

struct TailParams {
    int nt;
    TailLevel lv[kTailMaxLevels];
    const float *r_top;  // restricted residual of the first tail level (global)
    float *z_top;        // its correction (global)
    const __half *r_top_h;  // FP16 instead of r_top / z_top when not NULL (mixed precision)
    __half *z_top_h;
    int nu;        // red-black iterations per side at every level (< 0: 6 << level, the reference's)
    int nbottom;   // iterations of each of the two bottom orders (3 in the reference)
    float rscale;  // restriction scale (1 in the reference)
    // bottom64: the bottom level is smoothed in FP64 (z as doubles at byte
    // offset off_zd; r converted exactly from FP32), the result rounded to FP32
    // once for the prolongation.  No reference counterpart: the reference
    // smooths the bottom in FP32 (multigrid/mgpcg.py:319-336).
    int bottom64, off_zd;
};

// ---------------------------------------------------------------- lean smoothing
// Each thread owns up to kTailPairs pairs of k-adjacent cells (one of each
// colour) of the level being smoothed.  On entering a level it caches, per
// cell, its shared-memory index, a neighbour mask and its r, so the
// half-sweeps themselves are a handful of shared loads per update.
// mask bits: 0-5 neighbour (+i, -i, +j, -j, +k, -k) in the domain and not
// solid; 6-11 that neighbour is air; 12 the cell is fluid.
constexpr int kTailPairs = (kTailMaxCells / 2 + kTailThreads - 1) / kTailThreads;

struct TailCache {
    int idx[kTailPairs];      // index of the pair's even-k cell, -1 if unused
    uint32_t msk[kTailPairs]; // low 16 bits: even cell, high 16 bits: odd cell
    float r0[kTailPairs], r1[kTailPairs];
    int upd0;                 // bit q: in phase 0 the odd-k cell of pair q is updated
};

__device__ __forceinline__ uint32_t cell_mask(const uint8_t *code, const Dims D, int i, int j, int k, int c) {
    const int si = D.ny * D.nz, sj = D.nz;
    uint32_t m = 0;
    auto nb = [&](bool inside, int off, int bit) {
        const uint8_t cn = code[inside ? c + off : c];  // loaded either way: the loads issue together
        if (inside && cn != kCodeSolid) m |= 1u << bit;
        if (inside && cn == kCodeAir) m |= 1u << (bit + 6);
    };
    nb(i + 1 < D.nx, si, 0);
    nb(i > 0, -si, 1);
    nb(j + 1 < D.ny, sj, 2);
    nb(j > 0, -sj, 3);
    nb(k + 1 < D.nz, 1, 4);
    nb(k > 0, -1, 5);
    if (code[c] == kCodeFluid) m |= 1u << 12;
    return m;
}

// The masks of k-pair t (cells 2 kk and 2 kk + 1 of row (i, j)): even cell in
// the low 16 bits, odd cell in the high.
__device__ __forceinline__ uint32_t pair_mask(const uint8_t *code, const Dims D, int t) {
    const int hz = D.nz >> 1;
    const int kk = t % hz, qq = t / hz;
    const int j = qq % D.ny, i = qq / D.ny;
    const int c = (i * D.ny + j) * D.nz + 2 * kk;
    return cell_mask(code, D, i, j, 2 * kk, c) | (cell_mask(code, D, i, j, 2 * kk + 1, c + 1) << 16);
}

// set_tags: every pair's masks of a tail-sized level into pm (nz even).
__global__ void k_tail_masks(const uint8_t *__restrict__ code, Dims D, uint32_t *__restrict__ pm) {
    const int npairs = D.nx * D.ny * (D.nz >> 1);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npairs; t += gridDim.x * blockDim.x)
        pm[t] = pair_mask(code, D, t);
}

// pm: the masks from set_tags (one coalesced load per pair), else built from
// the codes.
__device__ __forceinline__ void tail_cache(TailCache &tc, const uint8_t *code, const float *r, const Dims D,
                                           const uint32_t *pm) {
    const int hz = D.nz >> 1, npairs = D.nx * D.ny * hz;
    tc.upd0 = 0;
#pragma unroll
    for (int q = 0; q < kTailPairs; q++) {
        const int t = threadIdx.x + q * kTailThreads;
        tc.idx[q] = -1;
        tc.msk[q] = 0;
        tc.r0[q] = tc.r1[q] = 0.0f;
        if (t < npairs) {
            const int kk = t % hz, qq = t / hz;
            const int j = qq % D.ny, i = qq / D.ny;
            const int c = (i * D.ny + j) * D.nz + 2 * kk;
            tc.idx[q] = c;
            tc.msk[q] = pm ? __ldg(pm + t) : pair_mask(code, D, t);
            tc.r0[q] = r[c];
            tc.r1[q] = r[c + 1];
            // phase 0 updates (i+j+k) odd cells: the odd-k cell iff i+j is even
            if (((i + j) & 1) == 0) tc.upd0 |= 1 << q;
        }
    }
}

// Neighbour sum of L z at a fluid cell from its mask, in the operation order
// of lap_at.  All six neighbours are loaded whether they count or not (an
// excluded one reads the cell itself), so the loads issue together instead of
// one after another behind each mask test: a dependent chain of shared loads
// was most of a half-sweep's time.
__device__ __forceinline__ float tail_lap(const float *z, int c, uint32_t m, int si, int sj) {
    const float xc = z[c];
    const float zip = z[(m & 1u) ? c + si : c], zim = z[(m & 2u) ? c - si : c];
    const float zjp = z[(m & 4u) ? c + sj : c], zjm = z[(m & 8u) ? c - sj : c];
    const float zkp = z[(m & 16u) ? c + 1 : c], zkm = z[(m & 32u) ? c - 1 : c];
    float tp, tm, ret = 0.0f;
    tp = (m & 1u) ? __fsub_rn((m & 64u) ? 0.0f : zip, xc) : 0.0f;
    tm = (m & 2u) ? __fsub_rn((m & 128u) ? 0.0f : zim, xc) : 0.0f;
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    tp = (m & 4u) ? __fsub_rn((m & 256u) ? 0.0f : zjp, xc) : 0.0f;
    tm = (m & 8u) ? __fsub_rn((m & 512u) ? 0.0f : zjm, xc) : 0.0f;
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    tp = (m & 16u) ? __fsub_rn((m & 1024u) ? 0.0f : zkp, xc) : 0.0f;
    tm = (m & 32u) ? __fsub_rn((m & 2048u) ? 0.0f : zkm, xc) : 0.0f;
    return __fadd_rn(ret, __fadd_rn(tp, tm));
}

// z update of one cell with the mask m (same operation order as lap_at).
__device__ __forceinline__ float tail_update(const float *z, int c, uint32_t m, float rc, int si, int sj,
                                             bool from_zero) {
    if (!(m & (1u << 12))) return 0.0f;
    const int d = __popc(m & 63u);
    if (d == 0) return 0.0f;
    if (from_zero) return __fdiv_rn(rc, (float)d);
    return __fadd_rn(z[c], __fdiv_rn(__fadd_rn(rc, tail_lap(z, c, m, si, sj)), (float)d));
}

// Threads that own a pair of the level: whole warps, all of them from 16^3
// up (2048 pairs), the first 8 warps at 8^3.
__device__ __forceinline__ int tail_threads(const Dims D) {
    const int npairs = D.nx * D.ny * (D.nz >> 1);
    const int w = (npairs + 31) & ~31;
    return w < kTailThreads ? w : kTailThreads;
}

// Barrier among the first nthr threads: the block barrier when all take part,
// else named barrier 1 (the threads above nthr own no cells of the level and
// wait at the next block barrier instead).
__device__ __forceinline__ void tail_sync(int nthr) {
    if (nthr >= kTailThreads)
        __syncthreads();
    else
        asm volatile("bar.sync 1, %0;" ::"r"(nthr) : "memory");
}

__device__ __forceinline__ void tail_half_lean(float *z, const TailCache &tc, const Dims D, int phase,
                                               bool from_zero, int nthr) {
    const int si = D.ny * D.nz, sj = D.nz;
#pragma unroll
    for (int q = 0; q < kTailPairs; q++) {
        const int c = tc.idx[q];
        if (c < 0) continue;
        const bool odd = (((tc.upd0 >> q) & 1) != 0) == (phase == 0);
        const uint32_t m = odd ? (tc.msk[q] >> 16) : (tc.msk[q] & 0xffffu);
        const int cu = c + (odd ? 1 : 0);
        const float zn = tail_update(z, cu, m, odd ? tc.r1[q] : tc.r0[q], si, sj, from_zero);
        z[cu] = zn;
        if (from_zero) z[odd ? c : c + 1] = 0.0f;
    }
    tail_sync(nthr);
}


// Restriction of the residual r + L z (multigrid/mgpcg.py:306-318): first
// every fine cell's r + L z (r alone off the fluid) into the scratch v, each
// thread for the pairs it caches, then each coarse fluid cell sums its 8
// children in (i, j, k) order and scales; coarse cells that are not fluid get
// 0.  Same values, bit for bit, as summing r + lap_at per child.
__device__ __forceinline__ void tail_restrict_cached(float *v, const float *zf, const TailCache &tc, const Dims F,
                                                     float *rc, const uint8_t *cc, const Dims C, float rscale) {
    const int si = F.ny * F.nz, sj = F.nz;
#pragma unroll
    for (int q = 0; q < kTailPairs; q++) {
        const int c = tc.idx[q];
        if (c < 0) continue;
        const uint32_t m0 = tc.msk[q] & 0xffffu, m1 = tc.msk[q] >> 16;
        v[c] = __fadd_rn(tc.r0[q], (m0 & (1u << 12)) ? tail_lap(zf, c, m0, si, sj) : 0.0f);
        v[c + 1] = __fadd_rn(tc.r1[q], (m1 & (1u << 12)) ? tail_lap(zf, c + 1, m1, si, sj) : 0.0f);
    }
    __syncthreads();
    const int n = C.nx * C.ny * C.nz;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        if (cc[q] != kCodeFluid) {
            rc[q] = 0.0f;
            continue;
        }
        const int K = q % C.nz, J = (q / C.nz) % C.ny, I = q / (C.nz * C.ny);
        const int c0 = ((2 * I) * F.ny + 2 * J) * F.nz + 2 * K;
        float s = v[c0];
        s = __fadd_rn(s, v[c0 + 1]);
        s = __fadd_rn(s, v[c0 + sj]);
        s = __fadd_rn(s, v[c0 + sj + 1]);
        s = __fadd_rn(s, v[c0 + si]);
        s = __fadd_rn(s, v[c0 + si + 1]);
        s = __fadd_rn(s, v[c0 + si + sj]);
        s = __fadd_rn(s, v[c0 + si + sj + 1]);
        rc[q] = __fmul_rn(s, rscale);
    }
    __syncthreads();
}

__device__ __forceinline__ void tail_prolong(float *zf, const float *zc, const Dims F) {
    const int n = F.nx * F.ny * F.nz;
    const int cy = F.ny >> 1, cz = F.nz >> 1;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const int k = c % F.nz, j = (c / F.nz) % F.ny, i = c / (F.nz * F.ny);
        zf[c] = __fadd_rn(zf[c], zc[((i >> 1) * cy + (j >> 1)) * cz + (k >> 1)]);
    }
    __syncthreads();
}

// ---------------------------------------------------------------- FP64 bottom
// No reference counterpart (the reference smooths its bottom level in FP32).
// The red-black Gauss-Seidel update of the other levels, z_c + (r + L z) / d
// with L z the sum over non-solid neighbours of (z_n - z_c), z_n = 0 for air,
// is in exact arithmetic (r + sum of the fluid neighbours' z) / d: the z_c
// terms cancel.  The bottom uses that form, which takes 6 FP64 additions and
// the division where the other takes 14 operations (this GPU issues FP64 at a
// small fraction of its FP32 rate, and the bottom runs on one SM): neighbours
// summed in the order i+, i-, j+, j-, k+, k- onto r, each non-fluid one adding
// +0.0, IEEE double rounding at each operation.  The oracle's FP64 bottom
// (oracle_bottom_half64) is the same sequence.

// a / d for d = 1..6, rounded to nearest as __ddiv_rn(a, d), by Markstein's
// FMA correction of a * RN(1/d) (P. Markstein, IBM J. Res. Dev. 34(1), 1990):
// two FMAs and a product instead of an FP64 division, which GB300 issues
// slowly.  tests/test_div6_exhaustive.py checks it bit for bit against IEEE
// division on 2^28 random doubles per d with |a| in [2^-900, 2^900] and on the
// zeros (which return a * RN(1/d), a zero of a's sign); other inputs take
// __ddiv_rn.
__device__ __forceinline__ double ddiv_small_rn(double a, int d) {
    const double y = d == 1 ? 1.0 : d == 2 ? 0.5 : d == 3 ? 1.0 / 3.0 : d == 4 ? 0.25 : d == 5 ? 0.2 : 1.0 / 6.0;
    const double m = fabs(a);
    const double q0 = __dmul_rn(a, y);
    if (m >= 0x1p-900 && m <= 0x1p900) return __fma_rn(__fma_rn(-q0, (double)d, a), y, q0);
    if (m == 0.0) return q0;
    return __ddiv_rn(a, (double)d);
}

// r + the fluid neighbours' z of cell c (mask m as in TailCache), in the
// order above.  All six neighbours are loaded (an excluded one reads the cell
// itself) so the loads issue together.
__device__ __forceinline__ double tail_gs_sum64(const double *z, int c, uint32_t m, double rc, int si, int sj) {
    const double zip = z[(m & 1u) ? c + si : c], zim = z[(m & 2u) ? c - si : c];
    const double zjp = z[(m & 4u) ? c + sj : c], zjm = z[(m & 8u) ? c - sj : c];
    const double zkp = z[(m & 16u) ? c + 1 : c], zkm = z[(m & 32u) ? c - 1 : c];
    // neighbour q is fluid: in the domain and not solid (bit q), not air (bit q + 6)
    const uint32_t fl = (m & 63u) & ~((m >> 6) & 63u);
    double s = rc;
    s = __dadd_rn(s, (fl & 1u) ? zip : 0.0);
    s = __dadd_rn(s, (fl & 2u) ? zim : 0.0);
    s = __dadd_rn(s, (fl & 4u) ? zjp : 0.0);
    s = __dadd_rn(s, (fl & 8u) ? zjm : 0.0);
    s = __dadd_rn(s, (fl & 16u) ? zkp : 0.0);
    return __dadd_rn(s, (fl & 32u) ? zkm : 0.0);
}

__device__ __forceinline__ void tail_half64(double *z, const TailCache &tc, const Dims D, int phase, int nthr) {
    const int si = D.ny * D.nz, sj = D.nz;
#pragma unroll
    for (int q = 0; q < kTailPairs; q++) {
        const int c = tc.idx[q];
        if (c < 0) continue;
        const bool odd = (((tc.upd0 >> q) & 1) != 0) == (phase == 0);
        const uint32_t m = odd ? (tc.msk[q] >> 16) : (tc.msk[q] & 0xffffu);
        const int cu = c + (odd ? 1 : 0);
        const double rc = (double)(odd ? tc.r1[q] : tc.r0[q]);
        double zn = 0.0;
        const int d = __popc(m & 63u);
        if ((m & (1u << 12)) && d != 0) zn = ddiv_small_rn(tail_gs_sum64(z, cu, m, rc, si, sj), d);
        z[cu] = zn;
    }
    tail_sync(nthr);
}

// The bottom's 2 x nbottom red-black iterations in FP64, starting from z = 0,
// then z rounded to FP32 into zf.  Not inlined: its FP64 registers would
// otherwise count against the whole tail / cluster kernel.
__device__ __noinline__ void tail_bottom64(double *zd, float *zf, const TailCache &tc, const Dims D, int nbottom) {
    const int n = D.nx * D.ny * D.nz;
    for (int q = threadIdx.x; q < n; q += blockDim.x) zd[q] = 0.0;
    __syncthreads();
    const int nthr = tail_threads(D);
    if ((int)threadIdx.x < nthr) {
        for (int it = 0; it < nbottom; it++) {
            tail_half64(zd, tc, D, 0, nthr);
            tail_half64(zd, tc, D, 1, nthr);
        }
        for (int it = 0; it < nbottom; it++) {
            tail_half64(zd, tc, D, 1, nthr);
            tail_half64(zd, tc, D, 0, nthr);
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < n; q += blockDim.x) zf[q] = __double2float_rn(zd[q]);
    __syncthreads();
}

// The tail sub-V-cycle on one block with the layout P in the shared memory at
// smem.  io: the first level's r comes from P.r_top / P.r_top_h and its z goes
// back to P.z_top / P.z_top_h; otherwise both stay in shared memory (the
// cluster kernel writes r there and reads z back through distributed shared
// memory).
__device__ __forceinline__ void tail_run(const TailParams &P, unsigned char *smem, bool io) {
    auto Z = [&](int t) { return reinterpret_cast<float *>(smem + P.lv[t].off_z); };
    auto R = [&](int t) { return reinterpret_cast<float *>(smem + P.lv[t].off_r); };
    auto C = [&](int t) { return reinterpret_cast<uint8_t *>(smem + P.lv[t].off_c); };
    auto V = [&](int t) { return reinterpret_cast<float *>(smem + P.lv[t].off_v); };
    // the sweeps of a level on the threads that own its pairs; the others
    // meet them at the block barrier after the loop
    auto sweeps = [&](int t, const TailCache &tc, int iters, bool down) {
        const Dims D = P.lv[t].D;
        const int nthr = tail_threads(D);
        if ((int)threadIdx.x < nthr)
            for (int it = 0; it < iters; it++) {
                tail_half_lean(Z(t), tc, D, down ? 0 : 1, down && it == 0, nthr);
                tail_half_lean(Z(t), tc, D, down ? 1 : 0, false, nthr);
            }
        if (nthr < kTailThreads) __syncthreads();
    };
    for (int t = 0; t < P.nt; t++) {
        const int n = P.lv[t].D.nx * P.lv[t].D.ny * P.lv[t].D.nz;
        uint8_t *c = C(t);
        for (int q = threadIdx.x; q < n; q += blockDim.x) c[q] = P.lv[t].code[q];
    }
    if (io) {
        const Dims D = P.lv[0].D;
        const int n = D.nx * D.ny * D.nz;
        float *r = R(0);
        if (P.r_top_h)
            for (int q = threadIdx.x; q < n; q += blockDim.x) r[q] = __half2float(P.r_top_h[q]);
        else
            for (int q = threadIdx.x; q < n; q += blockDim.x) r[q] = P.r_top[q];
    }
    __syncthreads();
    const int nb = P.nt - 1;
    TailCache tc;
    for (int t = 0; t < nb; t++) {
        const Dims D = P.lv[t].D;
        tail_cache(tc, C(t), R(t), D, P.lv[t].pmask);
        sweeps(t, tc, P.nu < 0 ? (6 << P.lv[t].abs_level) : P.nu, true);
        tail_restrict_cached(V(t), Z(t), tc, D, R(t + 1), C(t + 1), P.lv[t + 1].D, P.rscale);
    }
    tail_cache(tc, C(nb), R(nb), P.lv[nb].D, P.lv[nb].pmask);
    if (P.bottom64) {
        tail_bottom64(reinterpret_cast<double *>(smem + P.off_zd), Z(nb), tc, P.lv[nb].D, P.nbottom);
    } else {
        sweeps(nb, tc, P.nbottom, true);
        sweeps(nb, tc, P.nbottom, false);
    }
    for (int t = nb - 1; t >= 0; t--) {
        const Dims D = P.lv[t].D;
        tail_prolong(Z(t), Z(t + 1), D);
        tail_cache(tc, C(t), R(t), D, P.lv[t].pmask);
        sweeps(t, tc, P.nu < 0 ? (6 << P.lv[t].abs_level) : P.nu, false);
    }
    if (io) {
        const Dims D = P.lv[0].D;
        const int n = D.nx * D.ny * D.nz;
        const float *z = Z(0);
        if (P.z_top_h)
            for (int q = threadIdx.x; q < n; q += blockDim.x) P.z_top_h[q] = __float2half_rn(z[q]);
        else
            for (int q = threadIdx.x; q < n; q += blockDim.x) P.z_top[q] = z[q];
    }
}

__global__ void __launch_bounds__(kTailThreads) k_tail_vcycle(const TailParams P, unsigned long long *kc) {
    extern __shared__ __align__(16) unsigned char tail_smem[];
    count_kernel(kc);
    tail_run(P, tail_smem, true);
}

}  // namespace flub
