// The coarse part of the V-cycle (from a level of at most 32^3 cells down to
// the bottom) in ONE thread-block cluster.
//
// Below ~32^3 cells a red-black half-sweep is a few microseconds of launch
// latency for a fraction of a microsecond of work, and the reference schedule
// runs 6 << l iterations per side at level l.  Here a cluster of C blocks (16
// where the GPU allows it) keeps every coarse level in distributed shared
// memory: level l is split into slabs of P_l = nx_l / C_l consecutive i-planes
// over C_l = min(C, nx_l / 2) blocks.  Each slab carries one ghost plane on
// either side; a block that updates a cell on its first or last plane also
// stores the new value into the neighbour block's ghost plane (DSMEM), so one
// cluster barrier per half-sweep keeps every ghost plane current.  Restriction
// writes the coarse residual straight into the owning block's shared memory,
// prolongation reads the coarse correction from it.
//
// Same operations in the same order as the global kernels (mgpcg.py:72-116),
// so results are bit-identical.  All blocks run the same sequence of cluster
// barriers (uniform control flow); blocks that own no slab of a level simply
// wait at them.
#pragma once

#include <cooperative_groups.h>
#include <cuda_fp16.h>

#include "mg_kernels.cuh"
#include "restrict8.cuh"
#include "smooth8.cuh"
#include "tail.cuh"

namespace flub {

namespace cg = cooperative_groups;

constexpr int kClusterThreads = 1024;
constexpr int kClusterMaxLevels = 8;

struct ClusterLevel {
    Dims D;
    int abs_level;  // index in the full hierarchy (sets 6 << l)
    int ncta;       // blocks holding a slab of this level
    int P;          // i-planes per slab
    int lg_ny, lg_nz;
    const uint8_t *code;  // global cell codes of the level
    int off_z, off_c, off_r;  // shared-memory byte offsets
};

// The level just above the distributed ones, run by the same cluster in
// global memory (where it stays resident in L2) over its active list: its
// pre-smoothing and restriction before the distributed levels, its
// prolongation and post-smoothing after them, one cluster barrier between
// passes instead of one kernel launch per pass.  The passes are k_smooth8's
// and k_restrict8's (smooth8.cuh, restrict8.cuh) with L2-only loads of what
// other blocks of the cluster wrote.
struct ClusterGlobal {
    int on, half;  // half: FP16 level storage (mixed precision)
    Dims D;
    const uint8_t *code;
    const uint16_t *sw;
    const int *act, *act_n;
    void *r, *z, *z2;  // the level's residual and corrections (float or __half)
    int iters;         // red-black iterations per side
    float rscale;      // restriction output scale
    float zc_scale;    // prolongation input scale
    // the first distributed level (restriction target, prolongation source)
    Dims CD;
    const uint8_t *ccode;
    const int *cact, *cact_n;
    void *cr;
    const void *cz;
};

struct ClusterParams {
    ClusterGlobal g;
    int nl;
    ClusterLevel lv[kClusterMaxLevels];
    const float *r_top;  // residual of the first cluster level (global)
    float *z_top;        // its final correction (global)
    const __half *r_top_h;  // FP16 instead of r_top / z_top when not NULL (mixed precision)
    __half *z_top_h;
    int nu;        // red-black iterations per side at every level (< 0: 6 << level, the reference's)
    int nbottom;   // iterations of each of the two bottom orders (3 in the reference)
    float rscale;  // restriction scale (1 in the reference)
    // Levels below the distributed ones (at most kTailMaxCells cells) run in
    // block 0 alone, with block barriers: tail != 0, tp their layout at byte
    // offset tail_off of block 0's shared memory.
    int tail, tail_off;
    TailParams tp;
};

struct ClusterCtx {
    cg::cluster_group cl;
    unsigned rank;
    unsigned char *smem;
};

__device__ __forceinline__ float *cl_z(const ClusterCtx &x, const ClusterLevel &L) {
    return reinterpret_cast<float *>(x.smem + L.off_z);
}
__device__ __forceinline__ uint8_t *cl_c(const ClusterCtx &x, const ClusterLevel &L) {
    return reinterpret_cast<uint8_t *>(x.smem + L.off_c);
}
__device__ __forceinline__ float *cl_r(const ClusterCtx &x, const ClusterLevel &L) {
    return reinterpret_cast<float *>(x.smem + L.off_r);
}

// The codes and z of a cell's six neighbours from shared memory (zs/cs in
// the ghost-padded layout: plane 0 and P+1 are ghosts; c is the cell's index
// there).  Everything is loaded before anything is tested (a neighbour past
// the j or k edge reads the cell itself and counts as solid), so the loads
// issue together instead of one after another behind each test.
struct ClNb {
    uint8_t cc, cip, cim, cjp, cjm, ckp, ckm;
    float xc, zip, zim, zjp, zjm, zkp, zkm;
};

__device__ __forceinline__ ClNb cl_nb(const float *zs, const uint8_t *cs, int c, int j, int k, const Dims D) {
    const int sj = D.nz, si = D.ny * D.nz;
    const bool jp = j + 1 < D.ny, jm = j > 0, kp = k + 1 < D.nz, km = k > 0;
    const int ijp = jp ? c + sj : c, ijm = jm ? c - sj : c, ikp = kp ? c + 1 : c, ikm = km ? c - 1 : c;
    ClNb n;
    n.cc = cs[c];
    n.cip = cs[c + si];
    n.cim = cs[c - si];
    const uint8_t cjp = cs[ijp], cjm = cs[ijm], ckp = cs[ikp], ckm = cs[ikm];
    n.xc = zs[c];
    n.zip = zs[c + si];
    n.zim = zs[c - si];
    n.zjp = zs[ijp];
    n.zjm = zs[ijm];
    n.zkp = zs[ikp];
    n.zkm = zs[ikm];
    n.cjp = jp ? cjp : kCodeSolid;
    n.cjm = jm ? cjm : kCodeSolid;
    n.ckp = kp ? ckp : kCodeSolid;
    n.ckm = km ? ckm : kCodeSolid;
    return n;
}

// Neighbour sum of L z at a fluid cell (lap_at's operation order).
__device__ __forceinline__ float cl_nb_sum(const ClNb &n) {
    float ret = 0.0f;
    ret = __fadd_rn(ret, __fadd_rn(nb_term(n.cip, n.cip == kCodeFluid ? n.zip : 0.0f, n.xc),
                                   nb_term(n.cim, n.cim == kCodeFluid ? n.zim : 0.0f, n.xc)));
    ret = __fadd_rn(ret, __fadd_rn(nb_term(n.cjp, n.cjp == kCodeFluid ? n.zjp : 0.0f, n.xc),
                                   nb_term(n.cjm, n.cjm == kCodeFluid ? n.zjm : 0.0f, n.xc)));
    ret = __fadd_rn(ret, __fadd_rn(nb_term(n.ckp, n.ckp == kCodeFluid ? n.zkp : 0.0f, n.xc),
                                   nb_term(n.ckm, n.ckm == kCodeFluid ? n.zkm : 0.0f, n.xc)));
    return ret;
}

// Update of one cell from shared memory.
__device__ __forceinline__ float cl_update(const float *zs, const uint8_t *cs, int c, int j, int k, const Dims D,
                                           float rc, bool from_zero) {
    const ClNb n = cl_nb(zs, cs, c, j, k, D);
    if (n.cc != kCodeFluid) return 0.0f;
    const int d = (n.cip != kCodeSolid) + (n.cim != kCodeSolid) + (n.cjp != kCodeSolid) + (n.cjm != kCodeSolid) +
                  (n.ckp != kCodeSolid) + (n.ckm != kCodeSolid);
    if (d == 0) return 0.0f;
    if (from_zero) return __fdiv_rn(rc, (float)d);
    return __fadd_rn(n.xc, __fdiv_rn(__fadd_rn(rc, cl_nb_sum(n)), (float)d));
}

// r of an owned cell (the first level's r is copied from global memory at start).
__device__ __forceinline__ float cl_rval(const ClusterCtx &x, const ClusterLevel &L, const ClusterParams &P, int il,
                                         int j, int k) {
    return cl_r(x, L)[((il << L.lg_ny) + j) * L.D.nz + k];
}

// Store v into cell (il, j, k) of this block and, for a cell on the first or
// last plane of the slab, into the matching ghost plane of the neighbour.
__device__ __forceinline__ void cl_store(const ClusterCtx &x, const ClusterLevel &L, float *zs, int il, int j, int k,
                                         float v) {
    const int plane = L.D.ny * L.D.nz;
    const int off = (j << L.lg_nz) + k;
    zs[(il + 1) * plane + off] = v;
    if (il == 0 && x.rank > 0) {
        float *zn = x.cl.map_shared_rank(zs, x.rank - 1);
        zn[(L.P + 1) * plane + off] = v;
    }
    if (il == L.P - 1 && x.rank + 1 < (unsigned)L.ncta) {
        float *zn = x.cl.map_shared_rank(zs, x.rank + 1);
        zn[off] = v;
    }
}

// L z at an owned cell (0 off the fluid), for the restriction.
__device__ __forceinline__ float cl_lap(const float *zs, const uint8_t *cs, int c, int j, int k, const Dims D) {
    const ClNb n = cl_nb(zs, cs, c, j, k, D);
    return n.cc != kCodeFluid ? 0.0f : cl_nb_sum(n);
}

// One red-black half-sweep of level t (mgpcg.py:72-86), then a cluster barrier.
__device__ __forceinline__ void cl_half(const ClusterCtx &x, const ClusterParams &P, int t, int phase,
                                        bool from_zero) {
    const ClusterLevel &L = P.lv[t];
    if (x.rank < (unsigned)L.ncta) {
        float *zs = cl_z(x, L);
        const uint8_t *cs = cl_c(x, L);
        const int lg_hz = L.lg_nz - 1;
        const int npairs = L.P << (L.lg_ny + lg_hz);
        const int par = 1 - phase;
        for (int q = threadIdx.x; q < npairs; q += blockDim.x) {
            const int kk = q & ((1 << lg_hz) - 1);
            const int j = (q >> lg_hz) & (L.D.ny - 1);
            const int il = q >> (lg_hz + L.lg_ny);
            const int b = (par + (int)x.rank * L.P + il + j) & 1;
            const int k = 2 * kk + b;
            const int c = ((il + 1) << (L.lg_ny + L.lg_nz)) + (j << L.lg_nz) + k;
            const float v = cl_update(zs, cs, c, j, k, L.D, cl_rval(x, L, P, il, j, k), from_zero);
            cl_store(x, L, zs, il, j, k, v);
            if (from_zero) cl_store(x, L, zs, il, j, b ? k - 1 : k + 1, 0.0f);
        }
    }
    x.cl.sync();
}

// Residual + restriction of level t into level t+1 (mgpcg.py:94-101 as a
// gather, children summed in (ii, jj, kk) order), written into the shared
// memory of the block that owns the coarse plane; then a cluster barrier.
__device__ __forceinline__ void cl_restrict(const ClusterCtx &x, const ClusterParams &P, int t) {
    const ClusterLevel &F = P.lv[t], &C = P.lv[t + 1];
    if (x.rank < (unsigned)F.ncta) {
        const float *zs = cl_z(x, F);
        const uint8_t *cs = cl_c(x, F);
        const int cpl = F.P >> 1;
        const int n = cpl << (C.lg_ny + C.lg_nz);
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int K = q & (C.D.nz - 1), J = (q >> C.lg_nz) & (C.D.ny - 1), Il = q >> (C.lg_ny + C.lg_nz);
            const int gI = (int)x.rank * cpl + Il;
            const int owner = gI / C.P, lcp = gI - owner * C.P;
            float s = 0.0f;
            if (__ldg(C.code + (gI << (C.lg_ny + C.lg_nz)) + (J << C.lg_nz) + K) == kCodeFluid) {
                bool first = true;
#pragma unroll
                for (int ii = 0; ii < 2; ii++)
#pragma unroll
                    for (int jj = 0; jj < 2; jj++)
#pragma unroll
                        for (int kk = 0; kk < 2; kk++) {
                            const int il = 2 * Il + ii, j = 2 * J + jj, k = 2 * K + kk;
                            const int c = ((il + 1) << (F.lg_ny + F.lg_nz)) + (j << F.lg_nz) + k;
                            const float v = __fadd_rn(cl_rval(x, F, P, il, j, k), cl_lap(zs, cs, c, j, k, F.D));
                            s = first ? v : __fadd_rn(s, v);
                            first = false;
                        }
            }
            float *rdst = x.cl.map_shared_rank(cl_r(x, C), (unsigned)owner);
            rdst[(lcp << (C.lg_ny + C.lg_nz)) + (J << C.lg_nz) + K] = __fmul_rn(s, P.rscale);
        }
    }
    x.cl.sync();
}

// cl_restrict from the last distributed level t into the first tail level,
// whose dense r array lives in block 0's shared memory.
__device__ __forceinline__ void cl_restrict_tail(const ClusterCtx &x, const ClusterParams &P, int t) {
    const ClusterLevel &F = P.lv[t];
    const TailLevel &T = P.tp.lv[0];
    const int lg_cy = F.lg_ny - 1, lg_cz = F.lg_nz - 1;
    if (x.rank < (unsigned)F.ncta) {
        const float *zs = cl_z(x, F);
        const uint8_t *cs = cl_c(x, F);
        float *rdst = x.cl.map_shared_rank(reinterpret_cast<float *>(x.smem + P.tail_off + T.off_r), 0u);
        const int cpl = F.P >> 1;
        const int n = cpl << (lg_cy + lg_cz);
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int K = q & (T.D.nz - 1), J = (q >> lg_cz) & (T.D.ny - 1), Il = q >> (lg_cy + lg_cz);
            const int gI = (int)x.rank * cpl + Il;
            const int cq = (gI << (lg_cy + lg_cz)) + (J << lg_cz) + K;
            float s = 0.0f;
            if (__ldg(T.code + cq) == kCodeFluid) {
                bool first = true;
#pragma unroll
                for (int ii = 0; ii < 2; ii++)
#pragma unroll
                    for (int jj = 0; jj < 2; jj++)
#pragma unroll
                        for (int kk = 0; kk < 2; kk++) {
                            const int il = 2 * Il + ii, j = 2 * J + jj, k = 2 * K + kk;
                            const int c = ((il + 1) << (F.lg_ny + F.lg_nz)) + (j << F.lg_nz) + k;
                            const float v = __fadd_rn(cl_rval(x, F, P, il, j, k), cl_lap(zs, cs, c, j, k, F.D));
                            s = first ? v : __fadd_rn(s, v);
                            first = false;
                        }
            }
            rdst[cq] = __fmul_rn(s, P.rscale);
        }
    }
    x.cl.sync();
}

// cl_prolong into the last distributed level t from the first tail level's
// dense z array in block 0's shared memory.
__device__ __forceinline__ void cl_prolong_tail(const ClusterCtx &x, const ClusterParams &P, int t) {
    const ClusterLevel &F = P.lv[t];
    const TailLevel &T = P.tp.lv[0];
    const int lg_cy = F.lg_ny - 1, lg_cz = F.lg_nz - 1;
    if (x.rank < (unsigned)F.ncta) {
        float *zs = cl_z(x, F);
        const float *zc = x.cl.map_shared_rank(reinterpret_cast<float *>(x.smem + P.tail_off + T.off_z), 0u);
        const int n = F.P << (F.lg_ny + F.lg_nz);
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int k = q & (F.D.nz - 1), j = (q >> F.lg_nz) & (F.D.ny - 1), il = q >> (F.lg_ny + F.lg_nz);
            const int gI = ((int)x.rank * F.P + il) >> 1;
            const float add = zc[(gI << (lg_cy + lg_cz)) + ((j >> 1) << lg_cz) + (k >> 1)];
            const int c = ((il + 1) << (F.lg_ny + F.lg_nz)) + (j << F.lg_nz) + k;
            cl_store(x, F, zs, il, j, k, __fadd_rn(zs[c], add));
        }
    }
    x.cl.sync();
}

// z_t += z_{t+1}[I/2] (mgpcg.py:113-116), ghost planes included; then a barrier.
__device__ __forceinline__ void cl_prolong(const ClusterCtx &x, const ClusterParams &P, int t) {
    const ClusterLevel &F = P.lv[t], &C = P.lv[t + 1];
    if (x.rank < (unsigned)F.ncta) {
        float *zs = cl_z(x, F);
        const int n = F.P << (F.lg_ny + F.lg_nz);
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int k = q & (F.D.nz - 1), j = (q >> F.lg_nz) & (F.D.ny - 1), il = q >> (F.lg_ny + F.lg_nz);
            const int gI = ((int)x.rank * F.P + il) >> 1;
            const int owner = gI / C.P, lcp = gI - owner * C.P;
            const float *zc = x.cl.map_shared_rank(cl_z(x, C), (unsigned)owner);
            const float add = zc[((lcp + 1) << (C.lg_ny + C.lg_nz)) + ((j >> 1) << C.lg_nz) + (k >> 1)];
            const int c = ((il + 1) << (F.lg_ny + F.lg_nz)) + (j << F.lg_nz) + k;
            cl_store(x, F, zs, il, j, k, __fadd_rn(zs[c], add));
        }
    }
    x.cl.sync();
}

// Pre-smoothing of the global level, then its restriction into the first
// distributed level's global r (read back into shared memory afterwards).
template <typename T>
__device__ __noinline__ void cl_global_down(const ClusterCtx &x, const ClusterGlobal &G) {
    const int b = (int)x.rank, nb = (int)x.cl.num_blocks();
    const T *r = static_cast<const T *>(G.r);
    T *z2 = static_cast<T *>(G.z2);
    for (int it = 0; it < G.iters; it++) {
        if (it == 0)
            smooth8_pass<true, false, false, T, T, T, T>(z2, z2, nullptr, 1.0f, r, G.code, G.sw, G.D, 0, G.act,
                                                         G.act_n, b, nb);
        else
            smooth8_pass<false, false, false, T, T, T, T>(z2, z2, nullptr, 1.0f, r, G.code, G.sw, G.D, 0, G.act,
                                                          G.act_n, b, nb);
        x.cl.sync();
        smooth8_pass<false, false, false, T, T, T, T>(z2, z2, nullptr, 1.0f, r, G.code, G.sw, G.D, 1, G.act,
                                                      G.act_n, b, nb);
        x.cl.sync();
    }
    restrict8_pass<false, false>(r, (const T *)z2, G.code, G.sw, static_cast<T *>(G.cr), G.ccode, G.CD, G.rscale,
                                 G.cact, G.cact_n, b, nb);
    x.cl.sync();
}

// Prolongation of the first distributed level's z (written back to global
// memory) into the global level, fused with its first post-smoothing
// half-sweep, then the other half-sweeps.
template <typename T>
__device__ __noinline__ void cl_global_up(const ClusterCtx &x, const ClusterGlobal &G) {
    const int b = (int)x.rank, nb = (int)x.cl.num_blocks();
    const T *r = static_cast<const T *>(G.r);
    T *z = static_cast<T *>(G.z);
    for (int it = 0; it < G.iters; it++) {
        if (it == 0)
            smooth8_pass<false, true, false, T, T, T, T>(z, static_cast<const T *>(G.z2),
                                                         static_cast<const T *>(G.cz), G.zc_scale, r, G.code, G.sw,
                                                         G.D, 1, G.act, G.act_n, b, nb);
        else
            smooth8_pass<false, false, false, T, T, T, T>(z, z, nullptr, 1.0f, r, G.code, G.sw, G.D, 1, G.act,
                                                          G.act_n, b, nb);
        x.cl.sync();
        smooth8_pass<false, false, false, T, T, T, T>(z, z, nullptr, 1.0f, r, G.code, G.sw, G.D, 0, G.act,
                                                      G.act_n, b, nb);
        if (it + 1 < G.iters) x.cl.sync();
    }
}

// kGlobal: P.g holds the global level above the distributed ones (a separate
// instantiation, so that the kernel without it keeps its register budget).
template <bool kGlobal>
__global__ void __launch_bounds__(kClusterThreads, 1) k_cluster_vcycle(const ClusterParams P, unsigned long long *kc) {
    extern __shared__ __align__(16) unsigned char cluster_smem[];
    count_kernel(kc);
    ClusterCtx x{cg::this_cluster(), 0u, cluster_smem};
    x.rank = x.cl.block_rank();
    if (kGlobal) {
        if (P.g.half)
            cl_global_down<__half>(x, P.g);
        else
            cl_global_down<float>(x, P.g);
    }
    // cell codes of the owned planes and both ghost planes (0 outside the domain)
    for (int t = 0; t < P.nl; t++) {
        const ClusterLevel &L = P.lv[t];
        if (x.rank >= (unsigned)L.ncta) continue;
        uint8_t *cs = cl_c(x, L);
        float *zs = cl_z(x, L);
        const int lg_pl = L.lg_ny + L.lg_nz;
        const int n = (L.P + 2) << lg_pl;
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int gp = (int)x.rank * L.P - 1 + (q >> lg_pl);
            cs[q] = (gp >= 0 && gp < L.D.nx) ? __ldg(L.code + (gp << lg_pl) + (q & ((1 << lg_pl) - 1))) : kCodeSolid;
            zs[q] = 0.0f;
        }
    }
    {
        // the first level's residual comes from global memory once
        const ClusterLevel &L = P.lv[0];
        if (x.rank < (unsigned)L.ncta) {
            float *rs = cl_r(x, L);
            const int lg_pl = L.lg_ny + L.lg_nz;
            const int n = L.P << lg_pl;
            const int base = (int)x.rank * L.P << lg_pl;
            // L2-only loads: the global level's restriction above wrote r_top
            if (P.r_top_h)
                for (int q = threadIdx.x; q < n; q += blockDim.x) rs[q] = St<__half>::ld_cg(P.r_top_h + base + q);
            else
                for (int q = threadIdx.x; q < n; q += blockDim.x) rs[q] = __ldcg(P.r_top + base + q);
        }
    }
    x.cl.sync();
    if (P.tail) {
        // distributed levels 0 .. nl-1 down, the tail levels in block 0, then up
        const int nd = P.nl;
        for (int t = 0; t < nd; t++) {
            const int iters = P.nu < 0 ? (6 << P.lv[t].abs_level) : P.nu;
            for (int it = 0; it < iters; it++) {
                cl_half(x, P, t, 0, it == 0);
                cl_half(x, P, t, 1, false);
            }
            if (t + 1 < nd)
                cl_restrict(x, P, t);
            else
                cl_restrict_tail(x, P, t);
        }
        if (x.rank == 0) tail_run(P.tp, x.smem + P.tail_off, false);
        x.cl.sync();
        for (int t = nd - 1; t >= 0; t--) {
            if (t + 1 < nd)
                cl_prolong(x, P, t);
            else
                cl_prolong_tail(x, P, t);
            const int iters = P.nu < 0 ? (6 << P.lv[t].abs_level) : P.nu;
            for (int it = 0; it < iters; it++) {
                cl_half(x, P, t, 1, false);
                cl_half(x, P, t, 0, false);
            }
        }
    } else {
    const int nb = P.nl - 1;
    for (int t = 0; t < nb; t++) {
        const int iters = P.nu < 0 ? (6 << P.lv[t].abs_level) : P.nu;
        for (int it = 0; it < iters; it++) {
            cl_half(x, P, t, 0, it == 0);
            cl_half(x, P, t, 1, false);
        }
        cl_restrict(x, P, t);
    }
    for (int it = 0; it < P.nbottom; it++) {
        cl_half(x, P, nb, 0, it == 0);
        cl_half(x, P, nb, 1, false);
    }
    for (int it = 0; it < P.nbottom; it++) {
        cl_half(x, P, nb, 1, false);
        cl_half(x, P, nb, 0, false);
    }
    for (int t = nb - 1; t >= 0; t--) {
        cl_prolong(x, P, t);
        const int iters = P.nu < 0 ? (6 << P.lv[t].abs_level) : P.nu;
        for (int it = 0; it < iters; it++) {
            cl_half(x, P, t, 1, false);
            cl_half(x, P, t, 0, false);
        }
    }
    }
    const ClusterLevel &L = P.lv[0];
    if (x.rank < (unsigned)L.ncta) {
        const float *zs = cl_z(x, L);
        const int lg_pl = L.lg_ny + L.lg_nz;
        const int n = L.P << lg_pl;
        const int base = (int)x.rank * L.P << lg_pl;
        if (P.z_top_h)
            for (int q = threadIdx.x; q < n; q += blockDim.x) P.z_top_h[base + q] = __float2half_rn(zs[(1 << lg_pl) + q]);
        else
            for (int q = threadIdx.x; q < n; q += blockDim.x) P.z_top[base + q] = zs[(1 << lg_pl) + q];
    }
    if (kGlobal) {
        x.cl.sync();
        if (P.g.half)
            cl_global_up<__half>(x, P.g);
        else
            cl_global_up<float>(x, P.g);
    }
}

}  // namespace flub
