// MGPCG solver handle: level hierarchy, V-cycle schedule and the CG loop as a
// CUDA graph (multigrid/mgpcg.py:234-490).
//
// The whole solve is one graph:
//   prologue  [mean removal] rTr0/tol, z = M r, zTr, p = z,
//             first half of iteration 0: Ap = L p, alpha, r -= alpha Ap, rTr,
//             convergence test -> while-condition
//   while     second half of iteration m: z = M r, beta, x += alpha p,
//             p = z + beta p, it = m + 1;  first half of iteration m + 1
//   epilogue  x += alpha p if the last test converged
// which is the reference's loop (mgpcg.py:406-461) rotated so that the
// convergence test closes the loop body.  The host reads back the state once.
#include <cudaTypedefs.h>

#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "mg_kernels.cuh"
#include "cg8.cuh"
#include "cluster.cuh"
#include "mixed.cuh"
#include "persist.cuh"
#include "restrict8.cuh"
#include "smooth8.cuh"
#include "smooth_split.cuh"
#include "smooth_tile.cuh"
#include "tail.cuh"

namespace flub {

constexpr int kMaxLevels = 12;
constexpr size_t kTailMaxSmem = 200 * 1024;  // dynamic shared memory of the tail kernel

// Per level: cell codes, residual r, and two correction buffers.  Pre-smoothing
// and the restriction work on z2; the prolongation writes z2 + P z_coarse into
// z while it runs the first post-smoothing sweep, and post-smoothing finishes
// in place on z, which therefore holds the level's final correction (at level
// 0 the caller's z).
struct Level {
    Dims D;
    uint8_t *code;
    float *r;
    float *z;
    float *z2;
    // mixed precision: FP16 copies at scale 8^-l (level 0: rh is the FP16 copy
    // of the CG residual, zh is unused, z is the FP32 CG vector)
    __half *rh, *zh, *z2h;
    // active 8-cell groups (ascending) and their count on the device; NULL
    // when nz is not a multiple of 8 (the scalar kernels run there)
    int *act, *act_n;
    // stencil words (smooth8.cuh), same condition
    uint16_t *sw;
    // level 0 with nz % 8 == 0: the colour-split buffers of smooth_split.cuh --
    // stencil words, the residual (FP32 rs, or FP16 rsh in mixed precision) and
    // the post-smoothing correction zs; z2 / z2h hold the pre-smoothing
    // correction split the same way
    uint16_t *sws;
    float *rs, *zs;
    __half *rsh;
    // TMA-tiled smoothing (smooth_tile.cuh) on FP32 levels whose extents are
    // multiples of the tile: a third correction buffer for the ping-pong of
    // the out-of-place iterations, the tile flags, and the list of tiles that
    // hold fluid with its count on the device.  n_tiles == 0: not tiled.
    float *z3;
    unsigned char *tflags;
    int *tiles, *tiles_n;
    int n_tiles;
    // levels small enough for the one-block tail (tail.cuh), nz even: the
    // neighbour masks of each k-pair of cells the tail's sweeps use, built once
    // by set_tags (the tail otherwise rebuilds them from the codes at every
    // level entry of every V-cycle); NULL elsewhere
    uint32_t *pmask;
};

struct LaunchCtx {
    cudaStream_t s;
    unsigned long long *kc;  // device kernel counter when captured into a graph, else nullptr
    cudaGraphConditionalHandle h;
    int set_cond;
};

}  // namespace flub

struct flub_mg {
    int nx, ny, nz, levels, precision;
    int64_t n;
    void *ws;
    size_t ws_bytes;
    bool own_ws;
    int device;
    flub::Level lv[flub::kMaxLevels];
    float *x, *p, *Ap;
    float *r_old;  // mixed precision: the residual of the previous iteration (flexible CG)
    int *act_scratch;  // block counts for building the active lists
    flub::MgState *st;
    double *partials;
    double *hist;
    bool use_x0;
    cudaGraphExec_t graph[3];
    int graph_nodes[3];
    cudaStream_t cap_stream, cap_stream2;
    bool host_loop;
    bool skip_ok;   // internal z buffers keep z = 0 off the fluid (see k_smooth8)
    bool tile_ok;   // the TMA-tiled smoother runs where a level has tiles (FLUB_TILE=1)
    bool split_ok;  // level 0 smooths on colour-split storage (smooth_split.cuh); FLUB_NO_SPLIT=1 turns it off
    bool iter_toggle[flub::kMaxLevels];  // flub_mg_smooth_iteration: direction of the next tiled call
    bool r_masked;  // r is 0 off the fluid (mask_interior since the last init)
    int tail_start;  // first level run by the one-block tail kernel (== levels: none)
    size_t tail_smem;
    int persist_blocks;  // blocks of the persistent V-cycle legs (persist.cuh); 0: launch per pass
    int cl_start;    // first level run by the cluster kernel (== levels: none)
    int cl_size;     // blocks per cluster
    size_t cl_smem;
    // V-cycle schedule (flub_mg_set_schedule); the reference's: -1, 3, 1
    int sched_nu;        // red-black iterations per side at every level (< 0: 6 << level)
    int sched_bottom;    // bottom: this many (0, 1) iterations, then as many (1, 0)
    float sched_rscale;  // restriction scale
    bool bottom64;       // bottom level smoothed in FP64 (flub_mg_set_bottom_precision; mixed precision's default)
};

namespace flub {

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static inline void reference_schedule(flub_mg *mg) {
    mg->sched_nu = -1;
    mg->sched_bottom = 3;
    mg->sched_rscale = 1.0f;
}

// Red-black iterations per side at level l.
static inline int level_iters(const flub_mg *mg, int l) { return mg->sched_nu < 0 ? (6 << l) : mg->sched_nu; }

// Device address of the kernel counter inside the (device-resident) state.
static inline unsigned long long *kernel_counter(flub_mg *mg) {
    return reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(mg->st) + offsetof(MgState, kernels));
}

// Workspace carve-up; with base == nullptr only the size is computed.
static size_t carve(flub_mg *mg, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char * {
        char *p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    const int64_t n = mg->n;
    mg->st = (MgState *)take(sizeof(MgState));
    mg->partials = (double *)take(sizeof(double) * 2 * kMaxRedBlocks);
    mg->hist = (double *)take(sizeof(double) * kHistory);
    mg->x = (float *)take(sizeof(float) * n);
    mg->p = (float *)take(sizeof(float) * n);
    mg->Ap = (float *)take(sizeof(float) * n);
    for (int l = 0; l < mg->levels; l++) {
        Level &L = mg->lv[l];
        L.D = Dims{mg->nx >> l, mg->ny >> l, mg->nz >> l};
        const int64_t nl = L.D.n();
        L.code = (uint8_t *)take(nl);
        L.r = (float *)take(sizeof(float) * nl);
        L.z = (float *)take(sizeof(float) * nl);
        L.z2 = (float *)take(sizeof(float) * nl);
        L.rh = L.zh = L.z2h = nullptr;
        if (mg->precision == FLUB_PRECISION_MIXED) {
            L.rh = (__half *)take(sizeof(__half) * nl);
            L.zh = l ? (__half *)take(sizeof(__half) * nl) : nullptr;
            L.z2h = (__half *)take(sizeof(__half) * nl);
        }
        L.act = L.act_n = nullptr;
        L.sw = nullptr;
        L.sws = nullptr;
        L.rs = L.zs = nullptr;
        L.rsh = nullptr;
        if (L.D.nz % 8 == 0) {
            L.act = (int *)take(sizeof(int) * (size_t)(nl >> 3));
            L.act_n = (int *)take(sizeof(int));
            L.sw = (uint16_t *)take(sizeof(uint16_t) * (size_t)nl);
            if (l == 0 && mg->split_ok) {
                L.sws = (uint16_t *)take(sizeof(uint16_t) * (size_t)nl);
                L.zs = (float *)take(sizeof(float) * nl);
                if (mg->precision == FLUB_PRECISION_MIXED)
                    L.rsh = (__half *)take(sizeof(__half) * nl);
                else
                    L.rs = (float *)take(sizeof(float) * nl);
            }
        }
        L.z3 = nullptr;
        L.tflags = nullptr;
        L.tiles = L.tiles_n = nullptr;
        L.n_tiles = 0;
        // tiles where the level is a whole number of them and every extent is at
        // least a tile box (the coarse level below then holds the coarse box)
        if (mg->tile_ok && mg->precision == FLUB_PRECISION_FP32 && L.D.nz % 8 == 0 && L.D.nx % kTI == 0 &&
            L.D.ny % kTJ == 0 &&
            L.D.nz % kTK == 0 && L.D.nx >= 2 * kTI && L.D.ny >= 2 * kTJ && L.D.nz >= 2 * kTK) {
            L.n_tiles = (L.D.nx / kTI) * (L.D.ny / kTJ) * (L.D.nz / kTK);
            L.z3 = (float *)take(sizeof(float) * nl);
            L.tflags = (unsigned char *)take((size_t)L.n_tiles);
            L.tiles = (int *)take(sizeof(int) * (size_t)L.n_tiles);
            L.tiles_n = (int *)take(sizeof(int));
        }
        L.pmask = nullptr;
        if (nl <= kTailMaxCells && L.D.nz % 2 == 0) L.pmask = (uint32_t *)take(sizeof(uint32_t) * (size_t)(nl >> 1));
    }
    // per-block counts of the active-list build (level 0 has the most blocks)
    mg->act_scratch = (int *)take(sizeof(int) * (size_t)((n / 8 + kActPerBlock - 1) / kActPerBlock + 1));
    mg->r_old = mg->precision == FLUB_PRECISION_MIXED ? (float *)take(sizeof(float) * n) : nullptr;
    return off;
}

// Shared-memory layout of the tail kernel from level lt down; returns the
// bytes needed (0 if the tail does not qualify).
static size_t tail_layout(const flub_mg *mg, int lt, TailParams *P) {
    if (lt >= mg->levels || mg->levels - lt > kTailMaxLevels) return 0;
    size_t off = 0;
    auto take = [&](size_t b) {
        size_t o = off;
        off += (b + 15) & ~(size_t)15;
        return (int)o;
    };
    for (int l = lt; l < mg->levels; l++) {
        const Dims D{mg->nx >> l, mg->ny >> l, mg->nz >> l};
        const size_t n = (size_t)D.n();
        TailLevel &T = P->lv[l - lt];
        T.D = D;
        T.code = mg->lv[l].code;
        T.pmask = mg->lv[l].pmask;
        T.abs_level = l;
        T.off_z = take(sizeof(float) * n);
        T.off_r = take(sizeof(float) * n);
        T.off_c = take(n);
        T.off_v = l + 1 < mg->levels ? take(sizeof(float) * n) : -1;
    }
    P->nt = mg->levels - lt;
    P->nu = mg->sched_nu;
    P->nbottom = mg->sched_bottom;
    P->rscale = mg->sched_rscale;
    P->bottom64 = mg->bottom64 ? 1 : 0;
    P->off_zd = 0;
    if (mg->bottom64) P->off_zd = take(sizeof(double) * (size_t)P->lv[P->nt - 1].D.n());
    return off;
}

static int set_tail_smem_limit() {
    FLUB_CHECK_CUDA(cudaFuncSetAttribute(k_tail_vcycle, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailMaxSmem));
    return FLUB_OK;
}

static int choose_tail(flub_mg *mg) {
    mg->tail_start = mg->levels;
    mg->tail_smem = 0;
    for (int l = 0; l < mg->levels; l++) {
        const Dims D{mg->nx >> l, mg->ny >> l, mg->nz >> l};
        if (D.n() > kTailMaxCells) continue;
        TailParams P;
        const size_t b = tail_layout(mg, l, &P);
        if (b > 0 && b <= kTailMaxSmem) {
            mg->tail_start = l;
            mg->tail_smem = b;
        }
        break;
    }
    return FLUB_OK;
}

static inline bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
static inline int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

// Distributed-shared-memory layout of the cluster kernel from level lc down
// with C blocks; returns the bytes per block (0 if the levels do not qualify:
// every dimension a power of two, nx and nz at least 2 at every level).
static size_t cluster_layout(const flub_mg *mg, int lc, int C, ClusterParams *P) {
    if (lc >= mg->levels || mg->levels - lc > kClusterMaxLevels) return 0;
    size_t off = 0;
    auto take = [&](size_t b) {
        size_t o = off;
        off += (b + 15) & ~(size_t)15;
        return (int)o;
    };
    P->tail = 0;
    P->tail_off = 0;
    // block 0 takes over the <= 16^3 levels: their sweeps then synchronise
    // with block barriers instead of cluster barriers (measured at 256^3: the
    // reference schedule's solve 30.0 -> 27.4 ms, V(2,2) 3.03 -> 2.96 ms).
    // FLUB_CLUSTER_TAIL=0 keeps them in the cluster; both give the same bits.
    const char *ct = getenv("FLUB_CLUSTER_TAIL");
    const bool want_tail = !(ct && ct[0] == '0');
    int lt = mg->levels;  // first level run by block 0 alone (== levels: none)
    for (int l = lc; l < mg->levels; l++) {
        const Dims D{mg->nx >> l, mg->ny >> l, mg->nz >> l};
        if (want_tail && l > lc && D.n() <= kTailMaxCells && tail_layout(mg, l, &P->tp) > 0) {
            lt = l;
            break;
        }
        if (!is_pow2(D.nx) || !is_pow2(D.ny) || !is_pow2(D.nz) || D.nx < 2 || D.nz < 2) return 0;
        ClusterLevel &L = P->lv[l - lc];
        L.D = D;
        L.abs_level = l;
        L.ncta = D.nx / 2 < C ? D.nx / 2 : C;
        L.P = D.nx / L.ncta;
        L.lg_ny = ilog2(D.ny);
        L.lg_nz = ilog2(D.nz);
        L.code = mg->lv[l].code;
        const size_t plane = (size_t)D.ny * D.nz;
        L.off_z = take(sizeof(float) * (L.P + 2) * plane);
        L.off_c = take((L.P + 2) * plane);
        L.off_r = take(sizeof(float) * L.P * plane);
    }
    P->nl = lt - lc;
    if (lt < mg->levels) {
        // the coarsest levels in block 0: the tail layout after the distributed ones
        const size_t tb = tail_layout(mg, lt, &P->tp);
        P->tail = 1;
        P->tail_off = take(tb);
    }
    P->nu = mg->sched_nu;
    P->nbottom = mg->sched_bottom;
    P->rscale = mg->sched_rscale;
    return off;
}

static cudaError_t cluster_launch_config(int C, size_t smem, cudaStream_t s, cudaLaunchConfig_t *cfg,
                                         cudaLaunchAttribute *attr) {
    memset(cfg, 0, sizeof(*cfg));
    cfg->gridDim = dim3(C);
    cfg->blockDim = dim3(kClusterThreads);
    cfg->dynamicSmemBytes = smem;
    cfg->stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg->attrs = attr;
    cfg->numAttrs = 2;
    return cudaSuccess;
}

// Picks the first level of at most 32^3 cells whose coarse hierarchy fits one
// cluster (16 blocks, else 8); none if the GPU cannot run it or
// FLUB_NO_CLUSTER=1.
static int choose_cluster(flub_mg *mg) {
    mg->cl_start = mg->levels;
    mg->cl_size = 0;
    mg->cl_smem = 0;
    const char *off = getenv("FLUB_NO_CLUSTER");
    if (off && off[0] == '1') return FLUB_OK;
    int dev = 0, max_smem = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return FLUB_OK;
    }
    // larger levels keep the 152-SM global sweeps: on 8-16 SMs a 64^3 half-sweep
    // is bound by shared-memory bandwidth (FLUB_CLUSTER_MAX_CELLS overrides)
    int64_t max_cells = 32768;
    const char *mc = getenv("FLUB_CLUSTER_MAX_CELLS");
    if (mc && atoll(mc) > 0) max_cells = atoll(mc);
    for (int C : {16, 8}) {
        for (int l = 0; l < mg->levels; l++) {
            const Dims D{mg->nx >> l, mg->ny >> l, mg->nz >> l};
            if (D.n() > max_cells) continue;
            ClusterParams P;
            const size_t b = cluster_layout(mg, l, C, &P);
            if (b == 0 || b > (size_t)max_smem) break;
            if (cudaFuncSetAttribute(k_cluster_vcycle<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_cluster_vcycle<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_cluster_vcycle<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_cluster_vcycle<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem) !=
                    cudaSuccess) {
                cudaGetLastError();
                break;
            }
            cudaLaunchConfig_t cfg;
            cudaLaunchAttribute attr[2];
            cluster_launch_config(C, b, nullptr, &cfg, attr);
            cfg.numAttrs = 1;  // the cluster dimension only
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, k_cluster_vcycle<false>, &cfg) != cudaSuccess || nclusters < 1) {
                cudaGetLastError();
                break;
            }
            mg->cl_start = l;
            mg->cl_size = C;
            mg->cl_smem = b;
            return FLUB_OK;
        }
    }
    return FLUB_OK;
}

// The persistent cooperative V-cycle legs (persist.cuh), opt-in with
// FLUB_PERSIST=1 when the device can run them: one block count for all four
// kernels (the smallest co-resident count times the SMs).  Measured on the
// 256^3 dam break they are slower than one launch per pass (V(2,2) solve 2.93
// against 2.77 ms, the reference schedule 28.9 against 25.4 ms): a grid-wide
// barrier across both dies costs more than the kernel boundary it replaces.
static int choose_persist(flub_mg *mg) {
    mg->persist_blocks = 0;
    const char *on = getenv("FLUB_PERSIST");
    if (!(on && on[0] == '1')) return FLUB_OK;
    int dev = 0, coop = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || !coop) {
        cudaGetLastError();
        return FLUB_OK;
    }
    int occ = 1 << 30;
    const void *kerns[4] = {(const void *)k_vcycle_down<float>, (const void *)k_vcycle_up<float>,
                            (const void *)k_vcycle_down<__half>, (const void *)k_vcycle_up<__half>};
    for (const void *k : kerns) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, kPersistThreads, 0) != cudaSuccess) {
            cudaGetLastError();
            return FLUB_OK;
        }
        occ = b < occ ? b : occ;
    }
    if (occ < 1) return FLUB_OK;
    mg->persist_blocks = occ * nsm;
    return FLUB_OK;
}

// Levels 1 .. lg-1 go to the persistent legs when every one of them walks an
// active list with stencil words (nz % 8 == 0), the internal z buffers keep
// z = 0 off the fluid, and no tiled smoothing is asked for there.
static bool use_persist(const flub_mg *mg, int lg) {
    if (mg->persist_blocks <= 0 || !mg->skip_ok || lg < 2) return false;
    for (int l = 1; l < lg; l++) {
        const Level &L = mg->lv[l];
        if (L.D.nz % 8 != 0 || !L.act || !L.sw) return false;
        if (mg->tile_ok && L.n_tiles > 0) return false;
    }
    return true;
}

template <typename T>
static int launch_leg(flub_mg *mg, const LaunchCtx &c, bool down, int l0, int l1) {
    constexpr bool half = std::is_same<T, __half>::value;
    LegParams P = {};
    P.l0 = l0;
    P.l1 = l1;
    P.st = mg->st;
    P.rscale = (half ? 0.125f : 1.0f) * mg->sched_rscale;
    P.zc_scale = half ? 8.0f : 1.0f;
    for (int l = l0; l <= l1; l++) {
        const Level &L = mg->lv[l];
        LegLevel &Q = P.lv[l];
        Q.D = L.D;
        Q.code = L.code;
        Q.sw = L.sw;
        Q.act = L.act;
        Q.act_n = L.act_n;
        Q.iters = level_iters(mg, l);
        Q.r = half ? (void *)L.rh : (void *)L.r;
        Q.z = half ? (void *)L.zh : (void *)L.z;
        Q.z2 = half ? (void *)L.z2h : (void *)L.z2;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)mg->persist_blocks);
    cfg.blockDim = dim3(kPersistThreads);
    cfg.stream = c.s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = down ? cudaLaunchKernelEx(&cfg, k_vcycle_down<T>, (const LegParams)P, c.kc)
                               : cudaLaunchKernelEx(&cfg, k_vcycle_up<T>, (const LegParams)P, c.kc);
    if (e != cudaSuccess) {
        set_last_error("persistent V-cycle launch: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return FLUB_ERR_CUDA;
    }
    count_launches(1);
    return FLUB_OK;
}

// Opt-in (FLUB_CLUSTER_GLOBAL=1): the cluster kernel also runs the level just
// above its distributed levels (cluster.cuh, ClusterGlobal) when that level is
// below level 0, walks an active list with stencil words, the sweeps may skip
// fluid-free groups, and neither the persistent legs nor tiled smoothing are
// asked for there.  Measured on the 256^3 dam break it is slower than one
// launch per pass on all SMs (V(2,2) solve 2.89 against 2.68 ms, the
// reference schedule 25.5 against 23.3 ms): the 16 SMs of one cluster take
// longer over a 64^3 level's sweep than the launch boundary costs.
static bool use_cluster_global(const flub_mg *mg, int lt, int sk) {
    if (!(mg->cl_start < mg->levels) || lt != mg->cl_start) return false;
    const char *e = getenv("FLUB_CLUSTER_GLOBAL");
    if (!(e && e[0] == '1')) return false;
    const int G = lt - 1;
    if (G < 1 || sk != 1 || !mg->skip_ok || mg->persist_blocks > 0) return false;
    const Level &L = mg->lv[G];
    if (L.D.nz % 8 != 0 || !L.act || !L.sw) return false;
    return !(mg->tile_ok && L.n_tiles > 0);
}

static void fill_cluster_global(const flub_mg *mg, int G, bool half, ClusterGlobal *g) {
    const Level &L = mg->lv[G], &C = mg->lv[G + 1];
    g->on = 1;
    g->half = half ? 1 : 0;
    g->D = L.D;
    g->code = L.code;
    g->sw = L.sw;
    g->act = L.act;
    g->act_n = L.act_n;
    g->r = half ? (void *)L.rh : (void *)L.r;
    g->z = half ? (void *)L.zh : (void *)L.z;
    g->z2 = half ? (void *)L.z2h : (void *)L.z2;
    g->iters = level_iters(mg, G);
    g->rscale = (half ? 0.125f : 1.0f) * mg->sched_rscale;
    g->zc_scale = half ? 8.0f : 1.0f;
    g->CD = C.D;
    g->ccode = C.code;
    g->cact = C.act;
    g->cact_n = C.act_n;
    g->cr = half ? (void *)C.rh : (void *)C.r;
    g->cz = half ? (const void *)C.zh : (const void *)C.z;
}

// Whether the bottom level runs inside the one-block tail (tail.cuh), alone or
// inside the cluster kernel: the only place with an FP64 bottom.
static bool bottom_in_tail(flub_mg *mg) {
    if (mg->cl_start < mg->levels) {
        ClusterParams P;
        return cluster_layout(mg, mg->cl_start, mg->cl_size, &P) > 0 && P.tail;
    }
    return mg->tail_start < mg->levels;
}

static int validate_shape(int nx, int ny, int nz, int levels, int precision) {
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0, "MGPCG shape (%d, %d, %d) must be positive", nx, ny, nz);
    FLUB_REQUIRE(levels >= 1 && levels <= kMaxLevels, "n_mg_levels=%d outside [1, %d]", levels, kMaxLevels);
    FLUB_REQUIRE(precision == FLUB_PRECISION_FP32 || precision == FLUB_PRECISION_MIXED, "unknown precision %d",
                 precision);
    const int f = 1 << (levels - 1);
    FLUB_REQUIRE(nx % f == 0 && ny % f == 0 && nz % f == 0,
                 "shape (%d, %d, %d) is not divisible by 2**(n_mg_levels-1) = %d", nx, ny, nz, f);
    FLUB_REQUIRE(((nz >> (levels - 1)) % 2) == 0,
                 "nz >> (n_mg_levels-1) = %d must be even (red-black launch over k pairs)", nz >> (levels - 1));
    return FLUB_OK;
}

static inline unsigned red_blocks(int64_t n) { return blocks_for(n, kRedThreads, 152 * 6); }

// Grid of k8_matvec_pap over the level-0 groups: one resident wave (its
// registers allow fewer blocks per SM than red_blocks assumes, which left a
// second, partial wave).
static unsigned matvec_blocks(int64_t groups) {
    static int resident = 0;
    if (resident <= 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k8_matvec_pap, kRedThreads, 0) != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 4;
        }
        resident = b;
    }
    return blocks_for(groups + 1, kRedThreads, (int64_t)kNumSMs * resident);
}

// ---------------------------------------------------------------- enqueue helpers

#define FLUB_TRY(...)              \
    do {                           \
        int _s = (__VA_ARGS__);    \
        if (_s) return _s;         \
    } while (0)

// Kernel launch with programmatic stream serialisation (the kernel's entry
// waits on griddepcontrol.wait, see count_kernel), counted like the others.
template <typename... KArgs, typename... Args>
static int launch_pdl(void (*kern)(KArgs...), dim3 g, dim3 b, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
    if (e != cudaSuccess) {
        set_last_error("cudaLaunchKernelEx: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return FLUB_ERR_CUDA;
    }
    count_launches(1);
    return FLUB_OK;
}

enum SweepMode { kSweepInPlace = 0, kSweepFromZero = 1, kSweepProlong = 2 };

// One red-black half-sweep on level L (multigrid/mgpcg.py:72-86):
//   kSweepInPlace   zout = sweep(zout)
//   kSweepFromZero  zout = sweep(0)
//   kSweepProlong   zout = sweep(zin + P zc)   (mgpcg.py:113-116 fused in)
// Storage-generic form of the vectorised sweep (nz % 8 == 0): TO/TI/TR/TC are
// the types of zout, zin, r and the coarse correction zc (float or __half);
// zc is multiplied by zc_scale on load.
template <typename TO, typename TI, typename TR, typename TC>
static int sweep8(const LaunchCtx &c, const Level &L, int phase, int mode, int skip, const TR *r, const TI *zin,
                  TO *zout, const TC *zc, float zc_scale) {
    const Dims D = L.D;
    // skip: the caller asserts z = 0 off the fluid in zout, so only the active
    // groups are visited; one resident wave of blocks, grid-stride
    const int *act = skip ? L.act : nullptr;
    const int *act_n = skip ? L.act_n : nullptr;
    const dim3 blk(256), grd(blocks_for(D.n() >> 2, 256, kNumSMs * 6));  // two lanes per group, 6 resident blocks per SM
    if (mode == kSweepFromZero)
        return launch_pdl(k_smooth8<true, false, TO, TO, TR, TC>, grd, blk, 0, c.s, zout, (const TO *)zout,
                          (const TC *)nullptr, 1.0f, r, (const uint8_t *)L.code, (const uint16_t *)L.sw, D, phase,
                          act, act_n, c.kc);
    if (mode == kSweepProlong)
        return launch_pdl(k_smooth8<false, true, TO, TI, TR, TC>, grd, blk, 0, c.s, zout, zin, zc, zc_scale, r,
                          (const uint8_t *)L.code, (const uint16_t *)L.sw, D, phase, act, act_n, c.kc);
    return launch_pdl(k_smooth8<false, false, TO, TO, TR, TC>, grd, blk, 0, c.s, zout, (const TO *)zout,
                      (const TC *)nullptr, 1.0f, r, (const uint8_t *)L.code, (const uint16_t *)L.sw, D, phase, act,
                      act_n, c.kc);
}

static int sweep(const LaunchCtx &c, const Level &L, int phase, int mode, int skip, const float *r,
                 const float *zin, float *zout, const float *zc) {
    const Dims D = L.D;
    if (D.nz % 8 == 0) return sweep8<float, float, float, float>(c, L, phase, mode, skip, r, zin, zout, zc, 1.0f);
    // scalar path for levels whose nz is not a multiple of 8
    if (mode == kSweepProlong)
        FLUB_TRY(launch_pdl(k_prolong, dim3(blocks_for(D.n(), 256, 1 << 20)), dim3(256), 0, c.s, zout, zin, zc, D,
                            c.kc));
    const unsigned b = blocks_for(D.n() / 2, 256, 1 << 20);
    if (mode == kSweepFromZero)
        return launch_pdl(k_smooth_half<true>, dim3(b), dim3(256), 0, c.s, zout, r, (const uint8_t *)L.code, D, phase,
                          c.kc);
    return launch_pdl(k_smooth_half<false>, dim3(b), dim3(256), 0, c.s, zout, r, (const uint8_t *)L.code, D, phase,
                      c.kc);
}


// One level-0 half-sweep on colour-split storage (smooth_split.cuh).
template <int kMode, typename TRN, typename TR, typename TZI, typename TZ, typename TC>
static int split_sweep(const LaunchCtx &c, const Level &L, int phase, const TRN *rn, TR *rs, const TZI *zin, TZ *z,
                       const TC *zc, float zc_scale, float *zn, const SplitArgs *dot = nullptr) {
    SplitArgs A = {};
    if (dot) A = *dot;  // kLast with z.r folded in: dot, rdot, pinit, st, partials
    A.D = L.D;
    A.act = L.act;
    A.act_n = L.act_n;
    A.sws = L.sws;
    A.rn = rn;
    A.rs = rs;
    A.zin = zin;
    A.z = z;
    A.zc = zc;
    A.zc_scale = zc_scale;
    A.zn = zn;
    // one lane per active group, grid-stride with one resident wave of blocks
    static int resident = 0;
    if (resident <= 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_smooth_split<kMode, TRN, TR, TZI, TZ, TC>, 256, 0) !=
                cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 4;
        }
        resident = b;
    }
    const dim3 grd(blocks_for(L.D.n() >> 3, 256, (int64_t)kNumSMs * resident));
    return launch_pdl(k_smooth_split<kMode, TRN, TR, TZI, TZ, TC>, grd, dim3(256), 0, c.s, (const SplitArgs)A, phase,
                      c.kc);
}

// Colour-split level-0 smoothing unless FLUB_NO_SPLIT=1 (read when a handle is
// created or sized).
static bool split_requested() {
    const char *e = getenv("FLUB_NO_SPLIT");
    return !(e && e[0] == '1');
}

// Level 0 of the V-cycle on colour-split storage: the handle has the split
// buffers, level 0 hands on to a coarser level (lg >= 1), the sweeps may skip
// fluid-free groups, no tiled smoothing is asked for there, and the output z
// is not the input r.
static bool use_split(const flub_mg *mg, int lg, int sk, const void *r0, const void *z0) {
    const Level &L = mg->lv[0];
    return mg->split_ok && L.sws && lg >= 1 && sk == 1 && !(mg->tile_ok && L.n_tiles > 0) && r0 != z0;
}

// ---------------------------------------------------------------- tiled smoothing (smooth_tile.cuh)

static PFN_cuTensorMapEncodeTiled_v12000 g_tile_encode = nullptr;

// Driver entry point for tensor maps and the tile kernels' shared-memory limit.
static int tile_setup() {
    static std::mutex m;
    std::lock_guard<std::mutex> lock(m);
    if (g_tile_encode) return FLUB_OK;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return FLUB_ERR_CUDA;
    }
    if (cudaFuncSetAttribute(k_smooth_tile<kTileInPlaceInput>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTileSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_smooth_tile<kTileFromZero>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTileSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_smooth_tile<kTileProlong>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTileSmem) != cudaSuccess) {
        cudaGetLastError();
        return FLUB_ERR_CUDA;
    }
    g_tile_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return FLUB_OK;
}

// The tiled smoother is used (and its buffers carved) when FLUB_TILE=1 and the
// driver provides tensor maps; flub_mg_workspace_bytes and flub_mg_create
// must agree on it.
static bool tile_requested() {
    const char *tl = getenv("FLUB_TILE");
    return tl && tl[0] == '1' && tile_setup() == FLUB_OK;
}

// 3D tensor map over an (nx, ny, nz) C-order array (x = k innermost), box
// bk x bj x bi, zero fill outside the array.
static int tile_map(CUtensorMap *m, const void *base, CUtensorMapDataType dt, int esize, Dims D, int bk, int bj,
                    int bi) {
    cuuint64_t dims[3] = {(cuuint64_t)D.nz, (cuuint64_t)D.ny, (cuuint64_t)D.nx};
    cuuint64_t strides[2] = {(cuuint64_t)D.nz * esize, (cuuint64_t)D.nz * D.ny * esize};
    cuuint32_t box[3] = {(cuuint32_t)bk, (cuuint32_t)bj, (cuuint32_t)bi};
    cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = g_tile_encode(m, dt, 3, const_cast<void *>(base), dims, strides, box, es,
                                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_last_error("cuTensorMapEncodeTiled (%dx%dx%d, box %dx%dx%d) failed: %d", D.nx, D.ny, D.nz, bi, bj, bk,
                       (int)r);
        return FLUB_ERR_CUDA;
    }
    return FLUB_OK;
}

// One red-black iteration of level L (first_phase, then the other) by tiles,
// zin -> zout (different buffers); mode kTileFromZero ignores zin,
// kTileProlong adds the coarse correction zc first.
static int tile_iteration(flub_mg *mg, const LaunchCtx &c, int l, int first_phase, int mode, const float *r,
                          const float *zin, float *zout, const float *zc) {
    const Level &L = mg->lv[l];
    CUtensorMap mz, mr, mw, mc;
    FLUB_TRY(tile_map(&mr, r, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, L.D, kRK, kRJ, kRI));
    FLUB_TRY(tile_map(&mw, L.sw, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, L.D, kWK, kWJ, kWI));
    mz = mr;
    mc = mr;  // unused by the modes that do not read them
    if (mode != kTileFromZero) FLUB_TRY(tile_map(&mz, zin, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, L.D, kZK, kZJ, kZI));
    if (mode == kTileProlong)
        FLUB_TRY(tile_map(&mc, zc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, mg->lv[l + 1].D, kCK, kCJ, kCI));
    const dim3 grd(L.n_tiles < kNumSMs * kTileBlocksPerSM ? L.n_tiles : kNumSMs * kTileBlocksPerSM);
    int *status = &mg->st->status;
    const int *tl = L.tiles, *tn = L.tiles_n;
    if (mode == kTileFromZero)
        return launch_pdl(k_smooth_tile<kTileFromZero>, grd, dim3(kTileThreads), kTileSmem, c.s, mz, mr, mw, mc, zout,
                          L.D, first_phase, tl, tn, status, c.kc);
    if (mode == kTileProlong)
        return launch_pdl(k_smooth_tile<kTileProlong>, grd, dim3(kTileThreads), kTileSmem, c.s, mz, mr, mw, mc, zout,
                          L.D, first_phase, tl, tn, status, c.kc);
    return launch_pdl(k_smooth_tile<kTileInPlaceInput>, grd, dim3(kTileThreads), kTileSmem, c.s, mz, mr, mw, mc,
                      zout, L.D, first_phase, tl, tn, status, c.kc);
}

// Pre-smoothing (iters iterations from z = 0, phases 0 then 1) ending in
// z_fin, or post-smoothing (first iteration from z_pre + P zc, phases 1 then
// 0) ending in z_fin, by tiles; the iterations alternate between z_fin and
// the level's third buffer so that the last one writes z_fin.
static int tile_side(flub_mg *mg, const LaunchCtx &c, int l, bool post, int iters, const float *r,
                     const float *z_pre, float *z_fin, const float *zc) {
    float *z3 = mg->lv[l].z3;
    const float *prev = z_pre;
    for (int t = 0; t < iters; t++) {
        float *w = ((iters - 1 - t) % 2 == 0) ? z_fin : z3;
        const int mode = t == 0 ? (post ? kTileProlong : kTileFromZero) : kTileInPlaceInput;
        FLUB_TRY(tile_iteration(mg, c, l, post ? 1 : 0, mode, r, prev, w, zc));
        prev = w;
    }
    return FLUB_OK;
}

// multigrid/mgpcg.py:296-349 apply_preconditioner; level 0 uses (r0, z0).
// z0_clean: z0 holds 0 on every non-fluid cell (true for the handle's own z).
// dot_mode 1 / 2: the caller's next step is z.r (the prologue's p = z / the
// iteration's beta); when the last level-0 half-sweep can fold it in, it does
// and *dot_fused is set.
static int enqueue_vcycle(flub_mg *mg, const LaunchCtx &c, const float *r0, float *z0, bool z0_clean,
                          int dot_mode = 0, bool *dot_fused = nullptr) {
    if (dot_fused) *dot_fused = false;
    const bool use_cl = mg->cl_start < mg->levels;
    const int Lm = mg->levels, lt = use_cl ? mg->cl_start : mg->tail_start;
    const int sk = mg->skip_ok ? 1 : 0;
    auto SK = [&](int l) { return (l == 0 && !z0_clean) ? 0 : sk; };
    auto R = [&](int l) -> const float * { return l == 0 ? r0 : mg->lv[l].r; };
    auto ZF = [&](int l) -> float * { return l == 0 ? z0 : mg->lv[l].z; };
    auto ZP = [&](int l) -> float * { return mg->lv[l].z2; };
    const int lg = lt < Lm - 1 ? lt : Lm - 1;  // levels 0 .. lg-1 restrict to a coarser level
    // tiled smoothing where the level has tiles and the buffers written hold 0
    // off the fluid: pre-smoothing writes the level's own z2 / z3, post-
    // smoothing ends in ZF(l), the caller's z0 at level 0
    auto TILED_PRE = [&](int l) { return mg->tile_ok && mg->lv[l].n_tiles > 0 && sk == 1; };
    auto TILED_POST = [&](int l) { return mg->tile_ok && mg->lv[l].n_tiles > 0 && SK(l) == 1; };
    // levels 1 .. lg-1 in the persistent cooperative kernels, or one launch per pass
    const bool pers = use_persist(mg, lg);
    // the level above the cluster's in the cluster kernel: the launches per
    // pass stop one level earlier
    const bool clg = use_cl && use_cluster_global(mg, lt, sk);
    const int lge = clg ? lt - 1 : lg;
    // level 0 on colour-split storage (smooth_split.cuh)
    const bool split0 = use_split(mg, lge, sk, r0, z0);
    for (int l = 0; l < (pers ? 1 : lge); l++) {
        const Level &L = mg->lv[l];
        const int iters = level_iters(mg, l);
        if (l == 0 && split0) {
            float *z2 = ZP(0);
            for (int it = 0; it < iters; it++) {
                if (it == 0) {
                    FLUB_TRY((split_sweep<kFirst, float, float, float, float, float>(c, L, 0, r0, L.rs, nullptr, z2,
                                                                                   nullptr, 1.0f, nullptr)));
                    FLUB_TRY((split_sweep<kOwnZero, float, float, float, float, float>(
                        c, L, 1, nullptr, L.rs, nullptr, z2, nullptr, 1.0f, nullptr)));
                } else {
                    FLUB_TRY((split_sweep<kInPlace, float, float, float, float, float>(
                        c, L, 0, nullptr, L.rs, nullptr, z2, nullptr, 1.0f, nullptr)));
                    FLUB_TRY((split_sweep<kInPlace, float, float, float, float, float>(
                        c, L, 1, nullptr, L.rs, nullptr, z2, nullptr, 1.0f, nullptr)));
                }
            }
            const Level &C = mg->lv[1];
            FLUB_TRY(launch_pdl(k_restrict8_split<float, float, float>, dim3(blocks_for(C.D.n(), 256, kNumSMs * 4)),
                                dim3(256), 0, c.s, r0, (const float *)z2, (const uint8_t *)L.code,
                                (const uint16_t *)L.sw, C.r, (const uint8_t *)C.code, C.D, mg->sched_rscale,
                                (const int *)C.act, (const int *)C.act_n, c.kc));
            continue;
        }
        if (TILED_PRE(l)) {
            FLUB_TRY(tile_side(mg, c, l, false, iters, R(l), nullptr, ZP(l), nullptr));
        } else {
            for (int it = 0; it < iters; it++) {
                FLUB_TRY(sweep(c, L, 0, it == 0 ? kSweepFromZero : kSweepInPlace, sk, R(l), ZP(l), ZP(l), nullptr));
                FLUB_TRY(sweep(c, L, 1, kSweepInPlace, sk, R(l), ZP(l), ZP(l), nullptr));
            }
        }
        const Level &C = mg->lv[l + 1];
        if (L.D.nz % 8 == 0)
            FLUB_TRY(launch_pdl(k_restrict8<float, float, float>, dim3(blocks_for(C.D.n(), 256, kNumSMs * 4)),
                                dim3(256), 0, c.s, R(l), (const float *)ZP(l), (const uint8_t *)L.code,
                                (const uint16_t *)L.sw, C.r,
                                (const uint8_t *)C.code, C.D, mg->sched_rscale, (const int *)C.act,
                                (const int *)C.act_n, c.kc));
        else
            FLUB_TRY(launch_pdl(k_restrict, dim3(blocks_for(C.D.n(), 256, 1 << 20)), dim3(256), 0, c.s, R(l), ZP(l),
                                L.code, C.r, C.code, C.D, mg->sched_rscale, c.kc));
    }
    if (pers) FLUB_TRY(launch_leg<float>(mg, c, true, 1, lg));
    if (use_cl) {
        ClusterParams P = {};
        cluster_layout(mg, lt, mg->cl_size, &P);
        P.r_top = R(lt);
        P.z_top = ZF(lt);
        if (clg) fill_cluster_global(mg, lt - 1, false, &P.g);
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr[2];
        cluster_launch_config(mg->cl_size, mg->cl_smem, c.s, &cfg, attr);
        const cudaError_t e = P.g.on ? cudaLaunchKernelEx(&cfg, k_cluster_vcycle<true>, (const ClusterParams)P, c.kc)
                                     : cudaLaunchKernelEx(&cfg, k_cluster_vcycle<false>, (const ClusterParams)P, c.kc);
        if (e != cudaSuccess) {
            set_last_error("cluster V-cycle launch: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return FLUB_ERR_CUDA;
        }
        count_launches(1);
    } else if (lt < Lm) {
        TailParams P = {};
        tail_layout(mg, lt, &P);
        P.r_top = R(lt);
        P.z_top = ZF(lt);
        FLUB_TRY(launch_pdl(k_tail_vcycle, dim3(1), dim3(kTailThreads), mg->tail_smem, c.s, P, c.kc));
    } else {
        const int b = Lm - 1;
        const Level &L = mg->lv[b];
        for (int it = 0; it < mg->sched_bottom; it++) {
            FLUB_TRY(sweep(c, L, 0, it == 0 ? kSweepFromZero : kSweepInPlace, SK(b), R(b), ZF(b), ZF(b), nullptr));
            FLUB_TRY(sweep(c, L, 1, kSweepInPlace, SK(b), R(b), ZF(b), ZF(b), nullptr));
        }
        for (int it = 0; it < mg->sched_bottom; it++) {
            FLUB_TRY(sweep(c, L, 1, kSweepInPlace, SK(b), R(b), ZF(b), ZF(b), nullptr));
            FLUB_TRY(sweep(c, L, 0, kSweepInPlace, SK(b), R(b), ZF(b), ZF(b), nullptr));
        }
    }
    if (pers) FLUB_TRY(launch_leg<float>(mg, c, false, 1, lg));
    for (int l = pers ? 0 : lge - 1; l >= 0; l--) {
        const Level &L = mg->lv[l];
        const int iters = level_iters(mg, l);
        if (l == 0 && split0) {
            // the last half-sweep writes the groups with fluid of the natural z0;
            // a caller's z0 gets 0 everywhere else first
            if (!z0_clean) FLUB_CHECK_CUDA(cudaMemsetAsync(z0, 0, sizeof(float) * (size_t)mg->n, c.s));
            for (int it = 0; it < iters; it++) {
                if (it == 0)
                    FLUB_TRY((split_sweep<kProlong, float, float, float, float, float>(
                        c, L, 1, nullptr, L.rs, ZP(0), L.zs, mg->lv[1].z, 1.0f, nullptr)));
                else
                    FLUB_TRY((split_sweep<kInPlace, float, float, float, float, float>(
                        c, L, 1, nullptr, L.rs, nullptr, L.zs, nullptr, 1.0f, nullptr)));
                if (it + 1 == iters) {
                    SplitArgs D = {};
                    if (dot_mode && dot_fused) {
                        D.dot = dot_mode;
                        D.rdot = r0;
                        D.pinit = mg->p;
                        D.st = mg->st;
                        D.partials = mg->partials;
                        *dot_fused = true;
                    }
                    FLUB_TRY((split_sweep<kLast, float, float, float, float, float>(
                        c, L, 0, nullptr, L.rs, nullptr, L.zs, nullptr, 1.0f, z0, D.dot ? &D : nullptr)));
                }
                else
                    FLUB_TRY((split_sweep<kInPlace, float, float, float, float, float>(
                        c, L, 0, nullptr, L.rs, nullptr, L.zs, nullptr, 1.0f, nullptr)));
            }
            continue;
        }
        if (TILED_POST(l)) {
            FLUB_TRY(tile_side(mg, c, l, true, iters, R(l), ZP(l), ZF(l), mg->lv[l + 1].z));
            continue;
        }
        for (int it = 0; it < iters; it++) {
            FLUB_TRY(sweep(c, L, 1, it == 0 ? kSweepProlong : kSweepInPlace, SK(l), R(l), ZP(l), ZF(l),
                           mg->lv[l + 1].z));
            FLUB_TRY(sweep(c, L, 0, kSweepInPlace, SK(l), R(l), ZF(l), ZF(l), nullptr));
        }
    }
    return FLUB_OK;
}

// Cluster or one-block kernel for the coarse levels from lt down, with FP16
// (mixed precision) or FP32 top-level residual/correction.
static int launch_coarse(flub_mg *mg, const LaunchCtx &c, int lt, const float *r_top, float *z_top,
                         const __half *r_top_h, __half *z_top_h, bool global_half = false) {
    if (mg->cl_start < mg->levels) {
        ClusterParams P = {};
        cluster_layout(mg, lt, mg->cl_size, &P);
        P.r_top = r_top;
        P.z_top = z_top;
        P.r_top_h = r_top_h;
        P.z_top_h = z_top_h;
        if (global_half) fill_cluster_global(mg, lt - 1, true, &P.g);
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr[2];
        cluster_launch_config(mg->cl_size, mg->cl_smem, c.s, &cfg, attr);
        const cudaError_t e = P.g.on ? cudaLaunchKernelEx(&cfg, k_cluster_vcycle<true>, (const ClusterParams)P, c.kc)
                                     : cudaLaunchKernelEx(&cfg, k_cluster_vcycle<false>, (const ClusterParams)P, c.kc);
        if (e != cudaSuccess) {
            set_last_error("cluster V-cycle launch: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return FLUB_ERR_CUDA;
        }
        count_launches(1);
        return FLUB_OK;
    }
    TailParams P = {};
    tail_layout(mg, lt, &P);
    P.r_top = r_top;
    P.z_top = z_top;
    P.r_top_h = r_top_h;
    P.z_top_h = z_top_h;
    return launch_pdl(k_tail_vcycle, dim3(1), dim3(kTailThreads), mg->tail_smem, c.s, P, c.kc);
}

// Mixed-precision V-cycle: the levels in global memory are FP16 at scale 8^-l
// (mixed.cuh); the level-0 residual is read from its FP16 copy lv[0].rh, the
// result z0 is FP32.  Same schedule as enqueue_vcycle.
static int enqueue_vcycle_mixed(flub_mg *mg, const LaunchCtx &c, float *z0, bool z0_clean, int dot_mode = 0,
                                bool *dot_fused = nullptr) {
    if (dot_fused) *dot_fused = false;
    const bool use_cl = mg->cl_start < mg->levels;
    const int Lm = mg->levels, lt = use_cl ? mg->cl_start : mg->tail_start;
    const int sk = mg->skip_ok ? 1 : 0;
    const int sk0 = z0_clean ? sk : 0;
    const int lg = lt < Lm - 1 ? lt : Lm - 1;
    const bool pers = use_persist(mg, lg);
    const bool clg = use_cl && use_cluster_global(mg, lt, sk);
    const int lge = clg ? lt - 1 : lg;
    const bool split0 = use_split(mg, lge, sk0, mg->lv[0].rh, z0);
    for (int l = 0; l < (pers ? 1 : lge); l++) {
        const Level &L = mg->lv[l];
        const int iters = level_iters(mg, l);
        if (l == 0 && split0) {
            using H = __half;
            for (int it = 0; it < iters; it++) {
                if (it == 0) {
                    FLUB_TRY((split_sweep<kFirst, H, H, H, H, H>(c, L, 0, (const H *)L.rh, L.rsh, nullptr, L.z2h,
                                                                 nullptr, 1.0f, nullptr)));
                    FLUB_TRY((split_sweep<kOwnZero, H, H, H, H, H>(c, L, 1, nullptr, L.rsh, nullptr, L.z2h, nullptr,
                                                                   1.0f, nullptr)));
                } else {
                    FLUB_TRY((split_sweep<kInPlace, H, H, H, H, H>(c, L, 0, nullptr, L.rsh, nullptr, L.z2h, nullptr,
                                                                   1.0f, nullptr)));
                    FLUB_TRY((split_sweep<kInPlace, H, H, H, H, H>(c, L, 1, nullptr, L.rsh, nullptr, L.z2h, nullptr,
                                                                   1.0f, nullptr)));
                }
            }
            const Level &C = mg->lv[1];
            FLUB_TRY(launch_pdl(k_restrict8_split<H, H, H>, dim3(blocks_for(C.D.n(), 256, kNumSMs * 4)), dim3(256),
                                0, c.s, (const H *)L.rh, (const H *)L.z2h, (const uint8_t *)L.code,
                                (const uint16_t *)L.sw, C.rh, (const uint8_t *)C.code, C.D,
                                0.125f * mg->sched_rscale, (const int *)C.act, (const int *)C.act_n, c.kc));
            continue;
        }
        for (int it = 0; it < iters; it++) {
            FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, 0, it == 0 ? kSweepFromZero : kSweepInPlace, sk,
                                                            L.rh, L.z2h, L.z2h, nullptr, 1.0f));
            FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, 1, kSweepInPlace, sk, L.rh, L.z2h, L.z2h, nullptr,
                                                            1.0f));
        }
        const Level &C = mg->lv[l + 1];
        FLUB_TRY(launch_pdl(k_restrict8<__half, __half, __half>, dim3(blocks_for(C.D.n(), 256, kNumSMs * 4)),
                            dim3(256), 0, c.s, (const __half *)L.rh, (const __half *)L.z2h, (const uint8_t *)L.code,
                            (const uint16_t *)L.sw, C.rh, (const uint8_t *)C.code, C.D, 0.125f * mg->sched_rscale, (const int *)C.act,
                            (const int *)C.act_n, c.kc));
    }
    if (pers) FLUB_TRY(launch_leg<__half>(mg, c, true, 1, lg));
    if (lt < Lm) {
        if (lt == 0)
            FLUB_TRY(launch_coarse(mg, c, 0, nullptr, z0, mg->lv[0].rh, nullptr));
        else
            FLUB_TRY(launch_coarse(mg, c, lt, nullptr, nullptr, mg->lv[lt].rh, mg->lv[lt].zh, clg));
    } else {
        const int b = Lm - 1;
        const Level &L = mg->lv[b];
        for (int q = 0; q < 2 * mg->sched_bottom; q++) {
            // bottom: nbottom x (0, 1) from zero, then nbottom x (1, 0)
            const int ph0 = q < mg->sched_bottom ? 0 : 1, ph1 = 1 - ph0;
            const int m0 = q == 0 ? kSweepFromZero : kSweepInPlace;
            if (b == 0) {
                FLUB_TRY(sweep8<float, float, __half, float>(c, L, ph0, m0, sk0, L.rh, z0, z0, nullptr, 1.0f));
                FLUB_TRY(sweep8<float, float, __half, float>(c, L, ph1, kSweepInPlace, sk0, L.rh, z0, z0, nullptr,
                                                             1.0f));
            } else {
                FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, ph0, m0, sk, L.rh, L.zh, L.zh, nullptr, 1.0f));
                FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, ph1, kSweepInPlace, sk, L.rh, L.zh, L.zh,
                                                                nullptr, 1.0f));
            }
        }
    }
    if (pers) FLUB_TRY(launch_leg<__half>(mg, c, false, 1, lg));
    for (int l = pers ? 0 : lge - 1; l >= 0; l--) {
        const Level &L = mg->lv[l];
        const __half *zc = mg->lv[l + 1].zh;
        const int iters = level_iters(mg, l);
        if (l == 0 && split0) {
            using H = __half;
            if (!z0_clean) FLUB_CHECK_CUDA(cudaMemsetAsync(z0, 0, sizeof(float) * (size_t)mg->n, c.s));
            for (int it = 0; it < iters; it++) {
                if (it == 0)
                    FLUB_TRY((split_sweep<kProlong, H, H, H, float, H>(c, L, 1, nullptr, L.rsh, L.z2h, L.zs, zc, 8.0f,
                                                                       nullptr)));
                else
                    FLUB_TRY((split_sweep<kInPlace, H, H, float, float, float>(c, L, 1, nullptr, L.rsh, nullptr,
                                                                               L.zs, nullptr, 1.0f, nullptr)));
                if (it + 1 == iters) {
                    SplitArgs D = {};
                    if (dot_mode && dot_fused) {
                        D.dot = dot_mode;  // 1: p = zscale z and zr_old, 3: flexible beta
                        D.zscaled = 1;
                        D.rdot = mg->lv[0].r;
                        D.rold = mg->r_old;
                        D.pinit = mg->p;
                        D.st = mg->st;
                        D.partials = mg->partials;
                        *dot_fused = true;
                    }
                    FLUB_TRY((split_sweep<kLast, H, H, float, float, float>(c, L, 0, nullptr, L.rsh, nullptr, L.zs,
                                                                            nullptr, 1.0f, z0,
                                                                            D.dot ? &D : nullptr)));
                }
                else
                    FLUB_TRY((split_sweep<kInPlace, H, H, float, float, float>(c, L, 0, nullptr, L.rsh, nullptr,
                                                                               L.zs, nullptr, 1.0f, nullptr)));
            }
            continue;
        }
        for (int it = 0; it < iters; it++) {
            if (l == 0) {
                if (it == 0)
                    FLUB_TRY(sweep8<float, __half, __half, __half>(c, L, 1, kSweepProlong, sk0, L.rh, L.z2h, z0, zc,
                                                                   8.0f));
                else
                    FLUB_TRY(sweep8<float, float, __half, float>(c, L, 1, kSweepInPlace, sk0, L.rh, z0, z0, nullptr,
                                                                 1.0f));
                FLUB_TRY(sweep8<float, float, __half, float>(c, L, 0, kSweepInPlace, sk0, L.rh, z0, z0, nullptr, 1.0f));
            } else {
                if (it == 0)
                    FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, 1, kSweepProlong, sk, L.rh, L.z2h, L.zh, zc,
                                                                    8.0f));
                else
                    FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, 1, kSweepInPlace, sk, L.rh, L.zh, L.zh,
                                                                    nullptr, 1.0f));
                FLUB_TRY(sweep8<__half, __half, __half, __half>(c, L, 0, kSweepInPlace, sk, L.rh, L.zh, L.zh, nullptr,
                                                                1.0f));
            }
        }
    }
    return FLUB_OK;
}

static int enqueue_mean_removal(flub_mg *mg, const LaunchCtx &c, int guard) {
    const unsigned b = red_blocks(mg->n);
    FLUB_TRY(launch_pdl(k_fluid_mean, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, mg->lv[0].r, mg->lv[0].code, mg->n, mg->partials, guard, c.kc));
    FLUB_TRY(launch_pdl(k_sub_mean, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, mg->lv[0].r, mg->lv[0].code, mg->n, guard, c.kc));
    return FLUB_OK;
}

// ---- mixed precision: same loop, FP16 V-cycle, flexible beta
static int enqueue_prologue_mixed(flub_mg *mg, const LaunchCtx &c, int smoother) {
    const Level &L0 = mg->lv[0];
    const unsigned bg = red_blocks(mg->n / 8 + 1);
    if (smoother == FLUB_SMOOTHER_FRACTION) FLUB_TRY(enqueue_mean_removal(mg, c, 0));
    FLUB_TRY(launch_pdl(k8_dot_rr0, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.r, L0.code, mg->n, mg->partials,
                        (const int *)L0.act, (const int *)L0.act_n, c.kc));
    FLUB_TRY(launch_pdl(k8_residual_x0, dim3(blocks_for(mg->n / 8, 256, kNumSMs * 8)), dim3(256), 0, c.s, mg->st,
                        L0.r, (const float *)mg->x, (const uint8_t *)L0.code, (const uint16_t *)L0.sw, L0.D,
                        (const int *)L0.act,
                        (const int *)L0.act_n, c.kc));
    if (smoother == FLUB_SMOOTHER_FRACTION) FLUB_TRY(enqueue_mean_removal(mg, c, 2));
    FLUB_TRY(launch_pdl(k8_to_half, dim3(blocks_for(mg->n / 8, 256)), dim3(256), 0, c.s, mg->st, (const float *)L0.r, L0.rh,
                        mg->n, c.kc));
    bool fused = false;
    FLUB_TRY(enqueue_vcycle_mixed(mg, c, L0.z, true, 1, &fused));
    if (fused) return FLUB_OK;  // p = zscale z and z.r in the last level-0 half-sweep
    return launch_pdl(k8_dot_zr<true, true>, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.z, L0.r, mg->p, L0.code,
                      mg->n, mg->partials, (const int *)L0.act, (const int *)L0.act_n, c.kc);
}

static int enqueue_first_half_mixed(flub_mg *mg, const LaunchCtx &c, int smoother) {
    const Level &L0 = mg->lv[0];
    const unsigned b = red_blocks(mg->n), bg = red_blocks(mg->n / 8 + 1);
    FLUB_TRY(launch_pdl(k8_matvec_pap, dim3(matvec_blocks(mg->n / 8)), dim3(kRedThreads), 0, c.s, mg->st, mg->p,
                        mg->Ap, L0.code, (const uint16_t *)L0.sw, L0.D, mg->partials, (const int *)L0.act,
                        (const int *)L0.act_n, c.kc));
    if (smoother == FLUB_SMOOTHER_FRACTION) {
        FLUB_CHECK_CUDA(cudaMemcpyAsync(mg->r_old, L0.r, sizeof(float) * mg->n, cudaMemcpyDeviceToDevice, c.s));
        FLUB_TRY(launch_pdl(k_update_r, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap, mg->n, c.kc));
        FLUB_TRY(enqueue_mean_removal(mg, c, 1));
        FLUB_TRY(launch_pdl(k8_to_half, dim3(blocks_for(mg->n / 8, 256)), dim3(256), 0, c.s, mg->st, (const float *)L0.r,
                            L0.rh, mg->n, c.kc));
        return launch_pdl(k8_update_r_rr<false>, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap, L0.code,
                          mg->n, mg->partials, mg->hist, c.h, c.set_cond, (const int *)L0.act, (const int *)L0.act_n,
                          c.kc);
    }
    return launch_pdl(k8_update_r_rr_mixed, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->r_old, L0.rh,
                      mg->Ap, L0.code, mg->n, mg->partials, mg->hist, c.h, c.set_cond, (const int *)L0.act,
                      (const int *)L0.act_n, c.kc);
}

static int enqueue_second_half_mixed(flub_mg *mg, const LaunchCtx &c) {
    const Level &L0 = mg->lv[0];
    const unsigned bg = red_blocks(mg->n / 8 + 1);
    bool fused = false;
    FLUB_TRY(enqueue_vcycle_mixed(mg, c, L0.z, true, 3, &fused));
    if (!fused)  // else the flexible beta came with the last level-0 half-sweep
        FLUB_TRY(launch_pdl(k8_dot_zr_flex, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.z, L0.r, mg->r_old,
                            L0.code, mg->n, mg->partials, (const int *)L0.act, (const int *)L0.act_n, c.kc));
    return launch_pdl(k8_update_xp<true>, dim3(blocks_for(mg->n / 8, 256, kNumSMs * 8)), dim3(256), 0, c.s, mg->st,
                      mg->x, mg->p, L0.z, L0.code, mg->n, (const int *)L0.act, (const int *)L0.act_n, c.kc);
}

static int enqueue_prologue(flub_mg *mg, const LaunchCtx &c, int smoother) {
    if (mg->precision == FLUB_PRECISION_MIXED) return enqueue_prologue_mixed(mg, c, smoother);
    const unsigned b = red_blocks(mg->n);
    const Level &L0 = mg->lv[0];
    const bool v8 = (L0.D.nz % 8) == 0;  // group-of-8 kernels; the scalar ones otherwise
    const unsigned bg = red_blocks(mg->n / 8 + 1);
    if (smoother == FLUB_SMOOTHER_FRACTION) FLUB_TRY(enqueue_mean_removal(mg, c, 0));
    if (v8)
        FLUB_TRY(launch_pdl(k8_dot_rr0, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.r, L0.code, mg->n,
                            mg->partials, (const int *)L0.act, (const int *)L0.act_n, c.kc));
    else
        FLUB_TRY(launch_pdl(k_dot_rr0, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->n, mg->partials, c.kc));
    if (v8)
        FLUB_TRY(launch_pdl(k8_residual_x0, dim3(blocks_for(mg->n / 8, 256, kNumSMs * 8)), dim3(256), 0, c.s,
                            mg->st, L0.r, (const float *)mg->x, (const uint8_t *)L0.code, (const uint16_t *)L0.sw, L0.D,
                        (const int *)L0.act,
                            (const int *)L0.act_n, c.kc));
    else
        FLUB_TRY(launch_pdl(k_residual_x0, dim3(blocks_for(mg->n, 256)), dim3(256), 0, c.s, mg->st, L0.r, mg->x,
                            L0.code, L0.D, c.kc));
    if (smoother == FLUB_SMOOTHER_FRACTION) FLUB_TRY(enqueue_mean_removal(mg, c, 2));
    bool fused = false;
    FLUB_TRY(enqueue_vcycle(mg, c, L0.r, L0.z, true, 1, &fused));
    if (fused) return FLUB_OK;  // p = z and z.r in the last level-0 half-sweep
    if (v8)
        return launch_pdl(k8_dot_zr<true, false>, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.z, L0.r, mg->p, L0.code,
                          mg->n, mg->partials, (const int *)L0.act, (const int *)L0.act_n, c.kc);
    return launch_pdl(k_dot_zr_init, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.z, L0.r, mg->p, mg->n,
                      mg->partials, c.kc);
}

// Ap, alpha, r update, r.r, convergence test, loop condition.
static int enqueue_first_half(flub_mg *mg, const LaunchCtx &c, int smoother) {
    if (mg->precision == FLUB_PRECISION_MIXED) return enqueue_first_half_mixed(mg, c, smoother);
    const unsigned b = red_blocks(mg->n);
    const Level &L0 = mg->lv[0];
    const bool v8 = (L0.D.nz % 8) == 0;
    const unsigned bg = red_blocks(mg->n / 8 + 1);
    if (v8)
        FLUB_TRY(launch_pdl(k8_matvec_pap, dim3(matvec_blocks(mg->n / 8)), dim3(kRedThreads), 0, c.s, mg->st,
                            mg->p, mg->Ap, L0.code, (const uint16_t *)L0.sw, L0.D, mg->partials, (const int *)L0.act,
                            (const int *)L0.act_n, c.kc));
    else
        FLUB_TRY(launch_pdl(k_matvec_pap, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, mg->p, mg->Ap, L0.code, L0.D,
                            mg->partials, c.kc));
    if (smoother == FLUB_SMOOTHER_FRACTION) {
        FLUB_TRY(launch_pdl(k_update_r, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap, mg->n, c.kc));
        FLUB_TRY(enqueue_mean_removal(mg, c, 1));
        if (v8)
            return launch_pdl(k8_update_r_rr<false>, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap,
                              L0.code, mg->n, mg->partials, mg->hist, c.h, c.set_cond, (const int *)L0.act,
                              (const int *)L0.act_n, c.kc);
        return launch_pdl(k_update_r_rr<false>, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap, mg->n,
                          mg->partials, mg->hist, c.h, c.set_cond, c.kc);
    }
    if (v8)
        return launch_pdl(k8_update_r_rr<true>, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap, L0.code,
                          mg->n, mg->partials, mg->hist, c.h, c.set_cond, (const int *)L0.act,
                          (const int *)L0.act_n, c.kc);
    return launch_pdl(k_update_r_rr<true>, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.r, mg->Ap, mg->n,
                      mg->partials, mg->hist, c.h, c.set_cond, c.kc);
}

// z = M r, beta, x += alpha p, p = z + beta p, it += 1.
static int enqueue_second_half(flub_mg *mg, const LaunchCtx &c) {
    if (mg->precision == FLUB_PRECISION_MIXED) return enqueue_second_half_mixed(mg, c);
    const unsigned b = red_blocks(mg->n);
    const Level &L0 = mg->lv[0];
    bool fused = false;
    FLUB_TRY(enqueue_vcycle(mg, c, L0.r, L0.z, true, 2, &fused));
    if ((L0.D.nz % 8) == 0) {
        const unsigned bg = red_blocks(mg->n / 8 + 1);
        if (!fused)  // else beta came with the last level-0 half-sweep
            FLUB_TRY(launch_pdl(k8_dot_zr<false>, dim3(bg), dim3(kRedThreads), 0, c.s, mg->st, L0.z, L0.r,
                                (float *)nullptr, L0.code, mg->n, mg->partials, (const int *)L0.act,
                                (const int *)L0.act_n, c.kc));
        return launch_pdl(k8_update_xp<false>, dim3(blocks_for(mg->n / 8, 256, kNumSMs * 8)), dim3(256), 0, c.s,
                          mg->st, mg->x, mg->p, L0.z, L0.code, mg->n, (const int *)L0.act, (const int *)L0.act_n,
                          c.kc);
    }
    FLUB_TRY(launch_pdl(k_dot_zr_beta, dim3(b), dim3(kRedThreads), 0, c.s, mg->st, L0.z, L0.r, mg->n, mg->partials,
                        c.kc));
    return launch_pdl(k_update_xp, dim3(blocks_for(mg->n, 256)), dim3(256), 0, c.s, mg->st, mg->x, mg->p, L0.z, mg->n,
                      c.kc);
}

static int enqueue_epilogue(flub_mg *mg, const LaunchCtx &c) {
    const Level &L0 = mg->lv[0];
    if ((L0.D.nz % 8) == 0)
        return launch_pdl(k8_solve_end, dim3(blocks_for(mg->n / 8, 256, kNumSMs * 8)), dim3(256), 0, c.s, mg->st,
                          mg->x, mg->p, L0.code, mg->n, (const int *)L0.act, (const int *)L0.act_n, c.kc);
    return launch_pdl(k_solve_end, dim3(blocks_for(mg->n, 256)), dim3(256), 0, c.s, mg->st, mg->x, mg->p, mg->n,
                      c.kc);
}

// Builds prologue -> while(body) -> epilogue with stream capture.
static int build_graph(flub_mg *mg, int smoother, cudaGraphExec_t *out) {
    cudaStream_t s = mg->cap_stream, s2 = mg->cap_stream2;
    cudaGraph_t g = nullptr;
    int rc = FLUB_OK;
    const int64_t launches_before = flub_launch_count();
    FLUB_CHECK_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    auto abort_capture = [&](int code) {
        cudaGraph_t tmp = nullptr;
        cudaStreamEndCapture(s, &tmp);
        if (tmp) cudaGraphDestroy(tmp);
        cudaGetLastError();
        return code;
    };
    cudaStreamCaptureStatus cs;
    cudaGraph_t capg = nullptr;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &capg, nullptr, nullptr, nullptr) != cudaSuccess)
        return abort_capture((set_last_error("cudaStreamGetCaptureInfo failed"), FLUB_ERR_CUDA));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, capg, 0, 0);
    if (e != cudaSuccess)
        return abort_capture((set_last_error("cudaGraphConditionalHandleCreate: %s", cudaGetErrorString(e)),
                              FLUB_ERR_CUDA));
    LaunchCtx c{s, kernel_counter(mg), h, 1};
    if ((rc = enqueue_prologue(mg, c, smoother)) || (rc = enqueue_first_half(mg, c, smoother)))
        return abort_capture(rc);
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &capg, &deps, nullptr, &ndeps) != cudaSuccess)
        return abort_capture((set_last_error("cudaStreamGetCaptureInfo failed"), FLUB_ERR_CUDA));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    e = cudaGraphAddNode(&cnode, capg, deps, nullptr, ndeps, &cp);
    if (e != cudaSuccess)
        return abort_capture((set_last_error("cudaGraphAddNode(while): %s", cudaGetErrorString(e)), FLUB_ERR_CUDA));
    e = cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess)
        return abort_capture((set_last_error("cudaStreamUpdateCaptureDependencies: %s", cudaGetErrorString(e)),
                              FLUB_ERR_CUDA));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(s2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return abort_capture((set_last_error("cudaStreamBeginCaptureToGraph: %s", cudaGetErrorString(e)),
                              FLUB_ERR_CUDA));
    LaunchCtx c2{s2, kernel_counter(mg), h, 1};
    rc = enqueue_second_half(mg, c2);
    if (!rc) rc = enqueue_first_half(mg, c2, smoother);
    cudaGraph_t body_out = nullptr;
    e = cudaStreamEndCapture(s2, &body_out);
    if (rc || e != cudaSuccess) {
        if (!rc) set_last_error("cudaStreamEndCapture(body): %s", cudaGetErrorString(e));
        return abort_capture(rc ? rc : FLUB_ERR_CUDA);
    }
    if ((rc = enqueue_epilogue(mg, c))) return abort_capture(rc);
    FLUB_CHECK_CUDA(cudaStreamEndCapture(s, &g));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    // kernels captured into the graph are counted on the device when they run
    count_launches(launches_before - flub_launch_count());
    if (e != cudaSuccess) {
        set_last_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        return FLUB_ERR_CUDA;
    }
    return FLUB_OK;
}

static int read_info(flub_mg *mg, cudaStream_t s, flub_solve_info *info) {
    MgState h;
    FLUB_CHECK_CUDA(cudaMemcpyAsync(&h, mg->st, sizeof(MgState), cudaMemcpyDeviceToHost, s));
    FLUB_CHECK_CUDA(cudaStreamSynchronize(s));
    info->iterations = h.it;
    info->converged = h.converged;
    info->status = h.status;
    info->reserved = 0;
    info->rtr0 = h.rtr0;
    info->rtr = h.rtr;
    info->tol = h.tol;
    info->x0_scale = h.x0_scale;
    return FLUB_OK;
}

// Stencil words of every group of a level (nz % 8 == 0).
__global__ void __launch_bounds__(256) k_stencil_words(const uint8_t *__restrict__ code, uint16_t *__restrict__ sw,
                                                       Dims D) {
    const int ng = (int)(D.n() >> 3);
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int i, j, kg;
        group_ijk(g, D, i, j, kg);
        *reinterpret_cast<uint4 *>(sw + ((int64_t)g << 3)) = words8_from_codes(code, D, i, j, kg << 3, g << 3);
    }
}

// ---------------------------------------------------------------- warm-start support (no reference counterpart)

// Stencil words in the colour-split order of smooth_split.cuh: natural cell
// (i, j, k) -> element k >> 1 of row (i, j) in half (i + j + k) & 1.  One
// thread per natural 8-cell group.
__global__ void __launch_bounds__(256) k_split_words(const uint16_t *__restrict__ sw, uint16_t *__restrict__ sws,
                                                     Dims D) {
    const int ng = (int)(D.n() >> 3), hz = D.nz >> 1, hn = (int)(D.n() >> 1);
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        int i, j, kg;
        group_ijk(g, D, i, j, kg);
        const uint4 u = __ldg(reinterpret_cast<const uint4 *>(sw + ((size_t)g << 3)));
        const int h = (i * D.ny + j) * hz + 4 * kg, p = (i + j) & 1;
        uint32_t e[4], o[4];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const uint32_t w = word_at(u, m);
            if (((p + m) & 1) == 0) e[m >> 1] = w;
            else o[m >> 1] = w;
        }
        *reinterpret_cast<uint2 *>(sws + h) = make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
        *reinterpret_cast<uint2 *>(sws + hn + h) = make_uint2(o[0] | (o[1] << 16), o[2] | (o[3] << 16));
    }
}

__global__ void k_set_x0_scale(MgState *st, double v) { st->x0_scale = v; }

// gamma = (d . b) / (d . L d) over fluid cells: the multiple of d closest to
// the solution of L x = b in the energy norm.  Two FP64 sums, combined in a
// fixed order by the last block.
__global__ void __launch_bounds__(kRedThreads) k_x0_gamma(MgState *st, const float *__restrict__ d,
                                                          const float *__restrict__ b,
                                                          const uint8_t *__restrict__ code, Dims D,
                                                          double *partials) {
    __shared__ double red[32];
    const int64_t n = D.n();
    double s_ld = 0.0, s_b = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        if (code[c] != kCodeFluid) continue;
        int i, j, k, dd;
        unflatten(c, D, i, j, k);
        const float dc = d[c];
        const float ld = lap_at(d, code, i, j, k, D, c, dc, dd);
        s_ld = fma((double)dc, (double)ld, s_ld);
        s_b = fma((double)dc, (double)b[c], s_b);
    }
    const double bb = block_sum(s_b, red);
    __syncthreads();
    if (threadIdx.x == 0) partials[kMaxRedBlocks + blockIdx.x] = bb;
    double total;
    if (finish_partials(s_ld, partials, &st->ticket, red, &total)) {
        __syncthreads();
        double t2 = 0.0;
        for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) t2 += __ldcg(&partials[kMaxRedBlocks + q]);
        t2 = block_sum(t2, red);
        if (threadIdx.x == 0) {
            const double g = t2 / total;
            st->x0_scale = (total != 0.0 && isfinite(g)) ? g : 0.0;
        }
    }
}

// x = x0_scale * d on fluid cells, 0 elsewhere.
__global__ void __launch_bounds__(256) k_x0_apply(const MgState *__restrict__ st, const float *__restrict__ d,
                                                  const uint8_t *__restrict__ code, float *__restrict__ x, int64_t n) {
    const float g = (float)st->x0_scale;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        x[c] = code[c] == kCodeFluid ? __fmul_rn(g, d[c]) : 0.0f;
}

__global__ void __launch_bounds__(256) k_decode_codes(const uint8_t *__restrict__ code, int32_t *__restrict__ tag,
                                                      int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        tag[c] = decode_tag(code[c]);
}

// Coarse vector = sum of its 8 children (the V-cycle's restriction of a
// residual with z = 0), 0 at coarse cells that are not fluid.
__global__ void __launch_bounds__(256) k_restrict_vec(const float *__restrict__ f, const uint8_t *__restrict__ cc,
                                                      float *__restrict__ out, Dims C) {
    const int64_t n = C.n();
    const int64_t fy = 2 * (int64_t)C.ny, fz = 2 * (int64_t)C.nz;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        if (cc[q] != kCodeFluid) {
            out[q] = 0.0f;
            continue;
        }
        int I, J, K;
        unflatten(q, C, I, J, K);
        float s = 0.0f;
        for (int m = 0; m < 8; m++) {
            const int64_t c = ((2 * (int64_t)I + (m >> 2)) * fy + 2 * J + ((m >> 1) & 1)) * fz + 2 * K + (m & 1);
            s = __fadd_rn(s, f[c]);
        }
        out[q] = s;
    }
}

// Cell-centred trilinear interpolation from the coarse level to the fine
// level at fine fluid cells (0 elsewhere).  Fine cell 2I + e sits a quarter
// coarse cell from coarse cell I towards I - 1 (e = 0) or I + 1 (e = 1):
// weights 3/4 and 1/4 per axis.  Coarse fluid cells contribute their value,
// air cells 0 (Dirichlet), solid and out-of-domain cells are left out and
// the remaining weights renormalised.
// One thread per coarse cell (I, J, K) writes the 2 x 2 x 2 fine cells it
// covers (every level is half its parent on each axis).  The 27 coarse
// neighbours are loaded once into registers as a weight flag (inside the
// domain and not solid) and a value (0 unless fluid); each fine fluid cell
// accumulates its 8 corners in a fixed order (the coarse cell itself first,
// then the corners towards the fine cell, z fastest), w by adds and s by
// fmaf, and stores s / w.  A left-out corner adds 0 to w and fmaf(wt, 0, s)
// to s, which leave both unchanged (s starts at +0 and never becomes -0).
// Grid: row_grid(C.nx, C.ny, C.nz).
__global__ void __launch_bounds__(kRowThreads) k_prolong_trilinear(const float *__restrict__ xc,
                                                                    const uint8_t *__restrict__ cc, Dims C,
                                                                    const uint8_t *__restrict__ cf,
                                                                    float *__restrict__ xf) {
    const int K = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y, I = blockIdx.z;
    if (K >= C.nz) return;
    const int fy = 2 * C.ny, fz = 2 * C.nz;
    int64_t frow[4];
    uint16_t fcode[4];
    bool any = false;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        frow[r] = ((int64_t)(2 * I + (r >> 1)) * fy + 2 * J + (r & 1)) * fz + 2 * K;
        fcode[r] = __ldg(reinterpret_cast<const uint16_t *>(cf + frow[r]));
        any |= (fcode[r] & 0xff) == kCodeFluid || (fcode[r] >> 8) == kCodeFluid;
    }
    if (!any) {
#pragma unroll
        for (int r = 0; r < 4; r++) *reinterpret_cast<float2 *>(xf + frow[r]) = make_float2(0.0f, 0.0f);
        return;
    }
    float val[27];
    bool ok[27];
#pragma unroll
    for (int q = 0; q < 27; q++) {
        const int ii = I + q / 9 - 1, jj = J + (q / 3) % 3 - 1, kk = K + q % 3 - 1;
        const bool in = ii >= 0 && ii < C.nx && jj >= 0 && jj < C.ny && kk >= 0 && kk < C.nz;
        const int64_t cq = ((int64_t)ii * C.ny + jj) * C.nz + kk;
        const uint8_t code = in ? __ldg(cc + cq) : kCodeSolid;
        ok[q] = code != kCodeSolid;
        val[q] = code == kCodeFluid ? __ldg(xc + cq) : 0.0f;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
        float out[2];
#pragma unroll
        for (int ek = 0; ek < 2; ek++) {
            const int ei = r >> 1, ej = r & 1;
            const int oi = ei ? 1 : -1, oj = ej ? 1 : -1, ok3 = ek ? 1 : -1;
            float s = 0.0f, w = 0.0f;
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int a = (m >> 2) ? oi : 0, bq = ((m >> 1) & 1) ? oj : 0, e = (m & 1) ? ok3 : 0;
                const int q = (a + 1) * 9 + (bq + 1) * 3 + (e + 1);
                const float wt = (a ? 0.25f : 0.75f) * (bq ? 0.25f : 0.75f) * (e ? 0.25f : 0.75f);
                w += ok[q] ? wt : 0.0f;
                s = fmaf(wt, val[q], s);
            }
            const uint8_t fc = ek ? (uint8_t)(fcode[r] >> 8) : (uint8_t)(fcode[r] & 0xff);
            out[ek] = fc != kCodeFluid ? 0.0f : (w > 0.0f ? s / w : 0.0f);
        }
        *reinterpret_cast<float2 *>(xf + frow[r]) = make_float2(out[0], out[1]);
    }
}

}  // namespace flub

using namespace flub;

extern "C" {

size_t flub_mg_workspace_bytes(int nx, int ny, int nz, int levels, int precision) {
    if (validate_shape(nx, ny, nz, levels, precision)) return 0;
    flub_mg tmp;
    memset(&tmp, 0, sizeof(tmp));
    reference_schedule(&tmp);
    tmp.nx = nx; tmp.ny = ny; tmp.nz = nz; tmp.levels = levels; tmp.precision = precision;
    tmp.n = (int64_t)nx * ny * nz;
    tmp.tile_ok = tile_requested();
    tmp.split_ok = split_requested();
    return carve(&tmp, nullptr);
}

int flub_mg_create(int nx, int ny, int nz, int levels, int precision, void *workspace, size_t workspace_bytes,
                   flub_mg **out) {
    FLUB_REQUIRE(out != nullptr, "flub_mg_create: out is NULL");
    *out = nullptr;
    FLUB_TRY(validate_shape(nx, ny, nz, levels, precision));
    flub_mg *mg = new flub_mg;
    memset(mg, 0, sizeof(*mg));
    reference_schedule(mg);
    mg->nx = nx; mg->ny = ny; mg->nz = nz; mg->levels = levels; mg->precision = precision;
    mg->n = (int64_t)nx * ny * nz;
    mg->tile_ok = tile_requested();    // decides the tile buffers carved below
    mg->split_ok = split_requested();  // and the colour-split ones
    const size_t need = carve(mg, nullptr);
    if (workspace) {
        if (workspace_bytes < need || ((uintptr_t)workspace & 255)) {
            delete mg;
            set_last_error("workspace of %zu bytes at %p: need %zu bytes, 256-byte aligned", workspace_bytes,
                           workspace, need);
            return FLUB_ERR_INVALID_ARGUMENT;
        }
        mg->ws = workspace;
        mg->own_ws = false;
    } else {
        cudaError_t e = cudaMalloc(&mg->ws, need);
        if (e != cudaSuccess) {
            delete mg;
            set_last_error("cudaMalloc(%zu): %s", need, cudaGetErrorString(e));
            cudaGetLastError();
            return FLUB_ERR_OUT_OF_MEMORY;
        }
        mg->own_ws = true;
    }
    mg->ws_bytes = need;
    carve(mg, (char *)mg->ws);
    cudaGetDevice(&mg->device);
    if (cudaStreamCreateWithFlags(&mg->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&mg->cap_stream2, cudaStreamNonBlocking) != cudaSuccess) {
        flub_mg_destroy(mg);
        set_last_error("cudaStreamCreate failed");
        return FLUB_ERR_CUDA;
    }
    const char *hl = getenv("FLUB_SOLVE_HOST_LOOP");
    mg->host_loop = hl && hl[0] == '1';
    mg->skip_ok = true;  // the workspace is zeroed below and set_tags re-zeroes the z buffers
    choose_tail(mg);
    choose_cluster(mg);
    choose_persist(mg);
    if (precision == FLUB_PRECISION_MIXED && bottom_in_tail(mg)) {
        // mixed precision: FP64 at the coarsest level (the tail layouts grow by
        // the bottom's doubles, so they are chosen again)
        mg->bottom64 = true;
        choose_tail(mg);
        choose_cluster(mg);
        if (!bottom_in_tail(mg)) {
            mg->bottom64 = false;
            choose_tail(mg);
            choose_cluster(mg);
        }
    }
    if (precision == FLUB_PRECISION_MIXED) {
        // the FP16 sweeps work on rows of 8 cells: every level left to the global
        // kernels needs nz % 8 == 0
        const int lt = mg->cl_start < mg->levels ? mg->cl_start : mg->tail_start;
        const int last_global = lt < mg->levels ? lt - 1 : mg->levels - 1;
        for (int l = 0; l <= last_global; l++)
            if (mg->lv[l].D.nz % 8 != 0) {
                flub_mg_destroy(mg);
                set_last_error("mixed precision needs nz %% 8 == 0 on level %d (nz = %d)", l, nz >> l);
                return FLUB_ERR_UNSUPPORTED;
            }
    }
    if (set_tail_smem_limit() != FLUB_OK) {
        flub_mg_destroy(mg);
        return FLUB_ERR_CUDA;
    }
    // zero the state and all vectors once so that every buffer is defined
    if (cudaMemset(mg->ws, 0, need) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        flub_mg_destroy(mg);
        set_last_error("workspace initialisation failed");
        return FLUB_ERR_CUDA;
    }
    *out = mg;
    return FLUB_OK;
}

int flub_mg_destroy(flub_mg *mg) {
    if (!mg) return FLUB_OK;
    for (int s = 0; s < 3; s++)
        if (mg->graph[s]) cudaGraphExecDestroy(mg->graph[s]);
    if (mg->cap_stream) cudaStreamDestroy(mg->cap_stream);
    if (mg->cap_stream2) cudaStreamDestroy(mg->cap_stream2);
    if (mg->own_ws && mg->ws) cudaFree(mg->ws);
    delete mg;
    return FLUB_OK;
}

int flub_mg_set_tags(flub_mg *mg, const int32_t *tag, void *stream) {
    FLUB_REQUIRE(mg && tag, "flub_mg_set_tags: NULL argument");
    cudaStream_t s = as_stream(stream);
    if (mg->n % 4 == 0 && (uintptr_t)tag % 16 == 0)
        k_encode_tags4<<<blocks_for(mg->n / 4, 256), 256, 0, s>>>(reinterpret_cast<const int4 *>(tag),
                                                                  reinterpret_cast<uint32_t *>(mg->lv[0].code),
                                                                  mg->n / 4);
    else
        k_encode_tags<<<blocks_for(mg->n, 256), 256, 0, s>>>(tag, mg->lv[0].code, mg->n);
    FLUB_CHECK_LAUNCH();
    for (int l = 0; l + 1 < mg->levels; l++) {
        const Level &C = mg->lv[l + 1];
        k_restrict_codes<<<blocks_for(C.D.n(), 256), 256, 0, s>>>(mg->lv[l].code, C.code, C.D);
        FLUB_CHECK_LAUNCH();
    }
    for (int l = 0; l < mg->levels; l++) {
        const Level &L = mg->lv[l];
        if (!L.pmask) continue;
        k_tail_masks<<<blocks_for(L.D.n() >> 1, 256), 256, 0, s>>>(L.code, L.D, L.pmask);
        FLUB_CHECK_LAUNCH();
    }
    // stencil words and active 8-cell groups of every level that has them
    for (int l = 0; l < mg->levels; l++) {
        const Level &L = mg->lv[l];
        if (L.sw) {
            k_stencil_words<<<blocks_for(L.D.n() >> 3, 256), 256, 0, s>>>(L.code, L.sw, L.D);
            FLUB_CHECK_LAUNCH();
        }
        if (L.sws) {
            k_split_words<<<blocks_for(L.D.n() >> 3, 256), 256, 0, s>>>(L.sw, L.sws, L.D);
            FLUB_CHECK_LAUNCH();
            FLUB_CHECK_CUDA(cudaMemsetAsync(L.zs, 0, sizeof(float) * (size_t)L.D.n(), s));
        }
        if (!L.act) continue;
        const int ng = (int)(L.D.n() >> 3);
        const int nb = (ng + kActPerBlock - 1) / kActPerBlock;
        k_act_count<<<nb, kActThreads, 0, s>>>(L.code, ng, mg->act_scratch);
        FLUB_CHECK_LAUNCH();
        k_act_scan<<<1, kActThreads, 0, s>>>(mg->act_scratch, nb, L.act_n);
        FLUB_CHECK_LAUNCH();
        k_act_write<<<nb, kActThreads, 0, s>>>(L.code, ng, mg->act_scratch, L.act);
        FLUB_CHECK_LAUNCH();
        if (L.n_tiles) {
            FLUB_CHECK_CUDA(cudaMemsetAsync(L.tflags, 0, (size_t)L.n_tiles, s));
            FLUB_CHECK_CUDA(cudaMemsetAsync(L.tiles_n, 0, sizeof(int), s));
            k_tile_flags<<<blocks_for(ng, 256, kNumSMs * 8), 256, 0, s>>>(L.act, L.act_n, L.D, L.tflags);
            FLUB_CHECK_LAUNCH();
            k_tile_list<<<blocks_for(L.n_tiles, 256), 256, 0, s>>>(L.tflags, L.n_tiles, L.tiles, L.tiles_n);
            FLUB_CHECK_LAUNCH();
        }
    }
    // new tags: re-establish z = p = Ap = 0 off the fluid (the kernels skip
    // 8-cell groups without fluid and rely on it)
    for (int l = 0; l < mg->levels; l++) {
        const Level &L = mg->lv[l];
        const size_t b = sizeof(float) * (size_t)L.D.n();
        // one clear per level over the consecutive buffers carve() laid out
        // (r, z, z2, then the FP16 rh, zh, z2h): the coarse residuals (the
        // list-based restriction writes only groups with fluid, the others must
        // read 0) and every correction buffer; level 0 keeps its r (the CG
        // residual) and its FP16 copy is rewritten before each use
        char *first = l > 0 ? reinterpret_cast<char *>(L.r) : reinterpret_cast<char *>(L.z);
        char *last = L.z2h ? reinterpret_cast<char *>(L.z2h) + b / 2 : reinterpret_cast<char *>(L.z2) + b;
        FLUB_CHECK_CUDA(cudaMemsetAsync(first, 0, (size_t)(last - first), s));
        if (L.z3) FLUB_CHECK_CUDA(cudaMemsetAsync(L.z3, 0, b, s));
    }
    FLUB_CHECK_CUDA(cudaMemsetAsync(mg->p, 0, sizeof(float) * (size_t)mg->n, s));
    FLUB_CHECK_CUDA(cudaMemsetAsync(mg->Ap, 0, sizeof(float) * (size_t)mg->n, s));
    return FLUB_OK;
}

int flub_mg_init(flub_mg *mg, const float *rhs, float k, void *stream) {
    FLUB_REQUIRE(mg && rhs, "flub_mg_init: NULL argument");
    k_init<<<blocks_for(mg->n, 256), 256, 0, as_stream(stream)>>>(mg->lv[0].r, rhs, k, mg->x, mg->p, mg->n);
    FLUB_CHECK_LAUNCH();
    mg->use_x0 = false;
    mg->r_masked = false;
    return FLUB_OK;
}

int flub_mg_mask_interior(flub_mg *mg, void *stream) {
    FLUB_REQUIRE(mg, "flub_mg_mask_interior: NULL handle");
    if (mg->n % 4 == 0)
        k_mask_interior4<<<blocks_for(mg->n / 4, 256), 256, 0, as_stream(stream)>>>(
            reinterpret_cast<float4 *>(mg->lv[0].r), reinterpret_cast<const uint32_t *>(mg->lv[0].code), mg->n / 4);
    else
        k_mask_interior<<<blocks_for(mg->n, 256), 256, 0, as_stream(stream)>>>(mg->lv[0].r, mg->lv[0].code, mg->n);
    FLUB_CHECK_LAUNCH();
    mg->r_masked = true;
    return FLUB_OK;
}

int flub_mg_set_x0(flub_mg *mg, const float *x0, void *stream) {
    FLUB_REQUIRE(mg && x0, "flub_mg_set_x0: NULL argument");
    FLUB_CHECK_CUDA(cudaMemcpyAsync(mg->x, x0, sizeof(float) * mg->n, cudaMemcpyDeviceToDevice, as_stream(stream)));
    k_set_x0_scale<<<1, 1, 0, as_stream(stream)>>>(mg->st, 1.0);
    FLUB_CHECK_LAUNCH();
    mg->use_x0 = true;
    return FLUB_OK;
}

int flub_mg_solve(flub_mg *mg, int max_iters, double eps, double abs_tol, double rel_tol, int smoother,
                  void *stream, flub_solve_info *info) {
    FLUB_REQUIRE(mg, "flub_mg_solve: NULL handle");
    if (smoother != FLUB_SMOOTHER_PHASES && smoother != FLUB_SMOOTHER_FRACTION) {
        set_last_error("smoother %d not supported (only \"phases\" and \"fraction\"; the untagged \"default\" "
                       "smoother is not part of this library)", smoother);
        return FLUB_ERR_UNSUPPORTED;
    }
    if (max_iters < 0) max_iters = 100000;
    cudaStream_t s = as_stream(stream);
    // r.r may skip groups without fluid once r is 0 there: after mask_interior,
    // or with "fraction", whose mean removal zeroes r off the fluid first
    const int skip_r = (mg->r_masked || smoother == FLUB_SMOOTHER_FRACTION) ? 1 : 0;
    k_solve_begin<<<1, 1, 0, s>>>(mg->st, max_iters, eps, abs_tol, rel_tol, mg->use_x0 ? 1 : 0, skip_r);
    FLUB_CHECK_LAUNCH();
    mg->use_x0 = false;
    if (mg->host_loop) {
        LaunchCtx c{s, nullptr, 0, 0};
        FLUB_TRY(enqueue_prologue(mg, c, smoother));
        FLUB_TRY(enqueue_first_half(mg, c, smoother));
        for (int guard = 0; guard <= max_iters; guard++) {
            MgState h;
            FLUB_CHECK_CUDA(cudaMemcpyAsync(&h, mg->st, sizeof(MgState), cudaMemcpyDeviceToHost, s));
            FLUB_CHECK_CUDA(cudaStreamSynchronize(s));
            if (!h.cond) break;
            FLUB_TRY(enqueue_second_half(mg, c));
            FLUB_TRY(enqueue_first_half(mg, c, smoother));
        }
        FLUB_TRY(enqueue_epilogue(mg, c));
    } else {
        const int gi = smoother;
        if (!mg->graph[gi]) FLUB_TRY(build_graph(mg, smoother, &mg->graph[gi]));
        FLUB_CHECK_CUDA(cudaGraphLaunch(mg->graph[gi], s));
    }
    if (info) return read_info(mg, s, info);
    return FLUB_OK;
}

int flub_mg_get_info(flub_mg *mg, void *stream, flub_solve_info *info) {
    FLUB_REQUIRE(mg && info, "flub_mg_get_info: NULL argument");
    return read_info(mg, as_stream(stream), info);
}

int flub_mg_residual_history(flub_mg *mg, void *stream, double *out, int max_n, int *n_out) {
    FLUB_REQUIRE(mg && out && n_out && max_n >= 0, "flub_mg_residual_history: bad argument");
    flub_solve_info info;
    FLUB_TRY(read_info(mg, as_stream(stream), &info));
    int n = info.converged ? info.iterations + 1 : info.iterations;
    if (n > kHistory) n = kHistory;
    if (n > max_n) n = max_n;
    if (n > 0) {
        FLUB_CHECK_CUDA(cudaMemcpy(out, mg->hist, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    *n_out = n;
    return FLUB_OK;
}

int flub_mg_set_schedule(flub_mg *mg, int smooth_iters, int bottom_iters, float restrict_scale) {
    FLUB_REQUIRE(mg, "flub_mg_set_schedule: NULL handle");
    FLUB_REQUIRE(smooth_iters == -1 || (smooth_iters >= 1 && smooth_iters <= 64),
                 "flub_mg_set_schedule: smooth_iters must be -1 (the reference's 6 << level) or 1..64, got %d",
                 smooth_iters);
    FLUB_REQUIRE(bottom_iters >= 1 && bottom_iters <= 64, "flub_mg_set_schedule: bottom_iters must be 1..64, got %d",
                 bottom_iters);
    FLUB_REQUIRE(restrict_scale > 0.0f && restrict_scale <= 1.0f,
                 "flub_mg_set_schedule: restrict_scale must be in (0, 1], got %g", (double)restrict_scale);
    if (mg->sched_nu == smooth_iters && mg->sched_bottom == bottom_iters && mg->sched_rscale == restrict_scale)
        return FLUB_OK;
    // the captured solve graphs embed the schedule: drop them (recaptured by the next solve)
    FLUB_CHECK_CUDA(cudaDeviceSynchronize());
    for (int g = 0; g < 3; g++)
        if (mg->graph[g]) {
            cudaGraphExecDestroy(mg->graph[g]);
            mg->graph[g] = nullptr;
        }
    mg->sched_nu = smooth_iters;
    mg->sched_bottom = bottom_iters;
    mg->sched_rscale = restrict_scale;
    // the cluster kernel's layout depends on the schedule
    FLUB_TRY(choose_cluster(mg));
    return FLUB_OK;
}

int flub_mg_set_bottom_precision(flub_mg *mg, int bits) {
    FLUB_REQUIRE(mg, "flub_mg_set_bottom_precision: NULL handle");
    FLUB_REQUIRE(bits == 32 || bits == 64, "flub_mg_set_bottom_precision: bits must be 32 or 64, got %d", bits);
    const bool want = bits == 64;
    if (mg->bottom64 == want) return FLUB_OK;
    if (want && !bottom_in_tail(mg)) {
        set_last_error("flub_mg_set_bottom_precision: the bottom level does not run in the one-block tail here "
                       "(FP64 bottom needs it)");
        return FLUB_ERR_UNSUPPORTED;
    }
    FLUB_CHECK_CUDA(cudaDeviceSynchronize());
    for (int g = 0; g < 3; g++)
        if (mg->graph[g]) {
            cudaGraphExecDestroy(mg->graph[g]);
            mg->graph[g] = nullptr;
        }
    mg->bottom64 = want;
    choose_tail(mg);
    FLUB_TRY(choose_cluster(mg));
    if (want && !bottom_in_tail(mg)) {
        mg->bottom64 = false;
        choose_tail(mg);
        choose_cluster(mg);
        set_last_error("flub_mg_set_bottom_precision: the FP64 bottom does not fit the coarse-level kernels");
        return FLUB_ERR_UNSUPPORTED;
    }
    return FLUB_OK;
}

int flub_mg_get_bottom_precision(flub_mg *mg, int *bits) {
    FLUB_REQUIRE(mg && bits, "flub_mg_get_bottom_precision: NULL argument");
    *bits = mg->bottom64 ? 64 : 32;
    return FLUB_OK;
}

int flub_mg_set_x0_scaled(flub_mg *mg, const float *d, void *stream) {
    FLUB_REQUIRE(mg && d, "flub_mg_set_x0_scaled: NULL argument");
    FLUB_REQUIRE(d != mg->x, "flub_mg_set_x0_scaled: d must not be the solution vector itself");
    cudaStream_t s = as_stream(stream);
    const Level &L0 = mg->lv[0];
    if (L0.act)
        k8_x0_gamma<<<red_blocks(mg->n / 8 + 1), kRedThreads, 0, s>>>(mg->st, d, L0.r, L0.code, L0.sw, L0.D,
                                                                     mg->partials, L0.act, L0.act_n);
    else
        k_x0_gamma<<<red_blocks(mg->n), kRedThreads, 0, s>>>(mg->st, d, L0.r, L0.code, L0.D, mg->partials);
    FLUB_CHECK_LAUNCH();
    k_x0_apply<<<blocks_for(mg->n, 256), 256, 0, s>>>(mg->st, d, L0.code, mg->x, mg->n);
    FLUB_CHECK_LAUNCH();
    mg->use_x0 = true;
    return FLUB_OK;
}

int flub_mg_level_shape(flub_mg *mg, int level, int *nx, int *ny, int *nz) {
    FLUB_REQUIRE(mg && nx && ny && nz, "flub_mg_level_shape: NULL argument");
    FLUB_REQUIRE(level >= 0 && level < mg->levels, "flub_mg_level_shape: level %d outside [0, %d)", level,
                 mg->levels);
    *nx = mg->lv[level].D.nx;
    *ny = mg->lv[level].D.ny;
    *nz = mg->lv[level].D.nz;
    return FLUB_OK;
}

int flub_mg_level_tags(flub_mg *mg, int level, int32_t *tag, void *stream) {
    FLUB_REQUIRE(mg && tag, "flub_mg_level_tags: NULL argument");
    FLUB_REQUIRE(level >= 0 && level < mg->levels, "flub_mg_level_tags: level %d outside [0, %d)", level, mg->levels);
    const Level &L = mg->lv[level];
    k_decode_codes<<<blocks_for(L.D.n(), 256), 256, 0, as_stream(stream)>>>(L.code, tag, L.D.n());
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_mg_restrict_vector(flub_mg *mg, int level, const float *fine, float *coarse, void *stream) {
    FLUB_REQUIRE(mg && fine && coarse, "flub_mg_restrict_vector: NULL argument");
    FLUB_REQUIRE(level >= 1 && level < mg->levels, "flub_mg_restrict_vector: level %d outside [1, %d)", level,
                 mg->levels);
    const Level &L = mg->lv[level];
    k_restrict_vec<<<blocks_for(L.D.n(), 256), 256, 0, as_stream(stream)>>>(fine, L.code, coarse, L.D);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_mg_prolong_vector(flub_mg *mg, int level, const float *coarse, float *fine, void *stream) {
    FLUB_REQUIRE(mg && fine && coarse, "flub_mg_prolong_vector: NULL argument");
    FLUB_REQUIRE(level >= 1 && level < mg->levels, "flub_mg_prolong_vector: level %d outside [1, %d)", level,
                 mg->levels);
    const Level &C = mg->lv[level], &F = mg->lv[level - 1];
    k_prolong_trilinear<<<row_grid(C.D.nx, C.D.ny, C.D.nz), kRowThreads, 0, as_stream(stream)>>>(coarse, C.code,
                                                                                                 C.D, F.code, fine);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

float *flub_mg_x(flub_mg *mg) { return mg ? mg->x : nullptr; }
float *flub_mg_r(flub_mg *mg) { return mg ? mg->lv[0].r : nullptr; }

int flub_mg_get_x(flub_mg *mg, float *out, float scale, void *stream) {
    FLUB_REQUIRE(mg && out, "flub_mg_get_x: NULL argument");
    k_scale_copy<<<blocks_for(mg->n, 256), 256, 0, as_stream(stream)>>>(out, mg->x, scale, mg->n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_mg_apply_preconditioner(flub_mg *mg, const float *r, float *z, void *stream) {
    FLUB_REQUIRE(mg && r && z, "flub_mg_apply_preconditioner: NULL argument");
    LaunchCtx c{as_stream(stream), nullptr, 0, 0};
    if (mg->precision == FLUB_PRECISION_MIXED) {
        FLUB_TRY(launch_pdl(k8_to_half, dim3(blocks_for(mg->n / 8, 256)), dim3(256), 0, c.s, (MgState *)nullptr, r, mg->lv[0].rh, mg->n,
                            c.kc));
        return enqueue_vcycle_mixed(mg, c, z, false);
    }
    return enqueue_vcycle(mg, c, r, z, false);
}

int flub_mg_matvec(flub_mg *mg, const float *p, float *Ap, void *stream) {
    FLUB_REQUIRE(mg && p && Ap, "flub_mg_matvec: NULL argument");
    const Level &L0 = mg->lv[0];
    k_matvec<<<blocks_for(mg->n, 256), 256, 0, as_stream(stream)>>>(p, Ap, L0.code, L0.D);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_mg_smooth(flub_mg *mg, int level, int phase, void *stream) {
    FLUB_REQUIRE(mg, "flub_mg_smooth: NULL handle");
    FLUB_REQUIRE(level >= 0 && level < mg->levels, "flub_mg_smooth: level %d outside [0, %d)", level, mg->levels);
    FLUB_REQUIRE(phase == 0 || phase == 1, "flub_mg_smooth: phase must be 0 or 1");
    LaunchCtx c{as_stream(stream), nullptr, 0, 0};
    const Level &L = mg->lv[level];
    return sweep(c, L, phase, kSweepInPlace, mg->skip_ok ? 1 : 0, L.r, L.z, L.z, nullptr);
}

int flub_mg_smooth_iteration(flub_mg *mg, int level, int phase, int *tiled, void *stream) {
    FLUB_REQUIRE(mg, "flub_mg_smooth_iteration: NULL handle");
    FLUB_REQUIRE(level >= 0 && level < mg->levels, "flub_mg_smooth_iteration: level %d outside [0, %d)", level,
                 mg->levels);
    FLUB_REQUIRE(phase == 0 || phase == 1, "flub_mg_smooth_iteration: phase must be 0 or 1");
    LaunchCtx c{as_stream(stream), nullptr, 0, 0};
    const Level &L = mg->lv[level];
    const bool t = mg->tile_ok && L.n_tiles > 0 && mg->skip_ok;
    if (tiled) *tiled = t ? 1 : 0;
    if (!t && level == 0 && L.sws && mg->skip_ok) {
        // the colour-split kernels the V-cycle runs at level 0, in place on the
        // post-smoothing buffer with the split residual of the last V-cycle
        if (tiled) *tiled = 2;
        for (int ph : {phase, 1 - phase}) {
            if (mg->precision == FLUB_PRECISION_MIXED)
                FLUB_TRY((split_sweep<kInPlace, __half, __half, float, float, float>(
                    c, L, ph, nullptr, L.rsh, nullptr, L.zs, nullptr, 1.0f, nullptr)));
            else
                FLUB_TRY((split_sweep<kInPlace, float, float, float, float, float>(c, L, ph, nullptr, L.rs, nullptr,
                                                                                  L.zs, nullptr, 1.0f, nullptr)));
        }
        return FLUB_OK;
    }
    if (t) {
        // z -> z3 and z3 -> z on alternate calls (both keep 0 off the fluid);
        // the handle's pointers stay as the captured solve graphs know them
        const bool back = mg->iter_toggle[level];
        mg->iter_toggle[level] = !back;
        return tile_iteration(mg, c, level, phase, kTileInPlaceInput, L.r, back ? L.z3 : L.z, back ? L.z : L.z3,
                              nullptr);
    }
    FLUB_TRY(sweep(c, L, phase, kSweepInPlace, mg->skip_ok ? 1 : 0, L.r, L.z, L.z, nullptr));
    return sweep(c, L, 1 - phase, kSweepInPlace, mg->skip_ok ? 1 : 0, L.r, L.z, L.z, nullptr);
}

int flub_mg_kernels_executed(flub_mg *mg, void *stream, int64_t *out) {
    FLUB_REQUIRE(mg && out, "flub_mg_kernels_executed: NULL argument");
    unsigned long long v = 0;
    cudaStream_t s = as_stream(stream);
    FLUB_CHECK_CUDA(cudaMemcpyAsync(&v, kernel_counter(mg), sizeof(v), cudaMemcpyDeviceToHost, s));
    FLUB_CHECK_CUDA(cudaStreamSynchronize(s));
    *out = (int64_t)v;
    return FLUB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- allocation-free V-cycle
//
// For callers that cannot allocate device memory: a plugin whose host
// application owns every device allocation (and forbids cudaMalloc inside its
// frame loop), or a real-time caller that cannot afford cudaMalloc's implicit
// synchronisation.  flub_vcycle_noalloc keeps the whole level hierarchy in the
// file-scope device array below instead of a workspace; the caller only passes
// the tags, r and z.  The array holds grids of up to FLUB_NOALLOC_MAX_CELLS
// cells and stays resident on every device that loads this library until the
// process exits.

namespace flub {

constexpr size_t kNoallocScratchBytes = size_t(2) << 20;  // 2 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Layout inside the array: level-0 cell codes and pre-smoothing buffer, then
// (codes, r, z, z2) of every coarser level, each 256-byte aligned.  Returns
// the bytes used.
static size_t noalloc_layout(flub_mg *mg, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char * {
        char *p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    for (int l = 0; l < mg->levels; l++) {
        Level &L = mg->lv[l];
        L.D = Dims{mg->nx >> l, mg->ny >> l, mg->nz >> l};
        L.code = (uint8_t *)take((size_t)L.D.n());
        L.r = l ? (float *)take(sizeof(float) * L.D.n()) : nullptr;
        L.z = l ? (float *)take(sizeof(float) * L.D.n()) : nullptr;
        L.z2 = (float *)take(sizeof(float) * L.D.n());
        L.pmask = nullptr;  // the tail builds its masks from the codes
    }
    return off;
}

static std::mutex g_noalloc_mutex;
static void *g_noalloc_addr[64];

// Device address of g_noalloc_scratch on the current device, looked up once per
// device with that device current (a host-side use of the symbol's name is not
// a device address).
static int noalloc_scratch_address(void **out) {
    int dev = 0;
    FLUB_CHECK_CUDA(cudaGetDevice(&dev));
    FLUB_REQUIRE(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_last_error("cudaGetSymbolAddress(g_noalloc_scratch) on device %d: %s", dev, cudaGetErrorString(e));
            cudaGetLastError();
            return FLUB_ERR_CUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return FLUB_OK;
}

}  // namespace flub

extern "C" int flub_vcycle_noalloc(const int32_t *tag, const float *r, float *z, int nx, int ny, int nz, int levels,
                                   void *stream) {
    FLUB_REQUIRE(tag && r && z, "flub_vcycle_noalloc: NULL argument");
    FLUB_TRY(validate_shape(nx, ny, nz, levels, FLUB_PRECISION_FP32));
    const int64_t n = (int64_t)nx * ny * nz;
    FLUB_REQUIRE(n <= FLUB_NOALLOC_MAX_CELLS,
                 "flub_vcycle_noalloc: %lld cells exceed the allocation-free limit of %d cells (64^3)", (long long)n,
                 FLUB_NOALLOC_MAX_CELLS);
    flub_mg mg;  // host-side descriptor only; every level pointer points into the static array
    memset(&mg, 0, sizeof(mg));
    reference_schedule(&mg);
    mg.nx = nx; mg.ny = ny; mg.nz = nz; mg.levels = levels; mg.n = n;
    const size_t need = noalloc_layout(&mg, nullptr);
    FLUB_REQUIRE(need <= kNoallocScratchBytes, "flub_vcycle_noalloc: hierarchy needs %zu bytes > %zu", need,
                 kNoallocScratchBytes);
    void *base = nullptr;
    FLUB_TRY(noalloc_scratch_address(&base));
    noalloc_layout(&mg, (char *)base);
    choose_tail(&mg);
    choose_cluster(&mg);
    FLUB_TRY(set_tail_smem_limit());
    cudaStream_t s = as_stream(stream);
    // every scratch element is written before it is read: the codes by these two
    // kernels, z_l by the first (from-zero) sweep of its level, r_l by the
    // restriction, so nothing has to be cleared between calls
    k_encode_tags<<<blocks_for(n, 256), 256, 0, s>>>(tag, mg.lv[0].code, n);
    FLUB_CHECK_LAUNCH();
    for (int l = 0; l + 1 < levels; l++) {
        const Level &C = mg.lv[l + 1];
        k_restrict_codes<<<blocks_for(C.D.n(), 256), 256, 0, s>>>(mg.lv[l].code, C.code, C.D);
        FLUB_CHECK_LAUNCH();
    }
    LaunchCtx c{s, nullptr, 0, 0};
    return enqueue_vcycle(&mg, c, r, z, false);  // mg.skip_ok is false: every sweep writes every cell
}
