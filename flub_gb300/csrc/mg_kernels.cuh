// Device kernels of the MGPCG solver (multigrid/mgpcg.py).
//
// Operator conventions (multigrid/mgpcg.py:118-160): for a fluid cell,
//   L x = sum over axes (i, j, k) of [t(+1) + t(-1)],
//   t = (x_nb or 0 if the neighbour is air) - x_c for an in-domain non-solid
//   neighbour, 0 otherwise;  diag = number of such neighbours.
// L x = 0 at non-fluid cells.  Cells are stored as one byte code (common.cuh).
// All FP32 arithmetic uses explicit round-to-nearest intrinsics in the
// reference's order so that the CPU oracle reproduces it bit for bit.
#pragma once

#include "common.cuh"

namespace flub {

constexpr int kRedThreads = 256;
constexpr int kMaxRedBlocks = 2048;
constexpr int kHistory = 4096;

// Device-side solver state (one per handle).
struct MgState {
    double rtr0, tol, rtr, zr_old, pap, alpha, beta, eps, abs_tol, rel_tol;
    double mean;                 // zero_centered mean (FP64 sum / count)
    double x0_scale;             // scale applied to the initial guess (0: no guess)
    unsigned long long kernels;  // solver kernels executed inside graphs
    int it, max_iters, converged, status, cond, use_x0;
    unsigned int ticket;
    int skip_r;    // r is 0 off the fluid (masked), so r.r may skip groups without fluid
    float zscale;  // mixed precision: z = zscale * (V-cycle output); the FP16 residual copy is r / zscale
    float pad_;
    unsigned int bar_count, bar_gen;  // grid barrier of the persistent V-cycle kernels (persist.cuh)
};

// Power of two near 1 / RMS of a vector with squared norm rtr over n entries:
// the FP16 residual copy is stored at this scale so that it neither overflows
// nor underflows as CG drives the residual down by orders of magnitude.
__device__ __forceinline__ float fp16_residual_scale(double rtr, int64_t n) {
    if (!(rtr > 0.0) || !isfinite(rtr)) return 1.0f;
    int e = ilogb(sqrt(rtr / (double)n));
    e = e < -100 ? -100 : (e > 100 ? 100 : e);
    return ldexpf(1.0f, -e);
}

// fp16_residual_scale evaluated once per block by thread 0 and shared: the
// FP64 divide and square root cost tens of FP64 instructions, which at this
// GPU's FP64 rate dominate a streaming kernel when every thread repeats them.
// Every thread of the block must reach the call.
__device__ __forceinline__ float block_fp16_residual_scale(double rtr, int64_t n) {
    __shared__ float s_hs;
    if (threadIdx.x == 0) s_hs = fp16_residual_scale(rtr, n);
    __syncthreads();
    return s_hs;
}

struct Dims {
    int nx, ny, nz;
    __host__ __device__ int64_t n() const { return (int64_t)nx * ny * nz; }
};

// Sum of x[m] * y[m] over the 8 cells of a group, returned as a double.  Each
// product is split exactly into p + e with an FMA (Dekker), and the running
// sum is kept as an unevaluated pair (hi, lo) by two-sum (Knuth), all in FP32
// arithmetic; the pair is converted once.  The result agrees with an FP64
// accumulation of the exact products to about 2^-44 of sum |x y|, while the
// FP64 unit, which this GPU runs at a small fraction of the FP32 rate, sees
// one add per group instead of eight fused multiply-adds and sixteen
// conversions.
__device__ __forceinline__ double dot8_ff(const float *x, const float *y) {
    float hi = 0.0f, lo = 0.0f;
#pragma unroll
    for (int m = 0; m < 8; m++) {
        const float p = __fmul_rn(x[m], y[m]);
        const float e = __fmaf_rn(x[m], y[m], -p);
        const float t = __fadd_rn(hi, p);
        const float bp = __fsub_rn(t, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
        hi = t;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    return (double)hi + (double)lo;
}

// Entry of every solver kernel.  Programmatic dependent launch: let the next
// kernel of the stream start launching now, then wait until the previous one
// has completed and its writes are visible (both are no-ops for a launch
// without the programmatic-serialisation attribute).  Then one increment of the
// kernel counter per launch (first thread of the first block).
// Programmatic dependent launch in two steps, for kernels that first read
// data no earlier kernel of the solve writes (active lists, stencil words):
// pdl_open lets the next kernel launch, the reads of that constant data follow,
// and pdl_wait then waits for the previous kernel's results.
__device__ __forceinline__ void pdl_open() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void pdl_wait(unsigned long long *kc) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (kc && (blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y | threadIdx.z) == 0)
        atomicAdd(kc, 1ull);
}

__device__ __forceinline__ void count_kernel(unsigned long long *kc) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (kc && (blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y | threadIdx.z) == 0)
        atomicAdd(kc, 1ull);
}

// L x at cell c (i, j, k); returns the value and the diagonal count d.
__device__ __forceinline__ float lap_at(const float *__restrict__ x, const uint8_t *__restrict__ code, int i, int j,
                                        int k, const Dims D, int64_t c, float xc, int &d) {
    const int64_t si = (int64_t)D.ny * D.nz, sj = D.nz;
    float ret = 0.0f, tp, tm;
    uint8_t cn;
    d = 0;
    tp = 0.0f; tm = 0.0f;
    if (i + 1 < D.nx) { cn = code[c + si]; if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : x[c + si], xc); d++; } }
    if (i > 0)        { cn = code[c - si]; if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : x[c - si], xc); d++; } }
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    tp = 0.0f; tm = 0.0f;
    if (j + 1 < D.ny) { cn = code[c + sj]; if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : x[c + sj], xc); d++; } }
    if (j > 0)        { cn = code[c - sj]; if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : x[c - sj], xc); d++; } }
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    tp = 0.0f; tm = 0.0f;
    if (k + 1 < D.nz) { cn = code[c + 1]; if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : x[c + 1], xc); d++; } }
    if (k > 0)        { cn = code[c - 1]; if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : x[c - 1], xc); d++; } }
    ret = __fadd_rn(ret, __fadd_rn(tp, tm));
    return ret;
}

// Diagonal count only (multigrid/mgpcg.py:144-160 neighbor_sum_tag).
__device__ __forceinline__ int diag_at(const uint8_t *__restrict__ code, int i, int j, int k, const Dims D,
                                       int64_t c) {
    const int64_t si = (int64_t)D.ny * D.nz, sj = D.nz;
    int d = 0;
    if (i + 1 < D.nx && code[c + si] != kCodeSolid) d++;
    if (i > 0 && code[c - si] != kCodeSolid) d++;
    if (j + 1 < D.ny && code[c + sj] != kCodeSolid) d++;
    if (j > 0 && code[c - sj] != kCodeSolid) d++;
    if (k + 1 < D.nz && code[c + 1] != kCodeSolid) d++;
    if (k > 0 && code[c - 1] != kCodeSolid) d++;
    return d;
}

__device__ __forceinline__ void unflatten(int64_t c, const Dims D, int &i, int &j, int &k) {
    k = (int)(c % D.nz);
    const int64_t q = c / D.nz;
    j = (int)(q % D.ny);
    i = (int)(q / D.ny);
}

// ---------------------------------------------------------------- last-block reductions
// Each block stores its partial, the last block to finish combines all
// partials in index order (deterministic for a fixed grid size).
__device__ __forceinline__ bool finish_partials(double v, double *partials, unsigned int *ticket, double *red,
                                                double *total) {
    __shared__ bool am_last;
    double b = block_sum(v, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = b;
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    double s = 0.0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) s += __ldcg(&partials[q]);
    s = block_sum(s, red);
    if (threadIdx.x == 0) {
        *total = s;
        *ticket = 0u;
    }
    return true;
}

// ---------------------------------------------------------------- set-up kernels
__global__ void k_encode_tags(const int32_t *__restrict__ tag, uint8_t *__restrict__ code, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        code[c] = encode_tag(tag[c]);
}

// The same for n % 4 == 0 (aligned arrays): four tags in, four packed codes out.
__global__ void k_encode_tags4(const int4 *__restrict__ tag, uint32_t *__restrict__ code, int64_t n4) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += (int64_t)gridDim.x * blockDim.x) {
        const int4 t = __ldg(tag + q);
        code[q] = (uint32_t)encode_tag(t.x) | ((uint32_t)encode_tag(t.y) << 8) | ((uint32_t)encode_tag(t.z) << 16) |
                  ((uint32_t)encode_tag(t.w) << 24);
    }
}

// multigrid/mgpcg.py:162-174 restrict_tag on cell codes.
__global__ void k_restrict_codes(const uint8_t *__restrict__ cf, uint8_t *__restrict__ cc, Dims C) {
    const int64_t n = C.n();
    const Dims F{2 * C.nx, 2 * C.ny, 2 * C.nz};
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        int I, J, K;
        unflatten(q, C, I, J, K);
        bool any_air = false, any_fluid = false;
        for (int ii = 0; ii < 2; ii++)
            for (int jj = 0; jj < 2; jj++)
                for (int kk = 0; kk < 2; kk++) {
                    const uint8_t t = cf[((int64_t)(2 * I + ii) * F.ny + 2 * J + jj) * F.nz + 2 * K + kk];
                    any_air |= (t == kCodeAir);
                    any_fluid |= (t == kCodeFluid);
                }
        cc[q] = any_air ? kCodeAir : (any_fluid ? kCodeFluid : kCodeSolid);
    }
}

// (i, j, kg) of group g (8 cells along k starting at k = 8 kg) of a grid with
// nz % 8 == 0; shifts instead of divisions when nz / 8 and ny are powers of two.
__device__ __forceinline__ void group_ijk(int g, const Dims D, int &i, int &j, int &kg) {
    const int nz8 = D.nz >> 3;
    if (((nz8 & (nz8 - 1)) | (D.ny & (D.ny - 1))) == 0) {
        const int q = g >> (__ffs(nz8) - 1);
        kg = g & (nz8 - 1);
        j = q & (D.ny - 1);
        i = q >> (__ffs(D.ny) - 1);
    } else {
        const int q = g / nz8;
        kg = g - q * nz8;
        j = q % D.ny;
        i = q / D.ny;
    }
}

// ---------------------------------------------------------------- active 8-cell groups
// A level's "active list" holds, in ascending order, the index of every group
// of 8 consecutive cells along k that contains a fluid cell.  Kernels that
// only have work on fluid cells walk the list instead of the whole grid
// (in the 256^3 dam break 20 % of the groups are active).  Built once per
// set_tags in three deterministic passes: per-block counts, one-block scan,
// ordered write.
constexpr int kActThreads = 256;
constexpr int kActRounds = 4;
constexpr int kActPerBlock = kActThreads * kActRounds;

__device__ __forceinline__ bool group_active(const uint8_t *__restrict__ code, int g) {
    const uint2 c = __ldg(reinterpret_cast<const uint2 *>(code + ((int64_t)g << 3)));
    return ((c.x | c.y) & 0x02020202u) != 0u;  // a fluid byte (code 2) among the 8
}

__global__ void __launch_bounds__(kActThreads) k_act_count(const uint8_t *__restrict__ code, int ng,
                                                           int *__restrict__ bcount) {
    int total = 0;
    for (int q = 0; q < kActRounds; q++) {
        const int g = blockIdx.x * kActPerBlock + q * kActThreads + threadIdx.x;
        total += __syncthreads_count(g < ng && group_active(code, g));
    }
    if (threadIdx.x == 0) bcount[blockIdx.x] = total;
}

// Exclusive scan of nb block counts in place (one block of kActThreads), total to *act_n.
__global__ void __launch_bounds__(kActThreads) k_act_scan(int *__restrict__ bcount, int nb, int *__restrict__ act_n) {
    __shared__ int part[kActThreads];
    const int per = (nb + kActThreads - 1) / kActThreads;
    const int b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
    int s = 0;
    for (int b = b0; b < b1; b++) s += bcount[b];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < kActThreads; t++) {
            const int v = part[t];
            part[t] = run;
            run += v;
        }
        *act_n = run;
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int b = b0; b < b1; b++) {
        const int v = bcount[b];
        bcount[b] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kActThreads) k_act_write(const uint8_t *__restrict__ code, int ng,
                                                           const int *__restrict__ boff, int *__restrict__ act) {
    __shared__ int wcount[kActThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int base = boff[blockIdx.x];
    for (int q = 0; q < kActRounds; q++) {
        const int g = blockIdx.x * kActPerBlock + q * kActThreads + threadIdx.x;
        const bool f = g < ng && group_active(code, g);
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wcount[wid] = __popc(m);
        __syncthreads();
        int before = 0, round = 0;
        for (int w = 0; w < kActThreads / 32; w++) {
            before += w < wid ? wcount[w] : 0;
            round += wcount[w];
        }
        if (f) act[base + before + __popc(m & ((1u << lane) - 1u))] = g;
        base += round;
        __syncthreads();
    }
}

// Loop over the groups a kernel works on: the active list when act is not
// NULL (its length read from *act_n on the device), else every group 0..ng-1.
#define FLUB_ACT_LOOP(g, act, act_n, ng)                                                                   \
    for (int _t = blockIdx.x * blockDim.x + threadIdx.x, _tot = (act) ? *(act_n) : (ng); _t < _tot;     \
         _t += gridDim.x * blockDim.x)                                                                       \
        if (const int g = (act) ? __ldg((act) + _t) : _t; true)

// multigrid/mgpcg.py:276-284 init: r = k * rhs, x = p = 0.
__global__ void k_init(float *__restrict__ r, const float *__restrict__ rhs, float kk, float *__restrict__ x,
                       float *__restrict__ p, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        r[c] = __fmul_rn(rhs[c], kk);
        x[c] = 0.0f;
        p[c] = 0.0f;
    }
}

// multigrid/mgpcg.py:492-499 _mask_interior.
__global__ void k_mask_interior(float *__restrict__ r, const uint8_t *__restrict__ code, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (code[c] != kCodeFluid) r[c] = 0.0f;
}

// The same for n % 4 == 0 (aligned arrays), four cells per step; like the
// scalar kernel it only writes: one 16-byte zero store for four cells without
// fluid, single zero stores in a mixed quad.
__global__ void k_mask_interior4(float4 *__restrict__ r, const uint32_t *__restrict__ code, int64_t n4) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c4 = __ldg(code + q);
        bool fl[4];
#pragma unroll
        for (int e = 0; e < 4; e++) fl[e] = ((c4 >> (8 * e)) & 0xffu) == kCodeFluid;
        if (fl[0] && fl[1] && fl[2] && fl[3]) continue;  // r unchanged
        if (!fl[0] && !fl[1] && !fl[2] && !fl[3]) {
            r[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        float *rr = reinterpret_cast<float *>(r + q);
#pragma unroll
        for (int e = 0; e < 4; e++)
            if (!fl[e]) rr[e] = 0.0f;
    }
}

// Plain L p (flub_mg_matvec).
__global__ void k_matvec(const float *__restrict__ p, float *__restrict__ Ap, const uint8_t *__restrict__ code,
                         Dims D) {
    const int64_t n = D.n();
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k, d;
        unflatten(c, D, i, j, k);
        Ap[c] = code[c] == kCodeFluid ? lap_at(p, code, i, j, k, D, c, p[c], d) : 0.0f;
    }
}

// ---------------------------------------------------------------- V-cycle kernels

// multigrid/mgpcg.py:72-86 _smooth_mcadams, one half-sweep.  Phase 0 updates
// cells with (i+j+k) odd, phase 1 cells with (i+j+k) even.  One thread per
// (i, j, k-pair); the thread updates the member of the pair with the phase's
// parity.  kFromZero: z is implicitly 0 before the sweep (first sweep of a
// level in the V-cycle), the thread then writes both members of its pair.
template <bool kFromZero>
__global__ void __launch_bounds__(256) k_smooth_half(float *__restrict__ z, const float *__restrict__ r,
                                                     const uint8_t *__restrict__ code, Dims D, int phase,
                                                     unsigned long long *kc) {
    count_kernel(kc);
    const int hz = D.nz >> 1;
    const int64_t npairs = (int64_t)D.nx * D.ny * hz;
    const int par = 1 - phase;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < npairs;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int kk = (int)(t % hz);
        const int64_t q = t / hz;
        const int j = (int)(q % D.ny), i = (int)(q / D.ny);
        const int b = (par + i + j) & 1;
        const int k = 2 * kk + b;
        const int64_t c = ((int64_t)i * D.ny + j) * D.nz + k;
        float znew = 0.0f;
        if (code[c] == kCodeFluid) {
            int d;
            if (kFromZero) {
                // z = 0 + (r + L 0) / d with L 0 = 0 exactly
                d = diag_at(code, i, j, k, D, c);
                if (d != 0) znew = __fdiv_rn(r[c], (float)d);
            } else {
                const float zc = z[c];
                const float lz = lap_at(z, code, i, j, k, D, c, zc, d);
                if (d != 0) znew = __fadd_rn(zc, __fdiv_rn(__fadd_rn(r[c], lz), (float)d));
            }
        }
        z[c] = znew;
        if (kFromZero) z[c + (b ? -1 : 1)] = 0.0f;
    }
}

// multigrid/mgpcg.py:94-101 _restrict_mcadams as a gather: the coarse cell
// sums r + L z of its 8 children in (ii, jj, kk) order; 0 unless coarse fluid.
__global__ void __launch_bounds__(256) k_restrict(const float *__restrict__ rf, const float *__restrict__ zf,
                                                  const uint8_t *__restrict__ cf, float *__restrict__ rc,
                                                  const uint8_t *__restrict__ cc, Dims C, float scale,
                                                  unsigned long long *kc) {
    count_kernel(kc);
    const Dims F{2 * C.nx, 2 * C.ny, 2 * C.nz};
    const int64_t n = C.n();
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        if (cc[q] != kCodeFluid) {
            rc[q] = 0.0f;
            continue;
        }
        int I, J, K;
        unflatten(q, C, I, J, K);
        float s = 0.0f;
        bool first = true;
#pragma unroll
        for (int ii = 0; ii < 2; ii++)
#pragma unroll
            for (int jj = 0; jj < 2; jj++)
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                    const int i = 2 * I + ii, j = 2 * J + jj, k = 2 * K + kk;
                    const int64_t c = ((int64_t)i * F.ny + j) * F.nz + k;
                    float lz = 0.0f;
                    if (cf[c] == kCodeFluid) {
                        int d;
                        lz = lap_at(zf, cf, i, j, k, F, c, zf[c], d);
                    }
                    const float v = __fadd_rn(rf[c], lz);
                    s = first ? v : __fadd_rn(s, v);
                    first = false;
                }
        rc[q] = __fmul_rn(s, scale);  // scale 1: the reference's sum, exactly
    }
}

// multigrid/mgpcg.py:113-116 _prolongate: z_h += z_2h[I/2], written to zout
// (zout may equal zin).
__global__ void __launch_bounds__(256) k_prolong(float *zout, const float *zin, const float *__restrict__ zc, Dims F,
                                                 unsigned long long *kc) {
    count_kernel(kc);
    const int64_t n = F.n();
    const int cy = F.ny >> 1, cz = F.nz >> 1;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(c, F, i, j, k);
        zout[c] = __fadd_rn(zin[c], zc[((int64_t)(i >> 1) * cy + (j >> 1)) * cz + (k >> 1)]);
    }
}

// ---------------------------------------------------------------- CG kernels

__global__ void k_solve_begin(MgState *st, int max_iters, double eps, double abs_tol, double rel_tol, int use_x0,
                              int skip_r) {
    st->skip_r = skip_r;
    st->max_iters = max_iters;
    st->eps = eps;
    st->abs_tol = abs_tol;
    st->rel_tol = rel_tol;
    st->it = 0;
    st->converged = 0;
    st->status = FLUB_OK;
    st->cond = 0;
    st->use_x0 = use_x0;
    if (!use_x0) st->x0_scale = 0.0;
    st->zscale = 1.0f;
    st->alpha = 0.0;
    st->beta = 0.0;
    st->ticket = 0u;
}

// r -= L x0 when an initial guess was given (no reference counterpart).
__global__ void __launch_bounds__(256) k_residual_x0(MgState *st, float *__restrict__ r, const float *__restrict__ x,
                                                     const uint8_t *__restrict__ code, Dims D,
                                                     unsigned long long *kc) {
    count_kernel(kc);
    if (!st->use_x0) return;
    const int64_t n = D.n();
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        if (code[c] != kCodeFluid) continue;
        int i, j, k, d;
        unflatten(c, D, i, j, k);
        r[c] = __fsub_rn(r[c], lap_at(x, code, i, j, k, D, c, x[c], d));
    }
}

// Sum of r over fluid cells -> mean (zero_centered, multigrid/mgpcg.py:191-197).
// guard: 0 always run, 1 skip once the CG loop is finished, 2 run only when
// an initial guess was given.
// The count of fluid cells is accumulated as a double (exact below 2^53).
__global__ void __launch_bounds__(kRedThreads) k_fluid_mean(MgState *st, const float *__restrict__ r,
                                                            const uint8_t *__restrict__ code, int64_t n,
                                                            double *partials, int guard, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    if (guard == 1 && (st->it >= st->max_iters || st->converged || st->status)) return;
    if (guard == 2 && !st->use_x0) return;
    double s = 0.0, cnt = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (code[c] == kCodeFluid) {
            s += (double)r[c];
            cnt += 1.0;
        }
    double total;
    // two reductions share one ticket: pack the count into the second half of partials
    double bc = block_sum(cnt, red);
    __syncthreads();
    if (threadIdx.x == 0) partials[kMaxRedBlocks + blockIdx.x] = bc;
    if (finish_partials(s, partials, &st->ticket, red, &total)) {
        __syncthreads();
        double c2 = 0.0;
        for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) c2 += __ldcg(&partials[kMaxRedBlocks + q]);
        c2 = block_sum(c2, red);
        if (threadIdx.x == 0) st->mean = c2 > 0.0 ? total / c2 : 0.0;
    }
}

// _sub (multigrid/mgpcg.py:198-205): r -= mean on fluid cells, 0 elsewhere.
__global__ void __launch_bounds__(kRedThreads) k_sub_mean(MgState *st, float *__restrict__ r,
                                                          const uint8_t *__restrict__ code, int64_t n, int guard,
                                                          unsigned long long *kc) {
    count_kernel(kc);
    if (guard == 1 && (st->it >= st->max_iters || st->converged || st->status)) return;
    if (guard == 2 && !st->use_x0) return;
    const float m = (float)st->mean;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        r[c] = code[c] == kCodeFluid ? __fsub_rn(r[c], m) : 0.0f;
}

// rTr0 and the tolerance (multigrid/mgpcg.py:391-393).
__global__ void __launch_bounds__(kRedThreads) k_dot_rr0(MgState *st, const float *__restrict__ r, int64_t n,
                                                         double *partials, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    double s = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const double v = r[c];
        s = fma(v, v, s);
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        st->rtr0 = total;
        st->rtr = total;
        const double rel = total * st->rel_tol;
        st->tol = st->abs_tol > rel ? st->abs_tol : rel;
    }
}

// z.r after the first preconditioner application; p = z (mgpcg.py:396-401).
__global__ void __launch_bounds__(kRedThreads) k_dot_zr_init(MgState *st, const float *__restrict__ z,
                                                             const float *__restrict__ r, float *__restrict__ p,
                                                             int64_t n, double *partials, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    double s = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const float zc = z[c];
        s = fma((double)zc, (double)r[c], s);
        p[c] = zc;
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) st->zr_old = total;
}

// Ap = L p and p.Ap -> alpha (mgpcg.py:410-419).  Guarded: a no-op once the
// iteration budget is spent or the solve has converged / broken down.
__global__ void __launch_bounds__(kRedThreads) k_matvec_pap(MgState *st, const float *__restrict__ p,
                                                            float *__restrict__ Ap, const uint8_t *__restrict__ code,
                                                            Dims D, double *partials, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    if (st->it >= st->max_iters || st->converged || st->status) return;
    const int64_t n = D.n();
    double s = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        float a = 0.0f;
        const float pc = p[c];
        if (code[c] == kCodeFluid) {
            int i, j, k, d;
            unflatten(c, D, i, j, k);
            a = lap_at(p, code, i, j, k, D, c, pc, d);
        }
        Ap[c] = a;
        s = fma((double)pc, (double)a, s);
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        st->pap = total;
        const double alpha = st->zr_old / (total + st->eps);
        st->alpha = alpha;
        if (!isfinite(alpha)) st->status = FLUB_ERR_BREAKDOWN;
    }
}

// Sets the loop condition after the residual check (while-node handle).
__device__ __forceinline__ void publish_cond(MgState *st, int cond, cudaGraphConditionalHandle h, int set_cond) {
    st->cond = cond;
    if (set_cond) cudaGraphSetConditional(h, (unsigned)cond);
}

// r -= alpha Ap (skipped when kUpdate is false: "fraction" already updated r
// and removed the mean), r.r, convergence test (mgpcg.py:421-446).
template <bool kUpdate>
__global__ void __launch_bounds__(kRedThreads) k_update_r_rr(MgState *st, float *__restrict__ r,
                                                             const float *__restrict__ Ap, int64_t n,
                                                             double *partials, double *hist,
                                                             cudaGraphConditionalHandle h, int set_cond,
                                                             unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    if (st->it >= st->max_iters || st->converged || st->status) {
        if (blockIdx.x == 0 && threadIdx.x == 0) publish_cond(st, 0, h, set_cond);
        return;
    }
    const float a = (float)st->alpha;
    double s = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        float rv = r[c];
        if (kUpdate) {
            rv = __fmaf_rn(-a, Ap[c], rv);
            r[c] = rv;
        }
        s = fma((double)rv, (double)rv, s);
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        st->rtr = total;
        if (st->it < kHistory) hist[st->it] = total;
        if (!isfinite(total)) st->status = FLUB_ERR_BREAKDOWN;
        const int conv = total < st->tol;
        st->converged = conv;
        publish_cond(st, (!conv && st->status == FLUB_OK) ? 1 : 0, h, set_cond);
    }
}

// Fraction smoother: r -= alpha Ap only (mean removal and r.r follow).
__global__ void __launch_bounds__(kRedThreads) k_update_r(MgState *st, float *__restrict__ r,
                                                          const float *__restrict__ Ap, int64_t n,
                                                          unsigned long long *kc) {
    count_kernel(kc);
    if (st->it >= st->max_iters || st->converged || st->status) return;
    const float a = (float)st->alpha;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        r[c] = __fmaf_rn(-a, Ap[c], r[c]);
}

// z.r -> beta (mgpcg.py:451-455).
__global__ void __launch_bounds__(kRedThreads) k_dot_zr_beta(MgState *st, const float *__restrict__ z,
                                                             const float *__restrict__ r, int64_t n,
                                                             double *partials, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    double s = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        s = fma((double)z[c], (double)r[c], s);
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        const double beta = total / (st->zr_old + st->eps);
        st->beta = beta;
        st->zr_old = total;
        if (!isfinite(beta)) st->status = FLUB_ERR_BREAKDOWN;
    }
}

// x += alpha p; p = z + beta p; it += 1 (mgpcg.py:457-461).
__global__ void __launch_bounds__(256) k_update_xp(MgState *st, float *__restrict__ x, float *__restrict__ p,
                                                   const float *__restrict__ z, int64_t n, unsigned long long *kc) {
    count_kernel(kc);
    const float a = (float)st->alpha, b = (float)st->beta;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const float pc = p[c];
        x[c] = __fmaf_rn(a, pc, x[c]);
        p[c] = __fmaf_rn(b, pc, z[c]);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st->it += 1;
}

// On convergence: x += alpha p (mgpcg.py:444-446).
__global__ void __launch_bounds__(256) k_solve_end(MgState *st, float *__restrict__ x, const float *__restrict__ p,
                                                   int64_t n, unsigned long long *kc) {
    count_kernel(kc);
    if (!st->converged) return;
    const float a = (float)st->alpha;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        x[c] = __fmaf_rn(a, p[c], x[c]);
}

__global__ void k_scale_copy(float *__restrict__ out, const float *__restrict__ in, float s, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        out[c] = __fmul_rn(in[c], s);
}

}  // namespace flub
