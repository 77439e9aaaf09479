// CG vector kernels over groups of 8 consecutive cells (multigrid/mgpcg.py:
// 207-232 and the array_inner calls of :391-451), float4 rows, FP64 partial
// sums, 32-bit indices.
//
// Skipping: on a group without a fluid cell the CG vectors hold values that
// cannot change the result -- L p = Ap = 0, z = 0, p = 0 (p starts at 0 and is
// z + beta p) -- so such a group is not read at all.  The one vector that the
// caller could leave non-zero off the fluid is r (init without mask_interior);
// the r.r kernels therefore skip only when the solver state says r was
// masked (MgState::skip_r).
#pragma once

#include "mg_kernels.cuh"
#include "smooth8.cuh"

namespace flub {

__device__ __forceinline__ bool group_has_fluid(uint2 c) { return ((c.x | c.y) & 0x02020202u) != 0u; }

__device__ __forceinline__ void store_row8(float *p, const float v[8]) {
    float4 *o = reinterpret_cast<float4 *>(p);
    o[0] = make_float4(v[0], v[1], v[2], v[3]);
    o[1] = make_float4(v[4], v[5], v[6], v[7]);
}

// L x for the 8 cells of the row starting at c0 (group g), same operation
// order as lap_at, from the stencil words wd of the row.  Non-fluid cells get
// 0.
__device__ __forceinline__ void lap_row8_w(const float *__restrict__ x, const uint4 wd, const Dims D, int g,
                                           float out[8], Row8 &xc) {
    int i, j, kg;
    group_ijk(g, D, i, j, kg);
    const int k0 = kg << 3;
    const int sj = D.nz, si = D.ny * D.nz;
    const int c0 = g << 3;
    const bool hip = i + 1 < D.nx, him = i > 0, hjp = j + 1 < D.ny, hjm = j > 0;
    const bool hkp = k0 + 8 < D.nz, hkm = k0 > 0;
    Row8 xip, xim, xjp, xjm;
    load_row8(x + c0, xc);
    if (hip) load_row8(x + c0 + si, xip); else zero_row8(xip);
    if (him) load_row8(x + c0 - si, xim); else zero_row8(xim);
    if (hjp) load_row8(x + c0 + sj, xjp); else zero_row8(xjp);
    if (hjm) load_row8(x + c0 - sj, xjm); else zero_row8(xjm);
    const float xkm = hkm ? __ldg(x + c0 - 1) : 0.0f;
    const float xkp = hkp ? __ldg(x + c0 + 8) : 0.0f;
#pragma unroll
    for (int m = 0; m < 8; m++) {
        out[m] = 0.0f;
        const uint32_t w = word_at(wd, m);
        if (sw_code(w, 0) != kCodeFluid) continue;
        out[m] = sw_nbsum(w, xc.v[m], xip.v[m], xim.v[m], xjp.v[m], xjm.v[m], m < 7 ? xc.v[m + 1] : xkp,
                          m > 0 ? xc.v[m - 1] : xkm);
    }
}

// lap_row8_w with the words from sw, or from the codes when sw is NULL.
__device__ __forceinline__ void lap_row8(const float *__restrict__ x, const uint8_t *__restrict__ code,
                                         const uint16_t *__restrict__ sw, const Dims D, int g, float out[8], Row8 &xc) {
    int i, j, kg;
    group_ijk(g, D, i, j, kg);
    lap_row8_w(x, load_words8(sw, code, D, i, j, kg << 3, g << 3), D, g, out, xc);
}

// Ap = L p, p.Ap -> alpha (mgpcg.py:410-419); guarded like k_matvec_pap.
// The active-list length, the first list entry and the first group's stencil
// words do not change during a solve (set_tags writes them before it): they
// are read before the wait on the previous kernel, and each next list entry one
// group ahead.  Launched with one resident wave of blocks.
__global__ void __launch_bounds__(kRedThreads, 4) k8_matvec_pap(MgState *st, const float *__restrict__ p,
                                                             float *__restrict__ Ap, const uint8_t *__restrict__ code,
                                                             const uint16_t *__restrict__ sw, Dims D, double *partials,
                                                             const int *__restrict__ act,
                                                             const int *__restrict__ act_n, unsigned long long *kc) {
    __shared__ double red[32];
    pdl_open();
    const int ng = (int)(D.n() >> 3);
    const int tot = act ? *act_n : ng;
    const int stride = gridDim.x * blockDim.x;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int g_next = t < tot ? (act ? __ldg(act + t) : t) : 0;
    uint4 wd_first = make_uint4(0u, 0u, 0u, 0u);
    if (t < tot && sw) wd_first = __ldg(reinterpret_cast<const uint4 *>(sw + ((size_t)g_next << 3)));
    pdl_wait(kc);
    if (st->it >= st->max_iters || st->converged || st->status) return;
    double s = 0.0;
    bool first = true;
    for (; t < tot; t += stride) {
        const int g = g_next;
        const int tn = t + stride;
        g_next = tn < tot ? (act ? __ldg(act + tn) : tn) : 0;
        const bool use_first = first && sw;
        first = false;
        if (!act && !group_has_fluid(load_codes8(code + (g << 3)))) continue;  // Ap = 0 there already
        int i, j, kg;
        group_ijk(g, D, i, j, kg);
        const uint4 wd = use_first ? wd_first : load_words8(sw, code, D, i, j, kg << 3, g << 3);
        float a[8];
        Row8 pc;
        lap_row8_w(p, wd, D, g, a, pc);
        store_row8(Ap + (g << 3), a);
        s += dot8_ff(pc.v, a);
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        st->pap = total;
        const double alpha = st->zr_old / (total + st->eps);
        st->alpha = alpha;
        if (!isfinite(alpha)) st->status = FLUB_ERR_BREAKDOWN;
    }
}

// r -= alpha Ap, r.r, convergence test and loop condition (mgpcg.py:421-446).
template <bool kUpdate>
__global__ void __launch_bounds__(kRedThreads) k8_update_r_rr(MgState *st, float *__restrict__ r,
                                                              const float *__restrict__ Ap,
                                                              const uint8_t *__restrict__ code, int64_t n,
                                                              double *partials, double *hist,
                                                              cudaGraphConditionalHandle h, int set_cond,
                                                              const int *__restrict__ act,
                                                              const int *__restrict__ act_n, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    if (st->it >= st->max_iters || st->converged || st->status) {
        if ((blockIdx.x | threadIdx.x) == 0) publish_cond(st, 0, h, set_cond);
        return;
    }
    const float a = (float)st->alpha;
    const int skip = st->skip_r;
    const int *ga = skip ? act : nullptr;
    const int ng = (int)(n >> 3);
    double s = 0.0;
    FLUB_ACT_LOOP(g, ga, act_n, ng) {
        if (skip && !ga && !group_has_fluid(load_codes8(code + (g << 3)))) continue;
        Row8 rv;
        load_row8_rw(r + (g << 3), rv);
        if (kUpdate) {
            Row8 av;
            load_row8(Ap + (g << 3), av);
#pragma unroll
            for (int m = 0; m < 8; m++) rv.v[m] = __fmaf_rn(-a, av.v[m], rv.v[m]);
            store_row8(r + (g << 3), rv.v);
        }
        s += dot8_ff(rv.v, rv.v);
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

// rTr0 and the tolerance (mgpcg.py:391-393).
__global__ void __launch_bounds__(kRedThreads) k8_dot_rr0(MgState *st, const float *__restrict__ r,
                                                          const uint8_t *__restrict__ code, int64_t n,
                                                          double *partials, const int *__restrict__ act,
                                                          const int *__restrict__ act_n, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    const int skip = st->skip_r;
    const int *ga = skip ? act : nullptr;
    const int ng = (int)(n >> 3);
    double s = 0.0;
    FLUB_ACT_LOOP(g, ga, act_n, ng) {
        if (skip && !ga && !group_has_fluid(load_codes8(code + (g << 3)))) continue;
        Row8 rv;
        load_row8(r + (g << 3), rv);
        s += dot8_ff(rv.v, rv.v);
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        st->rtr0 = total;
        st->rtr = total;
        const double rel = total * st->rel_tol;
        st->tol = st->abs_tol > rel ? st->abs_tol : rel;
    }
}

// z.r; kInit: old_zTr = z.r and p = z (mgpcg.py:396-401), else beta (:451-455).
// kScaleZ: the V-cycle output is z / st->zscale (mixed precision), scaled back here.
template <bool kInit, bool kScaleZ = false>
__global__ void __launch_bounds__(kRedThreads) k8_dot_zr(MgState *st, const float *__restrict__ z,
                                                         const float *__restrict__ r, float *__restrict__ p,
                                                         const uint8_t *__restrict__ code, int64_t n,
                                                         double *partials, const int *__restrict__ act,
                                                         const int *__restrict__ act_n, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    const int ng = (int)(n >> 3);
    const float zs = kScaleZ ? st->zscale : 1.0f;
    double s = 0.0;
    FLUB_ACT_LOOP(g, act, act_n, ng) {
        if (!act && !group_has_fluid(load_codes8(code + (g << 3)))) continue;  // z = 0 (and p = 0) there
        Row8 zv, rv;
        load_row8(z + (g << 3), zv);
        if (kScaleZ) {
#pragma unroll
            for (int m = 0; m < 8; m++) zv.v[m] = __fmul_rn(zv.v[m], zs);
        }
        load_row8(r + (g << 3), rv);
        s += dot8_ff(zv.v, rv.v);
        if (kInit) store_row8(p + (g << 3), zv.v);
    }
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total) && threadIdx.x == 0) {
        if (kInit) {
            st->zr_old = total;
        } else {
            const double beta = total / (st->zr_old + st->eps);
            st->beta = beta;
            st->zr_old = total;
            if (!isfinite(beta)) st->status = FLUB_ERR_BREAKDOWN;
        }
    }
}

// x += alpha p; p = z + beta p; it += 1 (mgpcg.py:457-461).
template <bool kScaleZ = false>
__global__ void __launch_bounds__(256) k8_update_xp(MgState *st, float *__restrict__ x, float *__restrict__ p,
                                                    const float *__restrict__ z, const uint8_t *__restrict__ code,
                                                    int64_t n, const int *__restrict__ act,
                                                    const int *__restrict__ act_n, unsigned long long *kc) {
    count_kernel(kc);
    const float a = (float)st->alpha, b = (float)st->beta;
    const float zs = kScaleZ ? st->zscale : 1.0f;
    const int ng = (int)(n >> 3);
    FLUB_ACT_LOOP(g, act, act_n, ng) {
        if (!act && !group_has_fluid(load_codes8(code + (g << 3)))) continue;  // p = z = 0 there
        Row8 xv, pv, zv;
        load_row8_rw(x + (g << 3), xv);
        load_row8_rw(p + (g << 3), pv);
        load_row8(z + (g << 3), zv);
        if (kScaleZ) {
#pragma unroll
            for (int m = 0; m < 8; m++) zv.v[m] = __fmul_rn(zv.v[m], zs);
        }
#pragma unroll
        for (int m = 0; m < 8; m++) {
            xv.v[m] = __fmaf_rn(a, pv.v[m], xv.v[m]);
            pv.v[m] = __fmaf_rn(b, pv.v[m], zv.v[m]);
        }
        store_row8(x + (g << 3), xv.v);
        store_row8(p + (g << 3), pv.v);
    }
    if ((blockIdx.x | threadIdx.x) == 0) st->it += 1;
}

// r -= L x0 when an initial guess was given (no reference counterpart); L x0
// is 0 off the fluid, so only the active groups change.
__global__ void __launch_bounds__(256) k8_residual_x0(MgState *st, float *__restrict__ r, const float *__restrict__ x,
                                                      const uint8_t *__restrict__ code,
                                                      const uint16_t *__restrict__ sw, Dims D,
                                                      const int *__restrict__ act, const int *__restrict__ act_n,
                                                      unsigned long long *kc) {
    count_kernel(kc);
    if (!st->use_x0) return;
    const int ng = (int)(D.n() >> 3);
    FLUB_ACT_LOOP(g, act, act_n, ng) {
        const uint2 cc = load_codes8(code + (g << 3));
        if (!act && !group_has_fluid(cc)) continue;
        float lx[8];
        Row8 xc, rv;
        lap_row8(x, code, sw, D, g, lx, xc);
        load_row8_rw(r + (g << 3), rv);
#pragma unroll
        for (int m = 0; m < 8; m++)
            if (code_at(cc, m) == kCodeFluid) rv.v[m] = __fsub_rn(rv.v[m], lx[m]);
        store_row8(r + (g << 3), rv.v);
    }
}

// gamma = (d . b) / (d . L d) over fluid cells (no reference counterpart): the
// multiple of d closest to the solution of L x = b in the energy norm.
__global__ void __launch_bounds__(kRedThreads) k8_x0_gamma(MgState *st, const float *__restrict__ d,
                                                           const float *__restrict__ b,
                                                           const uint8_t *__restrict__ code,
                                                           const uint16_t *__restrict__ sw, Dims D, double *partials,
                                                           const int *__restrict__ act,
                                                           const int *__restrict__ act_n) {
    __shared__ double red[32];
    const int ng = (int)(D.n() >> 3);
    double s_ld = 0.0, s_b = 0.0;
    FLUB_ACT_LOOP(g, act, act_n, ng) {
        const uint2 cc = load_codes8(code + (g << 3));
        if (!act && !group_has_fluid(cc)) continue;
        float ld[8];
        Row8 dc, bv;
        lap_row8(d, code, sw, D, g, ld, dc);
        load_row8(b + (g << 3), bv);
        float dm[8];
#pragma unroll
        for (int m = 0; m < 8; m++) dm[m] = code_at(cc, m) == kCodeFluid ? dc.v[m] : 0.0f;
        s_ld += dot8_ff(dm, ld);
        s_b += dot8_ff(dm, bv.v);
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
            const double gm = t2 / total;
            st->x0_scale = (total != 0.0 && isfinite(gm)) ? gm : 0.0;
        }
    }
}

// On convergence: x += alpha p (mgpcg.py:444-446).
__global__ void __launch_bounds__(256) k8_solve_end(MgState *st, float *__restrict__ x, const float *__restrict__ p,
                                                    const uint8_t *__restrict__ code, int64_t n,
                                                    const int *__restrict__ act, const int *__restrict__ act_n,
                                                    unsigned long long *kc) {
    count_kernel(kc);
    if (!st->converged) return;
    const float a = (float)st->alpha;
    const int ng = (int)(n >> 3);
    FLUB_ACT_LOOP(g, act, act_n, ng) {
        if (!act && !group_has_fluid(load_codes8(code + (g << 3)))) continue;
        Row8 xv, pv;
        load_row8_rw(x + (g << 3), xv);
        load_row8(p + (g << 3), pv);
#pragma unroll
        for (int m = 0; m < 8; m++) xv.v[m] = __fmaf_rn(a, pv.v[m], xv.v[m]);
        store_row8(x + (g << 3), xv.v);
    }
}

}  // namespace flub
