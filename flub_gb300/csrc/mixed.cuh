// Mixed-precision preconditioner support (no reference counterpart).
//
// The V-cycle levels in global memory are stored in FP16; every operation is
// still computed in FP32 (store.cuh).  Level l is stored at scale 8^-l: the
// sum-restriction multiplies magnitudes by about 8 per level, the scaling keeps
// coarse values inside FP16's range, and because every V-cycle operation is
// linear and the factors are powers of two, scaling is exact: the restriction
// multiplies by 1/8 on store, the prolongation by 8 on load.
//
// FP16 rounding makes the preconditioner slightly non-symmetric, so CG uses
// the flexible (Polak-Ribiere) beta = z.(r - r_old) / (z_old . r_old).
#pragma once

#include "cg8.cuh"
#include "store.cuh"

namespace flub {

// Residual + restriction (mgpcg.py:94-101, gather form) between stored levels:
// r_c = out_scale * sum over children of (r_f + L z_f).
template <typename TRI, typename TZI, typename TRO>
__global__ void __launch_bounds__(256) k_restrict_t(const TRI *__restrict__ rf, const TZI *__restrict__ zf,
                                                    const uint8_t *__restrict__ cf, TRO *__restrict__ rc,
                                                    const uint8_t *__restrict__ cc, Dims C, float out_scale,
                                                    unsigned long long *kc) {
    count_kernel(kc);
    const Dims F{2 * C.nx, 2 * C.ny, 2 * C.nz};
    const int n = (int)C.n();
    const int si = F.ny * F.nz, sj = F.nz;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        if (cc[q] != kCodeFluid) {
            St<TRO>::st(rc + q, 0.0f);
            continue;
        }
        const int K = q % C.nz, J = (q / C.nz) % C.ny, I = q / (C.nz * C.ny);
        float s = 0.0f;
        bool first = true;
#pragma unroll
        for (int ii = 0; ii < 2; ii++)
#pragma unroll
            for (int jj = 0; jj < 2; jj++)
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                    const int i = 2 * I + ii, j = 2 * J + jj, k = 2 * K + kk;
                    const int c = (i * F.ny + j) * F.nz + k;
                    float lz = 0.0f;
                    if (cf[c] == kCodeFluid) {
                        const float xc = St<TZI>::ld_ro(zf + c);
                        float tp, tm;
                        uint8_t cn;
                        tp = 0.0f; tm = 0.0f;
                        if (i + 1 < F.nx) { cn = cf[c + si]; if (cn != kCodeSolid) tp = __fsub_rn(cn == kCodeAir ? 0.0f : St<TZI>::ld_ro(zf + c + si), xc); }
                        if (i > 0)        { cn = cf[c - si]; if (cn != kCodeSolid) tm = __fsub_rn(cn == kCodeAir ? 0.0f : St<TZI>::ld_ro(zf + c - si), xc); }
                        lz = __fadd_rn(lz, __fadd_rn(tp, tm));
                        tp = 0.0f; tm = 0.0f;
                        if (j + 1 < F.ny) { cn = cf[c + sj]; if (cn != kCodeSolid) tp = __fsub_rn(cn == kCodeAir ? 0.0f : St<TZI>::ld_ro(zf + c + sj), xc); }
                        if (j > 0)        { cn = cf[c - sj]; if (cn != kCodeSolid) tm = __fsub_rn(cn == kCodeAir ? 0.0f : St<TZI>::ld_ro(zf + c - sj), xc); }
                        lz = __fadd_rn(lz, __fadd_rn(tp, tm));
                        tp = 0.0f; tm = 0.0f;
                        if (k + 1 < F.nz) { cn = cf[c + 1]; if (cn != kCodeSolid) tp = __fsub_rn(cn == kCodeAir ? 0.0f : St<TZI>::ld_ro(zf + c + 1), xc); }
                        if (k > 0)        { cn = cf[c - 1]; if (cn != kCodeSolid) tm = __fsub_rn(cn == kCodeAir ? 0.0f : St<TZI>::ld_ro(zf + c - 1), xc); }
                        lz = __fadd_rn(lz, __fadd_rn(tp, tm));
                    }
                    const float v = __fadd_rn(St<TRI>::ld_ro(rf + c), lz);
                    s = first ? v : __fadd_rn(s, v);
                    first = false;
                }
        St<TRO>::st(rc + q, __fmul_rn(s, out_scale));
    }
}

// FP16 copy of the level-0 residual for the V-cycle (every group).  With a
// solver state, the copy is r / zscale with zscale a power of two near the
// RMS of r (fp16_residual_scale), recorded in st->zscale; without one
// (flub_mg_apply_preconditioner) the copy is unscaled.
__global__ void __launch_bounds__(256) k8_to_half(MgState *st, const float *__restrict__ r, __half *__restrict__ rh,
                                                  int64_t n, unsigned long long *kc) {
    count_kernel(kc);
    const float hs = st ? block_fp16_residual_scale(threadIdx.x == 0 ? st->rtr0 : 0.0, n) : 1.0f;
    if (st && (blockIdx.x | threadIdx.x) == 0) st->zscale = 1.0f / hs;
    const int ng = (int)(n >> 3);
    // every group: afterwards rh = r / zscale everywhere (0 off the fluid when r is masked)
    FLUB_ACT_LOOP(g, (const int *)nullptr, (const int *)nullptr, ng) {
        float v[8];
        St<float>::ld8_ro(r + (g << 3), v);
#pragma unroll
        for (int m = 0; m < 8; m++) v[m] = __fmul_rn(v[m], hs);
        St<__half>::st8(rh + (g << 3), v);
    }
}

// r_old = r; r -= alpha Ap; its FP16 copy; r.r, convergence test and loop
// condition (mgpcg.py:421-446 with the flexible-CG bookkeeping).
__global__ void __launch_bounds__(kRedThreads) k8_update_r_rr_mixed(MgState *st, float *__restrict__ r,
                                                                    float *__restrict__ r_old, __half *__restrict__ rh,
                                                                    const float *__restrict__ Ap,
                                                                    const uint8_t *__restrict__ code, int64_t n,
                                                                    double *partials, double *hist,
                                                                    cudaGraphConditionalHandle h, int set_cond,
                                                                    const int *__restrict__ act,
                                                                    const int *__restrict__ act_n,
                                                                    unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    if (st->it >= st->max_iters || st->converged || st->status) {
        if ((blockIdx.x | threadIdx.x) == 0) publish_cond(st, 0, h, set_cond);
        return;
    }
    const float a = (float)st->alpha;
    const int skip = st->skip_r;
    // with a masked r the groups without fluid keep r = r_old = rh = 0 (the
    // solve's first FP16 copy, k8_to_half, covered every group)
    const int *ga = skip ? act : nullptr;
    // scale of the FP16 copy from the previous residual norm (st->rtr is only
    // overwritten by the last block, after every block has read it)
    const float hs = block_fp16_residual_scale(threadIdx.x == 0 ? st->rtr : 0.0, n);
    if ((blockIdx.x | threadIdx.x) == 0) st->zscale = 1.0f / hs;
    const int ng = (int)(n >> 3);
    double s = 0.0;
    FLUB_ACT_LOOP(g, ga, act_n, ng) {
        if (skip && !ga && !group_has_fluid(load_codes8(code + (g << 3)))) continue;
        float rv[8], av[8], hv[8];
        St<float>::ld8(r + (g << 3), rv);
        St<float>::ld8_ro(Ap + (g << 3), av);
        St<float>::st8(r_old + (g << 3), rv);
#pragma unroll
        for (int m = 0; m < 8; m++) {
            rv[m] = __fmaf_rn(-a, av[m], rv[m]);
            hv[m] = __fmul_rn(rv[m], hs);
        }
        St<float>::st8(r + (g << 3), rv);
        St<__half>::st8(rh + (g << 3), hv);
        s += dot8_ff(rv, rv);
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

// Flexible beta = (z.r - z.r_old) / (old z.r_old): two sums in one pass.
__global__ void __launch_bounds__(kRedThreads) k8_dot_zr_flex(MgState *st, const float *__restrict__ z,
                                                              const float *__restrict__ r,
                                                              const float *__restrict__ r_old,
                                                              const uint8_t *__restrict__ code, int64_t n,
                                                              double *partials, const int *__restrict__ act,
                                                              const int *__restrict__ act_n, unsigned long long *kc) {
    __shared__ double red[32];
    count_kernel(kc);
    const int ng = (int)(n >> 3);
    const float zs = st->zscale;
    double s = 0.0, so = 0.0;
    FLUB_ACT_LOOP(g, act, act_n, ng) {
        if (!act && !group_has_fluid(load_codes8(code + (g << 3)))) continue;  // z = 0 there
        float zv[8], rv[8], ov[8];
        St<float>::ld8_ro(z + (g << 3), zv);
#pragma unroll
        for (int m = 0; m < 8; m++) zv[m] = __fmul_rn(zv[m], zs);
        St<float>::ld8_ro(r + (g << 3), rv);
        St<float>::ld8_ro(r_old + (g << 3), ov);
        s += dot8_ff(zv, rv);
        so += dot8_ff(zv, ov);
    }
    const double bo = block_sum(so, red);
    __syncthreads();
    if (threadIdx.x == 0) partials[kMaxRedBlocks + blockIdx.x] = bo;
    double total;
    if (finish_partials(s, partials, &st->ticket, red, &total)) {
        __syncthreads();
        double t2 = 0.0;
        for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) t2 += __ldcg(&partials[kMaxRedBlocks + q]);
        t2 = block_sum(t2, red);
        if (threadIdx.x == 0) {
            const double beta = (total - t2) / (st->zr_old + st->eps);
            st->beta = beta;
            st->zr_old = total;
            if (!isfinite(beta)) st->status = FLUB_ERR_BREAKDOWN;
        }
    }
}

}  // namespace flub
