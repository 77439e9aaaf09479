// Level-0 red-black smoothing on colour-split storage.
//
// In natural order (k fastest) the cells of one colour alternate along k, so
// a half-sweep that updates one colour still moves whole rows: half of every
// neighbour row it loads and half of the row it stores belong to the colour it
// does not update.  Inside the V-cycle the level-0 vectors are therefore kept
// split by colour: a buffer of n values holds the even cells ((i + j + k) even)
// in its first half and the odd cells in its second half, each half laid out
// [i][j][k / 2].  Natural cell (i, j, k) is element k >> 1 of row (i, j) in the
// half of parity (i + j + k) & 1, and
//   - its i and j neighbours (other colour) have the SAME index in the other
//     half's rows (i +- 1, j) and (i, j +- 1);
//   - its k neighbours are elements (k >> 1) - 1 + q and (k >> 1) + q of the
//     other half's row (i, j), with q = k & 1;
//   - its parent on the next level is (i >> 1, j >> 1, k >> 1) in natural order.
// An 8-cell group of the active lists (natural k = 8 kg .. 8 kg + 7) is
// elements 4 kg .. 4 kg + 3 of the row in each half.
//
// One lane updates the 4 cells of the active colour in one active group: one
// 8-byte load of their stencil words, 16-byte loads of their r and z and of
// the other colour's four neighbour rows and own row, one 16-byte store -- all
// of it data the update uses.  The arithmetic is smooth_cell (smooth8.cuh),
// cell by cell in the reference's order (multigrid/mgpcg.py:72-86), so results
// are bit-identical to the natural-order kernels.
//
// Modes of one half-sweep (phase 0 updates the odd cells, phase 1 the even):
//   kFirst    first pre-smoothing half-sweep (phase 0, from zero): reads the
//             natural residual rn, writes both halves of the split residual
//             rs and z = r / d on the odd cells; the even cells are not
//             touched (the next half-sweep runs kOwnZero).
//   kOwnZero  second half-sweep of the first iteration: the updated cells'
//             own z is 0 and is not read.
//   kInPlace  z updated in place.
//   kProlong  first post-smoothing half-sweep (phase 1): reads zin + zc[I/2]
//             (multigrid/mgpcg.py:113-116) and writes both halves of zout:
//             the updated even cells and the odd cells of the group with the
//             prolongation added (0 off the fluid).
//   kLast     last post-smoothing half-sweep (phase 0): writes the group's 8
//             cells to the natural-order output zn (float), the even cells
//             passed through (0 off the fluid).
// Only the groups of the active list are visited; the other groups of the
// split buffers are never read for a value that enters a fluid cell's update.
#pragma once

#include "smooth8.cuh"

namespace flub {

enum SplitMode { kFirst = 0, kOwnZero = 1, kInPlace = 2, kProlong = 3, kLast = 4 };

struct SplitArgs {
    Dims D;
    const int *act, *act_n;     // active 8-cell groups of level 0
    const uint16_t *sws;        // stencil words, colour-split
    const void *rn;             // kFirst: natural residual (TRN)
    void *rs;                   // colour-split residual (TR): written by kFirst, read by the others
    const void *zin;            // kProlong: colour-split input z (TZI)
    void *z;                    // colour-split z (TZ), in place / output
    const void *zc;             // kProlong: next level's correction, natural order (TC)
    float zc_scale;
    float *zn;                  // kLast: natural-order output
    // kLast: z.r of the CG step folded in (mgpcg.py:401, 451): dot 1 --
    // zr_old = z.r and p = z (the solve's prologue), dot 2 -- beta = z.r /
    // zr_old, zr_old = z.r (each iteration), dot 3 -- the flexible beta =
    // (z.r - z.r_old) / zr_old of the mixed-precision solve; 0 -- none.  rdot
    // and rold are natural-order FP32 vectors; zscaled: the CG's z is
    // st->zscale times the V-cycle's output (mixed precision).  The per-group
    // sums are k8_dot_zr's / k8_dot_zr_flex's.
    int dot, zscaled;
    const float *rdot, *rold;
    float *pinit;
    MgState *st;
    double *partials;
};

// Stencil word of a fluid cell whose six neighbours are all fluid (code 2 in
// all seven 2-bit fields), twice: the 4 words of a lane are all interior when
// both halves of its 8-byte word load equal this.
constexpr uint32_t kInteriorWord2 = 0x2AAA2AAAu;

// smooth_cell for an interior word (d = 6), without the per-cell word test.
__device__ __forceinline__ float smooth_interior(float xc, float xip, float xim, float xjp, float xjm, float xkp,
                                                 float xkm, float r) {
    return __fadd_rn(xc, div6_rn(__fadd_rn(r, interior_nbsum(xc, xip, xim, xjp, xjm, xkp, xkm))));
}

__device__ __forceinline__ uint32_t word4_at(uint2 w, int m) {
    const uint32_t v = m < 2 ? w.x : w.y;
    return (m & 1) ? (v >> 16) : (v & 0xffffu);
}

// The code of the cell on the other side of word w's k+ (kp = true) or k-
// neighbour bits.
__device__ __forceinline__ uint32_t word_kcode(uint32_t w, bool kp) { return sw_code(w, kp ? 5 : 6); }

// Register bound of 3 blocks of 256 threads per SM for the lean modes (the
// in-place FP32 sweep then takes 64 registers and 4 blocks are resident), 4
// for the prolongation and the natural-order output.  Measured on the 256^3
// and 512^3 dam breaks: the lean modes at 5 blocks (48 registers) are as fast
// at 256^3 and 10 % slower at 512^3 (fewer groups in flight at once stream
// from DRAM more efficiently), 6 spills, and 2 blocks, or two groups per lane
// with their loads issued together, are slower at both sizes.
template <int kMode, typename TRN, typename TR, typename TZI, typename TZ, typename TC>
__global__ void __launch_bounds__(256, (kMode == kProlong || kMode == kLast) ? 4 : 3)
    k_smooth_split(const SplitArgs A, int phase, unsigned long long *kc) {
    pdl_open();
    const Dims D = A.D;
    const int hz = D.nz >> 1;             // split row length
    const int hn = (int)(D.n() >> 1);     // elements per half
    const int sj = hz, si = D.ny * hz;    // split strides of j and i
    const int col = 1 - phase;            // colour of the updated cells: 1 odd, 0 even
    const int uoff = col ? hn : 0, voff = col ? 0 : hn;
    const TR *rs = static_cast<const TR *>(A.rs);
    TZ *z = static_cast<TZ *>(A.z);
    const int total = *A.act_n;
    const int stride = gridDim.x * blockDim.x;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int g_next = t < total ? __ldg(A.act + t) : 0;
    // the list and the first stencil words do not depend on the previous kernel
    uint2 wd_next = make_uint2(0u, 0u);
    if (t < total) {
        int i0, j0, kg0;
        group_ijk(g_next, D, i0, j0, kg0);
        wd_next = __ldg(reinterpret_cast<const uint2 *>(A.sws + uoff + (i0 * D.ny + j0) * hz + 4 * kg0));
    }
    pdl_wait(kc);
    bool first = true;
    double zr = 0.0, zro = 0.0;  // kLast with A.dot: this thread's parts of z.r and z.r_old
    const float zsc = (kMode == kLast && A.dot && A.zscaled) ? A.st->zscale : 1.0f;
    for (; t < total; t += stride) {
        const int g = g_next;
        const int tn = t + stride;
        g_next = tn < total ? __ldg(A.act + tn) : 0;
        int i, j, kg;
        group_ijk(g, D, i, j, kg);
        const int h = (i * D.ny + j) * hz + 4 * kg;  // split index of the group's first element
        const int q = (col + i + j) & 1;             // updated cell m sits at natural k = 8 kg + 2 m + q
        const uint2 wd = first ? wd_next : __ldg(reinterpret_cast<const uint2 *>(A.sws + uoff + h));
        first = false;
        float rr[4];
        if (kMode == kFirst) {
            // natural residual row -> both halves of the split residual
            float rv[8];
            St<TRN>::ld8_ro(static_cast<const TRN *>(A.rn) + ((size_t)g << 3), rv);
            const int p = (i + j) & 1;  // natural cell m is even when (p + m) is even
            float re[4], ro[4];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                if (((p + m) & 1) == 0) re[m >> 1] = rv[m];
                else ro[m >> 1] = rv[m];
            }
            TR *rsw = static_cast<TR *>(A.rs);
            St<TR>::st4(rsw + h, re);
            St<TR>::st4(rsw + hn + h, ro);
#pragma unroll
            for (int m = 0; m < 4; m++) rr[m] = col ? ro[m] : re[m];
            float out[4];
#pragma unroll
            for (int m = 0; m < 4; m++)
                out[m] = smooth_cell<true>(word4_at(wd, m), 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, rr[m]);
            St<TZ>::st4(z + uoff + h, out);
            continue;
        }
        St<TR>::ld4_ro(rs + uoff + h, rr);
        const bool hip = i + 1 < D.nx, him = i > 0, hjp = j + 1 < D.ny, hjm = j > 0;
        const bool hkm = kg > 0, hkp = 4 * kg + 4 < hz;
        // operands: own z, the other colour's row (i, j) as the window w[0..4]
        // (w[m] is cell m's k- neighbour, w[m + 1] its k+ neighbour), and its
        // four neighbour rows
        float xc[4] = {0.f, 0.f, 0.f, 0.f}, w[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        float zip[4] = {0.f, 0.f, 0.f, 0.f}, zim[4] = {0.f, 0.f, 0.f, 0.f};
        float zjp[4] = {0.f, 0.f, 0.f, 0.f}, zjm[4] = {0.f, 0.f, 0.f, 0.f};
        float vc[4];
        if (kMode == kProlong) {
            const TZI *zi = static_cast<const TZI *>(A.zin);
            const TC *zc = static_cast<const TC *>(A.zc);
            const float s = A.zc_scale;
            const int cy = D.ny >> 1;  // the coarse level is nx/2 x ny/2 x hz, natural order
            // coarse row (I, J) at K = 4 kg .. 4 kg + 3: the parents of elements h .. h + 3
            auto crow = [&](int ii, int jj, float o[4]) {
                St<TC>::ld4_ro(zc + ((size_t)((ii >> 1) * cy + (jj >> 1)) * hz + 4 * kg), o);
            };
            float cc[4], cn[4];
            crow(i, j, cc);
            St<TZI>::ld4(zi + uoff + h, xc);
            St<TZI>::ld4(zi + voff + h, vc);
#pragma unroll
            for (int m = 0; m < 4; m++) {
                xc[m] = __fadd_rn(xc[m], __fmul_rn(cc[m], s));
                vc[m] = __fadd_rn(vc[m], __fmul_rn(cc[m], s));
            }
            if (hip) {
                St<TZI>::ld4(zi + voff + h + si, zip);
                crow(i + 1, j, cn);
#pragma unroll
                for (int m = 0; m < 4; m++) zip[m] = __fadd_rn(zip[m], __fmul_rn(cn[m], s));
            }
            if (him) {
                St<TZI>::ld4(zi + voff + h - si, zim);
                crow(i - 1, j, cn);
#pragma unroll
                for (int m = 0; m < 4; m++) zim[m] = __fadd_rn(zim[m], __fmul_rn(cn[m], s));
            }
            if (hjp) {
                St<TZI>::ld4(zi + voff + h + sj, zjp);
                crow(i, j + 1, cn);
#pragma unroll
                for (int m = 0; m < 4; m++) zjp[m] = __fadd_rn(zjp[m], __fmul_rn(cn[m], s));
            }
            if (hjm) {
                St<TZI>::ld4(zi + voff + h - sj, zjm);
                crow(i, j - 1, cn);
#pragma unroll
                for (int m = 0; m < 4; m++) zjm[m] = __fadd_rn(zjm[m], __fmul_rn(cn[m], s));
            }
            // the window's fifth value: element h - 1 (q = 0) or h + 4 (q = 1),
            // whose parent is coarse K = 4 kg - 1 or 4 kg + 4
            const size_t crow0 = (size_t)((i >> 1) * cy + (j >> 1)) * hz;
            if (q == 0 && hkm)
                w[0] = __fadd_rn(St<TZI>::ld(zi + voff + h - 1), __fmul_rn(St<TC>::ld_ro(zc + crow0 + 4 * kg - 1), s));
            if (q == 1 && hkp)
                w[4] = __fadd_rn(St<TZI>::ld(zi + voff + h + 4), __fmul_rn(St<TC>::ld_ro(zc + crow0 + 4 * kg + 4), s));
        } else {
            if (kMode != kOwnZero) St<TZ>::ld4(z + uoff + h, xc);
            St<TZ>::ld4(z + voff + h, vc);
            if (hip) St<TZ>::ld4(z + voff + h + si, zip);
            if (him) St<TZ>::ld4(z + voff + h - si, zim);
            if (hjp) St<TZ>::ld4(z + voff + h + sj, zjp);
            if (hjm) St<TZ>::ld4(z + voff + h - sj, zjm);
            if (q == 0 && hkm) w[0] = St<TZ>::ld(z + voff + h - 1);
            if (q == 1 && hkp) w[4] = St<TZ>::ld(z + voff + h + 4);
        }
        // w[t] is element h - 1 + q + t of the other colour's row
#pragma unroll
        for (int m = 0; m < 4; m++) w[m + 1 - q] = vc[m];
        float out[4], vo[4];
        if (wd.x == kInteriorWord2 && wd.y == kInteriorWord2) {
            // four interior cells (most of a water body): their k neighbours, the
            // other colour's elements of the group, are fluid too
#pragma unroll
            for (int m = 0; m < 4; m++) {
                out[m] = smooth_interior(xc[m], zip[m], zim[m], zjp[m], zjm[m], w[m + 1], w[m], rr[m]);
                vo[m] = vc[m];
            }
        } else {
#pragma unroll
            for (int m = 0; m < 4; m++)
                out[m] = smooth_cell<false>(word4_at(wd, m), xc[m], zip[m], zim[m], zjp[m], zjm[m], w[m + 1], w[m],
                                            rr[m]);
            // the other colour's cells of the group: element m is the k+ neighbour
            // of updated cell m when q = 0, its k- neighbour when q = 1
#pragma unroll
            for (int m = 0; m < 4; m++)
                vo[m] = word_kcode(word4_at(wd, m), q == 0) == kCodeFluid ? vc[m] : 0.0f;
        }
        if (kMode == kLast) {
            // natural row of the group: updated cell m at offset 2 m + q, the
            // other colour's element m at 2 m + 1 - q
            float o8[8];
#pragma unroll
            for (int m = 0; m < 4; m++) {
                o8[2 * m + q] = out[m];
                o8[2 * m + 1 - q] = vo[m];
            }
            St<float>::st8(A.zn + ((size_t)g << 3), o8);
            if (A.dot) {
                float zv[8], rv[8];
#pragma unroll
                for (int m = 0; m < 8; m++) zv[m] = A.zscaled ? __fmul_rn(o8[m], zsc) : o8[m];
                St<float>::ld8_ro(A.rdot + ((size_t)g << 3), rv);
                zr += dot8_ff(zv, rv);
                if (A.dot == 3) {
                    float ov[8];
                    St<float>::ld8_ro(A.rold + ((size_t)g << 3), ov);
                    zro += dot8_ff(zv, ov);
                }
                if (A.dot == 1) St<float>::st8(A.pinit + ((size_t)g << 3), zv);
            }
        } else {
            St<TZ>::st4(z + uoff + h, out);
            if (kMode == kProlong) St<TZ>::st4(z + voff + h, vo);
        }
    }
    if (kMode == kLast && A.dot) {
        // the grid's z.r in FP64 (deterministic two-level reduction) and the
        // CG scalars, as k8_dot_zr sets them
        __shared__ double red[32];
        if (A.dot == 3) {
            const double bo = block_sum(zro, red);
            __syncthreads();
            if (threadIdx.x == 0) A.partials[kMaxRedBlocks + blockIdx.x] = bo;
        }
        double tot;
        if (finish_partials(zr, A.partials, &A.st->ticket, red, &tot)) {
            double t2 = 0.0;
            if (A.dot == 3) {
                __syncthreads();
                for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x)
                    t2 += __ldcg(&A.partials[kMaxRedBlocks + q]);
                t2 = block_sum(t2, red);
            }
            if (threadIdx.x == 0) {
                if (A.dot == 1) {
                    A.st->zr_old = tot;
                } else {
                    const double beta = (A.dot == 3 ? tot - t2 : tot) / (A.st->zr_old + A.st->eps);
                    A.st->beta = beta;
                    A.st->zr_old = tot;
                    if (!isfinite(beta)) A.st->status = FLUB_ERR_BREAKDOWN;
                }
            }
        }
    }
}

}  // namespace flub
