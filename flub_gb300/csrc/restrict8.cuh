// Residual + restriction (multigrid/mgpcg.py:94-101, written as a gather) on
// groups of 8 fine cells: four lanes produce 4 consecutive coarse cells
// (I, J, K0..K0+3) from the four fine rows (2I + ii, 2J + jj), k = 2 K0 .. 2 K0
// + 7, each one 8-cell group read with vector loads.  Per coarse cell the 8
// children are summed in the reference's order (ii, jj, kk), kk fastest, with
// the same FP32 operations as the scalar k_restrict, so results are
// bit-identical.
#pragma once

#include "cg8.cuh"
#include "store.cuh"

namespace flub {

// Natural-order row (ii, jj), cells 8 kg .. 8 kg + 7, of a colour-split
// level-0 vector (smooth_split.cuh): element m >> 1 of the half of parity
// (ii + jj + m) & 1.
template <typename TZ>
__device__ __forceinline__ void ld_row8_split(const TZ *__restrict__ z, const Dims D, int ii, int jj, int kg,
                                              float o[8]) {
    const int hz = D.nz >> 1, hn = (int)(D.n() >> 1);
    const int h = (ii * D.ny + jj) * hz + 4 * kg;
    const int p = (ii + jj) & 1;
    float e[4], od[4];
    St<TZ>::ld4_ro(z + h, e);
    St<TZ>::ld4_ro(z + hn + h, od);
#pragma unroll
    for (int m = 0; m < 8; m++) o[m] = ((p + m) & 1) ? od[m >> 1] : e[m >> 1];
}

// Natural cell (ii, jj, k) of a colour-split level-0 vector.
template <typename TZ>
__device__ __forceinline__ float ld_cell_split(const TZ *__restrict__ z, const Dims D, int ii, int jj, int k) {
    const int hz = D.nz >> 1, hn = (int)(D.n() >> 1);
    return St<TZ>::ld_ro(z + (((ii + jj + k) & 1) ? hn : 0) + (ii * D.ny + jj) * hz + (k >> 1));
}

// (r + L z) on the 8 cells of fine group g (L z is 0 at non-fluid cells),
// neighbour codes from the stencil words (sw, or the codes when sw is NULL).
// kNC: r and z may be read through the read-only path (see smooth8_pass).
// kSplitZ: z is a colour-split level-0 vector (r stays in natural order).
template <bool kNC, bool kSplitZ, typename TR, typename TZ>
__device__ __forceinline__ void residual_row8(const TR *__restrict__ r, const TZ *__restrict__ z,
                                              const uint8_t *__restrict__ code, const uint16_t *__restrict__ sw,
                                              const Dims D, int g, float out[8]) {
    int i, j, kg;
    group_ijk(g, D, i, j, kg);
    const int k0 = kg << 3;
    const int sj = D.nz, si = D.ny * D.nz;
    const int c0 = g << 3;
    float rv[8];
    if (kNC) St<TR>::ld8_ro(r + c0, rv); else St<TR>::ld8_cg(r + c0, rv);
    const uint4 wd = load_words8(sw, code, D, i, j, k0, c0);
    if (!words_have_fluid(wd)) {
#pragma unroll
        for (int m = 0; m < 8; m++) out[m] = __fadd_rn(rv[m], 0.0f);
        return;
    }
    const bool hip = i + 1 < D.nx, him = i > 0, hjp = j + 1 < D.ny, hjm = j > 0;
    const bool hkp = k0 + 8 < D.nz, hkm = k0 > 0;
    float xc[8], xip[8], xim[8], xjp[8], xjm[8];
    auto ld8 = [&](const TZ *p, float o[8]) {
        if (kNC) St<TZ>::ld8_ro(p, o); else St<TZ>::ld8_cg(p, o);
    };
    auto ld1 = [&](const TZ *p) { return kNC ? St<TZ>::ld_ro(p) : St<TZ>::ld_cg(p); };
#pragma unroll
    for (int m = 0; m < 8; m++) xip[m] = xim[m] = xjp[m] = xjm[m] = 0.0f;
    float xkm = 0.0f, xkp = 0.0f;
    if (kSplitZ) {
        ld_row8_split(z, D, i, j, kg, xc);
        if (hip) ld_row8_split(z, D, i + 1, j, kg, xip);
        if (him) ld_row8_split(z, D, i - 1, j, kg, xim);
        if (hjp) ld_row8_split(z, D, i, j + 1, kg, xjp);
        if (hjm) ld_row8_split(z, D, i, j - 1, kg, xjm);
        if (hkm) xkm = ld_cell_split(z, D, i, j, k0 - 1);
        if (hkp) xkp = ld_cell_split(z, D, i, j, k0 + 8);
    } else {
        ld8(z + c0, xc);
        if (hip) ld8(z + c0 + si, xip);
        if (him) ld8(z + c0 - si, xim);
        if (hjp) ld8(z + c0 + sj, xjp);
        if (hjm) ld8(z + c0 - sj, xjm);
        if (hkm) xkm = ld1(z + c0 - 1);
        if (hkp) xkp = ld1(z + c0 + 8);
    }
#pragma unroll
    for (int m = 0; m < 8; m++) {
        float lz = 0.0f;
        const uint32_t w = word_at(wd, m);
        if (sw_code(w, 0) == kCodeFluid)
            lz = sw_nbsum(w, xc[m], xip[m], xim[m], xjp[m], xjm[m], m < 7 ? xc[m + 1] : xkp, m > 0 ? xc[m - 1] : xkm);
        out[m] = __fadd_rn(rv[m], lz);
    }
}

// Coarse level C (fine = 2C).  Work items: the coarse half-groups of 4 cells
// (I, J, 4 K4 .. 4 K4 + 3): with a coarse active list, the 2 halves of every
// listed coarse group (the coarse cells outside the list are not fluid and keep
// r_c = 0, cleared at set_tags and never written otherwise); without one, every
// half-group.  Four adjacent lanes share an item, lane q = 2 ii + jj computing
// the residual of fine row (2I + ii, 2J + jj) -- a quarter of the registers
// and four times the lanes of one thread per item, to hide memory latency.
// The 8 children of each coarse cell are then summed in the reference's order
// (ii, jj, kk), kk fastest, from values broadcast by shuffles; the first
// lane of the four stores the 4 coarse values.
// out_scale: restriction scale (times 1/8 between FP16 levels at 8^-l).
// Grid: one-dimensional, grid-stride by warps (all lanes of a warp run the same
// iterations, so the shuffles see every lane).
// bid / nblk: this block's index and the number of blocks sharing the loop.
// pdl: called at the start of a kernel launched with programmatic dependent
// launch; the item count is read first, then pdl_wait(kc).
template <bool kNC, bool kSplitZ, typename TRI, typename TZI, typename TRO>
__device__ __forceinline__ void restrict8_pass(const TRI *__restrict__ rf, const TZI *__restrict__ zf,
                                               const uint8_t *__restrict__ cf, const uint16_t *__restrict__ swf,
                                               TRO *__restrict__ rc, const uint8_t *__restrict__ cc, const Dims C,
                                               float out_scale, const int *__restrict__ act,
                                               const int *__restrict__ act_n, int bid, int nblk, bool pdl = false,
                                               unsigned long long *kc = nullptr) {
    const Dims F{2 * C.nx, 2 * C.ny, 2 * C.nz};
    const int nh = (int)(C.n() >> 2);  // coarse half-groups of 4 cells
    const int items = act ? 2 * *act_n : nh;
    const int total = 4 * items;
    if (pdl) pdl_wait(kc);
    const int fz8 = F.nz >> 3;
    const int lane = threadIdx.x & 31, q = lane & 3;
    const int stride = nblk * blockDim.x;
    for (int base = bid * blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
        const int t = base + lane;
        const bool valid = t < total;  // the 4 lanes of an item agree (total is a multiple of 4)
        const int it = t >> 2;
        const int h = valid ? (act ? 2 * __ldg(act + (it >> 1)) + (it & 1) : it) : 0;  // half-group index
        const int q0 = h << 2;                                                          // first coarse cell
        const uint32_t codes4 = valid ? __ldg(reinterpret_cast<const uint32_t *>(cc + q0)) : 0u;
        const bool any = (codes4 & 0x02020202u) != 0u;  // a fluid coarse cell among the 4
        float v[8];
#pragma unroll
        for (int m = 0; m < 8; m++) v[m] = 0.0f;
        if (any) {
            // (I, J, K4) of the half-group: the coarse grid read as 4-cell groups
            int I, J, K4;
            group_ijk(h, Dims{C.nx, C.ny, C.nz << 1}, I, J, K4);  // C.nz / 4 half-groups per row
            const int g = ((2 * I + (q >> 1)) * F.ny + 2 * J + (q & 1)) * fz8 + K4;  // fine group at k = 8 K4
            residual_row8<kNC, kSplitZ>(rf, zf, cf, swf, F, g, v);
        }
        // coarse cell m gets (v[2m], v[2m + 1]) of lanes q = 0..3 in turn
        float s[4];
        const int src = lane & ~3;
#pragma unroll
        for (int m = 0; m < 4; m++) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const float a = __shfl_sync(0xffffffffu, v[2 * m], src + u);
                const float b = __shfl_sync(0xffffffffu, v[2 * m + 1], src + u);
                s[m] = u == 0 ? __fadd_rn(a, b) : __fadd_rn(__fadd_rn(s[m], a), b);
            }
        }
        if (!valid || q != 0) continue;
        if (any) {
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const uint8_t cm = (uint8_t)((codes4 >> (8 * m)) & 0xffu);
                s[m] = cm == kCodeFluid ? __fmul_rn(s[m], out_scale) : 0.0f;
            }
        } else {
#pragma unroll
            for (int m = 0; m < 4; m++) s[m] = 0.0f;
        }
        St<TRO>::st4(rc + q0, s);
    }
}

template <typename TRI, typename TZI, typename TRO>
__global__ void __launch_bounds__(256, 4) k_restrict8(const TRI *__restrict__ rf, const TZI *__restrict__ zf,
                                                      const uint8_t *__restrict__ cf, const uint16_t *__restrict__ swf,
                                                      TRO *__restrict__ rc,
                                                      const uint8_t *__restrict__ cc, Dims C, float out_scale,
                                                      const int *__restrict__ act, const int *__restrict__ act_n,
                                                      unsigned long long *kc) {
    pdl_open();
    restrict8_pass<true, false>(rf, zf, cf, swf, rc, cc, C, out_scale, act, act_n, blockIdx.x, gridDim.x, true, kc);
}

// Restriction out of level 0 whose pre-smoothed z is colour-split
// (smooth_split.cuh); r is the natural-order residual.
template <typename TRI, typename TZI, typename TRO>
__global__ void __launch_bounds__(256, 4) k_restrict8_split(const TRI *__restrict__ rf, const TZI *__restrict__ zf,
                                                            const uint8_t *__restrict__ cf,
                                                            const uint16_t *__restrict__ swf, TRO *__restrict__ rc,
                                                            const uint8_t *__restrict__ cc, Dims C, float out_scale,
                                                            const int *__restrict__ act,
                                                            const int *__restrict__ act_n, unsigned long long *kc) {
    pdl_open();
    restrict8_pass<true, true>(rf, zf, cf, swf, rc, cc, C, out_scale, act, act_n, blockIdx.x, gridDim.x, true, kc);
}

}  // namespace flub
