// Residual + restriction (multigrid/mgpcg.py:94-101, written as a gather) on
// groups of 8 fine cells: one thread produces 4 consecutive coarse cells
// (I, J, K0..K0+3) from the four fine rows (2I + ii, 2J + jj), k = 2 K0 .. 2 K0
// + 7, each one 8-cell group read with vector loads.  Per coarse cell the 8
// children are summed in the reference's order (ii, jj, kk), kk fastest, with
// the same FP32 operations as the scalar k_restrict, so results are
// bit-identical.
#pragma once

#include "cg8.cuh"
#include "store.cuh"

namespace flub {

// (r + L z) on the 8 cells of fine group g (L z is 0 at non-fluid cells),
// neighbour codes from the stencil words (sw, or the codes when sw is NULL).
template <typename TR, typename TZ>
__device__ __forceinline__ void residual_row8(const TR *__restrict__ r, const TZ *__restrict__ z,
                                              const uint8_t *__restrict__ code, const uint16_t *__restrict__ sw,
                                              const Dims D, int g, float out[8]) {
    int i, j, kg;
    group_ijk(g, D, i, j, kg);
    const int k0 = kg << 3;
    const int sj = D.nz, si = D.ny * D.nz;
    const int c0 = g << 3;
    float rv[8];
    St<TR>::ld8_ro(r + c0, rv);
    const uint4 wd = load_words8(sw, code, D, i, j, k0, c0);
    if (!words_have_fluid(wd)) {
#pragma unroll
        for (int m = 0; m < 8; m++) out[m] = __fadd_rn(rv[m], 0.0f);
        return;
    }
    const bool hip = i + 1 < D.nx, him = i > 0, hjp = j + 1 < D.ny, hjm = j > 0;
    const bool hkp = k0 + 8 < D.nz, hkm = k0 > 0;
    float xc[8], xip[8], xim[8], xjp[8], xjm[8];
    St<TZ>::ld8_ro(z + c0, xc);
#pragma unroll
    for (int m = 0; m < 8; m++) xip[m] = xim[m] = xjp[m] = xjm[m] = 0.0f;
    if (hip) St<TZ>::ld8_ro(z + c0 + si, xip);
    if (him) St<TZ>::ld8_ro(z + c0 - si, xim);
    if (hjp) St<TZ>::ld8_ro(z + c0 + sj, xjp);
    if (hjm) St<TZ>::ld8_ro(z + c0 - sj, xjm);
    const float xkm = hkm ? St<TZ>::ld_ro(z + c0 - 1) : 0.0f;
    const float xkp = hkp ? St<TZ>::ld_ro(z + c0 + 8) : 0.0f;
#pragma unroll
    for (int m = 0; m < 8; m++) {
        float lz = 0.0f;
        const uint32_t w = word_at(wd, m);
        if (sw_code(w, 0) == kCodeFluid) {
            const float c = xc[m];
            float tp, tm;
            uint32_t cn;
            tp = 0.0f; tm = 0.0f;
            cn = sw_code(w, 1); if (cn != kCodeSolid) tp = __fsub_rn(cn == kCodeAir ? 0.0f : xip[m], c);
            cn = sw_code(w, 2); if (cn != kCodeSolid) tm = __fsub_rn(cn == kCodeAir ? 0.0f : xim[m], c);
            lz = __fadd_rn(lz, __fadd_rn(tp, tm));
            tp = 0.0f; tm = 0.0f;
            cn = sw_code(w, 3); if (cn != kCodeSolid) tp = __fsub_rn(cn == kCodeAir ? 0.0f : xjp[m], c);
            cn = sw_code(w, 4); if (cn != kCodeSolid) tm = __fsub_rn(cn == kCodeAir ? 0.0f : xjm[m], c);
            lz = __fadd_rn(lz, __fadd_rn(tp, tm));
            tp = 0.0f; tm = 0.0f;
            cn = sw_code(w, 5); if (cn != kCodeSolid) tp = __fsub_rn(cn == kCodeAir ? 0.0f : (m < 7 ? xc[m + 1] : xkp), c);
            cn = sw_code(w, 6); if (cn != kCodeSolid) tm = __fsub_rn(cn == kCodeAir ? 0.0f : (m > 0 ? xc[m - 1] : xkm), c);
            lz = __fadd_rn(lz, __fadd_rn(tp, tm));
        }
        out[m] = __fadd_rn(rv[m], lz);
    }
}

// Coarse level C (fine = 2C).  Items: with a coarse active list, 2 per listed
// coarse group (its two halves of 4 cells); the coarse cells outside the list
// are not fluid and keep r_c = 0 (cleared at set_tags, never written
// otherwise).  Without a list, every half-group of the coarse grid.
// out_scale: restriction scale (times 1/8 between FP16 levels at 8^-l).
template <typename TRI, typename TZI, typename TRO>
__global__ void __launch_bounds__(256) k_restrict8(const TRI *__restrict__ rf, const TZI *__restrict__ zf,
                                                   const uint8_t *__restrict__ cf, const uint16_t *__restrict__ swf,
                                                   TRO *__restrict__ rc,
                                                   const uint8_t *__restrict__ cc, Dims C, float out_scale,
                                                   const int *__restrict__ act, const int *__restrict__ act_n,
                                                   unsigned long long *kc) {
    count_kernel(kc);
    const Dims F{2 * C.nx, 2 * C.ny, 2 * C.nz};
    const int nh = (int)(C.n() >> 2);  // coarse half-groups of 4 cells
    const int total = act ? 2 * *act_n : nh;
    const int fz8 = F.nz >> 3;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int h = act ? 2 * __ldg(act + (t >> 1)) + (t & 1) : t;  // half-group index
        const int q0 = h << 2;                                         // first coarse cell
        const uint32_t codes4 = __ldg(reinterpret_cast<const uint32_t *>(cc + q0));
        float s[4];
        if ((codes4 & 0x02020202u) == 0u) {
            // no fluid coarse cell among the 4
#pragma unroll
            for (int m = 0; m < 4; m++) s[m] = 0.0f;
        } else {
            // (I, J, K4) of the half-group: the coarse grid read as 4-cell groups
            int I, J, K4;
            group_ijk(h, Dims{C.nx, C.ny, C.nz << 1}, I, J, K4);  // C.nz / 4 half-groups per row
            bool first[4] = {true, true, true, true};
#pragma unroll
            for (int m = 0; m < 4; m++) s[m] = 0.0f;
#pragma unroll
            for (int ii = 0; ii < 2; ii++)
#pragma unroll
                for (int jj = 0; jj < 2; jj++) {
                    const int g = ((2 * I + ii) * F.ny + 2 * J + jj) * fz8 + K4;  // fine group at k = 8 K4
                    float v[8];
                    residual_row8(rf, zf, cf, swf, F, g, v);
#pragma unroll
                    for (int m = 0; m < 4; m++) {
#pragma unroll
                        for (int kk = 0; kk < 2; kk++) {
                            const float x = v[2 * m + kk];
                            s[m] = first[m] ? x : __fadd_rn(s[m], x);
                            first[m] = false;
                        }
                    }
                }
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const uint8_t cm = (uint8_t)((codes4 >> (8 * m)) & 0xffu);
                s[m] = cm == kCodeFluid ? __fmul_rn(s[m], out_scale) : 0.0f;
            }
        }
        St<TRO>::st4(rc + q0, s);
    }
}

}  // namespace flub
