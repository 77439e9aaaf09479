// Vectorised red-black smoothing: one thread owns 8 consecutive cells along k.
//
// Same arithmetic as k_smooth_half (multigrid/mgpcg.py:72-86) cell by cell, in
// the reference's order, so results stay bit-identical; the gain is in the
// instruction count: every row of 8 values is one pair of 16-byte loads (z, r)
// or one 8-byte load (cell codes), and indices are 32-bit.
#pragma once

#include "mg_kernels.cuh"
#include "store.cuh"

namespace flub {

struct Row8 {
    float v[8];
};

__device__ __forceinline__ void load_row8(const float *__restrict__ p, Row8 &o) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    const float4 b = __ldg(reinterpret_cast<const float4 *>(p) + 1);
    o.v[0] = a.x; o.v[1] = a.y; o.v[2] = a.z; o.v[3] = a.w;
    o.v[4] = b.x; o.v[5] = b.y; o.v[6] = b.z; o.v[7] = b.w;
}

// Row of z that may be written by other threads of the same launch (other
// colour only): plain loads, not the read-only path.
__device__ __forceinline__ void load_row8_rw(const float *p, Row8 &o) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0];
    const float4 b = reinterpret_cast<const float4 *>(p)[1];
    o.v[0] = a.x; o.v[1] = a.y; o.v[2] = a.z; o.v[3] = a.w;
    o.v[4] = b.x; o.v[5] = b.y; o.v[6] = b.z; o.v[7] = b.w;
}

__device__ __forceinline__ void zero_row8(Row8 &o) {
#pragma unroll
    for (int m = 0; m < 8; m++) o.v[m] = 0.0f;
}

__device__ __forceinline__ uint2 load_codes8(const uint8_t *__restrict__ p) {
    return __ldg(reinterpret_cast<const uint2 *>(p));
}

__device__ __forceinline__ uint8_t code_at(uint2 c, int m) {
    return (uint8_t)(((m < 4 ? c.x : c.y) >> (8 * (m & 3))) & 0xffu);
}

// ---------------------------------------------------------------- stencil words
// One 16-bit word per cell: bits 0-1 its code, then 2 bits per neighbour in
// the order i+, i-, j+, j-, k+, k- (code 0 -- excluded -- for a neighbour
// outside the domain).  set_tags stores them per level (Level::sw); a kernel
// then loads the 8 words of a group with one 16-byte load instead of five rows
// of codes.  Without stored words (sw == NULL) they are assembled from the
// codes by the same function set_tags uses.
__device__ __forceinline__ uint32_t sw_code(uint32_t w, int q) { return (w >> (2 * q)) & 3u; }

__device__ __forceinline__ uint32_t word_at(const uint4 &u, int m) {
    const uint32_t v = m < 2 ? u.x : (m < 4 ? u.y : (m < 6 ? u.z : u.w));
    return (m & 1) ? (v >> 16) : (v & 0xffffu);
}

// Words of the 8 cells of the row starting at c0 = (i, j, k0), from the codes.
__device__ __forceinline__ uint4 words8_from_codes(const uint8_t *__restrict__ code, const Dims D, int i, int j,
                                                   int k0, int c0) {
    const int sj = D.nz, si = D.ny * D.nz;
    const uint2 z2 = make_uint2(0u, 0u);
    const uint2 cc = load_codes8(code + c0);
    const uint2 cip = i + 1 < D.nx ? load_codes8(code + c0 + si) : z2;
    const uint2 cim = i > 0 ? load_codes8(code + c0 - si) : z2;
    const uint2 cjp = j + 1 < D.ny ? load_codes8(code + c0 + sj) : z2;
    const uint2 cjm = j > 0 ? load_codes8(code + c0 - sj) : z2;
    const uint32_t ckm = k0 > 0 ? __ldg(code + c0 - 1) : 0u;
    const uint32_t ckp = k0 + 8 < D.nz ? __ldg(code + c0 + 8) : 0u;
    uint32_t w[8];
#pragma unroll
    for (int m = 0; m < 8; m++)
        w[m] = (uint32_t)code_at(cc, m) | ((uint32_t)code_at(cip, m) << 2) | ((uint32_t)code_at(cim, m) << 4) |
               ((uint32_t)code_at(cjp, m) << 6) | ((uint32_t)code_at(cjm, m) << 8) |
               ((m < 7 ? (uint32_t)code_at(cc, m + 1) : ckp) << 10) |
               ((m > 0 ? (uint32_t)code_at(cc, m - 1) : ckm) << 12);
    return make_uint4(w[0] | (w[1] << 16), w[2] | (w[3] << 16), w[4] | (w[5] << 16), w[6] | (w[7] << 16));
}

__device__ __forceinline__ uint4 load_words8(const uint16_t *__restrict__ sw, const uint8_t *__restrict__ code,
                                             const Dims D, int i, int j, int k0, int c0) {
    return sw ? __ldg(reinterpret_cast<const uint4 *>(sw + c0)) : words8_from_codes(code, D, i, j, k0, c0);
}

__device__ __forceinline__ bool words_have_fluid(const uint4 &u) {
    // a centre code of 2 in any of the 8 words (bit 1 of each 16-bit half)
    return (((u.x | u.y | u.z | u.w) & 0x00020002u) != 0u);
}

// z_eff[m] += scale * zc[parent] for the 8 cells of a row whose coarse row
// starts at pc (4 coarse values: cell m has parent m / 2).  scale is 1 for FP32
// levels and 8 between FP16 levels stored at 8^-l (exact powers of two).
template <typename TC>
__device__ __forceinline__ void add_coarse_row8(Row8 &o, const TC *__restrict__ pc, float scale) {
    float cv[4];
    St<TC>::ld4_ro(pc, cv);
#pragma unroll
    for (int m = 0; m < 8; m++) o.v[m] = __fadd_rn(o.v[m], __fmul_rn(cv[m >> 1], scale));
}

template <typename TC>
__device__ __forceinline__ float coarse_at(const TC *__restrict__ p, float scale) {
    return __fmul_rn(St<TC>::ld_ro(p), scale);
}

// One half-sweep over 8 cells per thread.
//   kFromZero: z is 0 before the sweep (first sweep of a level in the V-cycle);
//              zin and zc are not read.
//   kProlong:  the sweep reads zin + zc[I/2] (multigrid/mgpcg.py:113-116 fused
//              into the first post-smoothing sweep) and writes every cell to
//              zout != zin; otherwise zout == zin (in place).
// TO/TI/TR/TC: storage of zout, zin, r and the coarse zc (float, or __half in
// the mixed-precision V-cycle); arithmetic is FP32 throughout.
// Every non-fluid cell is written as 0 (its value is never read by a fluid
// cell's update, and the reference's sweeps leave it 0 by the end of the
// V-cycle), so a buffer that starts at 0 keeps z = 0 off the fluid.  With an
// active list (act != NULL) the caller asserts that invariant for zout, and
// only the groups of the list (those holding a fluid cell) are visited;
// without one every group is.
// Grid: one-dimensional, grid-stride over the groups.  Requires nz % 8 == 0.
template <bool kFromZero, bool kProlong, typename TO, typename TI, typename TR, typename TC>
__global__ void __launch_bounds__(256, 3) k_smooth8(TO *zout, const TI *zin, const TC *__restrict__ zc,
                                                    float zc_scale, const TR *__restrict__ r,
                                                    const uint8_t *__restrict__ code,
                                                    const uint16_t *__restrict__ sw, Dims D, int phase,
                                                    const int *__restrict__ act, const int *__restrict__ act_n,
                                                    unsigned long long *kc) {
    count_kernel(kc);
    const int ng = (int)(D.n() >> 3);
    FLUB_ACT_LOOP(g, act, act_n, ng) {
    int i, j, kg;
    group_ijk(g, D, i, j, kg);
    const int k0 = kg << 3;
    const int sj = D.nz, si = D.ny * D.nz;
    const int c0 = (i * D.ny + j) * D.nz + k0;
    const bool hip = i + 1 < D.nx, him = i > 0, hjp = j + 1 < D.ny, hjm = j > 0;
    const bool hkp = k0 + 8 < D.nz, hkm = k0 > 0;
    const int par = 1 - phase;
    const int b0 = (i + j + k0 + par) & 1;  // cell m is updated iff (m & 1) == b0

    // stencil words of the 8 cells (codes of each cell and its 6 neighbours)
    const uint4 wd = load_words8(sw, code, D, i, j, k0, c0);

    Row8 rr;
    St<TR>::ld8_ro(r + c0, rr.v);
    Row8 zc0, zip, zim, zjp, zjm;
    float zkm = 0.0f, zkp = 0.0f;
    if (kFromZero) {
        zero_row8(zc0);
    } else {
        St<TI>::ld8(zin + c0, zc0.v);
        if (hip) St<TI>::ld8(zin + c0 + si, zip.v); else zero_row8(zip);
        if (him) St<TI>::ld8(zin + c0 - si, zim.v); else zero_row8(zim);
        if (hjp) St<TI>::ld8(zin + c0 + sj, zjp.v); else zero_row8(zjp);
        if (hjm) St<TI>::ld8(zin + c0 - sj, zjm.v); else zero_row8(zjm);
        if (hkm) zkm = St<TI>::ld(zin + c0 - 1);
        if (hkp) zkp = St<TI>::ld(zin + c0 + 8);
        if (kProlong) {
            const int cy = D.ny >> 1, cz = D.nz >> 1;
            const int ci = i >> 1, cj = j >> 1, ck = k0 >> 1;
            const int cb = (ci * cy + cj) * cz + ck;
            add_coarse_row8(zc0, zc + cb, zc_scale);
            if (hip) add_coarse_row8(zip, zc + (((i + 1) >> 1) * cy + cj) * cz + ck, zc_scale);
            if (him) add_coarse_row8(zim, zc + (((i - 1) >> 1) * cy + cj) * cz + ck, zc_scale);
            if (hjp) add_coarse_row8(zjp, zc + (ci * cy + ((j + 1) >> 1)) * cz + ck, zc_scale);
            if (hjm) add_coarse_row8(zjm, zc + (ci * cy + ((j - 1) >> 1)) * cz + ck, zc_scale);
            if (hkm) zkm = __fadd_rn(zkm, coarse_at(zc + cb - 1, zc_scale));
            if (hkp) zkp = __fadd_rn(zkp, coarse_at(zc + cb + 4, zc_scale));
        }
    }

    float out[8];
#pragma unroll
    for (int m = 0; m < 8; m++) {
        const uint32_t w = word_at(wd, m);
        const uint32_t cm = sw_code(w, 0);
        out[m] = cm == kCodeFluid ? zc0.v[m] : 0.0f;
        if ((m & 1) != b0) continue;
        float zn = 0.0f;
        if (cm == kCodeFluid) {
            const float xc = zc0.v[m];
            int d = 0;
            float tp, tm, ret = 0.0f;
            uint32_t cn;
            // axis i
            tp = 0.0f; tm = 0.0f;
            cn = sw_code(w, 1); if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : zip.v[m], xc); d++; }
            cn = sw_code(w, 2); if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : zim.v[m], xc); d++; }
            ret = __fadd_rn(ret, __fadd_rn(tp, tm));
            // axis j
            tp = 0.0f; tm = 0.0f;
            cn = sw_code(w, 3); if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : zjp.v[m], xc); d++; }
            cn = sw_code(w, 4); if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : zjm.v[m], xc); d++; }
            ret = __fadd_rn(ret, __fadd_rn(tp, tm));
            // axis k
            tp = 0.0f; tm = 0.0f;
            cn = sw_code(w, 5);
            if (cn != kCodeSolid) { tp = __fsub_rn(cn == kCodeAir ? 0.0f : (m < 7 ? zc0.v[m + 1] : zkp), xc); d++; }
            cn = sw_code(w, 6);
            if (cn != kCodeSolid) { tm = __fsub_rn(cn == kCodeAir ? 0.0f : (m > 0 ? zc0.v[m - 1] : zkm), xc); d++; }
            ret = __fadd_rn(ret, __fadd_rn(tp, tm));
            if (d != 0) {
                if (kFromZero)
                    zn = __fdiv_rn(rr.v[m], (float)d);  // 0 + (r + L 0) / d, L 0 = 0
                else
                    zn = __fadd_rn(xc, __fdiv_rn(__fadd_rn(rr.v[m], ret), (float)d));
            }
        }
        out[m] = zn;
    }
    St<TO>::st8(zout + c0, out);
    }
}

}  // namespace flub
