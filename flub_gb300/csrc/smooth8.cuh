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

// Bit q of sw_ns(w) (q = 2, 4, .., 12) is set when neighbour q / 2 is not
// solid: with solid 0, air 1, fluid 2 that is bit q | bit q + 1 of the word.
__device__ __forceinline__ uint32_t sw_ns(uint32_t w) { return (w | (w >> 1)) & 0x1554u; }

// Neighbour sum of L x at a fluid cell from its stencil word w, in lap_at's
// operation order: per neighbour (i+, i-, j+, j-, k+, k-) 0 when solid, else
// (x_n - x_c) with x_n = 0 for air, summed in pairs per axis.  Bit tests on
// the word replace the per-neighbour code compares.
// Stencil word of a fluid cell whose six neighbours are all fluid (code 2 in
// all seven 2-bit fields): most cells of a water body.
constexpr uint32_t kInteriorWord = 0x2AAAu;

// a / 6 rounded to nearest, as __fdiv_rn(a, 6.0f), with Markstein's FMA
// correction of the product by the rounded reciprocal (P. Markstein, IBM J.
// Res. Dev. 34(1), 1990; q0 = a y, r = a - 6 q0 exactly, q = q0 + r y): three
// FP32 operations instead of a division.  tests/test_div6_exhaustive.py checks
// it bit for bit against IEEE division for every float32 with |a| in
// [2^-100, 2^100] and for the zeros, which return q0 (a zero of a's sign, as
// a / 6); the other inputs (tiny, huge, inf, NaN) take __fdiv_rn.
__device__ __forceinline__ float div6_rn(float a) {
    constexpr float y = 0x1.555556p-3f;  // 1/6 rounded to nearest
    const float m = fabsf(a);
    const float q0 = __fmul_rn(a, y);
    if (m >= 0x1p-100f && m <= 0x1p100f) return __fmaf_rn(__fmaf_rn(-q0, 6.0f, a), y, q0);
    if (m == 0.0f) return q0;
    return __fdiv_rn(a, 6.0f);
}

// sw_nbsum for an interior word: every neighbour counts and enters with its
// value, so the bit tests and selects drop out; the FP32 operations and their
// order are sw_nbsum's (pair sums per axis).
__device__ __forceinline__ float interior_nbsum(float xc, float xip, float xim, float xjp, float xjm, float xkp,
                                                float xkm) {
    float ret = __fadd_rn(0.0f, __fadd_rn(__fsub_rn(xip, xc), __fsub_rn(xim, xc)));
    ret = __fadd_rn(ret, __fadd_rn(__fsub_rn(xjp, xc), __fsub_rn(xjm, xc)));
    return __fadd_rn(ret, __fadd_rn(__fsub_rn(xkp, xc), __fsub_rn(xkm, xc)));
}

__device__ __forceinline__ float sw_nbsum(uint32_t w, float xc, float xip, float xim, float xjp, float xjm,
                                          float xkp, float xkm) {
    if (w == kInteriorWord) return interior_nbsum(xc, xip, xim, xjp, xjm, xkp, xkm);
    const uint32_t ns = sw_ns(w);
    auto term = [&](int q, float xn) {
        const float v = (w & (2u << (2 * q))) ? xn : 0.0f;
        return (ns & (1u << (2 * q))) ? __fsub_rn(v, xc) : 0.0f;
    };
    float ret = 0.0f;
    ret = __fadd_rn(ret, __fadd_rn(term(1, xip), term(2, xim)));
    ret = __fadd_rn(ret, __fadd_rn(term(3, xjp), term(4, xjm)));
    return __fadd_rn(ret, __fadd_rn(term(5, xkp), term(6, xkm)));
}

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

template <bool kNC, typename TC>
__device__ __forceinline__ float coarse_at(const TC *__restrict__ p, float scale) {
    return __fmul_rn(kNC ? St<TC>::ld_ro(p) : St<TC>::ld_cg(p), scale);
}

// One cell's red-black update (multigrid/mgpcg.py:72-86 in the reference's
// order) from its stencil word w, its value xc, its six neighbours (i+, i-,
// j+, j-, k+, k-) and its residual r: xc + (r + L z) / d, or 0 for a cell that
// is not fluid or has no non-solid neighbour.  kFromZero: z was 0 before the
// sweep (then r / d).
template <bool kFromZero>
__device__ __forceinline__ float smooth_cell(uint32_t w, float xc, float xip, float xim, float xjp, float xjm,
                                             float xkp, float xkm, float r) {
    if (w == kInteriorWord)  // d = 6
        return kFromZero ? div6_rn(r)
                         : __fadd_rn(xc, div6_rn(__fadd_rn(r, interior_nbsum(xc, xip, xim, xjp, xjm, xkp, xkm))));
    if (sw_code(w, 0) != kCodeFluid) return 0.0f;
    const int d = __popc(sw_ns(w));
    if (d == 0) return 0.0f;
    const float ret = kFromZero ? 0.0f : sw_nbsum(w, xc, xip, xim, xjp, xjm, xkp, xkm);
    return kFromZero ? __fdiv_rn(r, (float)d) : __fadd_rn(xc, __fdiv_rn(__fadd_rn(r, ret), (float)d));
}

// One half-sweep over the 8-cell groups; a pair of adjacent lanes shares a
// group, each lane owning 4 consecutive cells (its "half") -- 4-wide vector
// loads per row and about half the registers of one lane per group, so twice
// as many lanes are resident to hide memory latency.  The k neighbours across
// the middle of the group come from the partner lane by a shuffle.
//   kFromZero: z is 0 before the sweep (first sweep of a level in the V-cycle);
//              zin and zc are not read.
//   kProlong:  the sweep reads zin + zc[I/2] (multigrid/mgpcg.py:113-116 fused
//              into the first post-smoothing sweep) and writes every cell to
//              zout != zin; otherwise zout == zin (in place).
// TO/TI/TR/TC: storage of zout, zin, r and the coarse zc (float, or __half in
// the mixed-precision V-cycle); arithmetic is FP32 throughout, cell by cell in
// the reference's order (multigrid/mgpcg.py:72-86), so results are bit-exact.
// Every non-fluid cell is written as 0 (its value is never read by a fluid
// cell's update, and the reference's sweeps leave it 0 by the end of the
// V-cycle), so a buffer that starts at 0 keeps z = 0 off the fluid.  With an
// active list (act != NULL) the caller asserts that invariant for zout, and
// only the groups of the list (those holding a fluid cell) are visited;
// without one every group is.
// Grid: one-dimensional; each warp walks 16 groups (32 halves) per step,
// grid-stride, so both lanes of a pair always run the same iterations.
// Requires nz % 8 == 0.  The prolongation variant holds the coarse values as
// well: 5 blocks per SM (51 registers) instead of 6 (40) keep it free of
// spills.
// kNC: r and zc may be read through the read-only (non-coherent) path, i.e.
// nothing writes them while the kernel runs; false inside the persistent and
// cluster V-cycle kernels (persist.cuh, cluster.cuh), where other blocks wrote
// them (and z) earlier in the same launch: then r, zc and z are read with
// L2-only loads.  bid / nblk: this block's index and the number of blocks that
// share the grid-stride loop.
// kc != NULL: called at the start of a kernel launched with programmatic
// dependent launch: the list reads come first, then pdl_wait(kc).
template <bool kFromZero, bool kProlong, bool kNC, typename TO, typename TI, typename TR, typename TC>
__device__ __forceinline__ void smooth8_pass(TO *zout, const TI *zin, const TC *__restrict__ zc, float zc_scale,
                                             const TR *__restrict__ r, const uint8_t *__restrict__ code,
                                             const uint16_t *__restrict__ sw, const Dims D, int phase,
                                             const int *__restrict__ act, const int *__restrict__ act_n, int bid,
                                             int nblk, bool pdl = false, unsigned long long *kc = nullptr) {
    const int lane = threadIdx.x & 31;
    const int total = 2 * (act ? *act_n : (int)(D.n() >> 3));
    const int stride = nblk * blockDim.x;
    // list entry of this lane's next group, fetched one grid-stride step ahead
    // so that the list read is off the critical path of the loads it feeds
    const int base0 = bid * blockDim.x + (threadIdx.x & ~31);
    int g_next = (base0 + lane < total) ? (act ? __ldg(act + ((base0 + lane) >> 1)) : ((base0 + lane) >> 1)) : 0;
    if (pdl) pdl_wait(kc);
    for (int base = base0; base < total; base += stride) {
        const int t = base + lane;
        const bool valid = t < total;  // both lanes of a pair agree (total is even)
        const int h = t & 1;           // half: cells 4h .. 4h + 3 of the group
        const int g = valid ? g_next : 0;
        const int tn = t + stride;
        g_next = tn < total ? (act ? __ldg(act + (tn >> 1)) : (tn >> 1)) : 0;
        int i, j, kg;
        group_ijk(g, D, i, j, kg);
        const int k0 = kg << 3;
        const int sj = D.nz, si = D.ny * D.nz;
        const int c0 = (i * D.ny + j) * D.nz + k0;
        const int ch = c0 + 4 * h;
        const bool hip = i + 1 < D.nx, him = i > 0, hjp = j + 1 < D.ny, hjm = j > 0;
        const bool hkp = k0 + 8 < D.nz, hkm = k0 > 0;
        const int par = 1 - phase;
        const int b0 = (i + j + k0 + par) & 1;  // cell m of the group is updated iff (m & 1) == b0

        uint2 wd = make_uint2(0u, 0u);
        float rr[4] = {0.0f, 0.0f, 0.0f, 0.0f}, zc0[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float zip[4] = {0.0f, 0.0f, 0.0f, 0.0f}, zim[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float zjp[4] = {0.0f, 0.0f, 0.0f, 0.0f}, zjm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float zout_k = 0.0f;  // the k neighbour outside the group (cell -1 for h = 0, cell 8 for h = 1)
        if (valid) {
            if (sw) {
                wd = __ldg(reinterpret_cast<const uint2 *>(sw + ch));
            } else {
                const uint4 w8 = words8_from_codes(code, D, i, j, k0, c0);
                wd = h ? make_uint2(w8.z, w8.w) : make_uint2(w8.x, w8.y);
            }
            if (kNC) St<TR>::ld4_ro(r + ch, rr); else St<TR>::ld4_cg(r + ch, rr);
            if (!kFromZero) {
                // z: plain loads (rows of the other colour do not change during the
                // launch), or L2-only ones where other blocks of the same launch
                // wrote it in an earlier pass (kNC false)
                auto ldz4 = [&](const TI *q, float o[4]) {
                    if (kNC) St<TI>::ld4(q, o); else St<TI>::ld4_cg(q, o);
                };
                auto ldz = [&](const TI *q) { return kNC ? St<TI>::ld(q) : St<TI>::ld_cg(q); };
                ldz4(zin + ch, zc0);
                if (hip) ldz4(zin + ch + si, zip);
                if (him) ldz4(zin + ch - si, zim);
                if (hjp) ldz4(zin + ch + sj, zjp);
                if (hjm) ldz4(zin + ch - sj, zjm);
                if (h == 0 && hkm) zout_k = ldz(zin + c0 - 1);
                if (h == 1 && hkp) zout_k = ldz(zin + c0 + 8);
                if (kProlong) {
                    const int cy = D.ny >> 1, cz = D.nz >> 1;
                    const int ci = i >> 1, cj = j >> 1, ck = (k0 >> 1) + 2 * h;
                    const int cb = (ci * cy + cj) * cz + ck;
                    float cv[2];
#define FLUB_ADD_COARSE(row, p)                                                         \
    {                                                                                   \
        if (kNC) St<TC>::ld2_ro((p), cv); else St<TC>::ld2_cg((p), cv);                 \
        _Pragma("unroll") for (int mm = 0; mm < 4; mm++)                                \
            row[mm] = __fadd_rn(row[mm], __fmul_rn(cv[mm >> 1], zc_scale));             \
    }
                    FLUB_ADD_COARSE(zc0, zc + cb)
                    if (hip) FLUB_ADD_COARSE(zip, zc + (((i + 1) >> 1) * cy + cj) * cz + ck)
                    if (him) FLUB_ADD_COARSE(zim, zc + (((i - 1) >> 1) * cy + cj) * cz + ck)
                    if (hjp) FLUB_ADD_COARSE(zjp, zc + (ci * cy + ((j + 1) >> 1)) * cz + ck)
                    if (hjm) FLUB_ADD_COARSE(zjm, zc + (ci * cy + ((j - 1) >> 1)) * cz + ck)
#undef FLUB_ADD_COARSE
                    if (h == 0 && hkm) zout_k = __fadd_rn(zout_k, coarse_at<kNC>(zc + cb - 1, zc_scale));
                    if (h == 1 && hkp) zout_k = __fadd_rn(zout_k, coarse_at<kNC>(zc + cb + 2, zc_scale));
                }
            }
        }
        // the partner's cell next to the middle of the group: h = 0 needs cell 4
        // (partner's first), h = 1 needs cell 3 (partner's last)
        const float send = h ? zc0[0] : zc0[3];
        const float zmid = __shfl_xor_sync(0xffffffffu, send, 1);
        const float zkm = h ? zmid : zout_k;  // neighbour below cell 4h
        const float zkp = h ? zout_k : zmid;  // neighbour above cell 4h + 3
        if (!valid) continue;

        float out[4];
        if constexpr (!kProlong) {
            // the two cells of the active colour are mm = b0 and mm = b0 + 2 (4h is
            // even): each gets one update body, its operands picked by selects, so
            // no lane runs the bodies of the other colour
            const uint32_t wa = b0 ? (wd.x >> 16) : (wd.x & 0xffffu), wb = b0 ? (wd.y >> 16) : (wd.y & 0xffffu);
            const float za = smooth_cell<kFromZero>(wa, b0 ? zc0[1] : zc0[0], b0 ? zip[1] : zip[0],
                                                    b0 ? zim[1] : zim[0], b0 ? zjp[1] : zjp[0], b0 ? zjm[1] : zjm[0],
                                                    b0 ? zc0[2] : zc0[1], b0 ? zc0[0] : zkm, b0 ? rr[1] : rr[0]);
            const float zb = smooth_cell<kFromZero>(wb, b0 ? zc0[3] : zc0[2], b0 ? zip[3] : zip[2],
                                                    b0 ? zim[3] : zim[2], b0 ? zjp[3] : zjp[2], b0 ? zjm[3] : zjm[2],
                                                    b0 ? zkp : zc0[3], b0 ? zc0[2] : zc0[1], b0 ? rr[3] : rr[2]);
            // the other colour passes through (0 off the fluid)
#pragma unroll
            for (int mm = 0; mm < 4; mm++) {
                const uint32_t w = (mm & 1) ? ((mm < 2 ? wd.x : wd.y) >> 16) : ((mm < 2 ? wd.x : wd.y) & 0xffffu);
                out[mm] = sw_code(w, 0) == kCodeFluid ? zc0[mm] : 0.0f;
            }
            out[0] = b0 ? out[0] : za;
            out[1] = b0 ? za : out[1];
            out[2] = b0 ? out[2] : zb;
            out[3] = b0 ? zb : out[3];
        } else {
            // (the prolongation variant keeps the per-cell form, which needs fewer
            // live registers)
#pragma unroll
            for (int mm = 0; mm < 4; mm++) {
                const uint32_t w = (mm & 1) ? ((mm < 2 ? wd.x : wd.y) >> 16) : ((mm < 2 ? wd.x : wd.y) & 0xffffu);
                out[mm] = sw_code(w, 0) == kCodeFluid ? zc0[mm] : 0.0f;
                if ((mm & 1) != b0) continue;  // 4h is even: cell 4h + mm has the parity of mm
                out[mm] = smooth_cell<kFromZero>(w, zc0[mm], zip[mm], zim[mm], zjp[mm], zjm[mm],
                                                 mm < 3 ? zc0[mm + 1] : zkp, mm > 0 ? zc0[mm - 1] : zkm, rr[mm]);
            }
        }
        St<TO>::st4(zout + ch, out);
    }
}

template <bool kFromZero, bool kProlong, typename TO, typename TI, typename TR, typename TC>
__global__ void __launch_bounds__(256, kProlong ? 5 : 6) k_smooth8(TO *zout, const TI *zin, const TC *__restrict__ zc,
                                                    float zc_scale, const TR *__restrict__ r,
                                                    const uint8_t *__restrict__ code,
                                                    const uint16_t *__restrict__ sw, Dims D, int phase,
                                                    const int *__restrict__ act, const int *__restrict__ act_n,
                                                    unsigned long long *kc) {
    pdl_open();
    smooth8_pass<kFromZero, kProlong, true>(zout, zin, zc, zc_scale, r, code, sw, D, phase, act, act_n, blockIdx.x,
                                            gridDim.x, true, kc);
}

}  // namespace flub
