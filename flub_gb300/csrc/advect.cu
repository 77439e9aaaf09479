// Semi-Lagrangian and MacCormack advection (advect.py), the first step of
// flub's time step (water_3d.py:34-37 advect, example_fluid.py:64-65).
//
// Positions are in grid units (cell i spans [i, i+1)); every sample clamps
// its index to the array it reads (utils/util.py:20-28 sample_3d).  FP32
// arithmetic through explicit round-to-nearest intrinsics in the reference's
// expression order, so the CPU oracle reproduces every value bit for bit.
//
// One thread per output element on a division-free row grid (k along
// threadIdx.x, j = blockIdx.y, i = blockIdx.z): the 32 threads of a warp read
// neighbouring k, so every gather instruction of the trace and the stencils
// touches one or two cache lines.  The kernels are bound by L1 gather
// throughput (about 280 loads per MacCormack element), not by HBM.
#include <cmath>

#include "common.cuh"

namespace flub {

// MAC face arrays of the cell grid (nx, ny, nz) and their strides: u
// (nx+1, ny, nz), v (nx, ny+1, nz), w (nx, ny, nz+1).
struct AdvVel {
    const float *__restrict__ u, *__restrict__ v, *__restrict__ w;
    int nx, ny, nz;
};

struct AdvVol {
    const float *__restrict__ q;
    int gx, gy, gz;
};

struct AdvF3 {
    float x, y, z;
};

// The trace's step factors (0.5 dt)/h, (0.75 dt)/h and dt/h for +dt and -dt,
// rounded to FP32 on the host exactly as the kernels would.
struct AdvSteps {
    float c1[2], c2[2], c3[2];
};

// floor(x) as an int (saturating; NaN -> 0) and the fraction x - floor(x).
__device__ __forceinline__ int adv_floor(float x) { return __float2int_rd(x); }
__device__ __forceinline__ float adv_fract(float x) { return __fsub_rn(x, floorf(x)); }

// clamp(i0, 0, hi) and clamp(i0 + 1, 0, hi), without forming i0 + 1.
struct AdvPair {
    int a, b;
};

__device__ __forceinline__ AdvPair adv_pair(int i0, int hi) {
    const int a = min(max(i0, 0), hi);
    return AdvPair{a, a + ((unsigned)i0 < (unsigned)hi ? 1 : 0)};
}

// wp.lerp(a, b, t) = a * (1 - t) + b * t.
__device__ __forceinline__ float adv_lerp(float a, float b, float t) {
    return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t));
}

// The eight corners (x.a|x.b, y.a|y.b, z.a|z.b) of q (plane stride sp, row
// stride sr) blended as utils/util.py:55-88 and :106-120 write it:
// lerp(lerp(lerp(a,b,fa), lerp(c,d,fa), fb), lerp(lerp(e,f,fa), lerp(g,h,fa), fb), fc).
__device__ __forceinline__ float adv_tri8(const float *__restrict__ q, int sp, int sr, AdvPair x, AdvPair y, AdvPair z,
                                          float fa, float fb, float fc) {
    const float *paa = q + (x.a * sp + y.a * sr), *pba = q + (x.b * sp + y.a * sr);
    const float *pab = q + (x.a * sp + y.b * sr), *pbb = q + (x.b * sp + y.b * sr);
    const float a = __ldg(paa + z.a), b = __ldg(pba + z.a), c = __ldg(pab + z.a), d = __ldg(pbb + z.a);
    const float e = __ldg(paa + z.b), f = __ldg(pba + z.b), g = __ldg(pab + z.b), h = __ldg(pbb + z.b);
    return adv_lerp(adv_lerp(adv_lerp(a, b, fa), adv_lerp(c, d, fa), fb),
                    adv_lerp(adv_lerp(e, f, fa), adv_lerp(g, h, fa), fb), fc);
}

// utils/util.py:34-88 sample_velocity_3d.  The three components share their
// clamped index pairs where their arrays share an extent.
__device__ __forceinline__ AdvF3 adv_velocity(const AdvVel &M, AdvF3 p) {
    const int nx = M.nx, ny = M.ny, nz = M.nz;
    const float s = __fsub_rn(p.x, 0.5f), t = __fsub_rn(p.y, 0.5f), r = __fsub_rn(p.z, 0.5f);
    const float fu = adv_fract(p.x), fv = adv_fract(p.y), fw = adv_fract(p.z);
    const float fs = adv_fract(s), ft = adv_fract(t), fr = adv_fract(r);
    const AdvPair xu = adv_pair(adv_floor(p.x), nx), xs = adv_pair(adv_floor(s), nx - 1);
    const AdvPair yv = adv_pair(adv_floor(p.y), ny), yt = adv_pair(adv_floor(t), ny - 1);
    const AdvPair zw = adv_pair(adv_floor(p.z), nz), zr = adv_pair(adv_floor(r), nz - 1);
    AdvF3 o;
    o.x = adv_tri8(M.u, ny * nz, nz, xu, yt, zr, fu, ft, fr);
    o.y = adv_tri8(M.v, (ny + 1) * nz, nz, xs, yv, zr, fs, fv, fr);
    o.z = adv_tri8(M.w, ny * (nz + 1), nz + 1, xs, yt, zw, fs, ft, fw);
    return o;
}

// advect.py:10-22 backtrace from p with its first velocity sample v1 given
// (c1, c2, c3: the step factors of the direction traced).
__device__ __forceinline__ AdvF3 adv_backtrace_v1(const AdvVel &M, AdvF3 p, AdvF3 v1, float c1, float c2, float c3) {
    const float k1 = 2.0f / 9.0f, k2 = 1.0f / 3.0f, k3 = 4.0f / 9.0f;
    const AdvF3 p1 = {__fsub_rn(p.x, __fmul_rn(c1, v1.x)), __fsub_rn(p.y, __fmul_rn(c1, v1.y)),
                      __fsub_rn(p.z, __fmul_rn(c1, v1.z))};
    const AdvF3 v2 = adv_velocity(M, p1);
    const AdvF3 p2 = {__fsub_rn(p.x, __fmul_rn(c2, v2.x)), __fsub_rn(p.y, __fmul_rn(c2, v2.y)),
                      __fsub_rn(p.z, __fmul_rn(c2, v2.z))};
    const AdvF3 v3 = adv_velocity(M, p2);
    AdvF3 o;
    o.x = __fsub_rn(p.x, __fmul_rn(c3, __fadd_rn(__fadd_rn(__fmul_rn(k1, v1.x), __fmul_rn(k2, v2.x)),
                                                 __fmul_rn(k3, v3.x))));
    o.y = __fsub_rn(p.y, __fmul_rn(c3, __fadd_rn(__fadd_rn(__fmul_rn(k1, v1.y), __fmul_rn(k2, v2.y)),
                                                 __fmul_rn(k3, v3.y))));
    o.z = __fsub_rn(p.z, __fmul_rn(c3, __fadd_rn(__fadd_rn(__fmul_rn(k1, v1.z), __fmul_rn(k2, v2.z)),
                                                 __fmul_rn(k3, v3.z))));
    return o;
}

// utils/util.py:122-129 cubic: the weights of the cubic through -1, 0, 1, 2
// at s, and the left-to-right dot product.
struct AdvW4 {
    float w0, w1, w2, w3;
};

__device__ __forceinline__ AdvW4 adv_cubic_w(float s) {
    const float m13 = -1.0f / 3.0f, k16 = 1.0f / 6.0f;
    const float ss = __fmul_rn(s, s), sss = __fmul_rn(ss, s);
    AdvW4 w;
    w.w0 = __fsub_rn(__fadd_rn(__fmul_rn(m13, s), __fmul_rn(__fmul_rn(0.5f, s), s)),
                     __fmul_rn(__fmul_rn(__fmul_rn(k16, s), s), s));
    w.w1 = __fadd_rn(__fsub_rn(1.0f, ss), __fmul_rn(0.5f, __fsub_rn(sss, s)));
    w.w2 = __fadd_rn(s, __fmul_rn(0.5f, __fsub_rn(ss, sss)));
    w.w3 = __fmul_rn(k16, __fsub_rn(sss, s));
    return w;
}

__device__ __forceinline__ float adv_dot4(float a, float b, float c, float d, const AdvW4 &w) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, w.w0), __fmul_rn(b, w.w1)), __fmul_rn(c, w.w2)),
                     __fmul_rn(d, w.w3));
}

// clamp(i0 + a - 1, 0, hi) * stride for a = 0..3 (i0 limited to
// [-2, hi + 2] first, which changes none of the four).
__device__ __forceinline__ void adv_quad(int i0, int hi, int stride, int o[4]) {
    const int c = min(max(i0, -2), hi + 2);
#pragma unroll
    for (int a = 0; a < 4; a++) o[a] = min(max(c + a - 1, 0), hi) * stride;
}

// utils/util.py:148-160 _tricubic (with _bicubic :139-146 and _cubic
// :131-137) at (s, t, r): cubics along the first axis innermost, then the
// second, then the third.
__device__ __forceinline__ float adv_tricubic(const AdvVol &Q, float s, float t, float r) {
    const AdvW4 wu = adv_cubic_w(adv_fract(s)), wv = adv_cubic_w(adv_fract(t)), ww = adv_cubic_w(adv_fract(r));
    int oi[4], oj[4], ok[4];
    adv_quad(adv_floor(s), Q.gx - 1, Q.gy * Q.gz, oi);
    adv_quad(adv_floor(t), Q.gy - 1, Q.gz, oj);
    adv_quad(adv_floor(r), Q.gz - 1, 1, ok);
    float qw[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
        float qv[4];
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const float *row = Q.q + (oj[n] + ok[m]);
            qv[n] = adv_dot4(__ldg(row + oi[0]), __ldg(row + oi[1]), __ldg(row + oi[2]), __ldg(row + oi[3]), wu);
        }
        qw[m] = adv_dot4(qv[0], qv[1], qv[2], qv[3], wv);
    }
    return adv_dot4(qw[0], qw[1], qw[2], qw[3], ww);
}

// utils/util.py:98-104 trilerp_stagger: the tricubic at p - stagger.
__device__ __forceinline__ float adv_sample_stagger(const AdvVol &Q, AdvF3 p, AdvF3 st) {
    return adv_tricubic(Q, __fsub_rn(p.x, st.x), __fsub_rn(p.y, st.y), __fsub_rn(p.z, st.z));
}

__device__ __forceinline__ float adv_min(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float adv_max(float a, float b) { return a > b ? a : b; }

// p / mh, as a multiplication when mh is a power of two (inv_mh = 1 / mh,
// then exact and equal to the quotient), else a division.
__device__ __forceinline__ float adv_div_mh(float p, float mh, float inv_mh) {
    return inv_mh != 0.0f ? __fmul_rn(p, inv_mh) : __fdiv_rn(p, mh);
}

// advect.py:103-122 sample_minmax: min and max of the eight values around
// floor(p / mh - stagger).  The reference passes h0 as mh while p is already
// in grid units (so the corner clamps to the far end of the array for
// p >= 1); mh = 1 gives the cell around p.
__device__ __forceinline__ void adv_minmax(const AdvVol &Q, AdvF3 p, float mh, float inv_mh, AdvF3 st, float &mn,
                                           float &mx) {
    const AdvPair x = adv_pair(adv_floor(__fsub_rn(adv_div_mh(p.x, mh, inv_mh), st.x)), Q.gx - 1);
    const AdvPair y = adv_pair(adv_floor(__fsub_rn(adv_div_mh(p.y, mh, inv_mh), st.y)), Q.gy - 1);
    const AdvPair z = adv_pair(adv_floor(__fsub_rn(adv_div_mh(p.z, mh, inv_mh), st.z)), Q.gz - 1);
    const int sp = Q.gy * Q.gz, sr = Q.gz;
    const float *q = Q.q;
    const float *paa = q + (x.a * sp + y.a * sr), *pba = q + (x.b * sp + y.a * sr);
    const float *pab = q + (x.a * sp + y.b * sr), *pbb = q + (x.b * sp + y.b * sr);
    const float v0 = __ldg(paa + z.a), v1 = __ldg(pba + z.a), v2 = __ldg(pab + z.a), v3 = __ldg(pbb + z.a);
    const float v4 = __ldg(paa + z.b), v5 = __ldg(pba + z.b), v6 = __ldg(pab + z.b), v7 = __ldg(pbb + z.b);
    mn = adv_min(adv_min(adv_min(adv_min(v0, v1), v2), v3), adv_min(adv_min(adv_min(v4, v5), v6), v7));
    mx = adv_max(adv_max(adv_max(adv_max(v0, v1), v2), v3), adv_max(adv_max(adv_max(v4, v5), v6), v7));
}

// advect.py:57-101 _advect_mc_1 (STAGE 1: q_out = the semi-Lagrangian
// sample), _advect_mc_2 (STAGE 2: q_tmp = the sample traced forward),
// _advect_mc_3 (STAGE 3: the MacCormack correction, kept where it lies
// strictly between the sample_minmax bounds, else the semi-Lagrangian
// sample), and STAGE 0: the three in one pass (stage 3 reads back exactly the
// values stages 1 and 2 wrote, so recomputing them in registers gives the
// same result without q_tmp).  The traces over dt and -dt start with the
// same velocity sample, taken once.  Grid: row_grid(qx, qy, qz).
template <int STAGE>
__global__ void __launch_bounds__(kRowThreads) k_advect_mc(const AdvVel M, const AdvVol Q, float *__restrict__ q_out,
                                                          float *__restrict__ q_tmp, AdvF3 st, const AdvSteps C,
                                                          float mh, float inv_mh) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= Q.gz) return;
    const int f = (i * Q.gy + j) * Q.gz + k;
    const AdvF3 p = {__fadd_rn((float)i, st.x), __fadd_rn((float)j, st.y), __fadd_rn((float)k, st.z)};
    const AdvF3 v1 = adv_velocity(M, p);
    if (STAGE == 1 || STAGE == 2) {
        const int s = STAGE - 1;
        const float q = adv_sample_stagger(Q, adv_backtrace_v1(M, p, v1, C.c1[s], C.c2[s], C.c3[s]), st);
        (STAGE == 1 ? q_out : q_tmp)[f] = q;
        return;
    }
    // foot over dt (pf) and over -dt (pb), and the tricubic samples there,
    // as one loop of two so that the code is held once
    AdvF3 pf = p, pb = p;
    float q_sl = 0.0f, q_bk = 0.0f;
#pragma unroll 1
    for (int s = 0; s < (STAGE == 0 ? 2 : 1); s++) {
        const AdvF3 e = adv_backtrace_v1(M, p, v1, s ? C.c1[1] : C.c1[0], s ? C.c2[1] : C.c2[0], s ? C.c3[1] : C.c3[0]);
        const float q = adv_sample_stagger(Q, e, st);
        if (s == 0) {
            pf = e;
            q_sl = q;
        } else {
            pb = e;
            q_bk = q;
        }
    }
    (void)pb;
    float qo, qt;
    if (STAGE == 3) {
        qo = q_out[f];
        qt = q_tmp[f];
    } else {
        qo = q_sl;
        qt = q_bk;
    }
    const float q = __fadd_rn(qo, __fmul_rn(0.5f, __fsub_rn(__ldg(Q.q + f), qt)));
    float mn, mx;
    adv_minmax(Q, pf, mh, inv_mh, st, mn, mx);
    q_out[f] = (mn < q && q < mx) ? q : q_sl;
}

// advect.py:39-54 advect_phi: the tricubic sample at the foot of the trace
// where it lies inside [0, extent) on every axis, else `outside` (the
// reference writes h0).  Grid: row_grid(px, py, pz).
__global__ void __launch_bounds__(kRowThreads) k_advect_phi(const AdvVel M, const AdvVol Q, float *__restrict__ out,
                                                           AdvF3 st, const AdvSteps C, float outside) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= Q.gz) return;
    const AdvF3 p0 = {__fadd_rn((float)i, st.x), __fadd_rn((float)j, st.y), __fadd_rn((float)k, st.z)};
    const AdvF3 p = adv_backtrace_v1(M, p0, adv_velocity(M, p0), C.c1[0], C.c2[0], C.c3[0]);
    const bool in = 0.0f <= p.x && p.x < (float)Q.gx && 0.0f <= p.y && p.y < (float)Q.gy && 0.0f <= p.z &&
                    p.z < (float)Q.gz;
    out[(i * Q.gy + j) * Q.gz + k] = in ? adv_sample_stagger(Q, p, st) : outside;
}

// advect.py:24-37 advect_simple_3d: a cell-centred q traced back from
// (i+0.5, j+0.5, k+0.5) and sampled trilinearly (utils/util.py:91-96
// trilerp).  Grid: row_grid(qx, qy, qz).
__global__ void __launch_bounds__(kRowThreads) k_advect_simple(const AdvVel M, const AdvVol Q, float *__restrict__ out,
                                                              const AdvSteps C) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= Q.gz) return;
    const AdvF3 p0 = {__fadd_rn((float)i, 0.5f), __fadd_rn((float)j, 0.5f), __fadd_rn((float)k, 0.5f)};
    const AdvF3 p = adv_backtrace_v1(M, p0, adv_velocity(M, p0), C.c1[0], C.c2[0], C.c3[0]);
    const float s = __fsub_rn(p.x, 0.5f), t = __fsub_rn(p.y, 0.5f), r = __fsub_rn(p.z, 0.5f);
    out[(i * Q.gy + j) * Q.gz + k] =
        adv_tri8(Q.q, Q.gy * Q.gz, Q.gz, adv_pair(adv_floor(s), Q.gx - 1), adv_pair(adv_floor(t), Q.gy - 1),
                 adv_pair(adv_floor(r), Q.gz - 1), adv_fract(s), adv_fract(t), adv_fract(r));
}

static inline AdvVel make_vel(const float *u, const float *v, const float *w, int nx, int ny, int nz) {
    return AdvVel{u, v, w, nx, ny, nz};
}

// The step factors of advect.py:16-21 for +dt (index 0) and -dt (index 1),
// each product and quotient rounded to FP32 as in the kernels.
static AdvSteps make_steps(float dt, float h) {
    AdvSteps C;
    for (int s = 0; s < 2; s++) {
        const float d = s ? -dt : dt;
        volatile float half = 0.5f * d, three_q = 0.75f * d;
        volatile float c1 = half / h, c2 = three_q / h, c3 = d / h;
        C.c1[s] = c1;
        C.c2[s] = c2;
        C.c3[s] = c3;
    }
    return C;
}

// 1 / mh when mh is a power of two (so that p * (1 / mh) == p / mh), else 0.
static float pow2_inverse(float mh) {
    int e = 0;
    const float m = std::frexp(mh, &e);
    if (std::fabs(m) != 0.5f || e < -120 || e > 120) return 0.0f;
    return std::ldexp(m > 0 ? 1.0f : -1.0f, 1 - e);
}

// Element counts stay below 2^31 so that the kernels index with int.
static inline bool adv_shape_ok(int x, int y, int z) {
    return x > 0 && y > 0 && z > 0 && x < 65536 && y < 65536 && (int64_t)x * y * z < ((int64_t)1 << 31);
}

static int launch_mc(const AdvVel &M, const float *q_in, float *q_out, float *q_tmp, int qx, int qy, int qz, AdvF3 st,
                     float dt, float h, float mh, int stage, cudaStream_t s) {
    const AdvVol Q{q_in, qx, qy, qz};
    const dim3 g = row_grid(qx, qy, qz);
    const AdvSteps C = make_steps(dt, h);
    const float inv = pow2_inverse(mh);
    switch (stage) {
        case 0: k_advect_mc<0><<<g, kRowThreads, 0, s>>>(M, Q, q_out, q_tmp, st, C, mh, inv); break;
        case 1: k_advect_mc<1><<<g, kRowThreads, 0, s>>>(M, Q, q_out, q_tmp, st, C, mh, inv); break;
        case 2: k_advect_mc<2><<<g, kRowThreads, 0, s>>>(M, Q, q_out, q_tmp, st, C, mh, inv); break;
        default: k_advect_mc<3><<<g, kRowThreads, 0, s>>>(M, Q, q_out, q_tmp, st, C, mh, inv); break;
    }
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_advect_mc(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *q_in,
                   float *q_out, float *q_tmp, int qx, int qy, int qz, float sx, float sy, float sz, float dt, float h,
                   float minmax_h, int stage, void *stream) {
    FLUB_REQUIRE(u && v && w && q_in && q_out, "flub_advect_mc: NULL argument");
    FLUB_REQUIRE(stage >= 0 && stage <= 3, "flub_advect_mc: stage=%d must be 0, 1, 2 or 3", stage);
    FLUB_REQUIRE(stage < 2 || q_tmp, "flub_advect_mc: stages 2 and 3 need q_tmp");
    FLUB_REQUIRE(q_out != q_in && q_tmp != q_in && (q_tmp == nullptr || q_tmp != q_out),
                 "flub_advect_mc: q_out and q_tmp must not alias q_in or each other");
    FLUB_REQUIRE(adv_shape_ok(nx + 1, ny + 1, nz + 1), "flub_advect_mc: bad velocity grid %dx%dx%d", nx, ny, nz);
    FLUB_REQUIRE(adv_shape_ok(qx, qy, qz), "flub_advect_mc: bad field shape %dx%dx%d", qx, qy, qz);
    FLUB_REQUIRE(h > 0.0f && minmax_h != 0.0f, "flub_advect_mc: h and minmax_h must be non-zero");
    return launch_mc(make_vel(u, v, w, nx, ny, nz), q_in, q_out, q_tmp, qx, qy, qz, AdvF3{sx, sy, sz}, dt, h,
                     minmax_h, stage, as_stream(stream));
}

int flub_advect_velocity_mc(const float *u, const float *v, const float *w, float *u_out, float *v_out, float *w_out,
                            int nx, int ny, int nz, float dt, float h, float minmax_h, void *stream) {
    FLUB_REQUIRE(u && v && w && u_out && v_out && w_out, "flub_advect_velocity_mc: NULL argument");
    FLUB_REQUIRE(u_out != u && v_out != v && w_out != w && u_out != v && u_out != w && v_out != u && v_out != w &&
                     w_out != u && w_out != v,
                 "flub_advect_velocity_mc: outputs must not alias the inputs");
    FLUB_REQUIRE(adv_shape_ok(nx + 1, ny + 1, nz + 1), "flub_advect_velocity_mc: bad grid %dx%dx%d", nx, ny, nz);
    FLUB_REQUIRE(h > 0.0f && minmax_h != 0.0f, "flub_advect_velocity_mc: h and minmax_h must be non-zero");
    const AdvVel M = make_vel(u, v, w, nx, ny, nz);
    cudaStream_t s = as_stream(stream);
    int st = launch_mc(M, u, u_out, nullptr, nx + 1, ny, nz, AdvF3{0.0f, 0.5f, 0.5f}, dt, h, minmax_h, 0, s);
    if (st == FLUB_OK)
        st = launch_mc(M, v, v_out, nullptr, nx, ny + 1, nz, AdvF3{0.5f, 0.0f, 0.5f}, dt, h, minmax_h, 0, s);
    if (st == FLUB_OK)
        st = launch_mc(M, w, w_out, nullptr, nx, ny, nz + 1, AdvF3{0.5f, 0.5f, 0.0f}, dt, h, minmax_h, 0, s);
    return st;
}

int flub_advect_phi(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *phi,
                    float *phi_out, int px, int py, int pz, float sx, float sy, float sz, float dt, float h,
                    float outside, void *stream) {
    FLUB_REQUIRE(u && v && w && phi && phi_out, "flub_advect_phi: NULL argument");
    FLUB_REQUIRE(phi_out != phi, "flub_advect_phi: phi_out must not alias phi");
    FLUB_REQUIRE(adv_shape_ok(nx + 1, ny + 1, nz + 1), "flub_advect_phi: bad velocity grid %dx%dx%d", nx, ny, nz);
    FLUB_REQUIRE(adv_shape_ok(px, py, pz), "flub_advect_phi: bad field shape %dx%dx%d", px, py, pz);
    FLUB_REQUIRE(h > 0.0f, "flub_advect_phi: h must be > 0");
    k_advect_phi<<<row_grid(px, py, pz), kRowThreads, 0, as_stream(stream)>>>(
        make_vel(u, v, w, nx, ny, nz), AdvVol{phi, px, py, pz}, phi_out, AdvF3{sx, sy, sz}, make_steps(dt, h),
        outside);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_advect_simple(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *q,
                       float *q_out, int qx, int qy, int qz, float dt, float h, void *stream) {
    FLUB_REQUIRE(u && v && w && q && q_out, "flub_advect_simple: NULL argument");
    FLUB_REQUIRE(q_out != q, "flub_advect_simple: q_out must not alias q");
    FLUB_REQUIRE(adv_shape_ok(nx + 1, ny + 1, nz + 1), "flub_advect_simple: bad velocity grid %dx%dx%d", nx, ny, nz);
    FLUB_REQUIRE(adv_shape_ok(qx, qy, qz), "flub_advect_simple: bad field shape %dx%dx%d", qx, qy, qz);
    FLUB_REQUIRE(h > 0.0f, "flub_advect_simple: h must be > 0");
    k_advect_simple<<<row_grid(qx, qy, qz), kRowThreads, 0, as_stream(stream)>>>(
        make_vel(u, v, w, nx, ny, nz), AdvVol{q, qx, qy, qz}, q_out, make_steps(dt, h));
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
