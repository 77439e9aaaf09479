// The step before the projection in flub's rigid-coupling path: rigid face
// velocities (rigid_coupling.py:51-70 precompute_solid_vel), face fractions
// (geometry.py phi_to_fraction with utils/util.py fraction_quad), and the
// cut-cell ("Batty") forms of the divergence and the pressure-gradient update
// (divergence.py:4-42 divergence_fractional_3d, subtract_gradient.py:7-122).
//
// FP32 arithmetic through explicit round-to-nearest intrinsics in the
// reference's expression order, so the CPU oracle reproduces every value bit
// for bit.
#include "common.cuh"

namespace flub {

constexpr int kMaxBodies = 64;

struct BodySet {
    int n;
    float x[kMaxBodies][3], v[kMaxBodies][3], w[kMaxBodies][3];
};

// Grid: row_grid over the face array (fx, fy, fz).
__global__ void __launch_bounds__(kRowThreads) k_solid_vel(float *__restrict__ ur, const int32_t *__restrict__ owner,
                                                          int fx, int fy, int fz, int d, float h0, const BodySet B) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= fz) return;
    const int64_t f = ((int64_t)i * fy + j) * fz + k;
    const int o = owner[f];
    const float eps = __fmul_rn(h0, 0.01f);
    const float tmp = __fmul_rn((float)i, h0);  // the reference tests the first index on every axis
    float res = 0.0f;
    if (eps < tmp && tmp < __fsub_rn(1.0f, eps) && o >= 0 && o < B.n) {
        const float si = d == 1 ? 0.0f : 0.5f, sj = d == 2 ? 0.0f : 0.5f, sk = d == 3 ? 0.0f : 0.5f;
        const float p0 = __fsub_rn(__fmul_rn(__fadd_rn((float)i, si), h0), B.x[o][0]);
        const float p1 = __fsub_rn(__fmul_rn(__fadd_rn((float)j, sj), h0), B.x[o][1]);
        const float p2 = __fsub_rn(__fmul_rn(__fadd_rn((float)k, sk), h0), B.x[o][2]);
        const float *w = B.w[o];
        float c;
        if (d == 1)
            c = __fsub_rn(__fmul_rn(w[1], p2), __fmul_rn(w[2], p1));
        else if (d == 2)
            c = __fsub_rn(__fmul_rn(w[2], p0), __fmul_rn(w[0], p2));
        else
            c = __fsub_rn(__fmul_rn(w[0], p1), __fmul_rn(w[1], p0));
        res = __fadd_rn(B.v[o][d - 1], c);
    }
    ur[f] = res;
}

__device__ __forceinline__ float fr_edge(float yl, float yr) {
    float ret;
    if (yl > 0.0f && yr > 0.0f) ret = 1.0f;
    else if (yl > 0.0f) ret = __fdiv_rn(yl, __fsub_rn(yl, yr));
    else if (yr > 0.0f) ret = __fdiv_rn(yr, __fsub_rn(yr, yl));
    else ret = 0.0f;
    if (ret < 0.1f) ret = 0.0f;
    else if (ret > 1.0f) ret = 1.0f;
    return ret;
}

__device__ __forceinline__ float fr_tri(float ya, float yb, float yc) {
    const float fab = fr_edge(ya, yb), fbc = fr_edge(yb, yc), fca = fr_edge(yc, ya);
    float ret;
    if (ya > 0.0f && yb > 0.0f && yc > 0.0f) ret = 1.0f;
    else if (ya > 0.0f && yb > 0.0f) ret = __fsub_rn(1.0f, __fmul_rn(__fsub_rn(1.0f, fca), __fsub_rn(1.0f, fbc)));
    else if (ya > 0.0f && yc > 0.0f) ret = __fsub_rn(1.0f, __fmul_rn(__fsub_rn(1.0f, fab), __fsub_rn(1.0f, fbc)));
    else if (yb > 0.0f && yc > 0.0f) ret = __fsub_rn(1.0f, __fmul_rn(__fsub_rn(1.0f, fab), __fsub_rn(1.0f, fca)));
    else if (ya > 0.0f) ret = __fmul_rn(fca, fab);
    else if (yb > 0.0f) ret = __fmul_rn(fab, fbc);
    else if (yc > 0.0f) ret = __fmul_rn(fbc, fca);
    else ret = 0.0f;
    return ret < 0.0f ? 0.0f : (ret > 1.0f ? 1.0f : ret);
}

__device__ __forceinline__ float fraction_quad(float ya, float yb, float yc, float yd, float yctr) {
    float f = __fadd_rn(__fadd_rn(__fadd_rn(fr_tri(ya, yb, yctr), fr_tri(yb, yc, yctr)), fr_tri(yc, yd, yctr)),
                        fr_tri(yd, ya, yctr));
    f = __fmul_rn(f, 0.25f);
    if (f < 0.1f) f = 0.0f;
    else if (f > 1.0f) f = 1.0f;
    return f;
}

// Grid: row_grid over the face array of axis d.
__global__ void __launch_bounds__(kRowThreads) k_phi_to_fraction(const float *__restrict__ phi, float *__restrict__ frac,
                                                                int nx, int ny, int nz, int d) {
    const int fy = ny + (d == 2), fz = nz + (d == 3);
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= fz) return;
    const int py = ny + 1, pz = nz + 1;
    auto PN = [&](int a, int b, int c) { return __ldg(phi + ((int64_t)a * py + b) * pz + c); };
    const float ya = PN(i, j, k);
    float yb, yc, yd;
    if (d == 1) { yb = PN(i, j + 1, k); yc = PN(i, j + 1, k + 1); yd = PN(i, j, k + 1); }
    else if (d == 2) { yb = PN(i + 1, j, k); yc = PN(i + 1, j, k + 1); yd = PN(i, j, k + 1); }
    else { yb = PN(i + 1, j, k); yc = PN(i + 1, j + 1, k); yd = PN(i, j + 1, k); }
    const int64_t f = ((int64_t)i * fy + j) * fz + k;
    frac[f] = fraction_quad(ya, yb, yc, yd, frac[f]);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Grid: row_grid(nx, ny, nz).
__global__ void __launch_bounds__(kRowThreads) k_divergence_fractional(
    const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w, float *__restrict__ div,
    const float *__restrict__ fu, const float *__restrict__ fv, const float *__restrict__ fw,
    const float *__restrict__ ur, const float *__restrict__ vr, const float *__restrict__ wr, int nx, int ny, int nz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    auto SU = [&](const float *a, int x, int y, int z) {
        return __ldg(a + ((int64_t)clampi(x, 0, nx) * ny + clampi(y, 0, ny - 1)) * nz + clampi(z, 0, nz - 1));
    };
    auto SV = [&](const float *a, int x, int y, int z) {
        return __ldg(a + ((int64_t)clampi(x, 0, nx - 1) * (ny + 1) + clampi(y, 0, ny)) * nz + clampi(z, 0, nz - 1));
    };
    auto SW = [&](const float *a, int x, int y, int z) {
        return __ldg(a + ((int64_t)clampi(x, 0, nx - 1) * ny + clampi(y, 0, ny - 1)) * (nz + 1) + clampi(z, 0, nz));
    };
    const float vl = SU(u, i, j, k), vR = SU(u, i + 1, j, k);
    const float vb = SV(v, i, j, k), vt = SV(v, i, j + 1, k);
    const float vf = SW(w, i, j, k), vn = SW(w, i, j, k + 1);
    const float l = SU(fu, i, j, k), r = SU(fu, i + 1, j, k);
    const float b = SV(fv, i, j, k), t = SV(fv, i, j + 1, k);
    const float f = SW(fw, i, j, k), n = SW(fw, i, j, k + 1);
    const float vls = SU(ur, i, j, k), vrs = SU(ur, i + 1, j, k);
    const float vbs = SV(vr, i, j, k), vts = SV(vr, i, j + 1, k);
    const float vfs = SW(wr, i, j, k), vns = SW(wr, i, j, k + 1);
    float a = __fsub_rn(__fmul_rn(vR, r), __fmul_rn(vl, l));
    a = __fadd_rn(a, __fmul_rn(vt, t));
    a = __fsub_rn(a, __fmul_rn(vb, b));
    a = __fadd_rn(a, __fmul_rn(vn, n));
    a = __fsub_rn(a, __fmul_rn(vf, f));
    float s = __fsub_rn(__fmul_rn(__fsub_rn(1.0f, r), vrs), __fmul_rn(__fsub_rn(1.0f, l), vls));
    s = __fadd_rn(s, __fmul_rn(__fsub_rn(1.0f, t), vts));
    s = __fsub_rn(s, __fmul_rn(__fsub_rn(1.0f, b), vbs));
    s = __fadd_rn(s, __fmul_rn(__fsub_rn(1.0f, n), vns));
    s = __fsub_rn(s, __fmul_rn(__fsub_rn(1.0f, f), vfs));
    div[((int64_t)i * ny + j) * nz + k] = __fadd_rn(a, s);
}

__device__ __forceinline__ float frac_fluid(float p1, float p2) {
    if (p1 < 0.0f && p2 < 0.0f) return 1.0f;
    if (p1 >= 0.0f && p2 >= 0.0f) return 0.0f;
    return __fsub_rn(1.0f, __fdiv_rn(fmaxf(p1, p2), fabsf(__fsub_rn(p1, p2))));
}

// Grid: row_grid over the face array of axis d.
__global__ void __launch_bounds__(kRowThreads) k_subtract_gradient_batty(
    float *__restrict__ uf, const float *__restrict__ p, const float *__restrict__ fr, const float *__restrict__ phi,
    const float *__restrict__ ur, int nx, int ny, int nz, int d, float lo, float h) {
    const int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= fz) return;
    const int gridn = (d == 1 ? fx : (d == 2 ? fy : fz)) - 1;
    const int64_t f = ((int64_t)i * fy + j) * fz + k;
    const int ii = d == 1 ? i : (d == 2 ? j : k);
    auto PC = [&](const float *a, int x, int y, int z) {
        return __ldg(a + ((int64_t)clampi(x, 0, nx - 1) * ny + clampi(y, 0, ny - 1)) * nz + clampi(z, 0, nz - 1));
    };
    if (0 < ii && ii < gridn) {
        const int il = i - (d == 1), jl = j - (d == 2), kl = k - (d == 3);
        const float ph = __ldg(phi + ((int64_t)i * ny + j) * nz + k);
        const float pl = __ldg(phi + ((int64_t)il * ny + jl) * nz + kl);
        if (ph < 0.0f || pl < 0.0f) {
            if (fr[f] == 0.0f) {
                uf[f] = ur[f];
            } else {
                const float plo = pl >= 0.0f ? 0.0f : PC(p, il, jl, kl);
                const float phi_ = ph >= 0.0f ? 0.0f : PC(p, i, j, k);
                float theta = d == 3 ? frac_fluid(pl, ph) : frac_fluid(ph, pl);
                theta = fmaxf(0.01f, theta);
                uf[f] = __fsub_rn(uf[f], __fdiv_rn(__fsub_rn(phi_, plo), theta));
            }
        } else {
            uf[f] = 0.0f;
        }
    } else if (lo <= 1e-5f || __fadd_rn(lo, __fmul_rn((float)ii, h)) >= __fsub_rn(1.0f, 1e-5f)) {
        uf[f] = 0.0f;
    }
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_solid_vel(float *ur, const int32_t *owner, int nx, int ny, int nz, int d, float h0, const float *bx,
                   const float *bv, const float *bw, int nbodies, void *stream) {
    FLUB_REQUIRE(ur && owner, "flub_solid_vel: NULL argument");
    FLUB_REQUIRE(d >= 1 && d <= 3, "flub_solid_vel: d=%d must be 1, 2 or 3", d);
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65535 && ny < 65535, "flub_solid_vel: bad shape");
    FLUB_REQUIRE(nbodies >= 0 && nbodies <= kMaxBodies && (nbodies == 0 || (bx && bv && bw)),
                 "flub_solid_vel: nbodies=%d outside [0, %d] or NULL body arrays", nbodies, kMaxBodies);
    BodySet B;
    B.n = nbodies;
    for (int o = 0; o < nbodies; o++)
        for (int a = 0; a < 3; a++) {
            B.x[o][a] = bx[3 * o + a];
            B.v[o][a] = bv[3 * o + a];
            B.w[o][a] = bw[3 * o + a];
        }
    const int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    k_solid_vel<<<row_grid(fx, fy, fz), kRowThreads, 0, as_stream(stream)>>>(ur, owner, fx, fy, fz, d, h0, B);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_phi_to_fraction(const float *phi_nodes, float *frac, int nx, int ny, int nz, int d, void *stream) {
    FLUB_REQUIRE(phi_nodes && frac, "flub_phi_to_fraction: NULL argument");
    FLUB_REQUIRE(d >= 1 && d <= 3, "flub_phi_to_fraction: d=%d must be 1, 2 or 3", d);
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65535 && ny < 65535, "flub_phi_to_fraction: bad shape");
    const int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    k_phi_to_fraction<<<row_grid(fx, fy, fz), kRowThreads, 0, as_stream(stream)>>>(phi_nodes, frac, nx, ny, nz, d);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_divergence_fractional(const float *u, const float *v, const float *w, float *div, const float *fu,
                               const float *fv, const float *fw, const float *ur, const float *vr, const float *wr,
                               int nx, int ny, int nz, void *stream) {
    FLUB_REQUIRE(u && v && w && div && fu && fv && fw && ur && vr && wr, "flub_divergence_fractional: NULL argument");
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65536 && ny < 65536, "flub_divergence_fractional: bad shape");
    k_divergence_fractional<<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(u, v, w, div, fu, fv, fw, ur,
                                                                                        vr, wr, nx, ny, nz);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_subtract_gradient_batty(float *uf, const float *p, const float *frac, const float *phi, const float *ur,
                                 int nx, int ny, int nz, int d, float lo, float h, void *stream) {
    FLUB_REQUIRE(uf && p && frac && phi && ur, "flub_subtract_gradient_batty: NULL argument");
    FLUB_REQUIRE(d >= 1 && d <= 3, "flub_subtract_gradient_batty: d=%d must be 1, 2 or 3", d);
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65535 && ny < 65535, "flub_subtract_gradient_batty: bad shape");
    const int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    k_subtract_gradient_batty<<<row_grid(fx, fy, fz), kRowThreads, 0, as_stream(stream)>>>(uf, p, frac, phi, ur, nx,
                                                                                          ny, nz, d, lo, h);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
