// Pressure-gradient velocity update.
//
// subtract_gradient.py:37-68 subtract_gradient_tag (one axis per launch, as
// the reference calls it at example_fluid.py:136-138) and a fused form that
// updates u, v and w in one pass over the (nx+1)(ny+1)(nz+1) face lattice with
// the pressure scale of example_fluid.py:134 folded into the read of p.
#include "common.cuh"

namespace flub {

// Update of face f between cells lo and hi (mirrors the reference's branch
// order: solid on either side, else fluid on either side, else 0).  Each
// branch reads only what it uses: a face between two air cells (most of a
// water scene) reads its two tags and writes 0.  ps: pressure scale.
__device__ __forceinline__ float grad_face(const float *__restrict__ uf, const float *__restrict__ urf,
                                          const float *__restrict__ p, float ps, int64_t f, int64_t clo, int64_t chi,
                                          int tlo, int thi) {
    if (tlo == 2 || thi == 2) return __ldg(&urf[f]);
    if (tlo == 1 || thi == 1)
        return __fsub_rn(uf[f], __fsub_rn(__fmul_rn(__ldg(&p[chi]), ps), __fmul_rn(__ldg(&p[clo]), ps)));
    return 0.0f;
}

// Grid: row_grid over the face array's extents (fx, fy, fz).
__global__ void __launch_bounds__(kRowThreads) k_subtract_gradient_axis(float *__restrict__ uf,
                                                                       const float *__restrict__ urf,
                                                                       const float *__restrict__ p,
                                                                       const int32_t *__restrict__ tag, int nx, int ny,
                                                                       int nz, int d) {
    const int fy = ny + (d == 2), fz = nz + (d == 3);
    const int nd = d == 1 ? nx : (d == 2 ? ny : nz);
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= fz) return;
    const int64_t f = ((int64_t)i * fy + j) * fz + k;
    {
        const int ii = d == 1 ? i : (d == 2 ? j : k);
        if (0 < ii && ii < nd) {
            const int64_t chi = ((int64_t)i * ny + j) * nz + k;
            const int64_t clo = chi - (d == 1 ? (int64_t)ny * nz : (d == 2 ? (int64_t)nz : 1));
            uf[f] = grad_face(uf, urf, p, 1.0f, f, clo, chi, __ldg(&tag[clo]), __ldg(&tag[chi]));
        } else {
            uf[f] = 0.0f;
        }
    }
}

__global__ void __launch_bounds__(kRowThreads) k_subtract_gradient_all(float *__restrict__ u, float *__restrict__ v,
                                                               float *__restrict__ w, const float *__restrict__ ur,
                                                               const float *__restrict__ vr,
                                                               const float *__restrict__ wr,
                                                               const float *__restrict__ p, float ps,
                                                               const int32_t *__restrict__ tag, int nx, int ny,
                                                               int nz) {
    // grid: row_grid(nx + 1, ny + 1, nz + 1), one thread per (i, j, k) of the extended index space
    const int ey = ny + 1, ez = nz + 1;
    const int64_t si = (int64_t)ny * nz, sj = nz;
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= ez) return;
    {
        const int64_t c = ((int64_t)i * ny + j) * nz + k;  // cell (i, j, k) when inside
        if (j < ny && k < nz) {  // u face (i, j, k), i in [0, nx]
            const int64_t f = ((int64_t)i * ny + j) * nz + k;
            if (0 < i && i < nx)
                u[f] = grad_face(u, ur, p, ps, f, c - si, c, __ldg(&tag[c - si]), __ldg(&tag[c]));
            else
                u[f] = 0.0f;
        }
        if (i < nx && k < nz) {  // v face (i, j, k), j in [0, ny]
            const int64_t f = ((int64_t)i * ey + j) * nz + k;
            if (0 < j && j < ny)
                v[f] = grad_face(v, vr, p, ps, f, c - sj, c, __ldg(&tag[c - sj]), __ldg(&tag[c]));
            else
                v[f] = 0.0f;
        }
        if (i < nx && j < ny) {  // w face (i, j, k), k in [0, nz]
            const int64_t f = ((int64_t)i * ny + j) * ez + k;
            if (0 < k && k < nz)
                w[f] = grad_face(w, wr, p, ps, f, c - 1, c, __ldg(&tag[c - 1]), __ldg(&tag[c]));
            else
                w[f] = 0.0f;
        }
    }
}

// grad_face on values already loaded.
__device__ __forceinline__ float grad_vals(int tlo, int thi, float urv, float uv, float plo, float phi, float ps) {
    if (tlo == 2 || thi == 2) return urv;
    if (tlo == 1 || thi == 1) return __fsub_rn(uv, __fsub_rn(__fmul_rn(phi, ps), __fmul_rn(plo, ps)));
    return 0.0f;
}

__device__ __forceinline__ int i4(const int4 &v, int e) { return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w)); }
__device__ __forceinline__ float f4(const float4 &v, int e) {
    return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}

// Four faces k = 4t .. 4t + 3 of a u or v row between cell rows lo and hi
// (16-byte aligned): the face, rigid-face and pressure vectors are loaded only
// when one of the four faces takes the branch that reads them.
__device__ __forceinline__ float4 grad_face4(const float *__restrict__ uf, const float *__restrict__ urf,
                                             const float *__restrict__ p, float ps, int64_t f, int64_t clo,
                                             int64_t chi, const int4 tlo, const int4 thi) {
    bool solid = false, fluid = false;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int a = i4(tlo, e), b = i4(thi, e);
        const bool s = a == 2 || b == 2;
        solid |= s;
        fluid |= !s && (a == 1 || b == 1);
    }
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 ur4 = solid ? __ldg(reinterpret_cast<const float4 *>(urf + f)) : z4;
    const float4 u4 = fluid ? *reinterpret_cast<const float4 *>(uf + f) : z4;
    const float4 plo = fluid ? __ldg(reinterpret_cast<const float4 *>(p + clo)) : z4;
    const float4 phi = fluid ? __ldg(reinterpret_cast<const float4 *>(p + chi)) : z4;
    float o[4];
#pragma unroll
    for (int e = 0; e < 4; e++)
        o[e] = grad_vals(i4(tlo, e), i4(thi, e), f4(ur4, e), f4(u4, e), f4(plo, e), f4(phi, e), ps);
    return make_float4(o[0], o[1], o[2], o[3]);
}

// k_subtract_gradient_all for nz % 4 == 0 with 16-byte aligned arrays: a
// thread updates the faces k = 4t .. 4t + 3 of point (i, j) of the extended
// lattice, u and v with 16-byte accesses, w (rows of nz + 1, not aligned) one
// face at a time; the thread of the last quad of a row also zeroes w face nz.
// Same values as k_subtract_gradient_all, face by face.
// Grid: row_grid(nx + 1, ny + 1, nz / 4).
__global__ void __launch_bounds__(kRowThreads) k_subtract_gradient_all4(float *__restrict__ u, float *__restrict__ v,
                                                                float *__restrict__ w, const float *__restrict__ ur,
                                                                const float *__restrict__ vr,
                                                                const float *__restrict__ wr,
                                                                const float *__restrict__ p, float ps,
                                                                const int32_t *__restrict__ tag, int nx, int ny,
                                                                int nz) {
    const int nz4 = nz >> 2, ey = ny + 1, ez = nz + 1;
    const int64_t si = (int64_t)ny * nz, sj = nz;
    const int t = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (t >= nz4) return;
    const int k0 = 4 * t;
    const int64_t c = ((int64_t)i * ny + j) * nz + k0;  // cell (i, j, k0) when inside
    const bool inside = i < nx && j < ny;
    const int4 tc = inside ? __ldg(reinterpret_cast<const int4 *>(tag + c)) : make_int4(0, 0, 0, 0);
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (j < ny) {  // u faces (i, j, k0 .. k0 + 3), i in [0, nx]
        float4 o = z4;
        if (0 < i && i < nx)
            o = grad_face4(u, ur, p, ps, c, c - si, c, __ldg(reinterpret_cast<const int4 *>(tag + c - si)), tc);
        *reinterpret_cast<float4 *>(u + c) = o;
    }
    if (i < nx) {  // v faces (i, j, k0 .. k0 + 3), j in [0, ny]
        const int64_t f = ((int64_t)i * ey + j) * nz + k0;
        float4 o = z4;
        if (0 < j && j < ny)
            o = grad_face4(v, vr, p, ps, f, c - sj, c, __ldg(reinterpret_cast<const int4 *>(tag + c - sj)), tc);
        *reinterpret_cast<float4 *>(v + f) = o;
    }
    if (inside) {  // w faces (i, j, k0 .. k0 + 3), face k between cells k - 1 and k
        const int64_t f = ((int64_t)i * ny + j) * ez + k0;
        const int tprev = k0 > 0 ? __ldg(&tag[c - 1]) : 0;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float o = 0.0f;
            if (k > 0) {
                const int tlo = e == 0 ? tprev : i4(tc, e - 1), thi = i4(tc, e);
                o = grad_face(w, wr, p, ps, f + e, c + e - 1, c + e, tlo, thi);
            }
            w[f + e] = o;
        }
        if (t == nz4 - 1) w[f + 4] = 0.0f;  // face nz
    }
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_subtract_gradient_tag(float *uf, const float *urf, const float *p, const int32_t *tag, int nx, int ny,
                               int nz, int d, void *stream) {
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0, "subtract_gradient: shape must be positive");
    FLUB_REQUIRE(d >= 1 && d <= 3, "subtract_gradient: d=%d must be 1, 2 or 3", d);
    FLUB_REQUIRE(uf && urf && p && tag, "subtract_gradient: NULL pointer argument");
    FLUB_REQUIRE(nx < 65535 && ny < 65535, "subtract_gradient: nx, ny must be below 65535");
    k_subtract_gradient_axis<<<row_grid(nx + (d == 1), ny + (d == 2), nz + (d == 3)), kRowThreads, 0,
                               as_stream(stream)>>>(uf, urf, p, tag, nx, ny, nz, d);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_subtract_gradient(float *u, float *v, float *w, const float *ur, const float *vr, const float *wr,
                           const float *p, float p_scale, const int32_t *tag, int nx, int ny, int nz, void *stream) {
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0, "subtract_gradient: shape must be positive");
    FLUB_REQUIRE(u && v && w && ur && vr && wr && p && tag, "subtract_gradient: NULL pointer argument");
    FLUB_REQUIRE(nx < 65535 && ny < 65535, "subtract_gradient: nx, ny must be below 65535");
    const bool v4 = nz % 4 == 0 && ((uintptr_t)u | (uintptr_t)v | (uintptr_t)ur | (uintptr_t)vr | (uintptr_t)p |
                                    (uintptr_t)tag) % 16 == 0;
    if (v4)
        k_subtract_gradient_all4<<<row_grid(nx + 1, ny + 1, nz / 4), kRowThreads, 0, as_stream(stream)>>>(
            u, v, w, ur, vr, wr, p, p_scale, tag, nx, ny, nz);
    else
        k_subtract_gradient_all<<<row_grid(nx + 1, ny + 1, nz + 1), kRowThreads, 0, as_stream(stream)>>>(
            u, v, w, ur, vr, wr, p, p_scale, tag, nx, ny, nz);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
