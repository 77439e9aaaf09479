// Cell classification: water level set -> air / fluid, solid primitives -> solid.
//
// geometry.py:335-344 _tag_dirichlet, :390-397 _tag_neumann,
// :225-239 precompute_grid_point_phi_prims with :148-169 sdf_argmin_prims,
// :82-113 compute_sdf_atom_prims and :17-32 _sdf_cube.
//
// Every FP32 operation is an explicit round-to-nearest intrinsic so that the
// compiler cannot contract or reorder it; the oracle performs the same
// operations in the same order, so tags and SDF values match bit for bit.
#include "common.cuh"

namespace flub {

struct PrimSet {
    int n;
    flub_prim p[FLUB_MAX_PRIMS];
};

__device__ __forceinline__ void quat_rotate_inv(const float q[4], const float v[3], float out[3]) {
    // v (2 w^2 - 1) - 2 w (q_v x v) + 2 (q_v . v) q_v
    const float w = q[3];
    const float c = __fsub_rn(__fmul_rn(__fmul_rn(2.0f, w), w), 1.0f);
    const float d = __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(q[0], v[0]), __fmul_rn(q[1], v[1])),
                                              __fmul_rn(q[2], v[2])));
    const float cx = __fsub_rn(__fmul_rn(q[1], v[2]), __fmul_rn(q[2], v[1]));
    const float cy = __fsub_rn(__fmul_rn(q[2], v[0]), __fmul_rn(q[0], v[2]));
    const float cz = __fsub_rn(__fmul_rn(q[0], v[1]), __fmul_rn(q[1], v[0]));
    const float w2 = __fmul_rn(w, 2.0f);
    out[0] = __fadd_rn(__fsub_rn(__fmul_rn(v[0], c), __fmul_rn(cx, w2)), __fmul_rn(q[0], d));
    out[1] = __fadd_rn(__fsub_rn(__fmul_rn(v[1], c), __fmul_rn(cy, w2)), __fmul_rn(q[1], d));
    out[2] = __fadd_rn(__fsub_rn(__fmul_rn(v[2], c), __fmul_rn(cz, w2)), __fmul_rn(q[2], d));
}

__device__ __forceinline__ float len3(float a, float b, float c) {
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c)));
}

__device__ float sdf_cube(const float p_in[3], const float radius[3], const float q[4]) {
    float p[3], m[3];
    quat_rotate_inv(q, p_in, p);
#pragma unroll
    for (int a = 0; a < 3; a++) m[a] = __fsub_rn(fmaxf(p[a], -p[a]), radius[a]);
    const float mx = fmaxf(fmaxf(m[0], m[1]), m[2]);
    if (mx < 0.0f) return mx;
    return len3(fmaxf(m[0], 0.0f), fmaxf(m[1], 0.0f), fmaxf(m[2], 0.0f));
}

__device__ __forceinline__ void quat_mul(const float a[4], const float b[4], float o[4]) {
    o[0] = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a[3], b[0]), __fmul_rn(b[3], a[0])), __fmul_rn(a[1], b[2])),
                     __fmul_rn(a[2], b[1]));
    o[1] = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a[3], b[1]), __fmul_rn(b[3], a[1])), __fmul_rn(a[2], b[0])),
                     __fmul_rn(a[0], b[2]));
    o[2] = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a[3], b[2]), __fmul_rn(b[3], a[2])), __fmul_rn(a[0], b[1])),
                     __fmul_rn(a[1], b[0]));
    o[3] = __fsub_rn(__fmul_rn(a[3], b[3]),
                     __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2])));
}

__device__ float sdf_atom(float u, float v, float w, const flub_prim &g) {
    const float p[3] = {__fsub_rn(u, g.x[0]), __fsub_rn(v, g.x[1]), __fsub_rn(w, g.x[2])};
    switch (g.geometry) {
    case 1:
    case 3:
        return sdf_cube(p, g.radius, g.q);
    case 2:
        return __fsub_rn(len3(p[0], p[1], p[2]), g.radius[0]);
    case 4: {
        const float s = 0.70710678118654752f;
        const float zq[4] = {0.0f, 0.0f, s, s}, zi[4] = {0.0f, 0.0f, -s, s};
        float t[4], q2[4];
        quat_mul(zq, g.q, t);
        quat_mul(t, zi, q2);
        return fminf(sdf_cube(p, g.radius, g.q), sdf_cube(p, g.radius, q2));
    }
    case 5:
        return 2.0f;
    default:
        return 1.0f;
    }
}

// sdf_argmin_prims: the smallest SDF below min(h0, running minimum), else 2.0.
__device__ __forceinline__ float phi_prims_at(int i, int j, int k, float h, float h0, float sx, float sy,
                                              float sz, const PrimSet &ps) {
    float u = __fmul_rn((float)i, h), v = __fmul_rn((float)j, h), w = __fmul_rn((float)k, h);
    u = __fadd_rn(u, __fmul_rn(sx, h));
    v = __fadd_rn(v, __fmul_rn(sy, h));
    w = __fadd_rn(w, __fmul_rn(sz, h));
    float interior = 2.0f;
    for (int o = 0; o < ps.n; o++) {
        const float s = sdf_atom(u, v, w, ps.p[o]);
        if (s < fminf(h0, interior)) interior = s;
    }
    return interior;
}

__global__ void k_tag_dirichlet(const float *__restrict__ phi, int32_t *__restrict__ tag, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        tag[c] = phi[c] > 0.0f ? 0 : 1;
}

__global__ void k_tag_neumann(const float *__restrict__ phr, int32_t *__restrict__ tag, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (phr[c] < 0.0f) tag[c] = 2;
}

// Grid: row_grid(nx, ny, nz) (one thread per cell, k along x).
__global__ void __launch_bounds__(kRowThreads) k_phi_prims(float *__restrict__ phi, int nx, int ny, int nz, float h,
                                                          float h0, float sx, float sy, float sz, const PrimSet ps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    const int64_t c = ((int64_t)i * ny + j) * nz + k;
    phi[c] = phi_prims_at(i, j, k, h, h0, sx, sy, sz, ps);
}

// Fused: tag from phi, then solid from the primitives' cell-centre SDF.
// Grid: row_grid(nx, ny, nz).
__global__ void __launch_bounds__(kRowThreads) k_classify(const float *__restrict__ phi, int32_t *__restrict__ tag,
                                                         float *__restrict__ phr, int nx, int ny, int nz, float h,
                                                         float h0, const PrimSet ps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    const int64_t c = ((int64_t)i * ny + j) * nz + k;
    int t = phi[c] > 0.0f ? 0 : 1;
    if (ps.n > 0 || phr) {
        const float s = phi_prims_at(i, j, k, h, h0, 0.5f, 0.5f, 0.5f, ps);
        if (phr) phr[c] = s;
        if (s < 0.0f) t = 2;
    }
    tag[c] = t;
}

// ---------------------------------------------------------------- four cells per thread
//
// k_classify for nz % 4 == 0: a thread classifies cells k = 4t .. 4t + 3 of
// row (i, j).  Within a row only w = (k + 1/2) h changes, so the SDF terms
// that involve only u, v and the primitive are computed once per row and
// primitive: the same operations on the same operands as phi_prims_at,
// sdf_atom, sdf_cube and quat_rotate_inv perform per cell, hence the same
// bits.

// Row-invariant part of sdf_cube's quat_rotate_inv(q, (p0, p1, p2)) for fixed p0, p1.
struct CubeRow {
    float c, w2, a01, q2p1, q2p0, cz, p0c, p1c, czw2;
    float q[4], r[3];
};

__device__ __forceinline__ void cube_row(CubeRow &cr, float p0, float p1, const float q[4], const float r[3]) {
    cr.c = __fsub_rn(__fmul_rn(__fmul_rn(2.0f, q[3]), q[3]), 1.0f);
    cr.a01 = __fadd_rn(__fmul_rn(q[0], p0), __fmul_rn(q[1], p1));
    cr.q2p1 = __fmul_rn(q[2], p1);
    cr.q2p0 = __fmul_rn(q[2], p0);
    cr.cz = __fsub_rn(__fmul_rn(q[0], p1), __fmul_rn(q[1], p0));
    cr.w2 = __fmul_rn(q[3], 2.0f);
    cr.p0c = __fmul_rn(p0, cr.c);
    cr.p1c = __fmul_rn(p1, cr.c);
    cr.czw2 = __fmul_rn(cr.cz, cr.w2);
#pragma unroll
    for (int a = 0; a < 4; a++) cr.q[a] = q[a];
#pragma unroll
    for (int a = 0; a < 3; a++) cr.r[a] = r[a];
}

// sdf_cube at (p0, p1, p2) from the row part.
__device__ __forceinline__ float cube_at(const CubeRow &cr, float p2) {
    const float d = __fmul_rn(2.0f, __fadd_rn(cr.a01, __fmul_rn(cr.q[2], p2)));
    const float cx = __fsub_rn(__fmul_rn(cr.q[1], p2), cr.q2p1);
    const float cy = __fsub_rn(cr.q2p0, __fmul_rn(cr.q[0], p2));
    float p[3], m[3];
    p[0] = __fadd_rn(__fsub_rn(cr.p0c, __fmul_rn(cx, cr.w2)), __fmul_rn(cr.q[0], d));
    p[1] = __fadd_rn(__fsub_rn(cr.p1c, __fmul_rn(cy, cr.w2)), __fmul_rn(cr.q[1], d));
    p[2] = __fadd_rn(__fsub_rn(__fmul_rn(p2, cr.c), cr.czw2), __fmul_rn(cr.q[2], d));
#pragma unroll
    for (int a = 0; a < 3; a++) m[a] = __fsub_rn(fmaxf(p[a], -p[a]), cr.r[a]);
    const float mx = fmaxf(fmaxf(m[0], m[1]), m[2]);
    if (mx < 0.0f) return mx;
    return len3(fmaxf(m[0], 0.0f), fmaxf(m[1], 0.0f), fmaxf(m[2], 0.0f));
}

__global__ void __launch_bounds__(kRowThreads) k_classify4(const float4 *__restrict__ phi, int4 *__restrict__ tag,
                                                          float4 *__restrict__ phr, int ny, int nz, float h,
                                                          float h0, const PrimSet ps) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    const int nz4 = nz >> 2;
    if (t >= nz4) return;
    const int64_t c4 = ((int64_t)i * ny + j) * nz4 + t;
    const float4 pv = __ldg(phi + c4);
    int tt[4] = {pv.x > 0.0f ? 0 : 1, pv.y > 0.0f ? 0 : 1, pv.z > 0.0f ? 0 : 1, pv.w > 0.0f ? 0 : 1};
    if (ps.n > 0 || phr) {
        const float hs = __fmul_rn(0.5f, h);
        const float u = __fadd_rn(__fmul_rn((float)i, h), hs), v = __fadd_rn(__fmul_rn((float)j, h), hs);
        float wv[4], in[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            wv[e] = __fadd_rn(__fmul_rn((float)(4 * t + e), h), hs);
            in[e] = 2.0f;
        }
        for (int o = 0; o < ps.n; o++) {
            const flub_prim &g = ps.p[o];
            const float p0 = __fsub_rn(u, g.x[0]), p1 = __fsub_rn(v, g.x[1]);
            float s[4];
            if (g.geometry == 1 || g.geometry == 3 || g.geometry == 4) {
                CubeRow cr;
                cube_row(cr, p0, p1, g.q, g.radius);
#pragma unroll
                for (int e = 0; e < 4; e++) s[e] = cube_at(cr, __fsub_rn(wv[e], g.x[2]));
                if (g.geometry == 4) {
                    const float sq = 0.70710678118654752f;
                    const float zq[4] = {0.0f, 0.0f, sq, sq}, zi[4] = {0.0f, 0.0f, -sq, sq};
                    float tq[4], q2[4];
                    quat_mul(zq, g.q, tq);
                    quat_mul(tq, zi, q2);
                    cube_row(cr, p0, p1, q2, g.radius);
#pragma unroll
                    for (int e = 0; e < 4; e++) s[e] = fminf(s[e], cube_at(cr, __fsub_rn(wv[e], g.x[2])));
                }
            } else if (g.geometry == 2) {
                const float s01 = __fadd_rn(__fmul_rn(p0, p0), __fmul_rn(p1, p1));
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float p2 = __fsub_rn(wv[e], g.x[2]);
                    s[e] = __fsub_rn(__fsqrt_rn(__fadd_rn(s01, __fmul_rn(p2, p2))), g.radius[0]);
                }
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++) s[e] = g.geometry == 5 ? 2.0f : 1.0f;
            }
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (s[e] < fminf(h0, in[e])) in[e] = s[e];
        }
        if (phr) phr[c4] = make_float4(in[0], in[1], in[2], in[3]);
#pragma unroll
        for (int e = 0; e < 4; e++)
            if (in[e] < 0.0f) tt[e] = 2;
    }
    tag[c4] = make_int4(tt[0], tt[1], tt[2], tt[3]);
}

static int make_primset(const flub_prim *prims, int nprims, PrimSet *ps) {
    FLUB_REQUIRE(nprims >= 0 && nprims <= FLUB_MAX_PRIMS, "nprims=%d outside [0, %d]", nprims, FLUB_MAX_PRIMS);
    FLUB_REQUIRE(nprims == 0 || prims != nullptr, "prims is NULL with nprims=%d", nprims);
    ps->n = nprims;
    for (int o = 0; o < nprims; o++) ps->p[o] = prims[o];
    return FLUB_OK;
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_tag_dirichlet(const float *phi, int32_t *tag, int64_t n, void *stream) {
    FLUB_REQUIRE(n >= 0 && (n == 0 || (phi && tag)), "flub_tag_dirichlet: bad arguments");
    if (n == 0) return FLUB_OK;
    k_tag_dirichlet<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(phi, tag, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_tag_neumann(const float *phr, int32_t *tag, int64_t n, void *stream) {
    FLUB_REQUIRE(n >= 0 && (n == 0 || (phr && tag)), "flub_tag_neumann: bad arguments");
    if (n == 0) return FLUB_OK;
    k_tag_neumann<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(phr, tag, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_phi_prims(float *phi, int nx, int ny, int nz, float h, float h0, float sx, float sy, float sz,
                   const flub_prim *prims, int nprims, void *stream) {
    FLUB_REQUIRE(nx >= 0 && ny >= 0 && nz >= 0, "flub_phi_prims: negative shape");
    const int64_t n = (int64_t)nx * ny * nz;
    if (n == 0) return FLUB_OK;
    FLUB_REQUIRE(phi != nullptr, "flub_phi_prims: phi is NULL");
    PrimSet ps;
    int st = make_primset(prims, nprims, &ps);
    if (st) return st;
    FLUB_REQUIRE(nx < 65536 && ny < 65536, "flub_phi_prims: nx, ny must be below 65536");
    k_phi_prims<<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(phi, nx, ny, nz, h, h0, sx, sy, sz, ps);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_classify(const float *phi, const flub_prim *prims, int nprims, int nx, int ny, int nz, float h, float h0,
                  int32_t *tag, float *phi_rigid, void *stream) {
    FLUB_REQUIRE(nx >= 0 && ny >= 0 && nz >= 0, "flub_classify: negative shape");
    const int64_t n = (int64_t)nx * ny * nz;
    if (n == 0) return FLUB_OK;
    FLUB_REQUIRE(phi && tag, "flub_classify: phi/tag is NULL");
    PrimSet ps;
    int st = make_primset(prims, nprims, &ps);
    if (st) return st;
    FLUB_REQUIRE(nx < 65536 && ny < 65536, "flub_classify: nx, ny must be below 65536");
    const bool v4 = nz % 4 == 0 && ((uintptr_t)phi | (uintptr_t)tag | (uintptr_t)phi_rigid) % 16 == 0;
    if (v4)
        k_classify4<<<row_grid(nx, ny, nz / 4), kRowThreads, 0, as_stream(stream)>>>(
            reinterpret_cast<const float4 *>(phi), reinterpret_cast<int4 *>(tag), reinterpret_cast<float4 *>(phi_rigid),
            ny, nz, h, h0, ps);
    else
        k_classify<<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(phi, tag, phi_rigid, nx, ny, nz, h,
                                                                              h0, ps);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
