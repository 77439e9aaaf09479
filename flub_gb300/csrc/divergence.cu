// Divergence right-hand side of the projection.
//
// divergence.py:43-99 divergence_tag, :173-180 mask_with_tag and
// utils/util.py:162-165 scale_by_3d, plus the fused form used by the
// projection (example_fluid.py:84-93).  Consecutive threads walk k, so every
// face array is read in coalesced rows: one cell per thread in general, four
// (k_divergence4) when nz % 4 == 0.
#include "common.cuh"

namespace flub {

template <bool kMasked>
__global__ void __launch_bounds__(kRowThreads) k_divergence(const float *__restrict__ u, const float *__restrict__ v,
                                                    const float *__restrict__ w, const float *__restrict__ ur,
                                                    const float *__restrict__ vr, const float *__restrict__ wr,
                                                    const int32_t *__restrict__ tag, float *__restrict__ div, int nx,
                                                    int ny, int nz, float scale) {
    // grid: row_grid(nx, ny, nz)
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    const int64_t sj = nz, si = (int64_t)ny * nz;
    const int64_t c = ((int64_t)i * ny + j) * nz + k;
    {
        if (kMasked && __ldg(&tag[c]) != 1) {
            div[c] = 0.0f;
            return;
        }
        // face indices: u (nx+1, ny, nz), v (nx, ny+1, nz), w (nx, ny, nz+1)
        const int64_t uL = c, uR = c + si;
        const int64_t vB = ((int64_t)i * (ny + 1) + j) * nz + k, vT = vB + nz;
        const int64_t wF = ((int64_t)i * ny + j) * (nz + 1) + k, wN = wF + 1;
        float fl = __ldg(&u[uL]), fr = __ldg(&u[uR]), fb = __ldg(&v[vB]), ft = __ldg(&v[vT]);
        float ff = __ldg(&w[wF]), fn = __ldg(&w[wN]);
        if (i == 0) fl = 0.0f; else if (__ldg(&tag[c - si]) == 2) fl = __ldg(&ur[uL]);
        if (i == nx - 1) fr = 0.0f; else if (__ldg(&tag[c + si]) == 2) fr = __ldg(&ur[uR]);
        if (j == 0) fb = 0.0f; else if (__ldg(&tag[c - sj]) == 2) fb = __ldg(&vr[vB]);
        if (j == ny - 1) ft = 0.0f; else if (__ldg(&tag[c + sj]) == 2) ft = __ldg(&vr[vT]);
        if (k == 0) ff = 0.0f; else if (__ldg(&tag[c - 1]) == 2) ff = __ldg(&wr[wF]);
        if (k == nz - 1) fn = 0.0f; else if (__ldg(&tag[c + 1]) == 2) fn = __ldg(&wr[wN]);
        const float d = __fsub_rn(__fadd_rn(__fsub_rn(__fadd_rn(__fsub_rn(fr, fl), ft), fb), fn), ff);
        div[c] = kMasked ? __fmul_rn(d, scale) : d;
    }
}

__device__ __forceinline__ int dv_i4(const int4 &v, int e) {
    return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}
__device__ __forceinline__ float dv_f4(const float4 &v, int e) {
    return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}

// k_divergence for nz % 4 == 0 with 16-byte aligned arrays: a thread takes
// cells k = 4t .. 4t + 3 of row (i, j), with 16-byte reads of the tags and of
// the u and v faces (the w faces, rows of nz + 1, one at a time).  A rigid
// face row is read only when one of the four cells has a solid neighbour
// across it; in the masked form nothing but the tags is read when none of the
// four cells is fluid.  Same values as k_divergence, cell by cell.
// Grid: row_grid(nx, ny, nz / 4).
template <bool kMasked>
__global__ void __launch_bounds__(kRowThreads) k_divergence4(const float *__restrict__ u, const float *__restrict__ v,
                                                     const float *__restrict__ w, const float *__restrict__ ur,
                                                     const float *__restrict__ vr, const float *__restrict__ wr,
                                                     const int32_t *__restrict__ tag, float *__restrict__ div, int nx,
                                                     int ny, int nz, float scale) {
    const int nz4 = nz >> 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (t >= nz4) return;
    const int k0 = 4 * t;
    const int64_t sj = nz, si = (int64_t)ny * nz;
    const int64_t c = ((int64_t)i * ny + j) * nz + k0;
    const int4 tc = __ldg(reinterpret_cast<const int4 *>(tag + c));
    if (kMasked && tc.x != 1 && tc.y != 1 && tc.z != 1 && tc.w != 1) {
        *reinterpret_cast<float4 *>(div + c) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const int4 zi = make_int4(0, 0, 0, 0);
    const float4 zf = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int64_t vB = ((int64_t)i * (ny + 1) + j) * nz + k0, vT = vB + nz;
    const int64_t wF = ((int64_t)i * ny + j) * (nz + 1) + k0;
    // neighbour tags (2 = solid: the face takes the rigid velocity)
    const int4 tim = i > 0 ? __ldg(reinterpret_cast<const int4 *>(tag + c - si)) : zi;
    const int4 tip = i < nx - 1 ? __ldg(reinterpret_cast<const int4 *>(tag + c + si)) : zi;
    const int4 tjm = j > 0 ? __ldg(reinterpret_cast<const int4 *>(tag + c - sj)) : zi;
    const int4 tjp = j < ny - 1 ? __ldg(reinterpret_cast<const int4 *>(tag + c + sj)) : zi;
    const int tkm = k0 > 0 ? __ldg(&tag[c - 1]) : 0, tkp = k0 + 4 < nz ? __ldg(&tag[c + 4]) : 0;
    const float4 ul = __ldg(reinterpret_cast<const float4 *>(u + c));
    const float4 uh = __ldg(reinterpret_cast<const float4 *>(u + c + si));
    const float4 vl = __ldg(reinterpret_cast<const float4 *>(v + vB));
    const float4 vh = __ldg(reinterpret_cast<const float4 *>(v + vT));
    float wv[5];
#pragma unroll
    for (int e = 0; e < 5; e++) wv[e] = __ldg(&w[wF + e]);
    auto any2 = [](const int4 &a) { return a.x == 2 || a.y == 2 || a.z == 2 || a.w == 2; };
    const float4 url = any2(tim) ? __ldg(reinterpret_cast<const float4 *>(ur + c)) : zf;
    const float4 urh = any2(tip) ? __ldg(reinterpret_cast<const float4 *>(ur + c + si)) : zf;
    const float4 vrl = any2(tjm) ? __ldg(reinterpret_cast<const float4 *>(vr + vB)) : zf;
    const float4 vrh = any2(tjp) ? __ldg(reinterpret_cast<const float4 *>(vr + vT)) : zf;
    float out[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int k = k0 + e;
        if (kMasked && dv_i4(tc, e) != 1) {
            out[e] = 0.0f;
            continue;
        }
        float fl = dv_f4(ul, e), fr = dv_f4(uh, e), fb = dv_f4(vl, e), ft = dv_f4(vh, e);
        float ff = wv[e], fn = wv[e + 1];
        if (i == 0) fl = 0.0f; else if (dv_i4(tim, e) == 2) fl = dv_f4(url, e);
        if (i == nx - 1) fr = 0.0f; else if (dv_i4(tip, e) == 2) fr = dv_f4(urh, e);
        if (j == 0) fb = 0.0f; else if (dv_i4(tjm, e) == 2) fb = dv_f4(vrl, e);
        if (j == ny - 1) ft = 0.0f; else if (dv_i4(tjp, e) == 2) ft = dv_f4(vrh, e);
        const int tb = e == 0 ? tkm : dv_i4(tc, e - 1), tf = e == 3 ? tkp : dv_i4(tc, e + 1);
        if (k == 0) ff = 0.0f; else if (tb == 2) ff = __ldg(&wr[wF + e]);
        if (k == nz - 1) fn = 0.0f; else if (tf == 2) fn = __ldg(&wr[wF + e + 1]);
        const float d = __fsub_rn(__fadd_rn(__fsub_rn(__fadd_rn(__fsub_rn(fr, fl), ft), fb), fn), ff);
        out[e] = kMasked ? __fmul_rn(d, scale) : d;
    }
    *reinterpret_cast<float4 *>(div + c) = make_float4(out[0], out[1], out[2], out[3]);
}

__global__ void k_mask_with_tag(float *__restrict__ div, const int32_t *__restrict__ tag, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (tag[c] != 1) div[c] = 0.0f;
}

__global__ void k_scale(float *__restrict__ q, float s, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        q[c] = __fmul_rn(q[c], s);
}

static int check_div_args(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                          const float *wr, const int32_t *tag, float *div, int nx, int ny, int nz) {
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0, "divergence: shape (%d, %d, %d) must be positive", nx, ny, nz);
    FLUB_REQUIRE(nx < 65536 && ny < 65536, "divergence: nx, ny must be below 65536");
    FLUB_REQUIRE(u && v && w && ur && vr && wr && tag && div, "divergence: NULL pointer argument");
    return FLUB_OK;
}

// k_divergence4 applies: nz % 4 == 0 and the arrays it reads 16 bytes at a time are 16-byte aligned.
static bool div4_ok(const float *u, const float *v, const float *ur, const float *vr, const int32_t *tag,
                    const float *div, int nz) {
    return nz % 4 == 0 && ((uintptr_t)u | (uintptr_t)v | (uintptr_t)ur | (uintptr_t)vr | (uintptr_t)tag |
                           (uintptr_t)div) % 16 == 0;
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_divergence_tag(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                        const float *wr, const int32_t *tag, float *div, int nx, int ny, int nz, void *stream) {
    int st = check_div_args(u, v, w, ur, vr, wr, tag, div, nx, ny, nz);
    if (st) return st;
    if (div4_ok(u, v, ur, vr, tag, div, nz))
        k_divergence4<false><<<row_grid(nx, ny, nz / 4), kRowThreads, 0, as_stream(stream)>>>(u, v, w, ur, vr, wr, tag,
                                                                                        div, nx, ny, nz, 1.0f);
    else
        k_divergence<false><<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(u, v, w, ur, vr, wr, tag, div,
                                                                                  nx, ny, nz, 1.0f);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_divergence_masked(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                           const float *wr, const int32_t *tag, float *div, float scale, int nx, int ny, int nz,
                           void *stream) {
    int st = check_div_args(u, v, w, ur, vr, wr, tag, div, nx, ny, nz);
    if (st) return st;
    if (div4_ok(u, v, ur, vr, tag, div, nz))
        k_divergence4<true><<<row_grid(nx, ny, nz / 4), kRowThreads, 0, as_stream(stream)>>>(u, v, w, ur, vr, wr, tag,
                                                                                        div, nx, ny, nz, scale);
    else
        k_divergence<true><<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(u, v, w, ur, vr, wr, tag, div,
                                                                                  nx, ny, nz, scale);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_mask_with_tag(float *div, const int32_t *tag, int64_t n, void *stream) {
    FLUB_REQUIRE(n >= 0 && (n == 0 || (div && tag)), "flub_mask_with_tag: bad arguments");
    if (n == 0) return FLUB_OK;
    k_mask_with_tag<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(div, tag, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_scale(float *q, float s, int64_t n, void *stream) {
    FLUB_REQUIRE(n >= 0 && (n == 0 || q), "flub_scale: bad arguments");
    if (n == 0) return FLUB_OK;
    k_scale<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(q, s, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
