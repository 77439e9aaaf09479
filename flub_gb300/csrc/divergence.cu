// Divergence right-hand side of the projection.
//
// divergence.py:43-99 divergence_tag, :173-180 mask_with_tag and
// utils/util.py:162-165 scale_by_3d, plus the fused form used by the
// projection (example_fluid.py:84-93).  One thread per cell; consecutive
// threads walk k, so every face array is read in coalesced rows.
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

}  // namespace flub

using namespace flub;

extern "C" {

int flub_divergence_tag(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                        const float *wr, const int32_t *tag, float *div, int nx, int ny, int nz, void *stream) {
    int st = check_div_args(u, v, w, ur, vr, wr, tag, div, nx, ny, nz);
    if (st) return st;
    k_divergence<false><<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(u, v, w, ur, vr, wr, tag, div, nx, ny,
                                                                           nz, 1.0f);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_divergence_masked(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                           const float *wr, const int32_t *tag, float *div, float scale, int nx, int ny, int nz,
                           void *stream) {
    int st = check_div_args(u, v, w, ur, vr, wr, tag, div, nx, ny, nz);
    if (st) return st;
    k_divergence<true><<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(u, v, w, ur, vr, wr, tag, div, nx, ny,
                                                                          nz, scale);
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
