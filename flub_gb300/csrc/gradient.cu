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
    k_subtract_gradient_all<<<row_grid(nx + 1, ny + 1, nz + 1), kRowThreads, 0, as_stream(stream)>>>(
        u, v, w, ur, vr, wr, p, p_scale, tag, nx, ny, nz);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
