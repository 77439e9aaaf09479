// Velocity extrapolation after the projection (water_3d.py:70-73 extrapolate,
// the step that follows project() in water_3d.step, :102).
//
// Face flags ("unknown", int32 per face, the reference's MACGridInt):
// 1 = to be extrapolated, 0 = known, -1 = extrapolated in the current pass.
#include "common.cuh"

namespace flub {

// utils/util.py:423-437 set_unknown over the cell grid: face (i, j, k) of
// every axis gets 1 where phi >= 0, else 0 (i < nx, j < ny, k < nz; the last
// face layer of each array is left as it was).  Grid: row_grid(nx, ny, nz).
__global__ void __launch_bounds__(kRowThreads) k_set_unknown(const float *__restrict__ phi, int32_t *__restrict__ tu,
                                                            int32_t *__restrict__ tv, int32_t *__restrict__ tw, int nx,
                                                            int ny, int nz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    const int32_t v = phi[((int64_t)i * ny + j) * nz + k] >= 0.0f ? 1 : 0;
    tu[((int64_t)i * ny + j) * nz + k] = v;
    tv[((int64_t)i * (ny + 1) + j) * nz + k] = v;
    tw[((int64_t)i * ny + j) * (nz + 1) + k] = v;
}

// extrapolate.py:8-30 extrapolate_3d on one face array q (fx, fy, fz): a face
// with flag 1 takes the mean of its in-bounds 3x3x3 neighbours (itself
// included) whose flag is 0, summed in (ii, jj, kk) order, kk fastest, FP32;
// with none it becomes 0.  kMark: set the flag of an extrapolated face to -1
// (the reference's kernel); otherwise leave it 1, which is the state its
// flush_1_3d (-1 -> 1) restores right after -- only flag-0 faces are ever
// read, so the two give the same values.
//
// One block owns a tile of kTi x kTj x kTk faces and stages the tile plus a
// one-face halo in shared memory (flags as bytes: 0 known, 1 to extrapolate,
// 2 any other flag or outside the array); each of its 256 threads then
// updates kTi faces along i.
// Known faces are never written during a pass and only known faces are read,
// so staging before other blocks write cannot change a result.
constexpr int kTi = 4, kTj = 8, kTk = 32;
constexpr int kHi = kTi + 2, kHj = kTj + 2, kHk = kTk + 2;

template <bool kMark>
__global__ void __launch_bounds__(kTj * kTk) k_extrapolate_tile(float *__restrict__ q, int32_t *__restrict__ unk,
                                                               int fx, int fy, int fz) {
    __shared__ float sv[kHi * kHj * kHk];
    __shared__ uint8_t sk[kHi * kHj * kHk];
    __shared__ int any_known;
    const int i0 = blockIdx.z * kTi, j0 = blockIdx.y * kTj, k0 = blockIdx.x * kTk;
    const int tid = threadIdx.y * kTk + threadIdx.x;
    if (tid == 0) any_known = 0;
    __syncthreads();
    int known = 0;
    for (int e = tid; e < kHi * kHj * kHk; e += kTj * kTk) {
        const int hk = e % kHk, hj = (e / kHk) % kHj, hi = e / (kHk * kHj);
        const int a = i0 + hi - 1, b = j0 + hj - 1, c = k0 + hk - 1;
        uint8_t kn = 2;
        float v = 0.0f;
        if (a >= 0 && a < fx && b >= 0 && b < fy && c >= 0 && c < fz) {
            const int64_t g = ((int64_t)a * fy + b) * fz + c;
            const int32_t fl = __ldg(unk + g);
            if (fl == 0) {
                kn = 0;
                v = __ldg(q + g);
                known = 1;
            } else if (fl == 1) {
                kn = 1;
            }
        }
        sk[e] = kn;
        sv[e] = v;
    }
    if (known) any_known = 1;
    __syncthreads();
    const int k = k0 + threadIdx.x, j = j0 + threadIdx.y;
    if (k >= fz || j >= fy) return;
    const bool none = any_known == 0;  // no known face in the tile and its halo: every unknown face becomes 0
#pragma unroll
    for (int ti = 0; ti < kTi; ti++) {
        const int i = i0 + ti;
        if (i >= fx) break;
        const int64_t f = ((int64_t)i * fy + j) * fz + k;
        const int hc = ((ti + 1) * kHj + threadIdx.y + 1) * kHk + threadIdx.x + 1;
        if (sk[hc] != 1) continue;  // known, or a flag other than 1: not touched, as in the reference
        if (none) {
            q[f] = 0.0f;
            continue;
        }
        int n = 0;
        float s = 0.0f;
#pragma unroll
        for (int ii = -1; ii <= 1; ii++)
#pragma unroll
            for (int jj = -1; jj <= 1; jj++)
#pragma unroll
                for (int kk = -1; kk <= 1; kk++) {
                    const int h = hc + (ii * kHj + jj) * kHk + kk;
                    if (sk[h] != 0) continue;
                    n++;
                    s = __fadd_rn(s, sv[h]);
                }
        if (n > 0) {
            q[f] = __fdiv_rn(s, (float)n);
            if (kMark) unk[f] = -1;
        } else {
            q[f] = 0.0f;
        }
    }
}

static inline dim3 tile_grid(int fx, int fy, int fz) {
    return dim3((unsigned)((fz + kTk - 1) / kTk), (unsigned)((fy + kTj - 1) / kTj), (unsigned)((fx + kTi - 1) / kTi));
}

// extrapolate.py:32-36 flush_1_3d.
__global__ void __launch_bounds__(256) k_flush_unknown(int32_t *__restrict__ unk, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (unk[c] == -1) unk[c] = 1;
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_set_unknown(const float *phi, int32_t *tu, int32_t *tv, int32_t *tw, int nx, int ny, int nz, void *stream) {
    FLUB_REQUIRE(phi && tu && tv && tw, "flub_set_unknown: NULL argument");
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65536 && ny < 65536, "flub_set_unknown: bad shape");
    k_set_unknown<<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(phi, tu, tv, tw, nx, ny, nz);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_extrapolate_axis(float *q, int32_t *unk, int nx, int ny, int nz, int d, void *stream) {
    FLUB_REQUIRE(q && unk, "flub_extrapolate_axis: NULL argument");
    FLUB_REQUIRE(d >= 1 && d <= 3, "flub_extrapolate_axis: d=%d must be 1, 2 or 3", d);
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65535 && ny < 65535, "flub_extrapolate_axis: bad shape");
    FLUB_REQUIRE(nx + 1 < 4 * 65535, "flub_extrapolate_axis: nx too large");
    const int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    k_extrapolate_tile<true><<<tile_grid(fx, fy, fz), dim3(kTk, kTj), 0, as_stream(stream)>>>(q, unk, fx, fy, fz);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_flush_unknown(int32_t *unk, int64_t n, void *stream) {
    FLUB_REQUIRE(unk && n >= 0, "flub_flush_unknown: bad arguments");
    if (n == 0) return FLUB_OK;
    k_flush_unknown<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(unk, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_extrapolate(float *u, float *v, float *w, int32_t *tu, int32_t *tv, int32_t *tw, const float *phi, int nx,
                     int ny, int nz, int n_passes, void *stream) {
    FLUB_REQUIRE(u && v && w && tu && tv && tw, "flub_extrapolate: NULL argument");
    FLUB_REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx < 65535 && ny < 65535, "flub_extrapolate: bad shape");
    FLUB_REQUIRE(n_passes >= 0, "flub_extrapolate: n_passes must be >= 0");
    cudaStream_t s = as_stream(stream);
    if (phi) {
        k_set_unknown<<<row_grid(nx, ny, nz), kRowThreads, 0, s>>>(phi, tu, tv, tw, nx, ny, nz);
        FLUB_CHECK_LAUNCH();
    }
    for (int p = 0; p < n_passes; p++) {
        k_extrapolate_tile<false><<<tile_grid(nx + 1, ny, nz), dim3(kTk, kTj), 0, s>>>(u, tu, nx + 1, ny, nz);
        FLUB_CHECK_LAUNCH();
        k_extrapolate_tile<false><<<tile_grid(nx, ny + 1, nz), dim3(kTk, kTj), 0, s>>>(v, tv, nx, ny + 1, nz);
        FLUB_CHECK_LAUNCH();
        k_extrapolate_tile<false><<<tile_grid(nx, ny, nz + 1), dim3(kTk, kTj), 0, s>>>(w, tw, nx, ny, nz + 1);
        FLUB_CHECK_LAUNCH();
    }
    return FLUB_OK;
}

}  // extern "C"
