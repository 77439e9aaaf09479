// Level-set redistance by fast sweeping (redistance.py), used by flub's
// particle level set (particles.py:255, :267-270).
//
// FP32 in the reference's operation order through explicit round-to-nearest
// intrinsics; x ** 2.0 is x * x, sqrt is the correctly rounded square root;
// the min and max of two values are a < b ? a : b and a > b ? a : b.
#include "common.cuh"

namespace flub {

__device__ __forceinline__ float rd_min(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float rd_max(float a, float b) { return a > b ? a : b; }

// utils/util.py:403-412 fraction_of_fluid.
__device__ __forceinline__ float rd_frac(float p1, float p2) {
    if (p1 < 0.0f && p2 < 0.0f) return 1.0f;
    if (p1 >= 0.0f && p2 >= 0.0f) return 0.0f;
    return __fsub_rn(1.0f, __fdiv_rn(fmaxf(p1, p2), fabsf(__fsub_rn(p1, p2))));
}

// redistance.py:66-119 _init_distance, out of place: every cell reads the
// values from before the launch (the reference rewrites phi in place inside
// one launch, where a cell may read a neighbour already rewritten).
// Neighbours outside the grid read 0.5 h; the neighbour test keeps the
// reference's precedence, (!boundary && left) || right || ... .
// Grid: row_grid(nx, ny, nz).
__global__ void __launch_bounds__(kRowThreads) k_redistance_init(const float *__restrict__ phi, float *__restrict__ out,
                                                                int nx, int ny, int nz, float h, int set_boundary) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    const int64_t c = ((int64_t)i * ny + j) * nz + k, sj = nz, si = (int64_t)ny * nz;
    const float hb = __fmul_rn(0.5f, h);
    const float pl = i > 0 ? __ldg(phi + c - si) : hb, pr = i < nx - 1 ? __ldg(phi + c + si) : hb;
    const float pb = j > 0 ? __ldg(phi + c - sj) : hb, pt = j < ny - 1 ? __ldg(phi + c + sj) : hb;
    const float pf = k > 0 ? __ldg(phi + c - 1) : hb, pn = k < nz - 1 ? __ldg(phi + c + 1) : hb;
    const float pc = __ldg(phi + c);
    const bool bnd = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1;
    float v = pc;
    if (bnd && !set_boundary) {
        v = pc;
    } else if (pc > 0.0f) {
        if ((!bnd && pl < 0.0f) || pr < 0.0f || pb < 0.0f || pt < 0.0f || pf < 0.0f || pn < 0.0f) {
            float m = __fsub_rn(1.0f, rd_frac(pc, pl));
            m = rd_min(m, __fsub_rn(1.0f, rd_frac(pc, pr)));
            m = rd_min(m, __fsub_rn(1.0f, rd_frac(pc, pb)));
            m = rd_min(m, __fsub_rn(1.0f, rd_frac(pc, pt)));
            m = rd_min(m, __fsub_rn(1.0f, rd_frac(pc, pf)));
            m = rd_min(m, __fsub_rn(1.0f, rd_frac(pc, pn)));
            v = __fmul_rn(h, m);
        } else {
            v = 2.0f;
        }
    } else if (pc < 0.0f) {
        if ((!bnd && pl > 0.0f) || pr > 0.0f || pb > 0.0f || pt > 0.0f || pf > 0.0f || pn > 0.0f) {
            float m = rd_frac(pc, pl);
            m = rd_min(m, rd_frac(pc, pr));
            m = rd_min(m, rd_frac(pc, pb));
            m = rd_min(m, rd_frac(pc, pt));
            m = rd_min(m, rd_frac(pc, pf));
            m = rd_min(m, rd_frac(pc, pn));
            v = __fmul_rn(-h, m);
        } else {
            v = -2.0f;
        }
    }
    out[c] = v;
}

// redistance.py:7-63 update over the cells of one parity (colour): the
// upwind-sorted neighbour values and the 1-, 2- or 3-neighbour Eikonal
// solution, kept where smaller than |phi|, for cells off the boundary with
// |phi| > h.  A cell reads only its six neighbours, all of the other parity,
// so the cells of one launch are independent.  Thread t of row (i, j) owns
// k = 2 t + ((colour + i + j) & 1).  Grid: row_grid(nx, ny, ceil(nz / 2)).
__global__ void __launch_bounds__(kRowThreads) k_redistance_sweep(float *phi, int nx, int ny, int nz, int incx, int incy,
                                                                 int incz, int colour, float h) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    const int k = 2 * t + ((colour + i + j) & 1);
    if (k >= nz) return;
    if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1) return;
    const int64_t c = ((int64_t)i * ny + j) * nz + k, sj = nz, si = (int64_t)ny * nz;
    const float pc = phi[c];
    if (!(fabsf(pc) > h)) return;
    const int64_t dx = incx * si, dy = incy * sj, dz = incz;
    float phii = __ldg(phi + c - dx), phij = __ldg(phi + c - dy), phik = __ldg(phi + c - dz);
    const float phiii = __ldg(phi + c + dx), phijj = __ldg(phi + c + dy), phikk = __ldg(phi + c + dz);
    float sgn = 1.0f;
    if (phii < 0.0f) {
        phii = -rd_max(phii, phiii);
        phij = -rd_max(phij, phijj);
        phik = -rd_max(phik, phikk);
        sgn = -1.0f;
    } else {
        phii = rd_min(phii, phiii);
        phij = rd_min(phij, phijj);
        phik = rd_min(phik, phikk);
    }
    const float phi0 = rd_min(rd_min(phii, phij), phik);
    const float phi2 = rd_max(rd_max(phii, phij), phik);
    const float phi1 = __fsub_rn(__fsub_rn(__fadd_rn(__fadd_rn(phii, phij), phik), phi0), phi2);
    float d = __fadd_rn(phi0, h);
    if (d > phi1) {
        const float e = __fsub_rn(phi0, phi1);
        d = __fmul_rn(0.5f, __fadd_rn(__fadd_rn(phi0, phi1),
                                      __fsqrt_rn(__fsub_rn(__fmul_rn(__fmul_rn(2.0f, h), h), __fmul_rn(e, e)))));
        if (d > phi2) {
            const float s = __fadd_rn(__fadd_rn(phi0, phi1), phi2);
            const float sq = __fadd_rn(__fadd_rn(__fmul_rn(phi0, phi0), __fmul_rn(phi1, phi1)), __fmul_rn(phi2, phi2));
            const float term = __fsub_rn(__fmul_rn(s, s), __fmul_rn(3.0f, __fsub_rn(sq, __fmul_rn(h, h))));
            d = __fmul_rn(1.0f / 3.0f, __fadd_rn(s, __fsqrt_rn(rd_max(0.0f, term))));
        }
    }
    phi[c] = __fmul_rn(sgn, rd_min(d, fabsf(pc)));
}

// redistance.py:128-136: the eight sweep directions of one round.
constexpr int kSweepDirs[8][3] = {{1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1},
                                  {1, 1, 1},  {-1, 1, 1},  {-1, -1, 1},  {1, -1, 1}};

// The parity of the cells the reference's launch _sweep(..., odd) updates:
// its thread (a, b, c) with (a + b + c) % 2 == odd writes the cell mirrored on
// every axis with a negative increment, which flips the parity by n - 1 on
// that axis.
static inline int sweep_colour(int nx, int ny, int nz, int incx, int incy, int incz, int odd) {
    int c = odd;
    if (incx < 0) c += nx - 1;
    if (incy < 0) c += ny - 1;
    if (incz < 0) c += nz - 1;
    return c & 1;
}

static int launch_sweep(float *phi, int nx, int ny, int nz, int incx, int incy, int incz, int odd, float h,
                        cudaStream_t s) {
    const int colour = sweep_colour(nx, ny, nz, incx, incy, incz, odd);
    k_redistance_sweep<<<row_grid(nx, ny, (nz + 1) / 2), kRowThreads, 0, s>>>(phi, nx, ny, nz, incx, incy, incz,
                                                                             colour, h);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

static inline bool rd_shape_ok(int nx, int ny, int nz) {
    return nx > 0 && ny > 0 && nz > 0 && nx < 65536 && ny < 65536;
}

}  // namespace flub

using namespace flub;

extern "C" {

int flub_redistance_init(const float *phi, float *out, int nx, int ny, int nz, float h, int set_boundary,
                         void *stream) {
    FLUB_REQUIRE(phi && out, "flub_redistance_init: NULL argument");
    FLUB_REQUIRE(phi != out, "flub_redistance_init: out must not alias phi");
    FLUB_REQUIRE(rd_shape_ok(nx, ny, nz), "flub_redistance_init: bad shape %dx%dx%d", nx, ny, nz);
    k_redistance_init<<<row_grid(nx, ny, nz), kRowThreads, 0, as_stream(stream)>>>(phi, out, nx, ny, nz, h,
                                                                                 set_boundary);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_redistance_sweep(float *phi, int nx, int ny, int nz, int incx, int incy, int incz, int odd, float h,
                          void *stream) {
    FLUB_REQUIRE(phi, "flub_redistance_sweep: NULL argument");
    FLUB_REQUIRE(rd_shape_ok(nx, ny, nz), "flub_redistance_sweep: bad shape %dx%dx%d", nx, ny, nz);
    FLUB_REQUIRE((incx == 1 || incx == -1) && (incy == 1 || incy == -1) && (incz == 1 || incz == -1),
                 "flub_redistance_sweep: increments must be +1 or -1");
    FLUB_REQUIRE(odd == 0 || odd == 1, "flub_redistance_sweep: odd must be 0 or 1");
    return launch_sweep(phi, nx, ny, nz, incx, incy, incz, odd, h, as_stream(stream));
}

int flub_redistance(const float *phi, float *phi_out, int nx, int ny, int nz, float h, int set_boundary, int n_rounds,
                    void *stream) {
    FLUB_REQUIRE(phi && phi_out, "flub_redistance: NULL argument");
    FLUB_REQUIRE(phi != phi_out, "flub_redistance: phi_out must not alias phi");
    FLUB_REQUIRE(rd_shape_ok(nx, ny, nz), "flub_redistance: bad shape %dx%dx%d", nx, ny, nz);
    FLUB_REQUIRE(n_rounds >= 0, "flub_redistance: n_rounds must be >= 0");
    cudaStream_t s = as_stream(stream);
    k_redistance_init<<<row_grid(nx, ny, nz), kRowThreads, 0, s>>>(phi, phi_out, nx, ny, nz, h, set_boundary);
    FLUB_CHECK_LAUNCH();
    for (int r = 0; r < n_rounds; r++)
        for (int d = 0; d < 8; d++)
            for (int odd = 0; odd < 2; odd++) {
                const int st = launch_sweep(phi_out, nx, ny, nz, kSweepDirs[d][0], kSweepDirs[d][1], kSweepDirs[d][2],
                                            odd, h, s);
                if (st != FLUB_OK) return st;
            }
    return FLUB_OK;
}

}  // extern "C"
