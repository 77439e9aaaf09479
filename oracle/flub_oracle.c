/*
 * flub_oracle -- CPU restatement of flub's pressure projection.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ as the parity checker, by
 * __graft_entry__.smoke() as the checker, and by bench.py as the timed CPU
 * baseline.  Never linked into or called by the product library.
 *
 * Parity status: the reference (pure Python + NVIDIA Warp) cannot be run on
 * these machines (warp is not installed and has no offline wheel), and the
 * reference ships no tests, fixtures or golden vectors for this path.  This
 * restatement is therefore "parity unpinned" against the reference's own
 * outputs; it is pinned instead against hand-derived known-answer vectors and
 * against an independent NumPy restatement (oracle/np_oracle.py) in tests/.
 *
 * Build: oracle/build.py (gcc -O3 -fopenmp -ffp-contract=off -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---------------- V-cycle schedule ----------------
 * No reference counterpart: the reference's counts (6 << l iterations per
 * side at level l, 3 + 3 at the bottom, restriction = plain sum) are the
 * defaults; oracle_set_schedule generalises them to check the library's
 * flub_mg_set_schedule. */
static int oracle_sched_nu = -1;
static int oracle_sched_bottom = 3;
static double oracle_sched_rscale = 1.0;
#define ORACLE_ITERS(l) (oracle_sched_nu < 0 ? (6 << (l)) : oracle_sched_nu)

void oracle_set_schedule(int nu, int bottom, double rscale) {
    oracle_sched_nu = nu;
    oracle_sched_bottom = bottom;
    oracle_sched_rscale = rscale;
}

/* FP64 bottom level for the FP32 V-cycle (no reference counterpart; the
 * library's flub_mg_set_bottom_precision(64)): the bottom's sweeps run on
 * doubles from z = 0 with the FP32 residual converted exactly, the result is
 * rounded to FP32 once.  Off by default (the reference smooths in FP32). */
static int oracle_bottom64 = 0;
void oracle_set_bottom_fp64(int on) { oracle_bottom64 = on; }
static void oracle_bottom_fp64_f32(float *z, const float *r, const int32_t *tag, int nx, int ny, int nz);

/* ---------------- precision-generic solver pieces ---------------- */
#define REAL float
#define FN(name) name##_f32
#include "oracle_impl.h"
static inline float axpy_fma_f32(float a, float x, float y) { return fmaf(a, x, y); }
#undef REAL
#undef FN

#define REAL double
#define FN(name) name##_f64
#include "oracle_impl.h"
static inline double axpy_fma_f64(double a, double x, double y) { return fma(a, x, y); }
#undef REAL
#undef FN

/* ---------------- geometry (FP32, as the reference computes it) ---------------- */

/* Primitive description, same layout as flub_prim in include/flub_gb300.h. */
typedef struct {
    int32_t geometry; /* 0 none, 1 box, 2 sphere, 3 box (rect), 4 "x", 5 mesh */
    float x[3];       /* centre */
    float q[4];       /* rotation quaternion (x, y, z, w) */
    float radius[3];  /* box half extents; sphere radius in radius[0] */
} oracle_prim;

/* Rotation of v by the conjugate of the unit quaternion q:
 * v (2w^2 - 1) - 2w (q_v x v) + 2 (q_v . v) q_v, evaluated left to right. */
static void quat_rotate_inv(const float q[4], const float v[3], float out[3]) {
    float w = q[3];
    float c = 2.0f * w * w - 1.0f;
    float d = 2.0f * ((q[0] * v[0] + q[1] * v[1]) + q[2] * v[2]);
    float cx = q[1] * v[2] - q[2] * v[1];
    float cy = q[2] * v[0] - q[0] * v[2];
    float cz = q[0] * v[1] - q[1] * v[0];
    float w2 = w * 2.0f;
    out[0] = (v[0] * c - cx * w2) + q[0] * d;
    out[1] = (v[1] * c - cy * w2) + q[1] * d;
    out[2] = (v[2] * c - cz * w2) + q[2] * d;
}

/* geometry.py:17-32 _sdf_cube. */
static float sdf_cube(const float p_in[3], const float radius[3], const float q[4]) {
    float p[3], m[3];
    quat_rotate_inv(q, p_in, p);
    for (int a = 0; a < 3; a++) m[a] = fmaxf(p[a], -p[a]) - radius[a];
    float mx = fmaxf(fmaxf(m[0], m[1]), m[2]);
    if (mx < 0.0f) return mx; /* -(min(-m)) */
    for (int a = 0; a < 3; a++) m[a] = fmaxf(m[a], 0.0f);
    return sqrtf((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]);
}

static void quat_mul(const float a[4], const float b[4], float out[4]) {
    /* Hamilton product, (x, y, z, w) storage */
    out[0] = ((a[3] * b[0] + b[3] * a[0]) + a[1] * b[2]) - a[2] * b[1];
    out[1] = ((a[3] * b[1] + b[3] * a[1]) + a[2] * b[0]) - a[0] * b[2];
    out[2] = ((a[3] * b[2] + b[3] * a[2]) + a[0] * b[1]) - a[1] * b[0];
    out[3] = a[3] * b[3] - ((a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]);
}

/* geometry.py:82-113 compute_sdf_atom_prims. */
static float sdf_atom_prims(float u, float v, float w, const oracle_prim *g) {
    float p[3] = {u - g->x[0], v - g->x[1], w - g->x[2]};
    switch (g->geometry) {
    case 1:
    case 3:
        return sdf_cube(p, g->radius, g->q);
    case 2:
        return sqrtf((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]) - g->radius[0];
    case 4: {
        const float h = 0.70710678118654752f; /* cos(pi/4) = sin(pi/4) */
        float zq[4] = {0.0f, 0.0f, h, h}, zi[4] = {0.0f, 0.0f, -h, h}, t[4], q2[4];
        quat_mul(zq, g->q, t);
        quat_mul(t, zi, q2);
        return fminf(sdf_cube(p, g->radius, g->q), sdf_cube(p, g->radius, q2));
    }
    case 5:
        return 2.0f;
    default:
        return 1.0f;
    }
}

/* geometry.py:225-239 precompute_grid_point_phi_prims + :148-169 sdf_argmin_prims. */
void oracle_phi_prims(float *phi, int nx, int ny, int nz, float h, float h0, const float stagger[3],
                      const oracle_prim *prims, int nprims) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                float u = (float)i * h, v = (float)j * h, w = (float)k * h;
                u = u + stagger[0] * h;
                v = v + stagger[1] * h;
                w = w + stagger[2] * h;
                float interior = 2.0f;
                for (int o = 0; o < nprims; o++) {
                    float s = sdf_atom_prims(u, v, w, &prims[o]);
                    if (s < fminf(h0, interior)) interior = s;
                }
                phi[IX(i, j, k)] = interior;
            }
}

/* geometry.py:335-344 _tag_dirichlet. */
void oracle_tag_dirichlet(const float *phi, int32_t *tag, int64_t n) {
    for (int64_t c = 0; c < n; c++) tag[c] = phi[c] > 0.0f ? 0 : 1;
}

/* geometry.py:390-397 _tag_neumann. */
void oracle_tag_neumann(const float *phi_rigid, int32_t *tag, int64_t n) {
    for (int64_t c = 0; c < n; c++)
        if (phi_rigid[c] < 0.0f) tag[c] = 2;
}

/* divergence.py:43-99 divergence_tag.  Boundary faces are 0 and a face whose
 * outer neighbour is solid takes the rigid velocity.  Per-axis extents are
 * used (the reference uses nx for all three axes, which only agrees on cubic
 * grids).  Sum order: vr - vl + vt - vb + vn - vf, left to right. */
void oracle_divergence(const float *u, const float *v, const float *w, const float *ur, const float *vr_,
                       const float *wr, const int32_t *tag, float *div, int nx, int ny, int nz) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                /* u: (nx+1, ny, nz), v: (nx, ny+1, nz), w: (nx, ny, nz+1) */
                int64_t uL = ((int64_t)i * ny + j) * nz + k, uR = ((int64_t)(i + 1) * ny + j) * nz + k;
                int64_t vB = ((int64_t)i * (ny + 1) + j) * nz + k, vT = ((int64_t)i * (ny + 1) + j + 1) * nz + k;
                int64_t wF = ((int64_t)i * ny + j) * (nz + 1) + k, wN = wF + 1;
                float fl = u[uL], fr = u[uR], fb = v[vB], ft = v[vT], ff = w[wF], fn = w[wN];
                if (i == 0) fl = 0.0f; else if (tag[IX(i - 1, j, k)] == 2) fl = ur[uL];
                if (i == nx - 1) fr = 0.0f; else if (tag[IX(i + 1, j, k)] == 2) fr = ur[uR];
                if (j == 0) fb = 0.0f; else if (tag[IX(i, j - 1, k)] == 2) fb = vr_[vB];
                if (j == ny - 1) ft = 0.0f; else if (tag[IX(i, j + 1, k)] == 2) ft = vr_[vT];
                if (k == 0) ff = 0.0f; else if (tag[IX(i, j, k - 1)] == 2) ff = wr[wF];
                if (k == nz - 1) fn = 0.0f; else if (tag[IX(i, j, k + 1)] == 2) fn = wr[wN];
                div[IX(i, j, k)] = ((((fr - fl) + ft) - fb) + fn) - ff;
            }
}

/* divergence.py:173-180 mask_with_tag. */
void oracle_mask_with_tag(float *div, const int32_t *tag, int64_t n) {
    for (int64_t c = 0; c < n; c++)
        if (tag[c] != 1) div[c] = 0.0f;
}

/* utils/util.py:162-165 scale_by_3d. */
void oracle_scale(float *q, float s, int64_t n) {
    for (int64_t c = 0; c < n; c++) q[c] = q[c] * s;
}

/* subtract_gradient.py:37-68 subtract_gradient_tag for axis d = 1, 2, 3 on the
 * face array uf of shape (nx+[d==1], ny+[d==2], nz+[d==3]). */
void oracle_subtract_gradient(float *uf, const float *urf, const float *p, const int32_t *tag, int nx, int ny,
                              int nz, int d) {
    int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    int nd = d == 1 ? nx : (d == 2 ? ny : nz);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < fx; i++)
        for (int j = 0; j < fy; j++)
            for (int k = 0; k < fz; k++) {
                int64_t f = ((int64_t)i * fy + j) * fz + k;
                int ii = d == 1 ? i : (d == 2 ? j : k);
                if (0 < ii && ii < nd) {
                    int il = i - (d == 1), jl = j - (d == 2), kl = k - (d == 3);
                    float pl = p[IX(il, jl, kl)], pr = p[IX(i, j, k)];
                    int tl = tag[IX(il, jl, kl)], tr = tag[IX(i, j, k)];
                    if (tl == 2 || tr == 2) uf[f] = urf[f];
                    else if (tl == 1 || tr == 1) uf[f] = uf[f] - (pr - pl);
                    else uf[f] = 0.0f;
                } else {
                    uf[f] = 0.0f;
                }
            }
}

/* ---------------- rigid face velocities and cut cells ---------------- */

/* rigid_coupling.py:51-70 precompute_solid_vel for the face array of axis d
 * (shape (fx, fy, fz)) with face owners owner (-1: none): the rigid velocity
 * v + omega x (pos - x) of the owner body at the face centre
 * pos = ((i, j, k) + stagger) * h0, component d-1, where i * h0 lies strictly
 * inside (0.01 h0, 1 - 0.01 h0) -- the reference tests the first index i for
 * every axis -- else 0.  Bodies: x, v, omega as n x 3 floats; an owner >= n
 * counts as none. */
void oracle_solid_vel(float *ur, const int32_t *owner, int fx, int fy, int fz, int d, float h0, const float *bx,
                      const float *bv, const float *bw, int n) {
    float st[3] = {0.5f, 0.5f, 0.5f};
    st[d - 1] = 0.0f;
    float eps = h0 * 0.01f;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < fx; i++)
        for (int j = 0; j < fy; j++)
            for (int k = 0; k < fz; k++) {
                int64_t f = ((int64_t)i * fy + j) * fz + k;
                int o = owner[f];
                float tmp = (float)i * h0;
                if (eps < tmp && tmp < 1.0f - eps && o >= 0 && o < n) {
                    float pos[3] = {((float)i + st[0]) * h0, ((float)j + st[1]) * h0, ((float)k + st[2]) * h0};
                    float p[3] = {pos[0] - bx[3 * o], pos[1] - bx[3 * o + 1], pos[2] - bx[3 * o + 2]};
                    const float *w = bw + 3 * o, *v = bv + 3 * o;
                    float c[3] = {w[1] * p[2] - w[2] * p[1], w[2] * p[0] - w[0] * p[2], w[0] * p[1] - w[1] * p[0]};
                    ur[f] = v[d - 1] + c[d - 1];
                } else {
                    ur[f] = 0.0f;
                }
            }
}

/* utils/util.py:169-187 fraction_edge, :190-219 fraction_triangle, :221-228
 * fraction_quad: the fraction of a face with sdf > 0 from its 4 corner values
 * and its centre value. */
static float fr_edge(float yl, float yr) {
    float ret;
    if (yl > 0.0f && yr > 0.0f) ret = 1.0f;
    else if (yl > 0.0f) ret = yl / (yl - yr);
    else if (yr > 0.0f) ret = yr / (yr - yl);
    else ret = 0.0f;
    if (ret < 0.1f) ret = 0.0f;
    else if (ret > 1.0f) ret = 1.0f;
    return ret;
}

static float fr_tri(float ya, float yb, float yc) {
    float fab = fr_edge(ya, yb), fbc = fr_edge(yb, yc), fca = fr_edge(yc, ya), ret;
    if (ya > 0.0f && yb > 0.0f && yc > 0.0f) ret = 1.0f;
    else if (ya > 0.0f && yb > 0.0f) ret = 1.0f - (1.0f - fca) * (1.0f - fbc);
    else if (ya > 0.0f && yc > 0.0f) ret = 1.0f - (1.0f - fab) * (1.0f - fbc);
    else if (yb > 0.0f && yc > 0.0f) ret = 1.0f - (1.0f - fab) * (1.0f - fca);
    else if (ya > 0.0f) ret = fca * fab;
    else if (yb > 0.0f) ret = fab * fbc;
    else if (yc > 0.0f) ret = fbc * fca;
    else ret = 0.0f;
    return ret < 0.0f ? 0.0f : (ret > 1.0f ? 1.0f : ret);
}

float oracle_fraction_quad(float ya, float yb, float yc, float yd, float yctr) {
    float f = fr_tri(ya, yb, yctr) + fr_tri(yb, yc, yctr) + fr_tri(yc, yd, yctr) + fr_tri(yd, ya, yctr);
    f = f * 0.25f;
    if (f < 0.1f) f = 0.0f;
    else if (f > 1.0f) f = 1.0f;
    return f;
}

/* geometry.py phi_to_fraction: face fractions of axis d in place; frac holds the
 * face-centre SDF on entry; phi is the SDF at the grid nodes, shape
 * (nx+1, ny+1, nz+1). */
void oracle_phi_to_fraction(const float *phi, float *frac, int nx, int ny, int nz, int d) {
    int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    int py = ny + 1, pz = nz + 1;
#define PN(a, b, c) phi[((int64_t)(a) * py + (b)) * pz + (c)]
#pragma omp parallel for schedule(static)
    for (int i = 0; i < fx; i++)
        for (int j = 0; j < fy; j++)
            for (int k = 0; k < fz; k++) {
                float ya = PN(i, j, k), yb, yc, yd;
                if (d == 1) { yb = PN(i, j + 1, k); yc = PN(i, j + 1, k + 1); yd = PN(i, j, k + 1); }
                else if (d == 2) { yb = PN(i + 1, j, k); yc = PN(i + 1, j, k + 1); yd = PN(i, j, k + 1); }
                else { yb = PN(i + 1, j, k); yc = PN(i + 1, j + 1, k); yd = PN(i, j + 1, k); }
                int64_t f = ((int64_t)i * fy + j) * fz + k;
                frac[f] = oracle_fraction_quad(ya, yb, yc, yd, frac[f]);
            }
#undef PN
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* divergence.py:4-42 divergence_fractional_3d: face-fraction weighted
 * divergence plus the rigid velocities on the solid parts of the faces. */
void oracle_divergence_fractional(const float *u, const float *v, const float *w, float *div, const float *fu,
                                  const float *fv, const float *fw, const float *ur, const float *vr, const float *wr,
                                  int nx, int ny, int nz) {
#define SU(a, q, i, j, k) a[((int64_t)clampi(i, 0, nx) * ny + clampi(j, 0, ny - 1)) * nz + clampi(k, 0, nz - 1)]
#define SV(a, q, i, j, k) a[((int64_t)clampi(i, 0, nx - 1) * (ny + 1) + clampi(j, 0, ny)) * nz + clampi(k, 0, nz - 1)]
#define SW(a, q, i, j, k) a[((int64_t)clampi(i, 0, nx - 1) * ny + clampi(j, 0, ny - 1)) * (nz + 1) + clampi(k, 0, nz)]
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                float vl = SU(u, 0, i, j, k), vr_ = SU(u, 0, i + 1, j, k);
                float vb = SV(v, 0, i, j, k), vt = SV(v, 0, i, j + 1, k);
                float vf = SW(w, 0, i, j, k), vn = SW(w, 0, i, j, k + 1);
                float l = SU(fu, 0, i, j, k), r = SU(fu, 0, i + 1, j, k);
                float b = SV(fv, 0, i, j, k), t = SV(fv, 0, i, j + 1, k);
                float f = SW(fw, 0, i, j, k), n = SW(fw, 0, i, j, k + 1);
                float vls = SU(ur, 0, i, j, k), vrs = SU(ur, 0, i + 1, j, k);
                float vbs = SV(vr, 0, i, j, k), vts = SV(vr, 0, i, j + 1, k);
                float vfs = SW(wr, 0, i, j, k), vns = SW(wr, 0, i, j, k + 1);
                float a = vr_ * r - vl * l + vt * t - vb * b + vn * n - vf * f;
                float s = (1.0f - r) * vrs - (1.0f - l) * vls + (1.0f - t) * vts - (1.0f - b) * vbs +
                          (1.0f - n) * vns - (1.0f - f) * vfs;
                div[IX(i, j, k)] = a + s;
            }
#undef SU
#undef SV
#undef SW
}

/* utils/util.py:404-412 fraction_of_fluid. */
static float frac_fluid(float p1, float p2) {
    if (p1 < 0.0f && p2 < 0.0f) return 1.0f;
    if (p1 >= 0.0f && p2 >= 0.0f) return 0.0f;
    return 1.0f - fmaxf(p1, p2) / fabsf(p1 - p2);
}

/* subtract_gradient.py:7-122 u/v/w_subtract_gradient_batty_3d on the face array
 * of axis d: ghost-fluid pressure gradient over the fluid fraction theta
 * (at least 0.01), the rigid velocity on faces of zero fraction, 0 on faces
 * between two air cells; on the domain-boundary face layers the face becomes 0
 * when lo <= 1e-5 or lo + index * h >= 1 - 1e-5 (lo: the domain's offset on
 * that axis), else it is left as it is. */
void oracle_subtract_gradient_batty(float *uf, const float *p, const float *fr, const float *phi, const float *ur,
                                    int nx, int ny, int nz, int d, float lo, float h) {
    const float eps = 1e-5f;
    int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    int gridn = (d == 1 ? fx : (d == 2 ? fy : fz)) - 1;
#define PC(a, i, j, k) a[((int64_t)clampi(i, 0, nx - 1) * ny + clampi(j, 0, ny - 1)) * nz + clampi(k, 0, nz - 1)]
#pragma omp parallel for schedule(static)
    for (int i = 0; i < fx; i++)
        for (int j = 0; j < fy; j++)
            for (int k = 0; k < fz; k++) {
                int64_t f = ((int64_t)i * fy + j) * fz + k;
                int ii = d == 1 ? i : (d == 2 ? j : k);
                if (0 < ii && ii < gridn) {
                    int il = i - (d == 1), jl = j - (d == 2), kl = k - (d == 3);
                    float ph = phi[IX(i, j, k)], pl = phi[IX(il, jl, kl)];
                    if (ph < 0.0f || pl < 0.0f) {
                        if (fr[f] == 0.0f) {
                            uf[f] = ur[f];
                        } else {
                            float plo = pl >= 0.0f ? 0.0f : PC(p, il, jl, kl);
                            float phi_ = ph >= 0.0f ? 0.0f : PC(p, i, j, k);
                            float theta = d == 3 ? frac_fluid(pl, ph) : frac_fluid(ph, pl);
                            theta = fmaxf(0.01f, theta);
                            uf[f] = uf[f] - (phi_ - plo) / theta;
                        }
                    } else {
                        uf[f] = 0.0f;
                    }
                } else if (lo <= eps || lo + (float)ii * h >= 1.0f - eps) {
                    uf[f] = 0.0f;
                }
            }
#undef PC
}

/* ---------------- velocity extrapolation ---------------- */

/* utils/util.py:423-437 set_unknown, launched over the cell grid (nx, ny, nz):
 * the face flag arrays tu (nx+1, ny, nz), tv (nx, ny+1, nz), tw (nx, ny, nz+1)
 * get 1 (unknown) where phi >= 0 and 0 (known) where phi < 0, at face index
 * (i, j, k) with i < nx, j < ny, k < nz; the last face layer of each array
 * keeps its previous flags. */
void oracle_set_unknown(const float *phi, int32_t *tu, int32_t *tv, int32_t *tw, int nx, int ny, int nz) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                int32_t v = phi[IX(i, j, k)] >= 0.0f ? 1 : 0;
                tu[((int64_t)i * ny + j) * nz + k] = v;
                tv[((int64_t)i * (ny + 1) + j) * nz + k] = v;
                tw[((int64_t)i * ny + j) * (nz + 1) + k] = v;
            }
}

/* extrapolate.py:8-30 extrapolate_3d on one face array q of shape (fx, fy, fz)
 * with flags unk: every face with flag 1 takes the mean of its in-bounds
 * neighbours (the 3x3x3 block, itself included) whose flag is 0, summed in
 * (ii, jj, kk) order from -1 to 1, kk fastest, and its flag becomes -1; with
 * no such neighbour the face becomes 0.  Only faces with flag 0 are read and
 * only faces with flag 1 are written, so the result does not depend on the
 * order the faces are visited in. */
void oracle_extrapolate_axis(float *q, int32_t *unk, int fx, int fy, int fz) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < fx; i++)
        for (int j = 0; j < fy; j++)
            for (int k = 0; k < fz; k++) {
                int64_t f = ((int64_t)i * fy + j) * fz + k;
                if (unk[f] != 1) continue;
                int n = 0;
                float s = 0.0f;
                for (int ii = -1; ii <= 1; ii++)
                    for (int jj = -1; jj <= 1; jj++)
                        for (int kk = -1; kk <= 1; kk++) {
                            int a = i + ii, b = j + jj, c = k + kk;
                            if (a < 0 || a >= fx || b < 0 || b >= fy || c < 0 || c >= fz) continue;
                            int64_t g = ((int64_t)a * fy + b) * fz + c;
                            if (unk[g] != 0) continue;
                            n++;
                            s = s + q[g];
                        }
                if (n > 0) {
                    q[f] = s / (float)n;
                    unk[f] = -1;
                } else {
                    q[f] = 0.0f;
                }
            }
}

/* extrapolate.py:32-36 flush_1_3d: flag -1 -> 1. */
void oracle_flush_unknown(int32_t *unk, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; c++)
        if (unk[c] == -1) unk[c] = 1;
}

/* ---------------- advection ----------------
 * FP32, every product and sum rounded on its own in the order the reference's
 * expressions give (this file is built with -ffp-contract=off).  Positions
 * are in grid units (cell i spans [i, i+1)); every sample clamps its index
 * to the array (utils/util.py:20-28 sample_3d). */

typedef struct {
    const float *q;
    int gx, gy, gz;
} adv_vol;

static inline int64_t adv_clamp64(int64_t v, int64_t hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

/* Indices are int64 so that an index +- 2 never overflows. */
static inline float adv_at(adv_vol V, int64_t u, int64_t v, int64_t w) {
    u = adv_clamp64(u, V.gx - 1);
    v = adv_clamp64(v, V.gy - 1);
    w = adv_clamp64(w, V.gz - 1);
    return V.q[(u * V.gy + v) * V.gz + w];
}

/* floor(x) as an int, saturating at the int range, NaN -> 0 (what a CUDA
 * float-to-int conversion gives), and the fraction x - floor(x) (equal to the
 * reference's x - float(int(floor(x))) wherever the int is exact). */
static inline int adv_ifloor(float x) {
    if (isnan(x)) return 0;
    float f = floorf(x);
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int)f;
}
static inline float adv_fract(float x) { return x - floorf(x); }

/* wp.lerp(a, b, t) = a * (1 - t) + b * t. */
static inline float adv_lerp(float a, float b, float t) { return a * (1.0f - t) + b * t; }

static inline float adv_min(float a, float b) { return a < b ? a : b; }
static inline float adv_max(float a, float b) { return a > b ? a : b; }

/* The eight corners (u0|u0+1, v0|v0+1, w0|w0+1) blended with fractions fa, fb,
 * fc: lerp(lerp(lerp(a,b,fa), lerp(c,d,fa), fb), lerp(lerp(e,f,fa),
 * lerp(g,h,fa), fb), fc), as utils/util.py:55-88 and :106-120 write it. */
static float adv_tri8(adv_vol V, int64_t u0, int64_t v0, int64_t w0, float fa, float fb, float fc) {
    float a = adv_at(V, u0, v0, w0), b = adv_at(V, u0 + 1, v0, w0);
    float c = adv_at(V, u0, v0 + 1, w0), d = adv_at(V, u0 + 1, v0 + 1, w0);
    float e = adv_at(V, u0, v0, w0 + 1), f = adv_at(V, u0 + 1, v0, w0 + 1);
    float g = adv_at(V, u0, v0 + 1, w0 + 1), h = adv_at(V, u0 + 1, v0 + 1, w0 + 1);
    return adv_lerp(adv_lerp(adv_lerp(a, b, fa), adv_lerp(c, d, fa), fb),
                    adv_lerp(adv_lerp(e, f, fa), adv_lerp(g, h, fa), fb), fc);
}

/* utils/util.py:34-88 sample_velocity_3d: the MAC velocity at p (u faces
 * sit at (i, j+0.5, k+0.5), v faces at (i+0.5, j, k+0.5), w faces at
 * (i+0.5, j+0.5, k)). */
static void adv_velocity(adv_vol U, adv_vol V, adv_vol W, const float p[3], float out[3]) {
    int iu = adv_ifloor(p[0]), iv = adv_ifloor(p[1]), iw = adv_ifloor(p[2]);
    float fu = adv_fract(p[0]), fv = adv_fract(p[1]), fw = adv_fract(p[2]);
    float s = p[0] - 0.5f, t = p[1] - 0.5f, r = p[2] - 0.5f;
    int is = adv_ifloor(s), it = adv_ifloor(t), ir = adv_ifloor(r);
    float fs = adv_fract(s), ft = adv_fract(t), fr = adv_fract(r);
    out[0] = adv_tri8(U, iu, it, ir, fu, ft, fr);
    out[1] = adv_tri8(V, is, iv, ir, fs, fv, fr);
    out[2] = adv_tri8(W, is, it, iw, fs, ft, fw);
}

/* advect.py:10-22 backtrace: three-stage Runge-Kutta (Ralston) from p over
 * -dt, positions in grid units (velocity / h). */
static void adv_backtrace(adv_vol U, adv_vol V, adv_vol W, float p[3], float dt, float h) {
    float v1[3], v2[3], v3[3], p1[3], p2[3];
    const float c1 = 0.5f * dt / h, c2 = 0.75f * dt / h, c3 = dt / h;
    const float k1 = 2.0f / 9.0f, k2 = 1.0f / 3.0f, k3 = 4.0f / 9.0f;
    adv_velocity(U, V, W, p, v1);
    for (int a = 0; a < 3; a++) p1[a] = p[a] - c1 * v1[a];
    adv_velocity(U, V, W, p1, v2);
    for (int a = 0; a < 3; a++) p2[a] = p[a] - c2 * v2[a];
    adv_velocity(U, V, W, p2, v3);
    for (int a = 0; a < 3; a++) p[a] = p[a] - c3 * ((k1 * v1[a] + k2 * v2[a]) + k3 * v3[a]);
}

/* utils/util.py:122-129 cubic: the cubic through (-1, a), (0, b), (1, c),
 * (2, d) at s; the weights are summed left to right (wp.dot). */
static float adv_cubic(float a, float b, float c, float d, float s) {
    const float m13 = -1.0f / 3.0f, k16 = 1.0f / 6.0f;
    float t0 = (m13 * s + 0.5f * s * s) - k16 * s * s * s;
    float t1 = (1.0f - s * s) + 0.5f * (s * s * s - s);
    float t2 = s + 0.5f * (s * s - s * s * s);
    float t3 = k16 * (s * s * s - s);
    return ((a * t0 + b * t1) + c * t2) + d * t3;
}

/* utils/util.py:148-160 _tricubic (with _bicubic :139-146 and _cubic
 * :131-137): cubic along the first axis innermost, then the second, then the
 * third, at (s, t, r) in index units. */
static float adv_tricubic(adv_vol Q, float s, float t, float r) {
    int64_t iu = adv_ifloor(s), iv = adv_ifloor(t), iw = adv_ifloor(r);
    float fu = adv_fract(s), fv = adv_fract(t), fw = adv_fract(r);
    float qw[4];
    for (int m = 0; m < 4; m++) {
        float qv[4];
        for (int n = 0; n < 4; n++) {
            int64_t b = iv + n - 1, c = iw + m - 1;
            qv[n] = adv_cubic(adv_at(Q, iu - 1, b, c), adv_at(Q, iu, b, c), adv_at(Q, iu + 1, b, c),
                              adv_at(Q, iu + 2, b, c), fu);
        }
        qw[m] = adv_cubic(qv[0], qv[1], qv[2], qv[3], fv);
    }
    return adv_cubic(qw[0], qw[1], qw[2], qw[3], fw);
}

/* utils/util.py:98-104 trilerp_stagger (the tricubic at p - stagger). */
static inline float adv_sample_stagger(adv_vol Q, const float p[3], const float st[3]) {
    return adv_tricubic(Q, p[0] - st[0], p[1] - st[1], p[2] - st[2]);
}

/* advect.py:103-122 sample_minmax: min and max of the eight values around
 * floor(p / h - stagger).  The reference passes h0 while p is already in
 * grid units, so the index is scaled by 1/h0 and clamps to the far corner of
 * the array for p >= 1; minmax_h = h0 reproduces that, 1 gives the cell
 * around p. */
static void adv_minmax(adv_vol Q, const float p[3], float mh, const float st[3], float *mn, float *mx) {
    int64_t a = adv_ifloor(p[0] / mh - st[0]), b = adv_ifloor(p[1] / mh - st[1]), c = adv_ifloor(p[2] / mh - st[2]);
    float v0 = adv_at(Q, a, b, c), v1 = adv_at(Q, a + 1, b, c), v2 = adv_at(Q, a, b + 1, c),
          v3 = adv_at(Q, a + 1, b + 1, c), v4 = adv_at(Q, a, b, c + 1), v5 = adv_at(Q, a + 1, b, c + 1),
          v6 = adv_at(Q, a, b + 1, c + 1), v7 = adv_at(Q, a + 1, b + 1, c + 1);
    float lo0 = adv_min(adv_min(adv_min(v0, v1), v2), v3), lo1 = adv_min(adv_min(adv_min(v4, v5), v6), v7);
    float hi0 = adv_max(adv_max(adv_max(v0, v1), v2), v3), hi1 = adv_max(adv_max(adv_max(v4, v5), v6), v7);
    *mn = adv_min(lo0, lo1);
    *mx = adv_max(hi0, hi1);
}

/* advect.py:57-101 _advect_mc_1 (stage 1), _advect_mc_2 (stage 2),
 * _advect_mc_3 (stage 3) on a field q of shape (qx, qy, qz) with stagger st,
 * advected by the MAC velocity (u, v, w) of the cell grid (nx, ny, nz);
 * stage 0 runs the three in order (advect.py:124-128 advect_mc). */
void oracle_advect_mc(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *q_in,
                      float *q_out, float *q_tmp, int qx, int qy, int qz, const float *st, float dt, float h,
                      float minmax_h, int stage) {
    if (stage == 0) {
        float *tmp = (float *)malloc(sizeof(float) * (size_t)qx * qy * qz);
        oracle_advect_mc(u, v, w, nx, ny, nz, q_in, q_out, tmp, qx, qy, qz, st, dt, h, minmax_h, 1);
        oracle_advect_mc(u, v, w, nx, ny, nz, q_in, q_out, tmp, qx, qy, qz, st, dt, h, minmax_h, 2);
        oracle_advect_mc(u, v, w, nx, ny, nz, q_in, q_out, tmp, qx, qy, qz, st, dt, h, minmax_h, 3);
        free(tmp);
        return;
    }
    adv_vol U = {u, nx + 1, ny, nz}, V = {v, nx, ny + 1, nz}, W = {w, nx, ny, nz + 1}, Q = {q_in, qx, qy, qz};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < qx; i++)
        for (int j = 0; j < qy; j++)
            for (int k = 0; k < qz; k++) {
                int64_t f = ((int64_t)i * qy + j) * qz + k;
                float p[3] = {(float)i + st[0], (float)j + st[1], (float)k + st[2]};
                if (stage == 2) {
                    adv_backtrace(U, V, W, p, -dt, h);
                    q_tmp[f] = adv_sample_stagger(Q, p, st);
                    continue;
                }
                adv_backtrace(U, V, W, p, dt, h);
                float q_sl = adv_sample_stagger(Q, p, st);
                if (stage == 1) {
                    q_out[f] = q_sl;
                    continue;
                }
                float q = q_out[f] + 0.5f * (q_in[f] - q_tmp[f]);
                float mn, mx;
                adv_minmax(Q, p, minmax_h, st, &mn, &mx);
                q_out[f] = (mn < q && q < mx) ? q : q_sl;
            }
}

/* advect.py:39-54 advect_phi: phi (px, py, pz) with stagger st traced back
 * by the velocity; the tricubic sample where the foot lies inside
 * [0, p*) on every axis, else `outside` (the reference writes h0). */
void oracle_advect_phi(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *phi,
                       float *phi_out, int px, int py, int pz, const float *st, float dt, float h, float outside) {
    adv_vol U = {u, nx + 1, ny, nz}, V = {v, nx, ny + 1, nz}, W = {w, nx, ny, nz + 1}, Q = {phi, px, py, pz};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < px; i++)
        for (int j = 0; j < py; j++)
            for (int k = 0; k < pz; k++) {
                float p[3] = {(float)i + st[0], (float)j + st[1], (float)k + st[2]};
                adv_backtrace(U, V, W, p, dt, h);
                int in = 0.0f <= p[0] && p[0] < (float)px && 0.0f <= p[1] && p[1] < (float)py && 0.0f <= p[2] &&
                         p[2] < (float)pz;
                phi_out[((int64_t)i * py + j) * pz + k] = in ? adv_sample_stagger(Q, p, st) : outside;
            }
}

/* advect.py:24-37 advect_simple_3d: a cell-centred q traced back from
 * (i+0.5, j+0.5, k+0.5), sampled trilinearly (utils/util.py:91-96 trilerp). */
void oracle_advect_simple(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *q,
                          float *q_out, int qx, int qy, int qz, float dt, float h) {
    adv_vol U = {u, nx + 1, ny, nz}, V = {v, nx, ny + 1, nz}, W = {w, nx, ny, nz + 1}, Q = {q, qx, qy, qz};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < qx; i++)
        for (int j = 0; j < qy; j++)
            for (int k = 0; k < qz; k++) {
                float p[3] = {(float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f};
                adv_backtrace(U, V, W, p, dt, h);
                float s = p[0] - 0.5f, t = p[1] - 0.5f, r = p[2] - 0.5f;
                q_out[((int64_t)i * qy + j) * qz + k] =
                    adv_tri8(Q, adv_ifloor(s), adv_ifloor(t), adv_ifloor(r), adv_fract(s), adv_fract(t), adv_fract(r));
            }
}

/* Single-point probes for known-answer tests. */
void oracle_sample_velocity(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *p,
                            float *out) {
    adv_vol U = {u, nx + 1, ny, nz}, V = {v, nx, ny + 1, nz}, W = {w, nx, ny, nz + 1};
    adv_velocity(U, V, W, p, out);
}

void oracle_backtrace(const float *u, const float *v, const float *w, int nx, int ny, int nz, float *p, float dt,
                      float h) {
    adv_vol U = {u, nx + 1, ny, nz}, V = {v, nx, ny + 1, nz}, W = {w, nx, ny, nz + 1};
    adv_backtrace(U, V, W, p, dt, h);
}

float oracle_tricubic(const float *q, int qx, int qy, int qz, float s, float t, float r) {
    adv_vol Q = {q, qx, qy, qz};
    return adv_tricubic(Q, s, t, r);
}

/* ---------------- level-set redistance ----------------
 * FP32 in the reference's operation order; x ** 2.0 is x * x; wp.min / wp.max
 * of two values are a < b ? a : b and a > b ? a : b; a vector's min / max
 * scans its components in order. */

static inline float rd_min(float a, float b) { return a < b ? a : b; }
static inline float rd_max(float a, float b) { return a > b ? a : b; }

/* redistance.py:66-119 _init_distance.  The reference rewrites phi in place
 * inside one launch, so a cell can read neighbours another thread has already
 * rewritten; here every cell reads the values from before the launch (phi) and
 * the results go to out.  Neighbours outside the grid read 0.5 h (the clamped
 * sample is replaced on each boundary side).  The neighbour test keeps the
 * reference's precedence: (!boundary && left) || right || bottom || ... */
void oracle_redistance_init(const float *phi, float *out, int nx, int ny, int nz, float h, int set_boundary) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const float hb = 0.5f * h;
                float pl = i > 0 ? phi[IX(i - 1, j, k)] : hb, pr = i < nx - 1 ? phi[IX(i + 1, j, k)] : hb;
                float pb = j > 0 ? phi[IX(i, j - 1, k)] : hb, pt = j < ny - 1 ? phi[IX(i, j + 1, k)] : hb;
                float pf = k > 0 ? phi[IX(i, j, k - 1)] : hb, pn = k < nz - 1 ? phi[IX(i, j, k + 1)] : hb;
                float pc = phi[IX(i, j, k)];
                int bnd = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1;
                float v = pc;
                if (bnd && !set_boundary) {
                    v = pc;
                } else if (pc > 0.0f) {
                    if ((!bnd && pl < 0.0f) || pr < 0.0f || pb < 0.0f || pt < 0.0f || pf < 0.0f || pn < 0.0f) {
                        float f[6] = {1.0f - frac_fluid(pc, pl), 1.0f - frac_fluid(pc, pr), 1.0f - frac_fluid(pc, pb),
                                      1.0f - frac_fluid(pc, pt), 1.0f - frac_fluid(pc, pf), 1.0f - frac_fluid(pc, pn)};
                        float m = f[0];
                        for (int a = 1; a < 6; a++) m = rd_min(m, f[a]);
                        v = h * m;
                    } else {
                        v = 2.0f;
                    }
                } else if (pc < 0.0f) {
                    if ((!bnd && pl > 0.0f) || pr > 0.0f || pb > 0.0f || pt > 0.0f || pf > 0.0f || pn > 0.0f) {
                        float f[6] = {frac_fluid(pc, pl), frac_fluid(pc, pr), frac_fluid(pc, pb),
                                      frac_fluid(pc, pt), frac_fluid(pc, pf), frac_fluid(pc, pn)};
                        float m = f[0];
                        for (int a = 1; a < 6; a++) m = rd_min(m, f[a]);
                        v = -h * m;
                    } else {
                        v = -2.0f;
                    }
                }
                out[IX(i, j, k)] = v;
            }
}

/* redistance.py:7-55 update at cell (i, j, k) for sweep direction
 * (incx, incy, incz): the upwind-sorted neighbour values, the 1-, 2- or
 * 3-neighbour Eikonal solution, kept if smaller than |phi|. */
static void rd_update(float *phi, int nx, int ny, int nz, int i, int j, int k, int incx, int incy, int incz, float h) {
    int bnd = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1;
    float pc = phi[IX(i, j, k)];
    if (!(fabsf(pc) > h) || bnd) return;
    float phii = phi[IX(i - incx, j, k)], phij = phi[IX(i, j - incy, k)], phik = phi[IX(i, j, k - incz)];
    float phiii = phi[IX(i + incx, j, k)], phijj = phi[IX(i, j + incy, k)], phikk = phi[IX(i, j, k + incz)];
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
    float phi0 = rd_min(rd_min(phii, phij), phik);
    float phi2 = rd_max(rd_max(phii, phij), phik);
    float phi1 = (((phii + phij) + phik) - phi0) - phi2;
    float d = phi0 + h;
    if (d > phi1) {
        float e = phi0 - phi1;
        d = 0.5f * ((phi0 + phi1) + sqrtf((2.0f * h) * h - e * e));
        if (d > phi2) {
            float s = (phi0 + phi1) + phi2;
            float term = s * s - 3.0f * (((phi0 * phi0 + phi1 * phi1) + phi2 * phi2) - h * h);
            d = (1.0f / 3.0f) * (((phi0 + phi1) + phi2) + sqrtf(rd_max(0.0f, term)));
        }
    }
    phi[IX(i, j, k)] = sgn * rd_min(d, fabsf(pc));
}

/* redistance.py:58-63 _sweep: the reference's thread (a, b, c) with
 * (a + b + c) % 2 == odd updates the cell (a, b, c) mirrored on every axis
 * whose increment is negative.  A cell reads only its six neighbours, all of
 * the other parity, so the cells of one launch can be visited in any order. */
void oracle_redistance_sweep(float *phi, int nx, int ny, int nz, int incx, int incy, int incz, int odd, float h) {
#pragma omp parallel for schedule(static)
    for (int a = 0; a < nx; a++)
        for (int b = 0; b < ny; b++)
            for (int c = 0; c < nz; c++) {
                if ((a + b + c) % 2 != odd) continue;
                int i = incx < 0 ? nx - 1 - a : a, j = incy < 0 ? ny - 1 - b : b, k = incz < 0 ? nz - 1 - c : c;
                rd_update(phi, nx, ny, nz, i, j, k, incx, incy, incz, h);
            }
}

/* redistance.py:121-136 redistance: _init_distance, then n_rounds times the
 * eight sweep directions, each as two launches (odd = 0, 1). */
static const int RD_DIRS[8][3] = {{1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1},
                                  {1, 1, 1},  {-1, 1, 1},  {-1, -1, 1},  {1, -1, 1}};

void oracle_redistance(float *phi, int nx, int ny, int nz, float h, int set_boundary, int n_rounds) {
    size_t n = (size_t)nx * ny * nz;
    float *tmp = (float *)malloc(n * sizeof(float));
    oracle_redistance_init(phi, tmp, nx, ny, nz, h, set_boundary);
    memcpy(phi, tmp, n * sizeof(float));
    free(tmp);
    for (int r = 0; r < n_rounds; r++)
        for (int s = 0; s < 8; s++)
            for (int odd = 0; odd < 2; odd++)
                oracle_redistance_sweep(phi, nx, ny, nz, RD_DIRS[s][0], RD_DIRS[s][1], RD_DIRS[s][2], odd, h);
}

/* multigrid/mgpcg.py:360-370 set_tags: coarse tag levels (restrict_tag). */
void oracle_tag_levels(int32_t **tagl, int levels, int nx, int ny, int nz) {
    for (int l = 0; l + 1 < levels; l++)
        oracle_restrict_tag_f32(tagl[l], tagl[l + 1], (nx >> l) / 2, (ny >> l) / 2, (nz >> l) / 2);
}

/* Level-hierarchy helpers so that Python can drive the V-cycle directly. */
/* FP64 bottom half-sweep (no reference counterpart; the red-black order of
 * oracle_smooth): the Gauss-Seidel update z_c + (r + L z) / d written as
 * (r + the fluid neighbours' z) / d, which it equals in exact arithmetic (the
 * z_c terms cancel).  The neighbours are added onto r in the order i+, i-,
 * j+, j-, k+, k-, each non-fluid or out-of-domain one adding +0.0; d counts
 * the in-domain non-solid neighbours (0: z = 0). */
static void oracle_bottom_half64(double *z, const double *r, const int32_t *tag, int nx, int ny, int nz, int phase) {
    int par = 1 - phase;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = (par - ((i + j) & 1) + 2) & 1; k < nz; k += 2) {
                int64_t c = IX(i, j, k);
                int d = divd_f64(tag, nx, ny, nz, i, j, k);
                if (d == 0) { z[c] = 0.0; continue; }
                double s = r[c];
                int64_t nb;
                nb = IX(i + 1, j, k); s = s + ((i + 1 < nx && tag[nb] == 1) ? z[nb] : 0.0);
                nb = IX(i - 1, j, k); s = s + ((i - 1 >= 0 && tag[nb] == 1) ? z[nb] : 0.0);
                nb = IX(i, j + 1, k); s = s + ((j + 1 < ny && tag[nb] == 1) ? z[nb] : 0.0);
                nb = IX(i, j - 1, k); s = s + ((j - 1 >= 0 && tag[nb] == 1) ? z[nb] : 0.0);
                nb = IX(i, j, k + 1); s = s + ((k + 1 < nz && tag[nb] == 1) ? z[nb] : 0.0);
                nb = IX(i, j, k - 1); s = s + ((k - 1 >= 0 && tag[nb] == 1) ? z[nb] : 0.0);
                z[c] = s / (double)d;
            }
}

static void oracle_bottom_fp64_f32(float *z, const float *r, const int32_t *tag, int nx, int ny, int nz) {
    int64_t n = (int64_t)nx * ny * nz;
    double *zd = (double *)calloc((size_t)n, sizeof(double));
    double *rd = (double *)malloc(sizeof(double) * (size_t)n);
    for (int64_t c = 0; c < n; c++) rd[c] = (double)r[c];
    for (int it = 0; it < oracle_sched_bottom; it++) {
        oracle_bottom_half64(zd, rd, tag, nx, ny, nz, 0);
        oracle_bottom_half64(zd, rd, tag, nx, ny, nz, 1);
    }
    for (int it = 0; it < oracle_sched_bottom; it++) {
        oracle_bottom_half64(zd, rd, tag, nx, ny, nz, 1);
        oracle_bottom_half64(zd, rd, tag, nx, ny, nz, 0);
    }
    for (int64_t c = 0; c < n; c++) z[c] = (float)zd[c];
    free(zd);
    free(rd);
}

void oracle_vcycle_levels_f32(float *r0, float *z0, int32_t **tagl, int levels, int nx, int ny, int nz) {
    float **rl = (float **)malloc(sizeof(float *) * (size_t)levels);
    float **zl = (float **)malloc(sizeof(float *) * (size_t)levels);
    rl[0] = r0;
    zl[0] = z0;
    for (int l = 1; l < levels; l++) {
        int64_t nl = (int64_t)(nx >> l) * (ny >> l) * (nz >> l);
        rl[l] = (float *)calloc((size_t)nl, sizeof(float));
        zl[l] = (float *)calloc((size_t)nl, sizeof(float));
    }
    oracle_vcycle_f32(rl, zl, tagl, levels, nx, ny, nz);
    for (int l = 1; l < levels; l++) { free(rl[l]); free(zl[l]); }
    free(rl); free(zl);
}

void oracle_vcycle_levels_f64(double *r0, double *z0, int32_t **tagl, int levels, int nx, int ny, int nz) {
    double **rl = (double **)malloc(sizeof(double *) * (size_t)levels);
    double **zl = (double **)malloc(sizeof(double *) * (size_t)levels);
    rl[0] = r0;
    zl[0] = z0;
    for (int l = 1; l < levels; l++) {
        int64_t nl = (int64_t)(nx >> l) * (ny >> l) * (nz >> l);
        rl[l] = (double *)calloc((size_t)nl, sizeof(double));
        zl[l] = (double *)calloc((size_t)nl, sizeof(double));
    }
    oracle_vcycle_f64(rl, zl, tagl, levels, nx, ny, nz);
    for (int l = 1; l < levels; l++) { free(rl[l]); free(zl[l]); }
    free(rl); free(zl);
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
