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

/* multigrid/mgpcg.py:360-370 set_tags: coarse tag levels (restrict_tag). */
void oracle_tag_levels(int32_t **tagl, int levels, int nx, int ny, int nz) {
    for (int l = 0; l + 1 < levels; l++)
        oracle_restrict_tag_f32(tagl[l], tagl[l + 1], (nx >> l) / 2, (ny >> l) / 2, (nz >> l) / 2);
}

/* Level-hierarchy helpers so that Python can drive the V-cycle directly. */
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
