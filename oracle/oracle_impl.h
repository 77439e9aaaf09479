/*
 * CPU restatement of flub's pressure projection -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is included twice by flub_oracle.c, once with REAL=float (the FP32
 * mirror of the CUDA kernels, same operation order, no FMA contraction except
 * where written as fmaf) and once with REAL=double (the FP64 oracle).  FN(name)
 * appends the precision suffix.
 *
 * Tags follow the reference's int32 convention: 0 air (Dirichlet p = 0),
 * 1 fluid (unknown), 2 solid (Neumann).  Arrays are C-order [i][j][k], k fastest.
 *
 * Every routine cites the reference function it restates (paths relative to the
 * flub repository).
 */

#define IX(i, j, k) ((((int64_t)(i)) * ny + (j)) * (int64_t)nz + (k))

/* multigrid/mgpcg.py:118-142 neighbor_dot_tag.  The reference clamps the
 * neighbour index at the domain wall; the clamped neighbour is the cell itself,
 * whose term (x_c - x_c) is exactly 0, so an out-of-domain neighbour is simply
 * skipped here.  Terms are summed per axis (i, j, k), "+" neighbour first. */
static inline REAL FN(ndot)(const REAL *x, const int32_t *tag, int nx, int ny,
                            int nz, int i, int j, int k) {
    int64_t c = IX(i, j, k);
    if (tag[c] != 1) return (REAL)0;
    REAL xc = x[c];
    REAL ret = (REAL)0;
    int64_t nb;
    REAL tp, tm;
    /* axis i */
    tp = (REAL)0; tm = (REAL)0;
    if (i + 1 < nx) { nb = IX(i + 1, j, k); if (tag[nb] < 2) tp = (tag[nb] == 0 ? (REAL)0 : x[nb]) - xc; }
    if (i - 1 >= 0) { nb = IX(i - 1, j, k); if (tag[nb] < 2) tm = (tag[nb] == 0 ? (REAL)0 : x[nb]) - xc; }
    ret = ret + (tp + tm);
    /* axis j */
    tp = (REAL)0; tm = (REAL)0;
    if (j + 1 < ny) { nb = IX(i, j + 1, k); if (tag[nb] < 2) tp = (tag[nb] == 0 ? (REAL)0 : x[nb]) - xc; }
    if (j - 1 >= 0) { nb = IX(i, j - 1, k); if (tag[nb] < 2) tm = (tag[nb] == 0 ? (REAL)0 : x[nb]) - xc; }
    ret = ret + (tp + tm);
    /* axis k */
    tp = (REAL)0; tm = (REAL)0;
    if (k + 1 < nz) { nb = IX(i, j, k + 1); if (tag[nb] < 2) tp = (tag[nb] == 0 ? (REAL)0 : x[nb]) - xc; }
    if (k - 1 >= 0) { nb = IX(i, j, k - 1); if (tag[nb] < 2) tm = (tag[nb] == 0 ? (REAL)0 : x[nb]) - xc; }
    ret = ret + (tp + tm);
    return ret;
}

/* multigrid/mgpcg.py:51-58 _compute_divd with :144-160 neighbor_sum_tag:
 * number of in-domain non-solid neighbours of a fluid cell, 0 elsewhere. */
static inline int FN(divd)(const int32_t *tag, int nx, int ny, int nz, int i, int j, int k) {
    if (tag[IX(i, j, k)] != 1) return 0;
    int d = 0;
    if (i + 1 < nx && tag[IX(i + 1, j, k)] < 2) d++;
    if (i - 1 >= 0 && tag[IX(i - 1, j, k)] < 2) d++;
    if (j + 1 < ny && tag[IX(i, j + 1, k)] < 2) d++;
    if (j - 1 >= 0 && tag[IX(i, j - 1, k)] < 2) d++;
    if (k + 1 < nz && tag[IX(i, j, k + 1)] < 2) d++;
    if (k - 1 >= 0 && tag[IX(i, j, k - 1)] < 2) d++;
    return d;
}

/* multigrid/mgpcg.py:36-39 compute_Ap_mcadams: Ap = L p. */
void FN(oracle_matvec)(const REAL *p, const int32_t *tag, REAL *Ap, int nx, int ny, int nz) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                Ap[IX(i, j, k)] = FN(ndot)(p, tag, nx, ny, nz, i, j, k);
}

/* multigrid/mgpcg.py:72-86 _smooth_mcadams: one red-black half-sweep.
 * Phase 0 updates cells with (i+j+k) odd, phase 1 cells with (i+j+k) even
 * (launch index (i, j, k/2), k = 2*_k+1 when (i+j)&1 == phase). */
void FN(oracle_smooth)(REAL *z, const REAL *r, const int32_t *tag, int nx, int ny, int nz, int phase) {
    int par = 1 - phase;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = (par - ((i + j) & 1) + 2) & 1; k < nz; k += 2) {
                int64_t c = IX(i, j, k);
                int d = FN(divd)(tag, nx, ny, nz, i, j, k);
                if (d != 0) {
                    REAL lz = FN(ndot)(z, tag, nx, ny, nz, i, j, k);
                    z[c] = z[c] + (r[c] + lz) / (REAL)d;
                } else {
                    z[c] = (REAL)0;
                }
            }
}

/* multigrid/mgpcg.py:94-101 _restrict_mcadams, written as a gather: each coarse
 * cell sums r + L z over its 8 children in the fixed order (ii, jj, kk) with kk
 * fastest (the reference sums them with atomics in an unspecified order), and
 * is 0 where the coarse tag is not fluid. */
void FN(oracle_restrict)(const REAL *rf, const REAL *zf, const int32_t *tagf, REAL *rc,
                         const int32_t *tagc, int nxc, int nyc, int nzc) {
    int nx = 2 * nxc, ny = 2 * nyc, nz = 2 * nzc;
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nxc; I++)
        for (int J = 0; J < nyc; J++)
            for (int K = 0; K < nzc; K++) {
                int64_t cc = ((int64_t)I * nyc + J) * nzc + K;
                if (tagc[cc] != 1) { rc[cc] = (REAL)0; continue; }
                REAL s = (REAL)0;
                int first = 1;
                for (int ii = 0; ii < 2; ii++)
                    for (int jj = 0; jj < 2; jj++)
                        for (int kk = 0; kk < 2; kk++) {
                            int i = 2 * I + ii, j = 2 * J + jj, k = 2 * K + kk;
                            int64_t c = IX(i, j, k);
                            REAL v = rf[c] + FN(ndot)(zf, tagf, nx, ny, nz, i, j, k);
                            if (first) { s = v; first = 0; } else s = s + v;
                        }
                rc[cc] = s * (REAL)oracle_sched_rscale;
            }
}

/* multigrid/mgpcg.py:113-116 _prolongate: z_h += z_2h[I/2]. */
void FN(oracle_prolong)(REAL *zf, const REAL *zc, int nx, int ny, int nz) {
    int nyc = ny / 2, nzc = nz / 2;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                zf[IX(i, j, k)] = zf[IX(i, j, k)] + zc[((int64_t)(i / 2) * nyc + j / 2) * nzc + k / 2];
}

/* multigrid/mgpcg.py:296-349 apply_preconditioner (smoother "phases" /
 * "fraction"): z = M r over the level hierarchy.  rl[0]/zl[0] are the finest
 * level; rl[l], zl[l] for l >= 1 are scratch of shape dims >> l.  Smoothing
 * counts: 6 << l per side (pre_and_post_smoothing = 6), 6 at the bottom
 * (bottom_smoothing = 6, split 3 x (0,1) then 3 x (1,0)).  The schedule
 * globals (oracle_set_schedule, no reference counterpart) generalise these
 * counts and scale the restriction; their defaults are the reference's. */
void FN(oracle_vcycle)(REAL **rl, REAL **zl, int32_t **tagl, int levels, int nx, int ny, int nz) {
    int64_t n0 = (int64_t)nx * ny * nz;
    memset(zl[0], 0, (size_t)n0 * sizeof(REAL));
    for (int l = 0; l < levels - 1; l++) {
        int ax = nx >> l, ay = ny >> l, az = nz >> l;
        for (int it = 0; it < ORACLE_ITERS(l); it++) {
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 0);
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 1);
        }
        int64_t nc = (int64_t)(ax / 2) * (ay / 2) * (az / 2);
        memset(zl[l + 1], 0, (size_t)nc * sizeof(REAL));
        FN(oracle_restrict)(rl[l], zl[l], tagl[l], rl[l + 1], tagl[l + 1], ax / 2, ay / 2, az / 2);
    }
    if (oracle_bottom64 && sizeof(REAL) == sizeof(float)) {
        int l = levels - 1;
        oracle_bottom_fp64_f32((float *)zl[l], (const float *)rl[l], tagl[l], nx >> l, ny >> l, nz >> l);
    } else {
        int l = levels - 1;
        int ax = nx >> l, ay = ny >> l, az = nz >> l;
        for (int it = 0; it < oracle_sched_bottom; it++) {
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 0);
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 1);
        }
        for (int it = 0; it < oracle_sched_bottom; it++) {
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 1);
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 0);
        }
    }
    for (int l = levels - 2; l >= 0; l--) {
        int ax = nx >> l, ay = ny >> l, az = nz >> l;
        FN(oracle_prolong)(zl[l], zl[l + 1], ax, ay, az);
        for (int it = 0; it < ORACLE_ITERS(l); it++) {
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 1);
            FN(oracle_smooth)(zl[l], rl[l], tagl[l], ax, ay, az, 0);
        }
    }
}

/* Deterministic FP64 inner product: sequential within each i-plane, planes
 * summed in order (independent of the thread count).  Stands in for
 * warp.utils.array_inner (multigrid/mgpcg.py:5), which accumulates in FP32. */
double FN(oracle_dot)(const REAL *a, const REAL *b, int nx, int ny, int nz) {
    int64_t plane = (int64_t)ny * nz;
    double *part = (double *)malloc(sizeof(double) * (size_t)nx);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        double s = 0.0;
        const REAL *pa = a + (int64_t)i * plane, *pb = b + (int64_t)i * plane;
        for (int64_t q = 0; q < plane; q++) s += (double)pa[q] * (double)pb[q];
        part[i] = s;
    }
    double s = 0.0;
    for (int i = 0; i < nx; i++) s += part[i];
    free(part);
    return s;
}

/* multigrid/mgpcg.py:191-205 _mean/_sub (zero_centered, :270-274): subtract the
 * mean over fluid cells, zero the rest. */
void FN(oracle_zero_centered)(REAL *r, const int32_t *tag, int nx, int ny, int nz) {
    int64_t n = (int64_t)nx * ny * nz;
    double s = 0.0;
    int64_t cnt = 0;
    for (int64_t c = 0; c < n; c++)
        if (tag[c] == 1) { s += (double)r[c]; cnt++; }
    REAL mean = cnt > 0 ? (REAL)(s / (double)cnt) : (REAL)0;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; c++) r[c] = tag[c] == 1 ? r[c] - mean : (REAL)0;
}

/* multigrid/mgpcg.py:162-174 restrict_tag: coarse = 0 if any child is air,
 * else 1 if any child is fluid, else 2. */
void FN(oracle_restrict_tag)(const int32_t *tagf, int32_t *tagc, int nxc, int nyc, int nzc) {
    int ny = 2 * nyc, nz = 2 * nzc;
    for (int I = 0; I < nxc; I++)
        for (int J = 0; J < nyc; J++)
            for (int K = 0; K < nzc; K++) {
                int t = 2;
                for (int ii = 0; ii < 2; ii++)
                    for (int jj = 0; jj < 2; jj++)
                        for (int kk = 0; kk < 2; kk++) {
                            int tg = tagf[IX(2 * I + ii, 2 * J + jj, 2 * K + kk)];
                            if (tg == 0) t = 0;
                            else if (t > 0 && tg == 1) t = 1;
                        }
                tagc[((int64_t)I * nyc + J) * nzc + K] = t;
            }
}

static inline REAL FN(axpy_fma)(REAL a, REAL x, REAL y);

/* multigrid/mgpcg.py:378-462 MGPCG.solve with smoother "phases" (zero_center=0)
 * or "fraction" (zero_center=1).  On entry r holds the masked right-hand side
 * (init + mask_interior, :276-284, :464-465); x, p are overwritten.  Vectors are
 * REAL, inner products and the scalars alpha/beta are FP64 (the reference keeps
 * them in FP32).  x += a p, r -= a Ap and p = z + b p are single fused
 * multiply-adds with a, b rounded to REAL.  The first-call graph-capture quirk
 * of graph_precondition (:286-294, first preconditioner application is recorded
 * but not executed) is not reproduced.
 * Returns the iteration count as the reference prints it; *rtr_out gets the
 * final squared residual norm, *rtr0_out the initial one and *converged
 * whether rTr < tol was reached.  x0 (may be NULL) is an initial guess: then
 * r <- r - L x0 first and the tolerance stays relative to the x0 = 0 residual. */
int FN(oracle_pcg)(REAL *x, REAL *r0, int32_t **tagl, int levels, int nx, int ny, int nz,
                   int max_iters, double eps, double abs_tol, double rel_tol, int zero_center,
                   const REAL *x0, double *rtr_out, double *rtr0_out, int *converged, double *hist) {
    int64_t n = (int64_t)nx * ny * nz;
    REAL **rl = (REAL **)malloc(sizeof(REAL *) * (size_t)levels);
    REAL **zl = (REAL **)malloc(sizeof(REAL *) * (size_t)levels);
    rl[0] = r0;
    zl[0] = (REAL *)calloc((size_t)n, sizeof(REAL));
    for (int l = 1; l < levels; l++) {
        int64_t nl = (int64_t)(nx >> l) * (ny >> l) * (nz >> l);
        rl[l] = (REAL *)calloc((size_t)nl, sizeof(REAL));
        zl[l] = (REAL *)calloc((size_t)nl, sizeof(REAL));
    }
    REAL *p = (REAL *)calloc((size_t)n, sizeof(REAL));
    REAL *Ap = (REAL *)calloc((size_t)n, sizeof(REAL));
    REAL *z = zl[0];

    if (zero_center) FN(oracle_zero_centered)(r0, tagl[0], nx, ny, nz);
    double rTr0 = FN(oracle_dot)(r0, r0, nx, ny, nz);
    double tol = abs_tol > rTr0 * rel_tol ? abs_tol : rTr0 * rel_tol;
    if (x0) {
        FN(oracle_matvec)(x0, tagl[0], Ap, nx, ny, nz);
        for (int64_t c = 0; c < n; c++) { x[c] = x0[c]; r0[c] = r0[c] - Ap[c]; }
        if (zero_center) FN(oracle_zero_centered)(r0, tagl[0], nx, ny, nz);
    } else {
        memset(x, 0, (size_t)n * sizeof(REAL));
    }
    FN(oracle_vcycle)(rl, zl, tagl, levels, nx, ny, nz);
    memcpy(p, z, (size_t)n * sizeof(REAL));
    double old_zTr = FN(oracle_dot)(z, r0, nx, ny, nz);
    int it = 0, conv = 0;
    double rTr = rTr0;
    int cap = max_iters < 0 ? 100000 : max_iters;
    while (it < cap) {
        FN(oracle_matvec)(p, tagl[0], Ap, nx, ny, nz);
        double pAp = FN(oracle_dot)(p, Ap, nx, ny, nz);
        double alpha = old_zTr / (pAp + eps);
        REAL a = (REAL)alpha;
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < n; c++) r0[c] = FN(axpy_fma)(-a, Ap[c], r0[c]);
        if (zero_center) FN(oracle_zero_centered)(r0, tagl[0], nx, ny, nz);
        rTr = FN(oracle_dot)(r0, r0, nx, ny, nz);
        if (hist) hist[it] = rTr;
        if (rTr < tol) {
#pragma omp parallel for schedule(static)
            for (int64_t c = 0; c < n; c++) x[c] = FN(axpy_fma)(a, p[c], x[c]);
            conv = 1;
            break;
        }
        FN(oracle_vcycle)(rl, zl, tagl, levels, nx, ny, nz);
        double zTr = FN(oracle_dot)(z, r0, nx, ny, nz);
        double beta = zTr / (old_zTr + eps);
        old_zTr = zTr;
        REAL b = (REAL)beta;
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < n; c++) {
            x[c] = FN(axpy_fma)(a, p[c], x[c]);
            p[c] = FN(axpy_fma)(b, p[c], z[c]);
        }
        it++;
    }
    if (rtr_out) *rtr_out = rTr;
    if (rtr0_out) *rtr0_out = rTr0;
    if (converged) *converged = conv;
    for (int l = 1; l < levels; l++) { free(rl[l]); free(zl[l]); }
    free(zl[0]); free(rl); free(zl); free(p); free(Ap);
    return it;
}
