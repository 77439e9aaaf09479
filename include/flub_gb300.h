/*
 * flub_gb300 -- C ABI of the GB300 (sm_103a) pressure projection.
 *
 * Drop-in replacement for the three stages of flub's projection path:
 * cell classification + divergence right-hand side, the MGPCG Poisson solve,
 * and the pressure-gradient velocity update.  Every entry point takes plain
 * device pointers (C-order [i][j][k] arrays, k fastest, FP32 fields, int32
 * tags with the reference's convention 0 air / 1 fluid / 2 solid), sizes and a
 * cudaStream_t passed as void*, and returns an int status (FLUB_OK == 0).
 * No entry point synchronises the stream unless its comment says so.
 *
 * Each declaration cites the reference code it replaces (paths inside the
 * flub repository, file:line).  In the reference these are Warp kernels
 * launched with wp.launch(kernel, dim, inputs=[...]) or methods of
 * multigrid/mgpcg.py:MGPCG; the Python module flub_gb300 exposes those same
 * names on top of this ABI.
 */
#ifndef FLUB_GB300_H
#define FLUB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define FLUB_OK 0
#define FLUB_ERR_INVALID_ARGUMENT 1 /* bad size, null pointer, unsupported shape */
#define FLUB_ERR_CUDA 2             /* a CUDA runtime call failed (see flub_last_error) */
#define FLUB_ERR_UNSUPPORTED 3      /* option not implemented (e.g. smoother "default") */
#define FLUB_ERR_OUT_OF_MEMORY 4
#define FLUB_ERR_BREAKDOWN 5        /* CG breakdown: non-finite alpha/beta or residual */
#define FLUB_ERR_TIMEOUT 6          /* a bounded device-side wait gave up */

/* Human-readable name of a status code. */
const char *flub_status_string(int status);
/* Detail of the last error raised on the calling host thread ("" if none). */
const char *flub_last_error(void);
/* ABI version (major * 10000 + minor * 100 + patch). */
int flub_version(void);

/* ---------------------------------------------------------------- classification */

/* Solid primitive, the fields of geometry.py:6-12 GeometryType3D that the
 * primitive SDF reads, with the body's position x and rotation q
 * (rigid_coupling.py x_pair.cur / theta_pair.cur).  geometry: 0 none, 1 box,
 * 2 sphere, 3 box, 4 "x" (two crossed boxes), 5 mesh (SDF 2.0: the mesh pass
 * is not part of this library). q is (x, y, z, w). */
typedef struct flub_prim {
    int32_t geometry;
    float x[3];
    float q[4];
    float radius[3];
} flub_prim;

#define FLUB_MAX_PRIMS 64

/* geometry.py:335-344 _tag_dirichlet: tag = (phi > 0) ? 0 : 1 over n cells. */
int flub_tag_dirichlet(const float *phi, int32_t *tag, int64_t n, void *stream);

/* geometry.py:225-239 precompute_grid_point_phi_prims (+ sdf_argmin_prims
 * :148-169, compute_sdf_atom_prims :82-113, _sdf_cube :17-32): phi at
 * ((i, j, k) + stagger) * h = min SDF over the primitives that is below h0,
 * else 2.0.  prims is a HOST array of nprims <= FLUB_MAX_PRIMS entries. */
int flub_phi_prims(float *phi, int nx, int ny, int nz, float h, float h0, float sx, float sy, float sz,
                   const flub_prim *prims, int nprims, void *stream);

/* geometry.py:390-397 _tag_neumann: tag = 2 where phi_rigid < 0. */
int flub_tag_neumann(const float *phi_rigid, int32_t *tag, int64_t n, void *stream);

/* The three above fused in one pass (the classification in
 * example_fluid.py:96-114 Dh() with water_3d.py:55-56): tag from the water
 * level set phi, then solid where the primitives' SDF at cell centres is < 0.
 * phi_rigid may be NULL; when given it receives the cell-centre solid SDF. */
int flub_classify(const float *phi, const flub_prim *prims, int nprims, int nx, int ny, int nz, float h,
                  float h0, int32_t *tag, float *phi_rigid, void *stream);

/* ---------------------------------------------------------------- divergence */

/* divergence.py:43-99 divergence_tag: div = (vr - vl) + (vt - vb) + (vn - vf)
 * per cell; domain-boundary faces count as 0, a face whose outer neighbour is
 * solid takes the rigid velocity.  u: (nx+1, ny, nz), v: (nx, ny+1, nz),
 * w: (nx, ny, nz+1); ur/vr/wr the rigid face velocities, same shapes. */
int flub_divergence_tag(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                        const float *wr, const int32_t *tag, float *div, int nx, int ny, int nz, void *stream);

/* divergence.py:173-180 mask_with_tag: div = 0 where tag != 1. */
int flub_mask_with_tag(float *div, const int32_t *tag, int64_t n, void *stream);

/* utils/util.py:162-165 scale_by_3d (and multigrid/mgpcg.py:9-12): q *= s. */
int flub_scale(float *q, float s, int64_t n, void *stream);

/* divergence_tag + mask_with_tag + scale_by_3d fused (the sequence of
 * example_fluid.py:84-93): div = (tag == 1) ? divergence * scale : 0. */
int flub_divergence_masked(const float *u, const float *v, const float *w, const float *ur, const float *vr,
                           const float *wr, const int32_t *tag, float *div, float scale, int nx, int ny, int nz,
                           void *stream);

/* ---------------------------------------------------------------- gradient */

/* subtract_gradient.py:37-68 subtract_gradient_tag for axis d (1 = u, 2 = v,
 * 3 = w) on the face array uf: solid on either side -> rigid velocity, else
 * fluid on either side -> uf -= p_hi - p_lo, else (and on domain-boundary
 * faces) 0. */
int flub_subtract_gradient_tag(float *uf, const float *urf, const float *p, const int32_t *tag, int nx, int ny,
                               int nz, int d, void *stream);

/* All three axes in one pass, with the pressure read as p * p_scale (the
 * scale_by_3d(p, 1/h0) of example_fluid.py:134 folded in). */
int flub_subtract_gradient(float *u, float *v, float *w, const float *ur, const float *vr, const float *wr,
                           const float *p, float p_scale, const int32_t *tag, int nx, int ny, int nz,
                           void *stream);

/* ---------------------------------------------------------------- rigid face velocities, cut cells */

/* rigid_coupling.py:51-70 precompute_solid_vel on the face array ur of axis d
 * (shape (nx+[d==1], ny+[d==2], nz+[d==3])) with face owners (int32, -1 none):
 * (v + omega x (pos - x))[d-1] of the owner body at the face centre
 * pos = ((i, j, k) + stagger) * h0 where 0.01 h0 < i * h0 < 1 - 0.01 h0 (the
 * reference tests the first index on every axis), else 0.  Bodies: HOST
 * arrays bx, bv, bw of nbodies x 3 floats (position, velocity, angular
 * velocity), nbodies <= 64; an owner >= nbodies counts as none. */
int flub_solid_vel(float *ur, const int32_t *owner, int nx, int ny, int nz, int d, float h0, const float *bx,
                   const float *bv, const float *bw, int nbodies, void *stream);

/* geometry.py phi_to_fraction with utils/util.py:169-228 fraction_edge /
 * fraction_triangle / fraction_quad: face fractions (sdf > 0 part) of axis d
 * in place on frac, which holds the face-centre SDF on entry; phi_nodes is
 * the SDF at the grid nodes, shape (nx+1, ny+1, nz+1). */
int flub_phi_to_fraction(const float *phi_nodes, float *frac, int nx, int ny, int nz, int d, void *stream);

/* divergence.py:4-42 divergence_fractional_3d: div (nx, ny, nz) = fraction-
 * weighted face velocities plus the rigid velocities on the solid parts. */
int flub_divergence_fractional(const float *u, const float *v, const float *w, float *div, const float *fu,
                               const float *fv, const float *fw, const float *ur, const float *vr, const float *wr,
                               int nx, int ny, int nz, void *stream);

/* subtract_gradient.py:7-122 u/v/w_subtract_gradient_batty_3d on the face
 * array uf of axis d: ghost-fluid pressure gradient divided by the fluid
 * fraction theta >= 0.01 of the face (phi: cell-centre level set), the rigid
 * velocity where the face fraction frac is 0, 0 between two air cells; the
 * domain-boundary face layers become 0 where lo <= 1e-5 or
 * lo + index * h >= 1 - 1e-5 (lo: the domain's offset on axis d). */
int flub_subtract_gradient_batty(float *uf, const float *p, const float *frac, const float *phi, const float *ur,
                                 int nx, int ny, int nz, int d, float lo, float h, void *stream);

/* ---------------------------------------------------------------- velocity extrapolation */

/* utils/util.py:423-437 set_unknown over the cell grid: the face flag arrays
 * tu (nx+1, ny, nz), tv (nx, ny+1, nz), tw (nx, ny, nz+1) get 1 where
 * phi >= 0 and 0 where phi < 0 at face index (i, j, k), i < nx, j < ny,
 * k < nz (the last face layer of each array keeps its flags, as in the
 * reference). */
int flub_set_unknown(const float *phi, int32_t *tu, int32_t *tv, int32_t *tw, int nx, int ny, int nz, void *stream);

/* extrapolate.py:8-30 extrapolate_3d on axis d of the face array q with flags
 * unk (same shape): every face with flag 1 takes the mean of its in-bounds
 * 3x3x3 neighbours with flag 0, summed in (ii, jj, kk) order, and its flag
 * becomes -1; with no such neighbour the face becomes 0. */
int flub_extrapolate_axis(float *q, int32_t *unk, int nx, int ny, int nz, int d, void *stream);

/* extrapolate.py:32-36 flush_1_3d: flags -1 -> 1 over n entries. */
int flub_flush_unknown(int32_t *unk, int64_t n, void *stream);

/* water_3d.py:70-73 extrapolate: set_unknown (skipped when phi is NULL), then
 * n_passes of extrapolate_by_1 (extrapolate.py:39-47) on the three axes.  Each
 * pass leaves the flags as the reference's flush does (extrapolated faces
 * back to 1), so the faces extrapolated and their values are the reference's
 * pass for pass. */
int flub_extrapolate(float *u, float *v, float *w, int32_t *tu, int32_t *tv, int32_t *tw, const float *phi, int nx,
                     int ny, int nz, int n_passes, void *stream);

/* ---------------------------------------------------------------- advection */

/* Velocity (u, v, w) below: MAC face arrays of the cell grid (nx, ny, nz),
 * shapes (nx+1, ny, nz), (nx, ny+1, nz), (nx, ny, nz+1).  Positions are in grid
 * units, samples clamp their indices to the array (utils/util.py:20-28).
 * Element counts must stay below 2^31. */

/* advect.py:57-101 _advect_mc_1 (stage 1: q_out = the tricubic sample of
 * q_in at the RK3 foot of the trace over dt), _advect_mc_2 (stage 2: q_tmp =
 * the sample traced over -dt), _advect_mc_3 (stage 3: q_out += (q_in - q_tmp)
 * / 2, replaced by the stage-1 value unless strictly inside the min/max of
 * sample_minmax, :103-122), or stage 0: all three in one pass
 * (advect.py:124-128 advect_mc; q_tmp may be NULL).  q_in has shape
 * (qx, qy, qz) and stagger (sx, sy, sz).  minmax_h: the divisor of
 * sample_minmax's position (the reference passes h0, as h; 1 centres the
 * bounds on the foot of the trace). */
int flub_advect_mc(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *q_in,
                   float *q_out, float *q_tmp, int qx, int qy, int qz, float sx, float sy, float sz, float dt, float h,
                   float minmax_h, int stage, void *stream);

/* advect.py:130-133 advect_uv_mc: the three face arrays advected by
 * themselves into (u_out, v_out, w_out), each by advect_mc. */
int flub_advect_velocity_mc(const float *u, const float *v, const float *w, float *u_out, float *v_out, float *w_out,
                            int nx, int ny, int nz, float dt, float h, float minmax_h, void *stream);

/* advect.py:39-54 advect_phi: phi (px, py, pz) with stagger (sx, sy, sz)
 * traced back over dt; the tricubic sample where the foot lies in
 * [0, extent) on every axis, else `outside` (the reference: h0). */
int flub_advect_phi(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *phi,
                    float *phi_out, int px, int py, int pz, float sx, float sy, float sz, float dt, float h,
                    float outside, void *stream);

/* advect.py:24-37 advect_simple_3d: cell-centred q traced back from the cell
 * centre, sampled trilinearly (utils/util.py:91-96 trilerp). */
int flub_advect_simple(const float *u, const float *v, const float *w, int nx, int ny, int nz, const float *q,
                       float *q_out, int qx, int qy, int qz, float dt, float h, void *stream);

/* ---------------------------------------------------------------- redistance */

/* redistance.py:66-119 _init_distance on phi (nx, ny, nz) into out: cells
 * next to a sign change get +-h times the smallest face fraction
 * (utils/util.py:403-412), other cells +-2; boundary cells keep phi unless
 * set_boundary.  Every cell reads the values from before the call (the
 * reference rewrites phi in place inside one launch, a data race). */
int flub_redistance_init(const float *phi, float *out, int nx, int ny, int nz, float h, int set_boundary,
                         void *stream);

/* redistance.py:58-63 _sweep(phi, incx, incy, incz, odd, h), in place: one
 * red-black half of a fast sweep in direction (incx, incy, incz) = +-1. */
int flub_redistance_sweep(float *phi, int nx, int ny, int nz, int incx, int incy, int incz, int odd, float h,
                          void *stream);

/* redistance.py:125-136 redistance: _init_distance from phi into phi_out,
 * then n_rounds (the reference: 2) rounds of the eight sweep directions on
 * phi_out. */
int flub_redistance(const float *phi, float *phi_out, int nx, int ny, int nz, float h, int set_boundary, int n_rounds,
                    void *stream);

/* ---------------------------------------------------------------- MGPCG */

/* multigrid/mgpcg.py:234-490 class MGPCG.  One handle = one level hierarchy
 * (shape // 2**l for l < levels) plus the CG vectors; not thread-safe; all
 * calls on a handle must use the same device.  Solves run entirely on the GPU
 * as one CUDA graph (a while-loop conditional node around one CG iteration);
 * the host reads back only the final status. */
typedef struct flub_mg flub_mg;

#define FLUB_SMOOTHER_PHASES 1   /* tagged red-black smoother, no mean removal (water_3d.py:66) */
#define FLUB_SMOOTHER_FRACTION 2 /* tagged smoother + zero_centered mean removal (example_fluid.py:43-49) */

#define FLUB_PRECISION_FP32 0    /* every vector FP32, inner products FP64 */
#define FLUB_PRECISION_MIXED 1   /* V-cycle levels stored in 16-bit floats, flexible CG */

typedef struct flub_solve_info {
    int iterations; /* as printed by the reference ("finished with N iterations") */
    int converged;  /* 1 if rTr < max(abs_tol, rel_tol * rTr0) was reached */
    int status;     /* FLUB_OK or FLUB_ERR_BREAKDOWN */
    int reserved;
    double rtr0;    /* initial squared residual norm (x0 = 0 residual) */
    double rtr;     /* final squared residual norm */
    double tol;     /* the squared-norm tolerance used */
    double x0_scale; /* scale applied to the initial guess: 0 none, 1 flub_mg_set_x0,
                        gamma for flub_mg_set_x0_scaled */
} flub_solve_info;

/* Bytes of device workspace a handle of this shape needs. */
size_t flub_mg_workspace_bytes(int nx, int ny, int nz, int levels, int precision);

/* multigrid/mgpcg.py:235-268 MGPCG.__init__(dim=3, shape, n_mg_levels, real).
 * Every dimension must be divisible by 2**(levels-1) and nz >> (levels-1)
 * must be even.  workspace: caller-owned device memory of
 * flub_mg_workspace_bytes(...) bytes (256-byte aligned), or NULL to let the
 * handle cudaMalloc its own. */
int flub_mg_create(int nx, int ny, int nz, int levels, int precision, void *workspace, size_t workspace_bytes,
                   flub_mg **out);
int flub_mg_destroy(flub_mg *mg);

/* multigrid/mgpcg.py:360-370 set_tags: copy the int32 tags, build the coarse
 * levels (restrict_tag :162-174) and the stencil diagonals. */
int flub_mg_set_tags(flub_mg *mg, const int32_t *tag, void *stream);

/* multigrid/mgpcg.py:276-284 init: x = p = 0, r0 = k * rhs. */
int flub_mg_init(flub_mg *mg, const float *rhs, float k, void *stream);

/* multigrid/mgpcg.py:464-465, :492-499 mask_interior: r0 = 0 where tag != 1. */
int flub_mg_mask_interior(flub_mg *mg, void *stream);

/* Optional initial guess (no reference counterpart: the reference always
 * starts from x = 0, mgpcg.py:282).  Call after init/mask_interior; the next
 * solve starts from x0 with r = r0 - L x0 and keeps its tolerance relative to
 * the x0 = 0 residual, so a guess can only change the iteration count. */
int flub_mg_set_x0(flub_mg *mg, const float *x0, void *stream);

/* multigrid/mgpcg.py:378-462 solve(max_iters, eps, abs_tol, rel_tol, verbose,
 * smoother).  max_iters = -1 means "no limit" (capped at 100000).  If info is
 * non-NULL the call synchronises the stream and fills it; with info == NULL
 * the solve is only enqueued (read the result later with flub_mg_get_info). */
int flub_mg_solve(flub_mg *mg, int max_iters, double eps, double abs_tol, double rel_tol, int smoother,
                  void *stream, flub_solve_info *info);

/* Synchronise the stream and read the outcome of the last solve. */
int flub_mg_get_info(flub_mg *mg, void *stream, flub_solve_info *info);

/* Squared residual norm after each iteration of the last solve (the
 * reference's verbose print, mgpcg.py:430-431).  Synchronises; returns the
 * number of entries written (<= max_n) in *n_out. */
int flub_mg_residual_history(flub_mg *mg, void *stream, double *out, int max_n, int *n_out);

/* Device pointers of the solution x (MGPCG.x) and of the level-0 residual r. */
float *flub_mg_x(flub_mg *mg);
float *flub_mg_r(flub_mg *mg);

/* x * scale into out (the wp.copy + scale_by_3d of water_3d.py:67-68). */
int flub_mg_get_x(flub_mg *mg, float *out, float scale, void *stream);

/* multigrid/mgpcg.py:296-349 apply_preconditioner: z = M r (one V-cycle).
 * Uses the handle's level hierarchy; r and z are N-cell device arrays. */
int flub_mg_apply_preconditioner(flub_mg *mg, const float *r, float *z, void *stream);

/* multigrid/mgpcg.py:36-39 compute_Ap_mcadams: Ap = L p with the level-0 tags. */
int flub_mg_matvec(flub_mg *mg, const float *p, float *Ap, void *stream);

/* multigrid/mgpcg.py:72-86 _smooth_mcadams: one red-black half-sweep (phase 0
 * updates (i+j+k)-odd cells, phase 1 even ones) on level `level` of the
 * handle's hierarchy, in place on that level's z with its r (level 0: the CG
 * vectors z and r).  The same kernel the V-cycle launches. */
int flub_mg_smooth(flub_mg *mg, int level, int phase, void *stream);

/* One red-black iteration (phase, then 1 - phase) on a level: the TMA-tiled
 * kernel where the level has tiles (out of place, between the level's
 * correction buffer and its spare, in alternate directions on successive
 * calls), else two half-sweeps in place.  *tiled (if not NULL) tells which
 * ran.  For timing and profiling. */
int flub_mg_smooth_iteration(flub_mg *mg, int level, int phase, int *tiled, void *stream);

/* Allocation-free V-cycle.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory themselves -- a plugin whose host
 * application owns every device allocation and forbids cudaMalloc in its frame
 * loop, or a real-time caller that cannot pay for cudaMalloc's implicit
 * synchronisation.  Always runs the reference's V-cycle schedule with FP32
 * level storage: it computes z = M r exactly as flub_mg_set_tags(tag) followed
 * by flub_mg_apply_preconditioner(r, z) would on an FP32 handle left at the
 * default schedule (same kernels, same results), but keeps the level
 * hierarchy in a 2 MiB array compiled into the library (resident on every
 * device that loads it, until the process exits) and allocates nothing.
 * Limits: nx * ny * nz <= FLUB_NOALLOC_MAX_CELLS, plus the shape rules of
 * flub_mg_create; larger grids are rejected with FLUB_ERR_INVALID_ARGUMENT.
 * The first call on each device looks up the array's device address and
 * keeps it for the life of the process; make that first call before any
 * stream capture, and do not call this entry point again on a device after
 * cudaDeviceReset (the kept address belongs to the context that was reset).
 * Every call shares the one array: calls that can overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller. */
#define FLUB_NOALLOC_MAX_CELLS 262144 /* 64^3 */
int flub_vcycle_noalloc(const int32_t *tag, const float *r, float *z, int nx, int ny, int nz, int levels,
                        void *stream);

/* V-cycle schedule of the handle's preconditioner (no reference counterpart;
 * the default is the reference's, mgpcg.py:296-349: smooth_iters = -1, i.e.
 * 6 << l red-black iterations per side at level l, bottom_iters = 3,
 * restrict_scale = 1).  smooth_iters = 1..64 runs that many iterations per
 * side at every level; bottom_iters (1..64) iterations of each bottom order;
 * the restriction multiplies its sum of 8 children by restrict_scale (0, 1].
 * With the unscaled 7-point operator on every level the sum of 8 children
 * over-corrects smooth errors about twice (the coarse operator is 4x the fine
 * one, the 8-child sum 8x): restrict_scale = 0.5 removes that, and a light
 * schedule (e.g. 2 iterations per side, 8 at the bottom) then converges in
 * fewer CG iterations at a fraction of the reference cycle's cost.  The solve
 * still stops at the same tolerance.  Synchronises the device when the
 * schedule changes (the captured solve graphs are rebuilt). */
int flub_mg_set_schedule(flub_mg *mg, int smooth_iters, int bottom_iters, float restrict_scale);

/* Arithmetic of the bottom level's smoothing (no reference counterpart: the
 * reference smooths its coarsest level in FP32, multigrid/mgpcg.py:319-336):
 * bits = 32, or 64 -- the bottom's red-black sweeps in FP64 on the FP32
 * restricted residual, the result rounded to FP32 once for the prolongation.
 * FP64 needs the bottom inside the one-block tail of the coarse-level kernels
 * (FLUB_ERR_UNSUPPORTED otherwise).  Handles created with
 * FLUB_PRECISION_MIXED start at 64, FP32 handles at 32 (the reference's
 * arithmetic).  Synchronises the device when the setting changes (the
 * captured solve graphs are rebuilt). */
int flub_mg_set_bottom_precision(flub_mg *mg, int bits);
int flub_mg_get_bottom_precision(flub_mg *mg, int *bits);

/* Warm start scaled on the device (no reference counterpart): x0 = gamma d
 * with gamma = (d . b) / (d . L d) over fluid cells, b the current right-hand
 * side (flub_mg_init + flub_mg_mask_interior), L the solver's operator --
 * the multiple of d closest to the solution in the energy norm, so the guess
 * is never worse than x0 = 0 in that norm.  Used by the next flub_mg_solve
 * only; gamma is reported in flub_solve_info.x0_scale.  No synchronisation. */
int flub_mg_set_x0_scaled(flub_mg *mg, const float *d, void *stream);

/* Extents of level l of the hierarchy (shape >> l). */
int flub_mg_level_shape(flub_mg *mg, int level, int *nx, int *ny, int *nz);
/* Cell tags of level l (the reference's convention, 0 air / 1 fluid /
 * 2 solid; levels >= 1 follow multigrid/mgpcg.py:162-174 restrict_tag), as set
 * by the last flub_mg_set_tags. */
int flub_mg_level_tags(flub_mg *mg, int level, int32_t *tag, void *stream);
/* coarse (level l) = sum of the 8 children in fine (level l - 1), 0 at coarse
 * cells that are not fluid: the V-cycle's restriction of a residual. */
int flub_mg_restrict_vector(flub_mg *mg, int level, const float *fine, float *coarse, void *stream);
/* fine (level l - 1) = cell-centred trilinear interpolation of coarse (level
 * l) at fine fluid cells, 0 elsewhere; coarse air cells count as 0, solid and
 * outside cells are left out with the weights renormalised. */
int flub_mg_prolong_vector(flub_mg *mg, int level, const float *coarse, float *fine, void *stream);

/* Solver kernels executed on the device inside solve graphs by this handle
 * since it was created (each kernel node counts once per execution).
 * Synchronises the stream. */
int flub_mg_kernels_executed(flub_mg *mg, void *stream, int64_t *out);

/* Kernels this library launched directly from the host in this process since
 * the counter was last reset (kernels inside solve graphs are not included:
 * see flub_mg_kernels_executed). */
int64_t flub_launch_count(void);
void flub_reset_launch_count(void);

/* ------------------------------------------------------------------------
 * Learned warm start: a small 3D U-Net whose output is CG's initial guess
 * (flub_mg_set_x0).  No counterpart in the reference (it always starts CG
 * from x = 0); these entry points exist for the network's forward pass,
 * backward pass and optimiser, which run on the GPU.
 *
 * Activations are channels-last BF16 [B][X][Y][Z][C] (C = 16, 32 or 64);
 * convolution weights are BF16 [27][Cout][Cin] with tap index
 * (dx+1)*9 + (dy+1)*3 + (dz+1); parameters, gradients and optimiser state are
 * FP32.  Activation and weight pointers must be 16-byte aligned.
 * ---------------------------------------------------------------------- */

/* y = [relu](conv3x3x3(x0, w0) + conv3x3x3(x1, w1) + bias), zero padding.
 * x1 / w1 optional (NULL, cin1 = 0): a second source accumulated into the same
 * output (a decoder's skip connection, so the concatenation is never formed).
 * bias may be NULL.  tcgen05 implicit GEMM with FP32 accumulation.  Shape
 * rules: NZ divides 128 or is a multiple of 128; NY a multiple of 128 / NZ
 * (when NZ < 128).  The data gradient is the same call on dy with the
 * flipped, transposed weights that flub_adam writes. */
int flub_conv3d_bf16(const void *x0, int cin0, const void *w0, const void *x1, int cin1, const void *w1,
                     const float *bias, void *y, int cout, int B, int NX, int NY, int NZ, int relu, void *stream);
/* Weight and bias gradients of one source of flub_conv3d_bf16, accumulated:
 * dw[27][cout][cin] += sum_v dy[v][co] x[v + tap][ci]; db[cout] += sum dy
 * (db may be NULL, e.g. for the second source of a two-source convolution).
 * tcgen05 GEMM over the voxels; same shape rules as flub_conv3d_bf16.
 * Accumulates with float atomics: the summation order is not fixed. */
int flub_conv3d_wgrad(const void *x, int cin, const void *dy, int cout, float *dw, float *db, int B, int NX, int NY,
                      int NZ, void *stream);
/* Non-zero in *out if a convolution kernel gave up on a bounded wait since the
 * last reset (its output is then incomplete).  Synchronises. */
int flub_conv_error(int *out, int reset);

/* Network input (16 channels): div / rms(div over fluid), fluid mask, solid
 * mask, zeros; tag is the reference's (0 air, 1 fluid, 2 solid) per sample of
 * ncell cells.  inv_scale[b] = 1 / rms (1 without fluid).  work: device
 * scratch of FLUB_UNET_INPUT_WORK(B) doubles. */
#define FLUB_UNET_INPUT_WORK(B) (2 * 152 * (B))
int flub_unet_input(const float *div, const int32_t *tag, int B, int64_t ncell, float *inv_scale, double *work,
                    void *out, void *stream);
/* 2x average pool and its gradient (dx = dy / 8, optionally added to dx);
 * NX, NY, NZ are the fine extents. */
int flub_pool2_bf16(const void *x, void *y, int B, int NX, int NY, int NZ, int C, void *stream);
int flub_pool2_bwd_bf16(const void *dy, void *dx, int B, int NX, int NY, int NZ, int C, int accumulate, void *stream);
/* Nearest 2x upsample and its gradient (sum over the 8 fine cells); NX, NY,
 * NZ are the fine extents. */
int flub_up2_bf16(const void *x, void *y, int B, int NX, int NY, int NZ, int C, void *stream);
int flub_up2_bwd_bf16(const void *dy, void *dx, int B, int NX, int NY, int NZ, int C, void *stream);
/* dx = dy where y > 0 else 0 (dx may alias dy). */
int flub_relu_bwd_bf16(const void *dy, const void *y, void *dx, int64_t n, void *stream);
/* 1x1x1 output head over 16 channels: out = x . w + b (FP32), and its
 * gradients (dx written, dw / db accumulated). */
int flub_head_fwd(const void *x, const float *w, const float *b, float *out, int64_t n, void *stream);
int flub_head_bwd(const void *x, const float *w, const float *dout, void *dx, float *dw, float *db, int64_t n,
                  void *stream);
/* Masked MSE against the normalised target t = x * inv_scale[b] over fluid
 * cells: *loss += sum of w_b (pred - t)^2 and dpred = d loss / d pred (0 off
 * fluid).  With sample_norm == NULL, w_b = inv_count (normally 1 / the
 * batch's fluid cells); otherwise sample_norm (B doubles of device memory)
 * receives |t_b|^2 and w_b = 1 / (B |t_b|^2): the mean relative squared
 * error of the samples. */
int flub_unet_loss(const float *pred, const float *x, const int32_t *tag, const float *inv_scale, int64_t ncell,
                   int B, double inv_count, double *sample_norm, float *dpred, double *loss, void *stream);
/* Pressure guess from the network output: x0 = out / inv_scale * gain on
 * fluid cells, 0 elsewhere. */
int flub_unet_output(const float *out, const int32_t *tag, const float *inv_scale, int64_t ncell, int B, float gain,
                     float *x0, void *stream);
/* One Adam step (bias-corrected, step >= 1) on FP32 parameters p with
 * gradient g and moments m, v.  For a convolution weight (w16 non-NULL,
 * n = 27 * cout * cin) also writes its BF16 copy [27][cout][cin] and the
 * flipped, transposed copy w16t [27][cin][cout] (tap 26 - t) for the data
 * gradient. */
int flub_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2, float eps,
              int step, void *w16, void *w16t, int cout, int cin, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FLUB_GB300_H */
