/*
 * omni3d.h -- C ABI of the GB300 (sm_103a) omni-directional 3D pressure reconstruction.
 *
 * The reference program (Omni3D_8.0/Omni3D_8.0/kernel.cu, "K" below) is a monolithic
 * executable with no library interface.  Each entry point here replaces one block of its
 * main() or one of its kernels; the block is cited beside the declaration.
 *
 * Conventions
 *   - Every function returns an int status: OMNI3D_OK (0) or a negative OMNI3D_ERR_*.
 *     omni3d_last_error(ctx) (or omni3d_global_error() for calls without a context)
 *     returns a text description of the last failure.
 *   - Volumes are float32, x fastest: index = i + j*nx + k*nx*ny (the order of the
 *     Tecplot rows the reference reads, K:8712-8792).
 *   - Pointers are host pointers unless the call's `device_ptrs` argument is non-zero, in
 *     which case they must be device pointers on the context's device.
 *   - A context is not reentrant; separate contexts may run concurrently on separate
 *     streams.
 */
#ifndef OMNI3D_H
#define OMNI3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OMNI3D_OK 0
#define OMNI3D_ERR_ARG (-1)      /* invalid argument */
#define OMNI3D_ERR_CUDA (-2)     /* CUDA runtime error (text in last_error) */
#define OMNI3D_ERR_IO (-3)       /* file missing, short or malformed */
#define OMNI3D_ERR_NOMEM (-4)    /* device or host allocation failed */
#define OMNI3D_ERR_STATE (-5)    /* call made in the wrong state */
#define OMNI3D_ERR_RANGE (-6)    /* size beyond a stated limit */
#define OMNI3D_ERR_NUMERIC (-7)  /* non-finite result or a line walk that failed */

/* Integration method (Tutorial p.1 "Standard / Selected"). */
#define OMNI3D_METHOD_PLAIN 0     /* bodyIntegralInner, K:1743-1863 */
#define OMNI3D_METHOD_SELECT 1    /* bodyIntegralInnerSelect, K:2280-2537 (what main runs) */
#define OMNI3D_METHOD_WEIGHTED 2  /* bodyIntegralInnerWeighted, K:1993-2135, launched by
                                     omni3dparallellinesESInnerWeighted K:6281-6345 (the
                                     commented-out alternative of main, K:8844): every step
                                     weighted by n / sum(curl/1e4) from the entry, no
                                     contribution to the entry itself */
/* Variants the reference keeps beside its three methods.  Fixed boundary: the walk never
 * steps into the j = 0 face (the Bernoulli face of main(), K:8805-8811), so that face keeps
 * its initial values.  Minimum curl: each step goes to the candidate voxel with the
 * smallest curl instead of the one nearest the line, so the paths depend on the field and
 * are re-walked for every solve. */
#define OMNI3D_METHOD_WEIGHTED_FIXED_BC 3  /* bodyIntegralInnerWeightedFixedBC, K:2136-2279 */
#define OMNI3D_METHOD_SELECT_FIXED_BC 4    /* bodyIntegralInnerSelectFixedBC, K:2538-2796 (also
                                              ties y before x before z) */
#define OMNI3D_METHOD_MINI_CURL 5          /* bodyIntegralInnerMiniCurl, K:2797-2936: the plain
                                              accumulation without the entry's own term */
#define OMNI3D_METHOD_WEIGHTED_MINI_CURL 6 /* bodyIntegralInnerWeightedMiniCurl, K:2937-3085
                                              (commented out in main, K:8847): weights n / sum
                                              of raw curl from the entry, the entry included,
                                              no zero-sum test */

/* Solver form.  Both produce the reference iteration's result; they differ in cost. */
#define OMNI3D_SOLVER_ANCHOR 0  /* iterate only the voxels whose values feed back (line
                                   entries / segment starts), then one full sweep */
#define OMNI3D_SOLVER_SWEEP 1   /* one full omni sweep per iteration, as K:8840-8861 */

/* Storage of the gradient field on the device. */
#define OMNI3D_GRAD_F32 0
#define OMNI3D_GRAD_BF16 1

/* Sweep engine.  Both give the same contributions; they differ in how the volume is read. */
#define OMNI3D_ENGINE_AUTO 0    /* the faster engine for the solve: lines (measured on GB300
                                   at 256^3 / 642 directions: lines 97 ms per sweep, bricks
                                   145 ms + 95 ms of per-field passes) */
#define OMNI3D_ENGINE_LINES 1   /* one thread per line, gathers and reductions through L2 */
#define OMNI3D_ENGINE_BRICKS 2  /* lines cut into 16^3-brick segments; each brick's field is
                                   staged in shared memory by TMA and its sums kept there */

/* Initial state of a solve when p_init is NULL. */
#define OMNI3D_INIT_ZERO 0      /* zero, as when main() is given no Bernoulli face */
#define OMNI3D_INIT_CENTRE 1    /* omni3d_centre_integration (initialIntegration.cpp) */

/* Gauge applied to the output (the reference applies none; K:8879-8915 is commented out). */
#define OMNI3D_GAUGE_NONE 0
#define OMNI3D_GAUGE_POINT 1    /* p -= p(ref voxel) */
#define OMNI3D_GAUGE_MEAN 2     /* p -= mean over voxels with count > 0 */

typedef struct omni3d_ctx omni3d_ctx;

/* Solver parameters.  The first block mirrors Parameter_Omni3D.dat (K:8541-8571). */
typedef struct {
    int nx, ny, nz;            /* grid after the ROI crop (lines 1-3, 16-21) */
    float dx, dy, dz;          /* spacing (lines 4-6) */
    float density;             /* rho (line 7) */
    float line_spacing;        /* spacing of the parallel lines (line 9) */
    int n_dirs;                /* number of direction vectors (line 10) */
    const float *dirs;         /* host, n_dirs x 3 (k1,k2,k3), as read from the direction file */
    int max_iter;              /* NoItr (line 14): iterations to run */
    float threshold;           /* curl threshold of the selected method (line 15) */
    int method;                /* OMNI3D_METHOD_* */
    /* additions of this implementation */
    int solver;                /* OMNI3D_SOLVER_* */
    int grad_storage;          /* OMNI3D_GRAD_* */
    double tol;                /* stop early when the gauged relative change of p falls below
                                  tol (0: run exactly max_iter, as the reference does) */
    int gauge;                 /* OMNI3D_GAUGE_* */
    int ref_i, ref_j, ref_k;   /* reference voxel of OMNI3D_GAUGE_POINT */
    int seed_first_iteration;  /* 1 (reference, K:8811): the first sweep accumulates on top of
                                  p_init; 0: on top of zero */
    int device;                /* CUDA device ordinal */
    long long anchor_max_links;/* anchor operator entries allowed before the solve falls back
                                  to the sweep form (0: what 80 % of the free device memory
                                  holds) */
    int engine;                /* OMNI3D_ENGINE_* */
    int initial_guess;         /* OMNI3D_INIT_*: the initial state when p_init is NULL */
    int sweep_fp64;            /* 1: full sweeps accumulate (pn, count) in FP64 and normalise in
                                  FP64 -- for the anchor solver its one final sweep, a
                                  defect-correction step from the FP32 iteration; for the sweep
                                  solver every sweep.  Line integrals stay FP32 sums. */
    int tile_width;            /* line order: a warp walks the lines of one direction through a
                                  tile of 32 lattice points, tile_width (4, 8 or 16) wide;
                                  0: 8 */
    int dir_group;             /* line order: neighbouring directions interleaved per tile
                                  (1-32); 0: 32 for grids of up to 2^24 voxels, 4 above */
    int autotune;              /* 1: omni3d_create picks tile_width and dir_group by timing one
                                  sweep of each of a few candidate pairs on this grid and
                                  direction set, and keeps the choice for the process, per
                                  device and size class (largest grid dimension rounded up to
                                  a multiple of 32, direction count, line spacing, walk rule);
                                  tile_width and dir_group are then ignored */
    int deterministic;         /* 1: bit-reproducible solves.  The sums whose order the GPU does
                                  not fix -- the voxels' (pn, count) of every full sweep, the
                                  anchor operator's rows (b, c) and the rows' sums in each
                                  iteration -- are taken in 64-bit fixed point (exact and
                                  order-independent) with power-of-two scales set on the device
                                  from bounds of the field, and normalised in FP64, so the same
                                  inputs give the same bits on every run.  Needs the line engine;
                                  returns OMNI3D_ERR_RANGE if a bound is not finite (a nonzero
                                  curl below about 1e-300 relative to the field).  The adjoint
                                  and omni3d_sweep are not covered. */
} omni3d_params;

typedef struct {
    int iterations;            /* iterations performed (<= max_iter) */
    double rel_change;         /* gauged relative change of the last iteration */
    long long n_lines;         /* lines that cross the volume (all directions) */
    long long n_units;         /* voxel-direction updates of one full sweep */
    long long walk_errors;     /* lines whose walk hit the reference's wrong-point branch */
    long long n_anchors;       /* anchor voxels (anchor solver) */
    long long n_links;         /* anchor operator entries (anchor solver) */
    double ms_geometry;        /* line tracing + walk (cached across solves) */
    double ms_setup;           /* per-field setup: anchor operator or precomputed terms */
    double ms_iterate;         /* iterations */
    double ms_final;           /* final full sweep + normalisation */
    double ms_total;           /* device time of the whole solve */
    double ms_sweep;           /* device time of the final full sweep kernel alone */
    long long kernel_launches; /* CUDA kernels this library launched during the call */
    int solver_used;           /* OMNI3D_SOLVER_*: the anchor solver falls back to the sweep
                                  solver when its operator would exceed anchor_max_links */
    int engine_used;           /* OMNI3D_ENGINE_LINES or OMNI3D_ENGINE_BRICKS */
    int tile_width;            /* the line order in use (see omni3d_params) */
    int dir_group;
} omni3d_stats;

/* Fill *p with the reference's defaults (K:8512-8535) and this implementation's. */
void omni3d_default_params(omni3d_params *p);

/* Create a solver context: validates the parameters, uploads the direction table and
 * traces the line geometry (the per-direction parallel-line generator of K:6153-6198 and
 * the entry/exit search cross2point, K:663-1113) into device line descriptors.
 * Replaces the setup of main(), K:8577-8672. */
int omni3d_create(const omni3d_params *params, omni3d_ctx **out);
int omni3d_destroy(omni3d_ctx *ctx);
const char *omni3d_last_error(const omni3d_ctx *ctx);
const char *omni3d_global_error(void);

/* The reference's initial guess by integration outward from the centre voxel,
 * initialIntegration.cpp:9-407 (uncalled by its main()): eight octant sweeps from
 * (nx/2, ny/2, nz/2); each voxel is the mean over its off-centre axes of the neighbour one
 * step nearer the centre plus the trapezoid increment -rho * a * spacing.  FP64 on the
 * device (wavefronts of equal distance from the centre), returned as float; bit-identical
 * to the reference's double result rounded to float.  The centre voxel is 0.  pref is
 * written to voxel 0 before the sweeps, as the reference does, and overwritten by them, so
 * it does not change the result (kept for the reference's signature). */
int omni3d_centre_integration(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az,
                              double pref, float *p_out, int device_ptrs);

/* Use this CUDA stream (cudaStream_t passed as void*) for all later work on ctx. */
int omni3d_set_stream(omni3d_ctx *ctx, void *stream);

/* Solve one snapshot: the whole per-file block of main(), K:8794-8863 (initial state,
 * NoItr x {omni sweep, devidecountInner}, read back p and count).
 *   ax, ay, az   material acceleration Du/Dt, Dv/Dt, Dw/Dt (grad p = -rho a)
 *   curl         |curl a| x mask (every method but PLAIN; NULL: computed on the device
 *                from ax..az and mask), see omni3d_curl
 *   mask         mask column of the input file (NULL: all ones); used only when curl is NULL
 *   p_init       initial pressure (NULL: zero), e.g. omni3d_bernoulli_face()
 *   p_out        pressure after the iterations (required)
 *   count_out    per-voxel line count of the last iteration (K:8857; NULL: not returned)
 *   stats        optional */
int omni3d_solve(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az,
                 const float *curl, const float *mask, const float *p_init, float *p_out,
                 float *count_out, int device_ptrs, omni3d_stats *stats);

/* One omni sweep from p without normalisation: pn += contributions, count += weights.
 * The loop body of omni3dparallellinesESInner (K:6151-6215) / ...Select (K:6414-6480)
 * over every (direction, lattice point) pair. */
int omni3d_sweep(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az,
                 const float *curl, const float *p, float *pn, float *count, int device_ptrs);

/* Remove the constant mode of a pressure field in place: p -= p[ref] (OMNI3D_GAUGE_POINT,
 * ref = i + j*nx + k*nx*ny) or p -= mean of p over voxels with count > 0
 * (OMNI3D_GAUGE_MEAN), with an FP64 reduction.  The reference's mean removal over the
 * measured voxels is commented out in its main() (K:8879-8915); omni3d_solve applies the
 * same operation when params.gauge is set.  n must equal the context's voxel count. */
int omni3d_gauge(omni3d_ctx *ctx, float *p, const float *count, long long n, int gauge,
                 long long ref, int device_ptrs);

/* Adjoint of the last omni3d_solve on ctx, for every method: writes the gradient of
 * <grad_p, p_out> with respect to ax, ay, az, i.e. the transpose of the solve's affine map
 * (scatter back along the lines and through the iterations, no stored iterates), including
 * the transpose of the output gauge.  The curl the solve used is held fixed: the weights and
 * segment splits of the selected and weighted methods (K:1993-2537) depend on it, and no
 * derivative is taken through it.  No counterpart in the reference; it serves pressure
 * sensitivities and torch.autograd (the omni3d Python package). */
int omni3d_adjoint(omni3d_ctx *ctx, const float *grad_p, float *grad_ax, float *grad_ay,
                   float *grad_az, int device_ptrs);

/* |curl a| x mask: calCurlofMaterialAccCPU, K:8352-8378 (GPU twin K:6863-6888). */
int omni3d_curl(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az,
                const float *mask, float *curl_out, int device_ptrs);

/* Lines and walk lengths of the traced geometry (diagnostics and tests). */
int omni3d_geometry_info(omni3d_ctx *ctx, long long *n_lines, long long *n_units,
                         long long *walk_errors);

/* Copy the line table to host memory: per line {entry voxel, exit voxel, direction, steps}
 * (4 x int32), n_max rows at most.  Lines are stored in the library's processing order
 * (groups of neighbouring directions, lattice tiles, direction, point: see tile_width and
 * dir_group); the direction column is the index in the caller's list. */
int omni3d_line_table(omni3d_ctx *ctx, int32_t *rows, long long n_max);

/* Copy the staircase of line `line` (one axis code 0/1/2 per step) to host memory. */
int omni3d_line_steps(omni3d_ctx *ctx, long long line, int8_t *axes, int cap);

/* Voxel limit of omni3d_sweep_noalloc (its scratch is sized for it at build time). */
#define OMNI3D_NOALLOC_MAX_VOXELS (64LL * 64 * 64)

/* omni3d_sweep without any device allocation, for callers that cannot call cudaMalloc at
 * that point: a framework whose own memory pool owns the device and forbids driver
 * allocations inside its step, a plugin loaded into an application with a fixed device
 * memory budget, a real-time loop that cannot take cudaMalloc's implicit synchronisation.
 * No counterpart in the reference.  Same arguments and result as
 * omni3d_sweep with device pointers (pn and count are added to), FP32 gradient storage
 * only, at most OMNI3D_NOALLOC_MAX_VOXELS voxels (larger grids are rejected with
 * OMNI3D_ERR_RANGE).  The packed field and the (pn, count) accumulator live in static
 * device arrays of that size that every GPU loading the library keeps until exit.  The
 * call only enqueues work on `stream` (NULL: the context's stream); the results are ready
 * when that stream reaches them.  All calls share the static arrays: calls that overlap on
 * the GPU (other streams, other contexts, other threads) race and must be serialised by
 * the caller.  The first call on a device looks up the arrays' device addresses (a
 * one-time set-up on that device), so make it before any stream capture.  The caller's
 * current device is left as it was. */
int omni3d_sweep_noalloc(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az,
                         const float *curl, const float *p, float *pn, float *count,
                         void *stream);

/* ---------------------------------------------------------------- batches of snapshots */

/* A batch solves several snapshots, each with its own context (grid sizes, methods and
 * tolerances may differ).  This replaces the reference's sequential per-file loop
 * (K:8701-8963).  When every member has the plain method, the anchor solver and tol = 0 (a
 * fixed iteration count), the batch is one CUDA-graph launch: every member's solve runs on
 * its own stream, forked from and joined to the batch stream, captured once and relaunched
 * while the buffers stay the same; the first omni3d_batch_solve prepares each member with
 * one regular solve.  Otherwise (a member with another method -- the selected method that
 * main runs rebuilds its operator per field --, the sweep solver, or its own tolerance) the
 * members are solved concurrently, each by omni3d_solve on its own context stream, shared
 * among a pool of host threads, so that one member's host synchronisations hold up only its
 * own thread; stats->ms_total is then the host wall time of the batch and
 * stats->iterations the most any member ran. */
typedef struct omni3d_batch omni3d_batch;
int omni3d_batch_create(omni3d_ctx *const *ctxs, int n, omni3d_batch **out);
int omni3d_batch_destroy(omni3d_batch *batch);
const char *omni3d_batch_last_error(const omni3d_batch *batch);
/* Per-member arrays of n pointers; mask, p_init and count_out (and their entries) may be
 * NULL.  mask is the members' mask column, from which the methods that read the curl
 * compute it (|curl a| x mask, as omni3d_solve with curl = NULL); a batch with any mask
 * runs in the concurrent form.  stats (optional) aggregates the members; ms_total is the
 * device time of the graph (the host wall time in the concurrent form). */
int omni3d_batch_solve(omni3d_batch *batch, const float *const *ax, const float *const *ay,
                       const float *const *az, const float *const *mask, const float *const *p_init,
                       float *const *p_out, float *const *count_out, int device_ptrs, omni3d_stats *stats);

/* ---------------------------------------------------------------- host-side helpers */

/* Direction set of an icosahedron subdivided `level` times (level 2: 42, 3: 162, 4: 642,
 * 5: 2562, ... vertices), sorted and rounded to six decimals the way the reference's
 * GridIcosahedronDivide<level>.dat files are.  Writes up to cap rows of (k1,k2,k3) into
 * out and returns the vertex count (or a negative status). */
int omni3d_icosphere(int level, float *out, int cap);

/* Direction file (K:8615-8649): rows "k1 k2 k3", a trailing count row ignored.  Reads n
 * rows into out (n x 3).  Returns the number of rows read or a negative status. */
int omni3d_read_directions(const char *path, int n, float *out);

/* Parameter_Omni3D.dat (K:8541-8571), including the hidden pref line and ROI lines. */
typedef struct {
    int nx_org, ny_org, nz_org;
    float dx, dy, dz, density, scale, line_spacing;
    int n_dirs;
    char dir_file[1024], accel_dir[1024], pressure_dir[1024];
    int n_iter;
    float threshold, pref;
    int roi[6];               /* i0, i1, j0, j1, k0, k1 (inclusive) */
} omni3d_file_params;
int omni3d_read_params(const char *path, omni3d_file_params *out);

/* Tecplot ASCII acceleration file (K:8708-8792): 3 header lines, then rows
 * "x y z u v w Du Dv Dw mask" (10 columns) or "x y z Du Dv Dw mask" (7 columns), i
 * fastest, cropped to the ROI.  Any output pointer may be NULL.  Arrays hold
 * (i1-i0+1)*(j1-j0+1)*(k1-k0+1) floats. */
int omni3d_read_tecplot(const char *path, const omni3d_file_params *fp, float *x, float *y,
                        float *z, float *u, float *v, float *w, float *ax, float *ay,
                        float *az, float *mask);

/* Initial pressure of K:8805-8811: pref - rho/2 |u|^2 on the j = 0 face, 0 elsewhere. */
int omni3d_bernoulli_face(int nx, int ny, int nz, float pref, float density, const float *u,
                          const float *v, const float *w, float *p_init);

/* PressureOmni3D_%05d.dat writer (K:8916-8935): header lines and rows of
 * "%15.9f %15.9f %15.9f %15.9f %15.9f" (x y z p count). */
int omni3d_write_pressure(const char *path, int nx, int ny, int nz, const float *x,
                          const float *y, const float *z, const float *p, const float *count);

/* CurlofMaterialAcc_Sample.dat writer (K:8938-8958). */
int omni3d_write_curl(const char *path, int nx, int ny, int nz, const float *x, const float *y,
                      const float *z, const float *curl);

#ifdef __cplusplus
}
#endif
#endif /* OMNI3D_H */
