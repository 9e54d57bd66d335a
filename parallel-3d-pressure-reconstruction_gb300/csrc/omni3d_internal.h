// Internal declarations shared by the CUDA translation units of libomni3d_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "omni3d.h"

namespace omni3d {

// Number of kernels this library has launched (process-wide, all contexts).
extern unsigned long long g_kernel_launches;
#define OM_COUNT_LAUNCH() (__atomic_fetch_add(&omni3d::g_kernel_launches, 1ull, __ATOMIC_RELAXED))

// Per-direction constants, computed once on the host (exact libm evaluation of the
// rotation of K:6175-6191) and read by the tracing kernels.
struct DirEntry {
    float ct, st, cp, sp;  // cos/sin of theta and phi
    float k1, k2, k3;      // the direction as read from the direction file
    int cas;               // which branch of cross2point (K:663-1113) applies: 1..7, 0 none
    int orig;              // index of the direction in the caller's list
    int pad_;
};

// Grid constants passed by value to every kernel.
struct Grid {
    int X, Y, Z;
    long long XY, V;
    float cx, cy, cz;       // (N-1)/2 in float, K:665-667
    float dx, dy, dz, rho;  // spacing and density
    float ls;               // line spacing
    float thr;              // select threshold the kernels compare against (thr_src, or with
                            // BF16 storage its BF16 stand-in, see k_pack)
    int ng;                 // lattice points per row, K:6159-6167
    float thr_src;          // select threshold as given
    int curl_map;           // 1: BF16 storage of a thresholded method (curl rounded so that
                            // every threshold decision is kept)
};

// One traced line (16 bytes): entry voxel, exit voxel (linear indices), direction and
// number of staircase steps.  The sign of every axis step is fixed per line: toward the
// exit.
struct LineRec {
    uint32_t e, x;
    int32_t dir;
    int32_t m;
};

// Device-resident geometry of one (grid, direction set, line spacing) triple.  Lines are
// grouped 32 per warp; group g's step words are interleaved lane by lane:
// word w of lane l lives at desc[32 * gbase[g] + 32 * w + l], 16 steps (2 bits each) per
// word.
struct Geometry {
    Grid grid;
    int nv = 0;
    int dir_group = 4;              // neighbouring directions interleaved per lattice tile
    int tile_width = 8;             // lattice tile width in points (4, 8 or 16; 32 points a tile)
    DirEntry *d_dirs = nullptr;
    float4 *d_off = nullptr;        // per line: centred offset (x, y, z) of its lattice point
    LineRec *d_lines = nullptr;
    uint32_t *d_gbase = nullptr;    // n_groups + 1 prefix sums of words per lane
    uint32_t *d_desc = nullptr;
    uint32_t *d_lines_through = nullptr;  // per voxel: lines through it (built on first use)
    unsigned max_through = 0;       // the most lines through one voxel (0: not computed)
    unsigned long long *d_counters = nullptr;  // walk counters (early stops, voxel visits)
    int walk_rule = 0;              // OmWalker rule of the staircases (3: per field, minimum curl)
    long long walk_generation = 0;  // incremented by every walk
    long long n_lines = 0, n_groups = 0, n_words = 0;
    long long n_units = 0;          // sum over lines of (steps + 1)
    long long walk_errors = 0;
};

// ---------------------------------------------------------------- launchers (kernels_*.cu)
// All launchers are asynchronous on `st` and return the launch status.

// Lines of every (direction, lattice point) pair, in that order.  Allocates and fills
// g->d_off, g->d_lines, g->d_gbase, g->d_desc; walks every line.  Synchronises `st`.
cudaError_t build_geometry(Geometry *g, cudaStream_t st, std::string *err);
void free_geometry(Geometry *g);
// (Re)walk every line with walk rule `rule` (curl: the field for rule 3).  Synchronises st,
// updates n_units / walk_errors and drops d_lines_through.
cudaError_t run_walk(Geometry *g, int rule, const float *curl, cudaStream_t st);
// Count the lines through every voxel into g->d_lines_through (once per geometry).
cudaError_t ensure_lines_through(Geometry *g, cudaStream_t st);
// The most lines through one voxel (once per geometry; synchronises st).
cudaError_t max_lines_through(Geometry *g, cudaStream_t st, unsigned *out);

// Exclusive scans (out has n + 1 entries; out[n] = total).  tmp must hold
// scan_tmp_elems(n) elements.
size_t scan_tmp_elems(long long n);
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, long long n, uint32_t *tmp,
                               cudaStream_t st);
cudaError_t exclusive_scan_u64(const unsigned long long *in, unsigned long long *out,
                               long long n, unsigned long long *tmp, cudaStream_t st);

// Brick-staged form of the geometry (kernels_brick.cu): every line cut at the boundaries of
// 16^3 voxel bricks into segments, stored brick-major; plus the per-solve segment
// summaries and carry-in states.
struct Bricks {
    bool built = false;
    int nbx = 0, nby = 0, nbz = 0;
    long long n_bricks = 0, n_segs = 0;
    uint4 *rec = nullptr;            // 2 x uint4 per segment, grouped by brick
    uint32_t *brick_off = nullptr;   // n_bricks + 1 segment offsets
    uint32_t *line_seg = nullptr;    // n_lines + 1: line-major id of each line's first segment
    uint4 *items = nullptr;          // work items (brick, first segment, end segment, 0)
    uint32_t n_items = 0;
    int grid = 0;                    // CTAs per brick pass (one per SM)
    uint32_t *work = nullptr;        // [0] work counter, [1] error flag (a TMA wait gave up)
    void *summ = nullptr;            // per-segment summaries of the prepared method
    void *carry = nullptr;           // per-segment carry-in states
    size_t summ_cap = 0, carry_cap = 0;
    int prepared_method = -1;
    const void *map_for = nullptr;   // field the tensor map describes
    alignas(64) unsigned char map[128];  // CUtensorMap of the float4 field
};

// Cut the lines into brick segments (once per geometry); cudaErrorNotSupported when the
// engine cannot be used (no tensor-map support, more than 2^32 segments).
cudaError_t build_bricks(const Geometry &geo, Bricks *B, cudaStream_t st, std::string *err);
void free_bricks(Bricks *B);

// Gradient field on the device: float4 (ax, ay, az, curl) per voxel, or its bf16 copy.
struct Field {
    float4 *f32 = nullptr;          // always present
    uint2 *bf16 = nullptr;          // {ax | ay << 16, az | curl << 16} as bf16 when grad_storage is BF16
    float *curl = nullptr;          // curl (methods that read it), also in f32[v].w; BF16-rounded
                                    // with BF16 storage
};

// Brick passes B1 + L for the field f (FP32) and the method: per-segment carry-in states.
cudaError_t brick_prepare(const Geometry &geo, Bricks *B, const Field &f, int method, cudaStream_t st,
                          std::string *err);
// Brick pass B2: one full sweep from p into pncnt, the same contributions as sweep_full.
cudaError_t brick_sweep(const Geometry &geo, Bricks *B, int method, const float *p, float2 *pncnt,
                        cudaStream_t st);
// The error flag of the brick passes (1: a TMA wait gave up).  Synchronises st.
cudaError_t brick_error(const Bricks &B, int *flag, cudaStream_t st);

// initialIntegration.cpp on the device: p integrated outward from the centre voxel in FP64
// (scratch: V doubles), written to out as float.  The components are read at
// ax[v * stride] (stride 1: three arrays; 4: the float4 field).  Synchronises st once.
cudaError_t centre_integration(const Grid &g, const float *ax, const float *ay, const float *az, int stride,
                               double pref, double *scratch, float *out, cudaStream_t st);

// Pack three component arrays (+ optional curl) into the interleaved field.  With make_bf16
// the BF16-rounded curl is also written to curl_rounded (when given; it may be curl).
cudaError_t pack_field(const Grid &g, const float *ax, const float *ay, const float *az,
                       const float *curl, Field *f, bool make_bf16, cudaStream_t st,
                       float *curl_rounded = nullptr);
// The curl a solve used (.w of its packed FP32 field) into out.
cudaError_t field_curl(long long V, const float4 *f32, float *out, cudaStream_t st);
// |curl a| x mask into out (and into field .w when f is given).
cudaError_t curl_field(const Grid &g, const float *ax, const float *ay, const float *az,
                       const float *mask, float *out, cudaStream_t st);

// One full sweep: pncnt[v] += (sum of contributions, sum of weights) over all lines.
// Every method but the plain one reads the curl indicator.
inline bool method_uses_curl(int method) { return method != OMNI3D_METHOD_PLAIN; }

// Walk rule of a method (OmWalker::step): 1 and 2 the fixed-boundary walks, 3 the
// minimum-curl walk (re-walked per field), 0 the nearest-candidate walk.
inline int method_walk_rule(int method)
{
    switch (method) {
    case OMNI3D_METHOD_WEIGHTED_FIXED_BC: return 1;
    case OMNI3D_METHOD_SELECT_FIXED_BC: return 2;
    case OMNI3D_METHOD_MINI_CURL:
    case OMNI3D_METHOD_WEIGHTED_MINI_CURL: return 3;
    default: return 0;
    }
}

// The accumulation along a line of a method: the variants share their base method's.
enum Accum { kAccPlain = 0, kAccSelect = 1, kAccWeighted = 2, kAccPlainNoEntry = 3, kAccWeightedRawCurl = 4 };
inline int method_accum(int method)
{
    switch (method) {
    case OMNI3D_METHOD_SELECT:
    case OMNI3D_METHOD_SELECT_FIXED_BC: return kAccSelect;
    case OMNI3D_METHOD_WEIGHTED:
    case OMNI3D_METHOD_WEIGHTED_FIXED_BC: return kAccWeighted;
    case OMNI3D_METHOD_MINI_CURL: return kAccPlainNoEntry;
    case OMNI3D_METHOD_WEIGHTED_MINI_CURL: return kAccWeightedRawCurl;
    default: return kAccPlain;
    }
}

// method: OMNI3D_METHOD_*; p is read at line entries / segment starts.
cudaError_t sweep_full(const Geometry &geo, const Field &f, int method, bool bf16,
                       const float *p, float2 *pncnt, cudaStream_t st);
// The same sweep accumulated in FP64 (two FP64 L2 reductions per contribution): the
// defect-correction sweep of params.sweep_fp64.
cudaError_t sweep_full64(const Geometry &geo, const Field &f, int method, bool bf16, const float *p,
                         double2 *pncnt, cudaStream_t st);
cudaError_t init_accum64(long long V, const float *p_init, bool seed, double2 *pncnt, cudaStream_t st);
// The same sweep accumulated in 64-bit fixed point (the bit-reproducible mode), with the
// voxel scales scale[kFixPn], scale[kFixCnt] (fixed.cuh).
struct Fix2;
cudaError_t sweep_full_fix(const Geometry &geo, const Field &f, int method, bool bf16, const float *p, Fix2 *pncnt,
                           const double *scale, cudaStream_t st);
cudaError_t normalize64(long long V, const double2 *pncnt, const float *p_keep, float *p_out, float *cnt_out,
                        cudaStream_t st);

// p_out[v] = cnt > 0 ? pn / cnt : p_keep[v]; cnt_out[v] = cnt (either may be null).
cudaError_t normalize(long long V, const float2 *pncnt, const float *p_keep, float *p_out,
                      float *cnt_out, cudaStream_t st);
// pn[v] += acc[v].x, cnt[v] += acc[v].y
cudaError_t accum_split(long long V, const float2 *acc, float *pn, float *cnt, cudaStream_t st);
// pncnt = (seed ? p_init : 0, 0)
cudaError_t init_accum(long long V, const float *p_init, bool seed, float2 *pncnt,
                       cudaStream_t st);

// Bit-reproducible mode (fixed.cuh, kernels_fixed.cu): device scales and bounds, and the
// operator rows' fixed-point (b, c) while filling.  Kernels that get a null Fixed pointer (or
// scale pointer) take the default FP32 sums.
struct Fixed {
    double *scale = nullptr;        // kFixSlots scales (device)
    unsigned *bits = nullptr;       // kBitsSlots float bits (device)
    long long *bc64 = nullptr;      // 2 per operator row (device)
    size_t cap_bc64 = 0;
    double lmax = 0.0;              // most lines through one voxel (geometry)
    int acc = 0;                    // the method's accumulation kind (weight bound)
    double hmax = 0.0;              // largest trapezoid coefficient rho * spacing / 2
    double path = 0.0;              // X + Y + Z: bound of a staircase's length
};
// Field bounds (max |a|, least nonzero curl) of the packed field into fx->bits.
cudaError_t fix_field_bounds(long long V, const float4 *f32, const Fixed &fx, cudaStream_t st);
// Scales for filling the operator (b, c), for the row sums of an iteration from the
// operator values pa (n of them), and for a full sweep reading the volume vol (V voxels).
cudaError_t fix_fill_scales(const Fixed &fx, cudaStream_t st);
cudaError_t fix_row_scale(long long n, const float *pa, const Fixed &fx, cudaStream_t st, const int *stop = nullptr);
cudaError_t fix_sweep_scales(long long V, const float *vol, const Fixed &fx, cudaStream_t st);
// bc = the fixed-point (b, c) rows as floats (only b when keep_c).
cudaError_t fix_rows_to_float(long long n, const Fixed &fx, float2 *bc, bool keep_c, cudaStream_t st);
// Fixed-point voxel sums: init (pn = seed ? p_init : 0, count = 0), one full sweep,
// normalisation (p = pn / count where count > 0, else p_keep) -- in FP64 from the exact sums.
struct Fix2;
cudaError_t init_accum_fix(long long V, const float *p_init, bool seed, const Fixed &fx, Fix2 *acc, cudaStream_t st);
cudaError_t normalize_fix(long long V, const Fix2 *acc, const Fixed &fx, const float *p_keep, float *p_out,
                          float *cnt_out, cudaStream_t st);

// Anchor operator (kernels_anchor.cu).
struct Anchor {
    long long n = 0, nnz = 0;
    uint8_t *flag = nullptr;        // V bytes: voxel is an anchor
    uint32_t *bits = nullptr;       // V bits
    int32_t *id = nullptr;          // V: anchor id or -1
    uint32_t *vox = nullptr;        // n: voxel of anchor
    unsigned long long *rowptr = nullptr;  // n + 1: row capacities (lines through the voxel)
    uint32_t *rowlen = nullptr;     // n: entries in each row
    uint32_t *col = nullptr;        // nnz, unit weights: the start anchor of each link
    uint2 *cw = nullptr;            // nnz, other methods: (start anchor, weight bits) of each link
    float2 *bc = nullptr;           // n: (b, c) = (sum of w * I, sum of w)
    float *pa = nullptr, *pb = nullptr;  // iterates
    double *red = nullptr;          // reduction scratch
    bool unit_weights = false;      // plain method: every w is 1 (the w array is unused)
    // build scratch (kept between builds)
    uint32_t *u = nullptr, *pos = nullptr, *tmp = nullptr;
    unsigned long long *cnt64 = nullptr, *tmp64 = nullptr;
    uint32_t *neg = nullptr;        // 1 word: some curl value has its sign bit set
    unsigned long long *next = nullptr;  // n: next free link slot of each row while filling
    // capacities in bytes, one per buffer above, so that rebuilding for a new field of the
    // same geometry allocates nothing
    size_t cap[20] = {};
};
// Builds the operator from the float4 entries of f (with BF16 storage they hold the stored
// values); returns cudaErrorNotSupported (nothing filled) when it would hold more than
// max_nnz entries (max_nnz < 0: no limit).
// fx (bit-reproducible mode): the rows' (b, c) are summed in fixed point with the scales of
// fix_fill_scales, which the caller sets before.
cudaError_t anchor_build(Geometry &geo, const Field &f, int method, long long ref_voxel,
                         long long max_nnz, Anchor *A, cudaStream_t st, std::string *err,
                         Fixed *fx = nullptr);
void anchor_free(Anchor *A);
// Plain method: recompute only b (the field-dependent part) of an operator built by
// anchor_build for the same geometry; rows, columns and c depend on the geometry alone.
cudaError_t anchor_refresh_rhs(const Geometry &geo, const Field &f, Anchor *A, cudaStream_t st,
                               const Fixed *fx = nullptr);
// One iteration p_next = (b + seed * p_init_a + M p_cur) / c; accumulates the gauged
// change / norm sums into red[0..1] for the relative change.  With stop, every kernel of the
// step returns at once while *stop != 0 (the gated steps of a graph-captured chunk).
cudaError_t anchor_step(const Anchor &A, const float *p_init, bool seed, int gauge,
                        long long ref_anchor, const float *p_cur, float *p_next, double *red2,
                        cudaStream_t st, const int *stop = nullptr, const Fixed *fx = nullptr);
// Launch the convergence test of step j of a chunk: rel_out[j] = sqrt(red2[0] / red2[1]),
// *stop = j + 1 when it is below tol (no-op while *stop != 0).
cudaError_t converged_test_launch(const double *red2, double tol, int j, int *stop, double *rel_out,
                                  cudaStream_t st);
// Gauged relative-change sums over the n values selected by mask (all when mask is null):
// out2 = {sum (d - d_ref)^2, sum (p - p_ref)^2} with d = pn - pc; the shift is the value at
// `ref` (point gauge), the mean (mean gauge) or zero.  Deterministic FP64 reduction;
// scratch holds change_scratch_doubles().
size_t change_scratch_doubles();
cudaError_t change_sums(long long n, const float *pc, const float *pn, int gauge, long long ref,
                        double *scratch, double *out2, cudaStream_t st, const uint8_t *mask,
                        const int *stop = nullptr);
// Flag the anchor voxels (line entries, or the segment starts of the selected method or a
// small superset of them, plus ref_voxel when >= 0) into a V-byte array.  count1 is one
// device word of scratch.
cudaError_t anchor_mark(const Geometry &geo, const Field &f, int method, long long ref_voxel,
                        uint8_t *flag, unsigned long long *count1, cudaStream_t st);
// Scatter anchor values into a volume.
cudaError_t anchor_scatter(const Anchor &A, const float *pa, float *vol, cudaStream_t st);
// Gather anchor values from a volume.
cudaError_t anchor_gather(const Anchor &A, const float *vol, float *pa, cudaStream_t st);

// Adjoint of the plain-method solve (kernels_adjoint.cu).
struct AdjointBuffers {
    unsigned long long *tptr = nullptr;  // transposed operator (built once per operator)
    uint32_t *trow = nullptr;
    float *tw = nullptr;                 // weights of the transposed entries (weighted operators)
    unsigned long long *tmp = nullptr;
    float *mu = nullptr, *lam = nullptr, *nxt = nullptr, *acc = nullptr;
};
void adjoint_free(AdjointBuffers *B);
// gx, gy, gz = d<g, p_K>/d(ax, ay, az) for `method` after K iterations with the curl held
// fixed, given the operator A of that solve, its per-voxel count cnt and its packed FP32
// field f32 (whose .w holds the curl the solve used).
cudaError_t adjoint_solve(const Geometry &geo, const Anchor &A, AdjointBuffers *B, int K, int method,
                          const float4 *f32, const float *g, const float *cnt, float *gx, float *gy,
                          float *gz, cudaStream_t st);
// out = G^T g for the output gauge G (part: gauge_transpose_scratch_doubles()).
cudaError_t gauge_transpose(long long V, int gauge, long long ref, const float *g,
                            const float *cnt, float *out, double *part, cudaStream_t st);
size_t gauge_transpose_scratch_doubles();

// Gauge: subtract p[ref] (mode POINT) or the mean over count > 0 (MEAN), FP64 reduction.
cudaError_t apply_gauge(long long V, int gauge, long long ref, const float *cnt, float *p,
                        double *scratch, cudaStream_t st);
size_t gauge_scratch_doubles();

}  // namespace omni3d
