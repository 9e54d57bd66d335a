// Anchor operator: the reference iteration restricted to the voxels whose values feed back.
//
// In one iteration of the reference (K:8840-8861) a voxel v receives, from every line
// segment through it, w * (p[start] + I(v)) in pn and w in count (w = 1 for the plain
// method; the start is the line entry, K:1760-1761; for the weighted method the start is
// the entry and w = n / sum(curl/1e4) along the line, K:2086-2130; for the selected method
// the start is the voxel where the segment began or restarted, K:2301-2411, and
// w = n / sum(curl/1e4) along the segment).
// I(v) and w depend only on the gradient field, so
//     p_new(v) = (b(v) + sum_j w_j p_old(start_j)) / c(v),  b = sum w I,  c = sum w.
// Only the start voxels ("anchors") are ever read, so the iteration closes on the anchors:
// iterate p_a <- (b_a + M p_a) / c_a on them alone, then evaluate every voxel once from
// the final anchor values with one full sweep.  This gives the reference's iterate exactly
// (up to the order of floating-point sums) at a fraction of the cost.
//
// The operator is built from the same line descriptors as the sweep: a marking pass finds
// the anchors, the geometry's line counts size each anchor's row, a filling pass writes
// (column = start anchor, weight) pairs and accumulates b and c.  The filling pass learns
// whether a visited voxel is an anchor from the field gather itself: for the duration of
// the pass the anchors' packed field entries carry a flag in a bit no value uses (the sign
// of the curl in .w, curl being non-negative), so a step costs one gather instead of a
// gather and a bitmap load.  A field with a negative curl value keeps the bitmap.  The
// operator passes read the float4 entries, which with BF16 storage hold the stored values
// (k_pack): they are bound by instruction issue, not by their gathers, and so read nothing
// that needs unpacking.
//
// The filling pass sums each line's integral in plain FP32 in step order, as the reference
// does (K:1816-1834); the final sweep, whose integrals reach every voxel directly, keeps
// compensated sums.  The filling pass is bound by instruction issue, and the three
// additions of the compensation took 2.7 ms of its 52.7 ms at 256^3 / 642 directions.
#include <algorithm>

#include "fixed.cuh"
#include "omni3d_internal.h"
#include "walk.cuh"

namespace omni3d {

// Steps whose gathers a walk issues together (walk.cuh): 4 beat 3 and 2 by 0.3 and 1.5 ms at
// 256^3 / 642 directions; 5 and 6 spill.
constexpr int kWalkBatch = 4;
// Launch shape of the operator passes: the filling pass waits on its gathers and issues many
// instructions per step, and 40 resident warps per SM (48 registers, a few bytes spilled to
// L1) beat 32 (64 registers, no spill) and 48 (more spills): with CTAs of 256 threads 50.0
// against 55.1 and 56.2 ms at 256^3 / 642 directions.  Small CTAs then free their slots as
// soon as their own few lines end, where a CTA of 8 warps waits for its longest line: 20
// CTAs of 64 threads took the pass from 46.9 to 44.2 ms (10 of 128: 44.8 ms; 32 warps
// without spills, 32 CTAs of 32 threads or 16 of 64: 48.1 ms).
constexpr int kFillBlocks = 20;
constexpr int kFillThreads = 64;  // threads per CTA (whole warps: one line per thread)

namespace {

// Anchor flag of a gathered voxel: with FB the sign bit of its .w (the flag the filling
// pass sets in the field), else its bit of the bitmap word gathered beside it.
template <bool FB>
__device__ __forceinline__ bool anchor_of(const float4 &gv, uint32_t word, long long v)
{
    return FB ? (__float_as_uint(gv.w) >> 31) != 0u : ((word >> (v & 31)) & 1u) != 0u;
}

// Curl from .w of the FP32 field: under FB its sign bit is the anchor flag.
template <bool FB>
__device__ __forceinline__ float curl_of(const float4 &gv)
{
    return FB ? fabsf(gv.w) : gv.w;
}

__device__ __forceinline__ float sel3(int a, float x, float y, float z)
{
    return a == 0 ? x : (a == 1 ? y : z);
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ __forceinline__ bool is_anchor(const uint32_t *bits, long long v)
{
    return (__ldg(bits + (v >> 5)) >> (v & 31)) & 1u;
}

enum Pass { kMark = 0, kFill = 2, kRhs = 3 };

struct Sink {
    const uint32_t *bits;
    const int32_t *id;
    uint8_t *flag;
    unsigned long long *next;  // per row: the next free link slot (starts at the row's first slot)
    uint32_t *col;   // unit-weight operators: the start anchor of each link
    uint2 *cw;       // weighted operators: (start anchor, weight bits) of each link
    float2 *bc;      // per row: (b, c)
    long long *bc64; // bit-reproducible mode: per row the fixed-point (b, c) instead of bc
    const double *fix;  // its scales (fixed.cuh)
};

// Record one contribution of weight wt and integral I into voxel v from the segment whose
// start anchor is scol (its id, loaded once per segment).  A link costs one row lookup, one
// 64-bit slot atomic, one store and one vector reduction of (b, c); UNIT operators (every
// weight 1) store no weight.
template <int PASS, bool UNIT>
__device__ __forceinline__ void emit_w(const Sink &S, uint32_t v, uint32_t scol, float wt, float I, bool anchor)
{
    if (PASS == kMark) return;
    if (!anchor) return;
    int row = __ldg(S.id + v);
    if (row < 0) return;  // not an anchor after all: nothing to index
    if (PASS == kFill && (int)scol < 0) return;  // a start that is no anchor: no column to link
    if (PASS == kRhs) {  // plain method, operator cached: only b = sum I is field-dependent
        if (S.bc64) fix_add(S.bc64 + 2 * row, I, S.fix[kFixB]);
        else atomicAdd(&S.bc[row].x, I);
        return;
    }
    const unsigned long long slot = atomicAdd(S.next + row, 1ull);
    const float bt = UNIT ? I : wt * I, ct = UNIT ? 1.0f : wt;
    if (UNIT) S.col[slot] = scol;
    else S.cw[slot] = make_uint2(scol, __float_as_uint(wt));
    if (S.bc64) {  // bit-reproducible: exact, order-independent fixed-point row sums
        fix_add(S.bc64 + 2 * row, bt, S.fix[kFixB]);
        fix_add(S.bc64 + 2 * row + 1, ct, S.fix[kFixC]);
    } else {
        atomicAdd(S.bc + row, make_float2(bt, ct));
    }
}

// The anchor id of a segment's start voxel, for the filling pass's links.
template <int PASS>
__device__ __forceinline__ uint32_t start_col(const Sink &S, uint32_t start)
{
    return PASS == kFill ? (uint32_t)__ldg(S.id + start) : 0u;
}

struct Walk {
    uint32_t v;
    int d0, d1, d2;
    float h0, h1, h2;
    int m;
    const uint32_t *dp;
    __device__ __forceinline__ void init(const Grid &g, const LineRec &r, const uint32_t *gbase,
                                         const uint32_t *desc, long long li)
    {
        int ie = (int)(r.e % (uint32_t)g.X), je = (int)((r.e / (uint32_t)g.X) % (uint32_t)g.Y),
            ke = (int)(r.e / (uint32_t)g.XY);
        int ix = (int)(r.x % (uint32_t)g.X), jx = (int)((r.x / (uint32_t)g.X) % (uint32_t)g.Y),
            kx = (int)(r.x / (uint32_t)g.XY);
        int si = ix > ie ? 1 : -1, sj = jx > je ? 1 : -1, sk = kx > ke ? 1 : -1;
        d0 = si;
        d1 = sj * g.X;
        d2 = sk * (int)g.XY;
        h0 = __fmul_rn(-g.rho * (float)si, g.dx) * 0.5f;
        h1 = __fmul_rn(-g.rho * (float)sj, g.dy) * 0.5f;
        h2 = __fmul_rn(-g.rho * (float)sk, g.dz) * 0.5f;
        v = r.e;
        m = r.m;
        dp = desc + 32ull * gbase[li >> 5] + (li & 31);
    }
};

// The trapezoid increment of a step along axis a, h_a (g_a(v) + g_a(previous voxel)), formed
// for all three axes and then selected: one selection instead of three.  The filling pass is
// bound by instruction issue with the selections' pipe the busiest, and this took 0.8 ms off
// its 50 ms at 256^3 / 642 directions.
__device__ __forceinline__ float step_term(int a, const Walk &L, const float4 &gv, const float4 &gl)
{
    return sel3(a, L.h0 * (gv.x + gl.x), L.h1 * (gv.y + gl.y), L.h2 * (gv.z + gl.z));
}

// Plain method: anchors are the entries; every voxel of a line takes (p[entry] + I, 1).
// SELF = false leaves the entry's own term out (the minimum-curl plain variant).
template <int PASS, bool SELF, bool FB>
__global__ void __launch_bounds__(kFillThreads, kFillBlocks)
k_anchor_plain(Grid g, const LineRec *__restrict__ lines,
               const uint32_t *__restrict__ gbase,
               const uint32_t *__restrict__ desc, long long n_lines,
               const float4 *__restrict__ f32, Sink S)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    if (PASS == kMark) {
        S.flag[r.e] = 1;
        return;
    }
    Walk L;
    L.init(g, r, gbase, desc, li);
    const uint32_t e = r.e;
    const uint32_t ecol = start_col<PASS>(S, e);
    if (SELF) emit_w<PASS, true>(S, e, ecol, 1.0f, 0.0f, is_anchor(S.bits, e));
    float4 gl = __ldg(f32 + e);
    float I = 0.0f;
    // the field (and without FB the anchor bitmap word) of every voxel gathered in batches
    walk_steps<kWalkBatch, kGradF32, !FB>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, nullptr, S.bits, [&](int a, uint32_t v, const float4 &gv, uint32_t word) {
            I += step_term(a, L, gv, gl);
            gl = gv;
            emit_w<PASS, true>(S, v, ecol, 1.0f, I, anchor_of<FB>(gv, word, v));
        });
}

// Weighted method: the walk of k_sweep_weighted (K:1993-2135); anchors are the entries
// (the marking pass is the plain method's), the entry itself receives nothing.
template <int PASS, bool FB>
__global__ void __launch_bounds__(kFillThreads, kFillBlocks)
k_anchor_weighted(Grid g, const LineRec *__restrict__ lines,
                  const uint32_t *__restrict__ gbase,
                  const uint32_t *__restrict__ desc, long long n_lines,
                  const float4 *__restrict__ f32,
                  const float *__restrict__ curl, Sink S)
{
    static_assert(PASS == kFill, "the weighted operator has only a filling pass");
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    Walk L;
    L.init(g, r, gbase, desc, li);
    const uint32_t e = r.e;
    const uint32_t ecol = start_col<PASS>(S, e);
    float4 gl = __ldg(f32 + e);
    float I = 0.0f, csum = 0.0f, nseg = 0.0f;
    walk_steps<kWalkBatch, kGradF32, !FB>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, nullptr, S.bits, [&](int a, uint32_t v, const float4 &gv, uint32_t word) {
            float cn = curl_of<FB>(gv);
            I += step_term(a, L, gv, gl);
            csum += __fdiv_rn(cn, 1.0e4f);  // the weights as in k_sweep_weighted
            nseg += 1.0f;
            if (csum != 0.0f) emit_w<PASS, false>(S, v, ecol, __fdividef(nseg, csum), I, anchor_of<FB>(gv, word, v));
            gl = gv;
        });
}

// Weighted method with raw curl sums (the minimum-curl variant): the walk of
// k_sweep_weighted_raw; anchors are the entries, the entry takes its own term.
template <int PASS, bool FB>
__global__ void __launch_bounds__(kFillThreads, kFillBlocks)
k_anchor_weighted_raw(Grid g, const LineRec *__restrict__ lines,
                      const uint32_t *__restrict__ gbase,
                      const uint32_t *__restrict__ desc, long long n_lines,
                      const float4 *__restrict__ f32,
                      const float *__restrict__ curl, Sink S)
{
    static_assert(PASS == kFill, "the raw-curl weighted operator has only a filling pass");
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    Walk L;
    L.init(g, r, gbase, desc, li);
    const uint32_t e = r.e;
    const uint32_t ecol = start_col<PASS>(S, e);
    float4 gl = __ldg(f32 + e);
    float csum = curl_of<FB>(gl), nseg = 1.0f;
    emit_w<PASS, false>(S, e, ecol, __frcp_rn(csum), 0.0f, FB ? anchor_of<FB>(gl, 0u, e) : is_anchor(S.bits, e));
    float I = 0.0f;
    walk_steps<kWalkBatch, kGradF32, !FB>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, nullptr, S.bits, [&](int a, uint32_t v, const float4 &gv, uint32_t word) {
            float cn = curl_of<FB>(gv);
            I += step_term(a, L, gv, gl);
            csum += cn;
            nseg += 1.0f;
            emit_w<PASS, false>(S, v, ecol, __fdividef(nseg, csum), I, anchor_of<FB>(gv, word, v));
            gl = gv;
        });
}

// Selected method: the state machine of k_sweep_select (K:2280-2537); anchors are the
// segment starts.
template <int PASS, bool FB>
__global__ void __launch_bounds__(kFillThreads, kFillBlocks)
k_anchor_select(Grid g, const LineRec *__restrict__ lines,
                const uint32_t *__restrict__ gbase,
                const uint32_t *__restrict__ desc, long long n_lines,
                const float4 *__restrict__ f32,
                const float *__restrict__ curl, Sink S)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    Walk L;
    L.init(g, r, gbase, desc, li);
    const float thr = g.thr;
    float4 gl = make_float4(0.f, 0.f, 0.f, 0.f);
    if (PASS == kFill) gl = __ldg(f32 + L.v);
    // the field carries curl (.w of its entries): one gather per step in the filling pass
    constexpr bool kW = PASS == kFill;
    float ce = kW ? curl_of<FB>(gl) : __ldg(curl + L.v);
    bool started = !(ce == 0.0f || ce > thr);
    bool paused = false;
    uint32_t start = L.v;
    if (PASS == kMark && started) S.flag[start] = 1;
    uint32_t scol = started ? start_col<PASS>(S, start) : 0u;
    float I = 0.0f, csum = 0.0f, nseg = 0.0f;
    // the filling pass gathers the field (and without FB the anchor bitmap word) of every
    // voxel in batches
    constexpr int kGrad = PASS == kFill ? kGradF32 : kNoGrad;
    walk_steps<kWalkBatch, kGrad, PASS == kFill && !FB>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, nullptr, S.bits, [&](int a, uint32_t v, const float4 &gv, uint32_t word) {
            const float cn = kW ? curl_of<FB>(gv) : __ldg(curl + v);
            if (!started) {
                bool ok = (a == 0) ? (cn != 0.0f && cn < thr) : (cn != 0.0f);
                if (ok) {
                    start = v;
                    if (PASS == kMark) S.flag[start] = 1;
                    scol = start_col<PASS>(S, start);
                    started = true;
                    I = 0.0f; nseg = 0.0f; csum = 0.0f;
                }
            } else {
                bool good = cn < thr && cn != 0.0f;
                if (!paused && good) {
                    if (PASS == kFill)
                        I += step_term(a, L, gv, gl);
                    csum += cn * 1.0e-4f;  // the weights as in k_sweep_select
                    nseg += 1.0f;
                    if (PASS == kFill)
                        emit_w<PASS, false>(S, v, scol, __fdividef(nseg, csum), I, anchor_of<FB>(gv, word, v));
                }
                bool enter_bad = (a == 0) ? ((!paused && cn >= thr) || cn == 0.0f) : (!paused && cn >= thr);
                if (enter_bad) paused = true;
                if (paused && good) {
                    start = v;
                    if (PASS == kMark) S.flag[start] = 1;
                    scol = start_col<PASS>(S, start);
                    I = 0.0f;
                    paused = false;
                    if (a != 2) { nseg = 0.0f; csum = 0.0f; }
                }
            }
            gl = gv;
        });
}

// Selected method: a voxel can start a segment only if it is on the boundary (a line entry)
// or if the voxel before it on some line is "bad" (curl == 0 or curl >= thr): a start
// before the first good voxel follows a voxel that failed the start test, and a restart
// follows a voxel that paused or kept the pause (K:2300-2506); and every start voxel has
// curl != 0.  Flags that superset and counts it into *count.
__global__ void k_select_candidates(Grid g, const float *__restrict__ curl, uint8_t *flag,
                                    unsigned long long *count)
{
    const long long X = g.X, Y = g.Y, Z = g.Z, XY = g.XY;
    unsigned long long local = 0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.V;
         v += (long long)gridDim.x * blockDim.x) {
        long long i = v % X, j = (v / X) % Y, k = v / XY;
        bool c = i == 0 || i == X - 1 || j == 0 || j == Y - 1 || k == 0 || k == Z - 1;
        if (!c) {
            const long long nb[6] = {v - 1, v + 1, v - X, v + X, v - XY, v + XY};
#pragma unroll
            for (int q = 0; q < 6; q++) {
                float cu = __ldg(curl + nb[q]);
                c |= (cu == 0.0f || cu >= g.thr);
            }
        }
        // every start rule needs curl != 0 at the start voxel (the masked interior drops out)
        c = c && __ldg(curl + v) != 0.0f;
        flag[v] = c ? 1 : 0;
        local += c ? 1 : 0;
    }
    for (int o = 16; o; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

__global__ void k_flag_to_u32(long long V, const uint8_t *flag, uint32_t *out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        out[v] = flag[v];
}

// id[v] = position among anchors or -1; vox[id] = v; bits = one bit per voxel.
__global__ void k_assign_ids(long long V, const uint8_t *flag, const uint32_t *pos, int32_t *id, uint32_t *vox,
                             uint32_t *bits)
{
    long long nthr = ((V + 31) / 32) * 32;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nthr;
         v += (long long)gridDim.x * blockDim.x) {
        bool f = v < V && flag[v];
        unsigned b = __ballot_sync(0xffffffffu, f);
        if (v < V) {
            id[v] = f ? (int32_t)pos[v] : -1;
            if (f) vox[pos[v]] = (uint32_t)v;
        }
        if ((threadIdx.x & 31) == 0) bits[v >> 5] = b;
    }
}

__global__ void k_row_capacity(long long n, const uint32_t *vox, const uint32_t *lines_through,
                               unsigned long long *out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = lines_through[vox[i]];
}

// Row sums of the anchor iteration: compensated (Kahan) FP32 per lane, the 32 lane sums
// and the numerator in FP64.  A row gathers about as many terms as lines cross its voxel
// (~1000 at 642 directions); plain FP32 sums of that many terms leave a rounding floor near
// 1e-6 in the iteration's relative change, above the tolerances the solver is asked for.
__device__ __forceinline__ double warp_sum_compensated(float s, float comp)
{
    double d = (double)s - (double)comp;
    for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    return d;
}

// The warp's exact sum of fixed-point lane sums (integer additions: order-independent).
__device__ __forceinline__ long long warp_sum_fixed(long long t)
{
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

__device__ __forceinline__ float anchor_update(double sum, long long row, const float2 *bc,
                                               const uint32_t *vox, const float *p_init, int seed, const float *pc)
{
    const float2 q = bc[row];
    const float cc = q.y;
    double numer = (double)q.x + sum;
    if (seed && p_init) numer += (double)p_init[vox[row]];
    return cc > 0.0f ? (float)(numer / (double)cc) : pc[row];
}

// One anchor iteration, a warp per row.
__global__ void __launch_bounds__(256) k_anchor_spmv(long long n, const unsigned long long *__restrict__ rowptr,
                                                     const uint32_t *__restrict__ rowlen,
                                                     const uint2 *__restrict__ cw, const float2 *__restrict__ bc,
                                                     const uint32_t *__restrict__ vox, const float *__restrict__ p_init,
                                                     int seed, const float *__restrict__ pc, float *__restrict__ pn,
                                                     const int *stop, const double *__restrict__ fix)
{
    if (stop && *stop) return;  // a graph-captured chunk that has met its tolerance
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;  // whole warps
    unsigned long long j0 = rowptr[row], j1 = j0 + rowlen[row];
    double sum;
    if (fix) {  // bit-reproducible: exact fixed-point sum, whatever the entries' order
        const double sr = fix[kFixRow];
        long long t = 0;
        for (unsigned long long j = j0 + lane; j < j1; j += 32) {
            const uint2 q = __ldg(cw + j);
            t += (long long)fix_term(__uint_as_float(q.y) * __ldg(pc + q.x), sr);
        }
        sum = (double)warp_sum_fixed(t) / sr;
    } else {
        float s = 0.0f, comp = 0.0f;
        for (unsigned long long j = j0 + lane; j < j1; j += 32) {
            const uint2 q = __ldg(cw + j);
            kahan_add(s, comp, __uint_as_float(q.y) * __ldg(pc + q.x));
        }
        sum = warp_sum_compensated(s, comp);
    }
    if (lane == 0) pn[row] = anchor_update(sum, row, bc, vox, p_init, seed, pc);
}

// Plain method: every weight is 1, so a row is a plain sum of gathered anchor values.
__global__ void __launch_bounds__(256) k_anchor_spmv_unit(long long n, const unsigned long long *__restrict__ rowptr,
                                                          const uint32_t *__restrict__ rowlen,
                                                          const uint32_t *__restrict__ col, const float2 *__restrict__ bc,
                                                          const uint32_t *__restrict__ vox,
                                                          const float *__restrict__ p_init, int seed,
                                                          const float *__restrict__ pc, float *__restrict__ pn,
                                                          const int *stop, const double *__restrict__ fix)
{
    if (stop && *stop) return;
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;  // whole warps
    unsigned long long j0 = rowptr[row], j1 = j0 + rowlen[row];
    double sum;
    if (fix) {  // bit-reproducible: exact fixed-point sum, whatever the entries' order
        const double sr = fix[kFixRow];
        long long t = 0;
        for (unsigned long long j = j0 + lane; j < j1; j += 32) t += (long long)fix_term(__ldg(pc + __ldg(col + j)), sr);
        sum = (double)warp_sum_fixed(t) / sr;
    } else {
        float s = 0.0f, comp = 0.0f;
        for (unsigned long long j = j0 + lane; j < j1; j += 32) kahan_add(s, comp, __ldg(pc + __ldg(col + j)));
        sum = warp_sum_compensated(s, comp);
    }
    if (lane == 0) pn[row] = anchor_update(sum, row, bc, vox, p_init, seed, pc);
}

constexpr int kRedBlocks = 256, kRedThreads = 256;

__device__ __forceinline__ double block_sum(double x, double *sh)
{
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
    __syncthreads();
    return s;
}

// Sums of (d, p, 1) over the selected entries (for the mean gauge).
__global__ void k_sum_dp(long long n, const float *pc, const float *pn, const uint8_t *mask, double *part,
                         const int *stop)
{
    if (stop && *stop) return;
    __shared__ double sh[32];
    double sd = 0.0, sp = 0.0, cn = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (mask && !mask[i]) continue;
        sd += (double)pn[i] - (double)pc[i];
        sp += (double)pn[i];
        cn += 1.0;
    }
    double a = block_sum(sd, sh), bb = block_sum(sp, sh), cc = block_sum(cn, sh);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = a;
        part[3 * blockIdx.x + 1] = bb;
        part[3 * blockIdx.x + 2] = cc;
    }
}

__global__ void k_finish(const double *part, int nblk, int width, double *out, const int *stop)
{
    if (stop && *stop) return;
    if ((int)threadIdx.x < width) {
        double s = 0.0;
        for (int i = 0; i < nblk; i++) s += part[width * i + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

// Gauged squared change and squared norm over the selected entries: sum (d - sd)^2 and
// sum (p - sp)^2.  The shifts are the reference entry's change and value (point gauge),
// the means (mean gauge: sums[0..2] = sum d, sum p, count) or 0.
__global__ void k_change(long long n, const float *pc, const float *pn, const uint8_t *mask, int gauge,
                         long long ref, const double *sums, double *part, const int *stop)
{
    if (stop && *stop) return;
    __shared__ double sh[32];
    double sd = 0.0, sp = 0.0;
    if (gauge == OMNI3D_GAUGE_POINT && ref >= 0) {
        sp = (double)pn[ref];
        sd = sp - (double)pc[ref];
    } else if (gauge == OMNI3D_GAUGE_MEAN && sums[2] > 0) {
        sd = sums[0] / sums[2];
        sp = sums[1] / sums[2];
    }
    double a = 0.0, bb = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (mask && !mask[i]) continue;
        double d = (double)pn[i] - (double)pc[i] - sd;
        double q = (double)pn[i] - sp;
        a += d * d;
        bb += q * q;
    }
    double ta = block_sum(a, sh), tb = block_sum(bb, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = ta; part[2 * blockIdx.x + 1] = tb; }
}

// The gauged squared change and norm of one anchor iteration in one block (operators of up to
// kChangeBlockMax anchors): the means (mean gauge) in a first pass, then the sums of
// (d - d_mean)^2 and (p - p_mean)^2 -- one kernel instead of four, and one fixed order of
// the sums.  red2 = {change, norm}.  One SM's FP64 rate limits it: at 5.8 K anchors it saves
// 20 us per iteration against the four-kernel form, at 97 K anchors it costs 250 us more.
constexpr long long kChangeBlockMax = 16384;
__global__ void __launch_bounds__(1024) k_change_block(long long n, const float *__restrict__ pc,
                                                       const float *__restrict__ pn, int gauge, long long ref,
                                                       double *red2, const int *stop)
{
    if (stop && *stop) return;
    __shared__ double sh[32];
    __shared__ double shift[2];
    double sd = 0.0, sp = 0.0;
    if (gauge == OMNI3D_GAUGE_POINT && ref >= 0) {
        sp = (double)pn[ref];
        sd = sp - (double)pc[ref];
    } else if (gauge == OMNI3D_GAUGE_MEAN) {
        double a = 0.0, b = 0.0;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) {
            a += (double)pn[i] - (double)pc[i];
            b += (double)pn[i];
        }
        a = block_sum(a, sh);
        b = block_sum(b, sh);
        if (threadIdx.x == 0) {
            shift[0] = n > 0 ? a / (double)n : 0.0;
            shift[1] = n > 0 ? b / (double)n : 0.0;
        }
        __syncthreads();
        sd = shift[0];
        sp = shift[1];
    }
    double x = 0.0, y = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double d = (double)pn[i] - (double)pc[i] - sd;
        const double q = (double)pn[i] - sp;
        x += d * d;
        y += q * q;
    }
    x = block_sum(x, sh);
    y = block_sum(y, sh);
    if (threadIdx.x == 0) {
        red2[0] = x;
        red2[1] = y;
    }
}

// Convergence test of step j of a graph-captured chunk: rel = sqrt(change / norm) (the host
// loop's formula), recorded in rel_out[j]; *stop = j + 1 when rel < tol, which turns the
// chunk's remaining kernels into no-ops.
__global__ void k_converged(const double *red2, double tol, int j, int *stop, double *rel_out)
{
    if (*stop) return;
    const double rel = red2[1] > 0 ? sqrt(red2[0] / red2[1]) : 0.0;
    rel_out[j] = rel;
    if (rel < tol) *stop = j + 1;
}

__global__ void k_scatter(long long n, const uint32_t *vox, const float *pa, float *vol)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        vol[vox[i]] = pa[i];
}

__global__ void k_gather(long long n, const uint32_t *vox, const float *vol, float *pa)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        pa[i] = vol[vox[i]];
}

unsigned grid_for(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 64) b = 152LL * 64;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// b = 0 on every row, c kept (the cached plain operator's refresh).
__global__ void k_clear_b(long long n, float2 *bc)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        bc[i].x = 0.0f;
}

// After the filling pass: each row's length from its next free slot, and (flags = 1) the
// anchor flags cleared from the field entries.
__global__ void k_fill_finish(long long n, const unsigned long long *__restrict__ rowptr,
                              const unsigned long long *__restrict__ next, uint32_t *rowlen, int flags,
                              const uint32_t *__restrict__ vox, float4 *f32)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        rowlen[i] = (uint32_t)(next[i] - rowptr[i]);
        if (flags) {
            uint32_t *u = reinterpret_cast<uint32_t *>(&f32[vox[i]].w);
            *u &= 0x7fffffffu;
        }
    }
}

// Set (set = 1) or clear the anchor flag, the sign bit of .w, in the field entries of the n
// anchors.
__global__ void k_field_flags(long long n, const uint32_t *__restrict__ vox, float4 *f32, int set)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t *u = reinterpret_cast<uint32_t *>(&f32[vox[i]].w);
        *u = set ? (*u | 0x80000000u) : (*u & 0x7fffffffu);
    }
}

// *any = 1 when some curl value has its sign bit set (negative, or -0).
__global__ void k_sign_any(long long V, const float *__restrict__ curl, uint32_t *any)
{
    bool neg = false;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        neg |= (__float_as_uint(curl[v]) >> 31) != 0u;
    if (__any_sync(0xffffffffu, neg) && (threadIdx.x & 31) == 0) *any = 1u;
}

// Launch the pass for the method's accumulation kind.  FB: the anchors are flagged in the
// field (bitmap otherwise).
template <int PASS, bool FB>
void launch_pass(int acc, const Geometry &geo, const Field &f, const Sink &S, cudaStream_t st)
{
    const unsigned blocks = (unsigned)((geo.n_lines + kFillThreads - 1) / kFillThreads);
    const Grid &g = geo.grid;
    if constexpr (PASS == kFill) {
        if (acc == kAccWeightedRawCurl) {
            k_anchor_weighted_raw<kFill, FB><<<blocks, kFillThreads, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                                     geo.n_lines, f.f32, f.curl, S);
            OM_COUNT_LAUNCH();
            return;
        }
        if (acc == kAccWeighted) {
            k_anchor_weighted<kFill, FB><<<blocks, kFillThreads, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines,
                                                                 f.f32, f.curl, S);
            OM_COUNT_LAUNCH();
            return;
        }
        if (acc == kAccPlainNoEntry) {
            k_anchor_plain<kFill, false, FB><<<blocks, kFillThreads, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                                     geo.n_lines, f.f32, S);
            OM_COUNT_LAUNCH();
            return;
        }
    }
    if constexpr (PASS != kRhs) {
        if (acc == kAccSelect) {
            k_anchor_select<PASS, FB><<<blocks, kFillThreads, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines,
                                                              f.f32, f.curl, S);
            OM_COUNT_LAUNCH();
            return;
        }
    }
    // plain method, and the marking pass of every method whose anchors are the entries
    k_anchor_plain<PASS, true, FB><<<blocks, kFillThreads, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines,
                                                           f.f32, S);
    OM_COUNT_LAUNCH();
}

// fb: the anchors' field entries carry the anchor flag (k_field_flags): possible when no
// curl value has its sign bit set.
template <int PASS>
cudaError_t run_pass(const Geometry &geo, const Field &f, int method, bool fb, const Sink &S, cudaStream_t st)
{
    if (geo.n_lines == 0) return cudaSuccess;
    // every pointer the pass dereferences must be set: refuse to launch otherwise
    const bool need_field = PASS == kFill || PASS == kRhs;
    bool ok = geo.d_lines && geo.d_gbase && geo.d_desc;
    if (PASS == kMark) ok = ok && S.flag;
    else ok = ok && S.bits && S.id && S.bc;
    const bool unit_links = method_accum(method) == kAccPlain || method_accum(method) == kAccPlainNoEntry;
    if (PASS == kFill) ok = ok && S.next && (unit_links ? S.col != nullptr : S.cw != nullptr);
    if (need_field) ok = ok && f.f32 != nullptr;
    const int acc = method_accum(method);
    const bool weighted = acc == kAccWeighted || acc == kAccWeightedRawCurl;
    if (acc == kAccSelect || (weighted && PASS == kFill)) ok = ok && f.curl && f.f32;
    if (PASS == kRhs && acc != kAccPlain) ok = false;  // only the plain operator is cached
    if (!ok) return cudaErrorInvalidValue;
    if (PASS == kMark) launch_pass<kMark, false>(acc, geo, f, S, st);  // reads no field
    else if (fb) launch_pass<PASS, true>(acc, geo, f, S, st);
    else launch_pass<PASS, false>(acc, geo, f, S, st);
    return cudaGetLastError();
}

}  // namespace

#define AN_TRY(x)                                                              \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess) {                                               \
            if (err) *err = std::string(#x) + ": " + cudaGetErrorString(e_);   \
            return e_;                                                         \
        }                                                                      \
    } while (0)

size_t change_scratch_doubles();

// Grow-only device buffer: reallocates only when `bytes` exceeds the recorded capacity.
template <typename T>
cudaError_t grow(T *&p, size_t &cap, size_t bytes)
{
    if (bytes == 0) bytes = 1;
    if (bytes <= cap && p) return cudaSuccess;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    return e;
}

void anchor_free(Anchor *A)
{
    cudaFree(A->flag); cudaFree(A->bits); cudaFree(A->id); cudaFree(A->vox); cudaFree(A->rowptr);
    cudaFree(A->col); cudaFree(A->cw); cudaFree(A->bc); cudaFree(A->pa); cudaFree(A->pb);
    cudaFree(A->red); cudaFree(A->rowlen); cudaFree(A->u); cudaFree(A->pos); cudaFree(A->tmp); cudaFree(A->cnt64); cudaFree(A->tmp64);
    cudaFree(A->neg); cudaFree(A->next);
    *A = Anchor();
}

cudaError_t anchor_build(Geometry &geo, const Field &f, int method, long long ref_voxel,
                         long long max_nnz, Anchor *A, cudaStream_t st, std::string *err, Fixed *fx)
{
    const long long V = geo.grid.V;
    size_t *cap = A->cap;
    AN_TRY(grow(A->flag, cap[0], (size_t)V));
    AN_TRY(grow(A->bits, cap[1], sizeof(uint32_t) * (size_t)((V + 31) / 32)));
    AN_TRY(grow(A->id, cap[2], sizeof(int32_t) * (size_t)V));
    AN_TRY(grow(A->u, cap[3], sizeof(uint32_t) * (size_t)V));
    AN_TRY(grow(A->pos, cap[4], sizeof(uint32_t) * (size_t)(V + 1)));
    AN_TRY(grow(A->tmp, cap[5], sizeof(uint32_t) * scan_tmp_elems(V)));
    AN_TRY(grow(A->red, cap[6], sizeof(double) * change_scratch_doubles()));
    Sink S{};
    S.flag = A->flag;
    bool marked = false;
    if (method_accum(method) == kAccSelect) {
        // cheap superset of the segment starts; used when it stays small
        AN_TRY(grow(A->cnt64, cap[8], sizeof(unsigned long long) * 1));
        unsigned long long *dcount = A->cnt64;
        AN_TRY(cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), st));
        k_select_candidates<<<grid_for(V), 256, 0, st>>>(geo.grid, f.curl, A->flag, dcount);
        OM_COUNT_LAUNCH();
        AN_TRY(cudaGetLastError());
        unsigned long long nc = 0;
        AN_TRY(cudaMemcpyAsync(&nc, dcount, sizeof(nc), cudaMemcpyDeviceToHost, st));
        AN_TRY(cudaStreamSynchronize(st));
        marked = (long long)nc <= V / 16;
    }
    if (!marked) {
        AN_TRY(cudaMemsetAsync(A->flag, 0, (size_t)V, st));
        AN_TRY(run_pass<kMark>(geo, f, method, false, S, st));
    }
    if (ref_voxel >= 0 && ref_voxel < V) AN_TRY(cudaMemsetAsync(A->flag + ref_voxel, 1, 1, st));
    // the field carries curl in .w: its sign bit can flag the anchors unless a curl value
    // already has it set
    const bool check_sign = f.curl != nullptr;
    AN_TRY(grow(A->neg, cap[18], sizeof(uint32_t)));
    AN_TRY(cudaMemsetAsync(A->neg, 0, sizeof(uint32_t), st));
    if (check_sign) {
        k_sign_any<<<grid_for(V), 256, 0, st>>>(V, f.curl, A->neg);
        OM_COUNT_LAUNCH();
        AN_TRY(cudaGetLastError());
    }

    k_flag_to_u32<<<grid_for(V), 256, 0, st>>>(V, A->flag, A->u);
    OM_COUNT_LAUNCH();
    AN_TRY(cudaGetLastError());
    AN_TRY(exclusive_scan_u32(A->u, A->pos, V, A->tmp, st));
    uint32_t n = 0, neg = 0;
    AN_TRY(cudaMemcpyAsync(&n, A->pos + V, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AN_TRY(cudaMemcpyAsync(&neg, A->neg, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AN_TRY(cudaStreamSynchronize(st));
    A->n = n;
    const bool fb = neg == 0u;
    AN_TRY(grow(A->vox, cap[7], sizeof(uint32_t) * (size_t)n));
    k_assign_ids<<<grid_for(V), 256, 0, st>>>(V, A->flag, A->pos, A->id, A->vox, A->bits);
    OM_COUNT_LAUNCH();
    AN_TRY(cudaGetLastError());

    // rows: a voxel receives at most one contribution per line through it, so the
    // geometry-only line counts size the rows and no counting pass is needed
    AN_TRY(ensure_lines_through(&geo, st));
    AN_TRY(grow(A->cnt64, cap[8], sizeof(unsigned long long) * (size_t)n));
    AN_TRY(grow(A->tmp64, cap[9], sizeof(unsigned long long) * scan_tmp_elems(n)));
    AN_TRY(grow(A->rowptr, cap[10], sizeof(unsigned long long) * (size_t)(n + 1)));
    k_row_capacity<<<grid_for(n), 256, 0, st>>>(n, A->vox, geo.d_lines_through, A->cnt64);
    OM_COUNT_LAUNCH();
    AN_TRY(cudaGetLastError());
    AN_TRY(exclusive_scan_u64(A->cnt64, A->rowptr, n, A->tmp64, st));
    unsigned long long nnz = 0;
    AN_TRY(cudaMemcpyAsync(&nnz, A->rowptr + n, sizeof(nnz), cudaMemcpyDeviceToHost, st));
    AN_TRY(cudaStreamSynchronize(st));
    A->nnz = (long long)nnz;
    if (max_nnz >= 0 && (long long)nnz > max_nnz) {
        if (err) *err = "anchor operator larger than its limit";
        return cudaErrorNotSupported;
    }

    const bool unit_links = method_accum(method) == kAccPlain || method_accum(method) == kAccPlainNoEntry;
    if (unit_links) AN_TRY(grow(A->col, cap[11], sizeof(uint32_t) * (size_t)nnz));
    else AN_TRY(grow(A->cw, cap[12], sizeof(uint2) * (size_t)nnz));
    AN_TRY(grow(A->bc, cap[13], sizeof(float2) * (size_t)n));
    AN_TRY(grow(A->pa, cap[15], sizeof(float) * (size_t)n));
    AN_TRY(grow(A->pb, cap[16], sizeof(float) * (size_t)n));
    AN_TRY(grow(A->rowlen, cap[17], sizeof(uint32_t) * (size_t)n));
    AN_TRY(grow(A->next, cap[19], sizeof(unsigned long long) * (size_t)std::max<long long>(n, 1)));
    if (n) AN_TRY(cudaMemcpyAsync(A->next, A->rowptr, sizeof(unsigned long long) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    AN_TRY(cudaMemsetAsync(A->bc, 0, sizeof(float2) * (size_t)std::max<long long>(n, 1), st));
    S.bits = A->bits;
    S.id = A->id;
    S.next = A->next;
    S.col = unit_links ? A->col : nullptr;
    S.cw = unit_links ? nullptr : A->cw;
    S.bc = A->bc;
    if (fx) {  // bit-reproducible: the rows' (b, c) in fixed point (scales set by the caller)
        AN_TRY(grow(fx->bc64, fx->cap_bc64, sizeof(long long) * 2 * (size_t)std::max<long long>(n, 1)));
        AN_TRY(cudaMemsetAsync(fx->bc64, 0, sizeof(long long) * 2 * (size_t)std::max<long long>(n, 1), st));
        S.bc64 = fx->bc64;
        S.fix = fx->scale;
    }
    if (fb && n) {
        k_field_flags<<<grid_for(n), 256, 0, st>>>(n, A->vox, f.f32, 1);
        OM_COUNT_LAUNCH();
        AN_TRY(cudaGetLastError());
    }
    AN_TRY(run_pass<kFill>(geo, f, method, fb, S, st));
    if (fx) AN_TRY(fix_rows_to_float(n, *fx, A->bc, false, st));
    if (n) {  // row lengths; the sweeps read the field unflagged
        k_fill_finish<<<grid_for(n), 256, 0, st>>>(n, A->rowptr, A->next, A->rowlen, fb ? 1 : 0, A->vox, f.f32);
        OM_COUNT_LAUNCH();
        AN_TRY(cudaGetLastError());
    }
    A->unit_weights = method_accum(method) == kAccPlain || method_accum(method) == kAccPlainNoEntry;
    return cudaGetLastError();
}

size_t change_scratch_doubles() { return 8 + 3 * kRedBlocks; }

cudaError_t change_sums(long long n, const float *pc, const float *pn, int gauge, long long ref, double *scratch,
                        double *out2, cudaStream_t st, const uint8_t *mask, const int *stop)
{
    double *part = scratch + 8;
    if (gauge == OMNI3D_GAUGE_MEAN) {
        k_sum_dp<<<kRedBlocks, kRedThreads, 0, st>>>(n, pc, pn, mask, part, stop);
        OM_COUNT_LAUNCH();
        k_finish<<<1, 32, 0, st>>>(part, kRedBlocks, 3, scratch + 4, stop);
        OM_COUNT_LAUNCH();
    }
    k_change<<<kRedBlocks, kRedThreads, 0, st>>>(n, pc, pn, mask, gauge, ref, scratch + 4, part, stop);
    OM_COUNT_LAUNCH();
    k_finish<<<1, 32, 0, st>>>(part, kRedBlocks, 2, out2, stop);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t anchor_mark(const Geometry &geo, const Field &f, int method, long long ref_voxel,
                        uint8_t *flag, unsigned long long *count1, cudaStream_t st)
{
    const long long V = geo.grid.V;
    cudaError_t e;
    bool marked = false;
    if (method_accum(method) == kAccSelect) {
        e = cudaMemsetAsync(count1, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) return e;
        k_select_candidates<<<grid_for(V), 256, 0, st>>>(geo.grid, f.curl, flag, count1);
        OM_COUNT_LAUNCH();
        unsigned long long nc = 0;
        e = cudaMemcpyAsync(&nc, count1, sizeof(nc), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        marked = (long long)nc <= V / 16;
    }
    if (!marked) {
        e = cudaMemsetAsync(flag, 0, (size_t)V, st);
        if (e != cudaSuccess) return e;
        Sink S{};
        S.flag = flag;
        e = run_pass<kMark>(geo, f, method, false, S, st);
        if (e != cudaSuccess) return e;
    }
    if (ref_voxel >= 0 && ref_voxel < geo.grid.V) e = cudaMemsetAsync(flag + ref_voxel, 1, 1, st);
    return e;
}

cudaError_t anchor_step(const Anchor &A, const float *p_init, bool seed, int gauge, long long ref_anchor,
                        const float *p_cur, float *p_next, double *red2, cudaStream_t st, const int *stop,
                        const Fixed *fx)
{
    if (A.n == 0) return cudaSuccess;
    long long threads = A.n * 32;
    const double *fix = nullptr;
    if (fx) {  // bit-reproducible: the row sums' scale from this iterate's largest value
        cudaError_t e = fix_row_scale(A.n, p_cur, *fx, st, stop);
        if (e != cudaSuccess) return e;
        fix = fx->scale;
    }
    if (A.unit_weights)
        k_anchor_spmv_unit<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(A.n, A.rowptr, A.rowlen, A.col, A.bc, A.vox,
                                                                               p_init, seed ? 1 : 0, p_cur, p_next, stop,
                                                                               fix);
    else
        k_anchor_spmv<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(A.n, A.rowptr, A.rowlen, A.cw, A.bc,
                                                                          A.vox, p_init, seed ? 1 : 0, p_cur, p_next,
                                                                          stop, fix);
    OM_COUNT_LAUNCH();
    if (red2 && A.n <= kChangeBlockMax) {
        k_change_block<<<1, 1024, 0, st>>>(A.n, p_cur, p_next, gauge, ref_anchor, red2, stop);
        OM_COUNT_LAUNCH();
    } else if (red2) {
        return change_sums(A.n, p_cur, p_next, gauge, ref_anchor, A.red, red2, st, nullptr, stop);
    }
    return cudaGetLastError();
}

cudaError_t converged_test_launch(const double *red2, double tol, int j, int *stop, double *rel_out,
                                  cudaStream_t st)
{
    k_converged<<<1, 1, 0, st>>>(red2, tol, j, stop, rel_out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t anchor_refresh_rhs(const Geometry &geo, const Field &f, Anchor *A, cudaStream_t st,
                               const Fixed *fx)
{
    if (A->n == 0) return cudaSuccess;
    if (fx && (!fx->bc64 || fx->cap_bc64 < sizeof(long long) * 2 * (size_t)A->n)) return cudaErrorInvalidValue;
    k_clear_b<<<grid_for(A->n), 256, 0, st>>>(A->n, A->bc);
    OM_COUNT_LAUNCH();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    Sink S{};
    S.bits = A->bits;
    S.id = A->id;
    S.bc = A->bc;
    if (fx) {
        if ((e = cudaMemsetAsync(fx->bc64, 0, sizeof(long long) * 2 * (size_t)A->n, st)) != cudaSuccess) return e;
        S.bc64 = fx->bc64;
        S.fix = fx->scale;
    }
    // the plain method's field carries no curl (.w = +0), so the anchors can be flagged in it
    const bool fb = f.curl == nullptr;
    if (fb) {
        k_field_flags<<<grid_for(A->n), 256, 0, st>>>(A->n, A->vox, f.f32, 1);
        OM_COUNT_LAUNCH();
    }
    e = run_pass<kRhs>(geo, f, OMNI3D_METHOD_PLAIN, fb, S, st);
    if (e == cudaSuccess && fx) e = fix_rows_to_float(A->n, *fx, A->bc, true, st);
    if (e != cudaSuccess || !fb) return e;
    k_field_flags<<<grid_for(A->n), 256, 0, st>>>(A->n, A->vox, f.f32, 0);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t anchor_scatter(const Anchor &A, const float *pa, float *vol, cudaStream_t st)
{
    if (A.n == 0) return cudaSuccess;
    k_scatter<<<grid_for(A.n), 256, 0, st>>>(A.n, A.vox, pa, vol);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t anchor_gather(const Anchor &A, const float *vol, float *pa, cudaStream_t st)
{
    if (A.n == 0) return cudaSuccess;
    k_gather<<<grid_for(A.n), 256, 0, st>>>(A.n, A.vox, vol, pa);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

}  // namespace omni3d
