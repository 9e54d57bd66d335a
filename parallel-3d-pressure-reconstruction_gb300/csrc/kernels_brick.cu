// Brick-staged omni sweep.
//
// The line-major sweep (kernels_sweep.cu) gathers the gradient and reduces into the
// accumulators through L2 once per voxel visit.  This engine instead cuts every traced line
// at the boundaries of 16^3 voxel bricks and processes the volume brick by brick: the
// brick's gradient record (ax, ay, az, curl), with a one-voxel halo, is staged into shared
// memory by one TMA tensor copy, and all line segments crossing the brick are walked there.
// What a segment needs from the earlier part of its line -- the running integral, the
// curl-weight sums, the segment start of the selected method -- is carried in by three
// passes:
//   B1  per brick: each segment's summary (the change of the line state across it),
//   L   per line: the summaries composed in line order into each segment's carry-in state,
//   B2  per brick: the segments re-walked from their carry-in states, contributions added
//       to the brick's (pn, count) in shared memory, the brick flushed once to the volume.
// B1 and L depend only on the field, so a solve runs them once and B2 once per sweep.
//
// Segment record (two uint4, brick-major, grouped by brick):
//   a.x  line-major segment id (segments of a line are numbered consecutively)
//   a.y  bits 0-11: first voxel in brick coordinates (x | y << 4 | z << 8);
//        bits 12-17: voxels in the segment (1..46); bits 18-20: step signs (+1 if set)
//        per axis; bit 21: the segment starts at the line entry
//   a.z  line entry voxel (linear index)
//   a.w, b.x, b.y  2-bit steps into the segment's voxels (the entry voxel has none), 16 per word
//   b.z  line index
// A staircase moves monotonically along every axis, so a line visits each brick at most
// once and a segment holds at most 16 + 15 + 15 = 46 voxels.  Within a brick the records
// are ordered by segment length (a counting sort over (brick, voxels)), so the 32 lanes of a
// warp walk segments of equal length and the walk loop does not diverge.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <vector>

#include "omni3d_internal.h"

namespace omni3d {

namespace {

constexpr int kB = 16;                   // brick edge
constexpr int kP = kB + 2;               // padded edge (halo of one voxel)
constexpr int kP2 = kP * kP;
constexpr int kP3 = kP * kP * kP;
constexpr int kFieldBytes = kP3 * 16;    // float4 per padded voxel: 93,312 B
constexpr int kAccBytes = kB * kB * kB * 8;  // float2 per brick voxel: 32,768 B
constexpr int kThreads = 1024;
constexpr long long kSpinLimit = 1ll << 24;  // mbarrier polls before a wait gives up

__device__ __forceinline__ float sel3(int a, float x, float y, float z)
{
    return a == 0 ? x : (a == 1 ? y : z);
}

__device__ __forceinline__ int sel3i(int a, int x, int y, int z)
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

// ------------------------------------------------------------------ TMA and mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of the barrier: false if it did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    for (long long i = 0; i < kSpinLimit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// One 4-D tile (4 floats x 18 x 18 x 18 voxels) of the float4 field into shared memory.
__device__ __forceinline__ void tma_load_brick(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y,
                                               int z)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ------------------------------------------------------------------ segment building
struct LineStart {
    int i, j, k;          // entry voxel coordinates
    int si, sj, sk;       // step signs
    int m;
    const uint32_t *dp;
};

__device__ __forceinline__ LineStart line_start(const Grid &g, const LineRec &r, const uint32_t *gbase,
                                                const uint32_t *desc, long long li)
{
    LineStart s;
    s.i = (int)(r.e % (uint32_t)g.X);
    s.j = (int)((r.e / (uint32_t)g.X) % (uint32_t)g.Y);
    s.k = (int)(r.e / (uint32_t)g.XY);
    int ix = (int)(r.x % (uint32_t)g.X), jx = (int)((r.x / (uint32_t)g.X) % (uint32_t)g.Y),
        kx = (int)(r.x / (uint32_t)g.XY);
    s.si = ix > s.i ? 1 : -1;
    s.sj = jx > s.j ? 1 : -1;
    s.sk = kx > s.k ? 1 : -1;
    s.m = r.m;
    s.dp = desc + 32ull * gbase[li >> 5] + (li & 31);
    return s;
}

// Does a step of sign s that ends at coordinate c cross a brick boundary?
__device__ __forceinline__ bool crossed(int c, int s)
{
    return s > 0 ? (c & (kB - 1)) == 0 : (c & (kB - 1)) == kB - 1;
}

// Counting key of a segment: (brick, voxels in the segment), voxels < 64.
constexpr int kLenKeys = 64;

__device__ __forceinline__ long long seg_key(int i, int j, int k, int nbx, int nby, int nv)
{
    return ((i >> 4) + (long long)(j >> 4) * nbx + (long long)(k >> 4) * nbx * nby) * kLenKeys + nv;
}

__global__ void __launch_bounds__(256) k_seg_count(Grid g, const LineRec *__restrict__ lines,
                                                   const uint32_t *__restrict__ gbase,
                                                   const uint32_t *__restrict__ desc, long long n_lines, int nbx,
                                                   int nby, uint32_t *key_count, uint32_t *line_nseg)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    LineStart L = line_start(g, r, gbase, desc, li);
    int i = L.i, j = L.j, k = L.k;
    uint32_t nseg = 1;
    int nv = 1;
    for (int s0 = 0; s0 < L.m; s0 += 16) {
        uint32_t w = __ldg(L.dp + 32 * (s0 >> 4));
        int n = min(16, L.m - s0);
        for (int t = 0; t < n; t++, w >>= 2) {
            int a = (int)(w & 3u);
            bool cr;
            if (a == 0) { i += L.si; cr = crossed(i, L.si); }
            else if (a == 1) { j += L.sj; cr = crossed(j, L.sj); }
            else { k += L.sk; cr = crossed(k, L.sk); }
            if (cr) {
                // close the segment in the brick just left
                int pi = i, pj = j, pk = k;
                if (a == 0) pi -= L.si; else if (a == 1) pj -= L.sj; else pk -= L.sk;
                atomicAdd(key_count + seg_key(pi, pj, pk, nbx, nby, nv), 1u);
                nseg++;
                nv = 0;
            }
            nv++;
        }
    }
    atomicAdd(key_count + seg_key(i, j, k, nbx, nby, nv), 1u);
    line_nseg[li] = nseg;
}

struct SegOut {
    uint4 *rec;
    const uint32_t *key_off;   // first slot of every (brick, length) key
    uint32_t *cursor;
    const uint32_t *line_seg;
    int nbx, nby;
};

__device__ __forceinline__ void emit_segment(const SegOut &O, int fi, int fj, int fk, int nv, int signs, int first_entry,
                                             uint32_t entry, const uint32_t w[3], uint32_t id, uint32_t line)
{
    const long long key = seg_key(fi, fj, fk, O.nbx, O.nby, nv);
    uint32_t slot = O.key_off[key] + atomicAdd(O.cursor + key, 1u);
    uint4 ra, rb;
    ra.x = id;
    ra.y = (uint32_t)((fi & 15) | ((fj & 15) << 4) | ((fk & 15) << 8)) | ((uint32_t)nv << 12) |
           ((uint32_t)signs << 18) | ((uint32_t)first_entry << 21);
    ra.z = entry;
    ra.w = w[0];
    rb.x = w[1];
    rb.y = w[2];
    rb.z = line;
    rb.w = 0;
    O.rec[2ull * slot] = ra;
    O.rec[2ull * slot + 1] = rb;
}

__global__ void __launch_bounds__(256) k_seg_fill(Grid g, const LineRec *__restrict__ lines,
                                                  const uint32_t *__restrict__ gbase,
                                                  const uint32_t *__restrict__ desc, long long n_lines, SegOut O)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    LineStart L = line_start(g, r, gbase, desc, li);
    const int signs = (L.si > 0 ? 1 : 0) | (L.sj > 0 ? 2 : 0) | (L.sk > 0 ? 4 : 0);
    int i = L.i, j = L.j, k = L.k;
    int fi = i, fj = j, fk = k;  // first voxel of the open segment
    int nv = 1, ns = 0, first_entry = 1;
    uint32_t w3[3] = {0u, 0u, 0u};
    uint32_t id = O.line_seg[li];
    for (int s0 = 0; s0 < L.m; s0 += 16) {
        uint32_t w = __ldg(L.dp + 32 * (s0 >> 4));
        int n = min(16, L.m - s0);
        for (int t = 0; t < n; t++, w >>= 2) {
            int a = (int)(w & 3u);
            bool cr;
            if (a == 0) { i += L.si; cr = crossed(i, L.si); }
            else if (a == 1) { j += L.sj; cr = crossed(j, L.sj); }
            else { k += L.sk; cr = crossed(k, L.sk); }
            if (cr) {
                emit_segment(O, fi, fj, fk, nv, signs, first_entry, r.e, w3, id, (uint32_t)li);
                id++;
                fi = i; fj = j; fk = k;
                nv = 0; ns = 0; first_entry = 0;
                w3[0] = w3[1] = w3[2] = 0u;
            }
            // the step into the current voxel
            int pos = 2 * ns;
            uint32_t bits = (uint32_t)a << (pos & 31);
            if (pos < 32) w3[0] |= bits; else if (pos < 64) w3[1] |= bits; else w3[2] |= bits;
            ns++;
            nv++;
        }
    }
    emit_segment(O, fi, fj, fk, nv, signs, first_entry, r.e, w3, id, (uint32_t)li);
}

// ------------------------------------------------------------------ segment decoding
struct SegWalk {
    uint32_t id, entry, w0, w1, w2;
    int cur;         // padded index of the voxel before the first step
    int acur;        // brick index (0..4095) of that voxel (meaningless for halo voxels)
    int ns;          // steps in the segment
    int first_entry;
    int p0, p1, p2;  // signed padded strides per axis
    int q0, q1, q2;  // signed brick strides per axis
    float h0, h1, h2;  // -rho * sign * spacing / 2 per axis

    __device__ __forceinline__ void init(const Grid &g, const uint4 &ra, const uint4 &rb)
    {
        id = ra.x;
        entry = ra.z;
        w0 = ra.w;
        w1 = rb.x;
        w2 = rb.y;
        const uint32_t bits = ra.y;
        const int lx = bits & 15, ly = (bits >> 4) & 15, lz = (bits >> 8) & 15;
        const int nv = (bits >> 12) & 63;
        const int sg = (bits >> 18) & 7;
        first_entry = (bits >> 21) & 1;
        ns = nv - first_entry;
        const int s0 = (sg & 1) ? 1 : -1, s1 = (sg & 2) ? 1 : -1, s2 = (sg & 4) ? 1 : -1;
        p0 = s0; p1 = s1 * kP; p2 = s2 * kP2;
        q0 = s0; q1 = s1 * kB; q2 = s2 * kB * kB;
        h0 = __fmul_rn(-g.rho * (float)s0, g.dx) * 0.5f;
        h1 = __fmul_rn(-g.rho * (float)s1, g.dy) * 0.5f;
        h2 = __fmul_rn(-g.rho * (float)s2, g.dz) * 0.5f;
        cur = (lz + 1) * kP2 + (ly + 1) * kP + (lx + 1);
        acur = lz * kB * kB + ly * kB + lx;
        if (!first_entry) {
            const int a0 = (int)(w0 & 3u);
            cur -= pst(a0);
            acur -= ast(a0);
        }
    }
    __device__ __forceinline__ uint32_t word(int t0) const { return t0 == 0 ? w0 : (t0 == 16 ? w1 : w2); }
    __device__ __forceinline__ int pst(int a) const { return sel3i(a, p0, p1, p2); }
    __device__ __forceinline__ int ast(int a) const { return sel3i(a, q0, q1, q2); }
    __device__ __forceinline__ float h(int a) const { return sel3(a, h0, h1, h2); }
};

// Linear voxel index of a padded brick index.
__device__ __forceinline__ uint32_t global_of(const Grid &g, int bx, int by, int bz, int q)
{
    const int pz = q / kP2, py = (q / kP) % kP, px = q % kP;
    return (uint32_t)((bx * kB + px - 1) + (long long)(by * kB + py - 1) * g.X + (long long)(bz * kB + pz - 1) * g.XY);
}

// Selected-method state machine (the rules of k_sweep_select).
enum Mode : uint32_t { kNotStarted = 0, kRunning = 1, kPaused = 2 };

struct SelState {
    uint32_t mode;
    bool restarted, reset;
    int start;        // padded brick index of the last (re)start inside the segment
    float I, comp, csum;
    int nseg;
};

__device__ __forceinline__ void sel_init_variant(SelState &s, uint32_t mode)
{
    s.mode = mode;
    s.restarted = false;
    s.reset = false;
    s.start = 0;
    s.I = s.comp = s.csum = 0.0f;
    s.nseg = 0;
}

// One step into padded voxel q (axis a, curl cn, trapezoid term t) for a B1 variant.
__device__ __forceinline__ void sel_step(SelState &s, int a, float cn, float t, float thr, int q)
{
    if (s.mode == kNotStarted) {
        bool ok = (a == 0) ? (cn != 0.0f && cn < thr) : (cn != 0.0f);
        if (ok) {
            s.mode = kRunning;
            s.restarted = true;
            s.reset = true;
            s.start = q;
            s.I = s.comp = s.csum = 0.0f;
            s.nseg = 0;
        }
        return;
    }
    bool paused = s.mode == kPaused;
    bool good = cn < thr && cn != 0.0f;
    if (!paused && good) {
        kahan_add(s.I, s.comp, t);
        s.csum += cn * 1.0e-4f;
        s.nseg += 1;
    }
    bool enter_bad = (a == 0) ? ((!paused && cn >= thr) || cn == 0.0f) : (!paused && cn >= thr);
    if (enter_bad) paused = true;
    if (paused && good) {
        s.start = q;
        s.restarted = true;
        s.I = s.comp = 0.0f;
        paused = false;
        if (a != 2) {
            s.csum = 0.0f;
            s.nseg = 0;
            s.reset = true;
        }
    }
    s.mode = paused ? kPaused : kRunning;
}

__device__ __forceinline__ uint4 sel_pack(const SelState &s, const Grid &g, int bx, int by, int bz)
{
    uint4 o;
    o.x = s.mode | ((uint32_t)s.restarted << 2) | ((uint32_t)s.reset << 3) | ((uint32_t)s.nseg << 4);
    o.y = s.restarted ? global_of(g, bx, by, bz, s.start) : 0u;
    o.z = __float_as_uint(s.I);
    o.w = __float_as_uint(s.csum);
    return o;
}

struct BrickArgs {
    Grid g;
    int nbx, nby, nbz;
    const uint4 *rec;
    const uint4 *items;      // x = brick, y = first segment, z = end segment (brick-major)
    uint32_t n_items;
    uint32_t *work;          // work counter (zeroed before the launch)
    int *err;                // set when a TMA wait gave up
    void *summ;              // B1 output (line-major)
    const void *carry;       // B2 input (line-major)
    const float *p;          // B2: values read at line entries / segment starts
    float2 *pncnt;           // B2: accumulators of the volume
};

// B1: per-segment summaries.
template <int METHOD>
__device__ __forceinline__ void b1_segment(const BrickArgs &A, const float4 *F, const uint4 &ra, const uint4 &rb,
                                           int bx, int by, int bz)
{
    SegWalk W;
    W.init(A.g, ra, rb);
    const float thr = A.g.thr;
    int cur = W.cur;
    float4 gl = F[cur];
    if (METHOD == OMNI3D_METHOD_SELECT) {
        SelState v[3];
        int nvar = 3;
        if (W.first_entry) {
            // the line's own start test at the entry (ce <= thr and nonzero), then the walk
            nvar = 1;
            sel_init_variant(v[0], kNotStarted);
            const float ce = gl.w;
            if (!(ce == 0.0f || ce > thr)) {
                v[0].mode = kRunning;
                v[0].restarted = true;
                v[0].reset = true;
                v[0].start = cur;  // the entry voxel
            }
        } else {
            sel_init_variant(v[0], kNotStarted);
            sel_init_variant(v[1], kRunning);
            sel_init_variant(v[2], kPaused);
        }
        for (int t0 = 0; t0 < W.ns; t0 += 16) {
            uint32_t w = W.word(t0);
            const int n = min(16, W.ns - t0);
            for (int t = 0; t < n; t++, w >>= 2) {
                const int a = (int)(w & 3u);
                const int nxt = cur + W.pst(a);
                const float4 gv = F[nxt];
                const float term = W.h(a) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z));
                sel_step(v[0], a, gv.w, term, thr, nxt);
                if (nvar == 3) {
                    sel_step(v[1], a, gv.w, term, thr, nxt);
                    sel_step(v[2], a, gv.w, term, thr, nxt);
                }
                gl = gv;
                cur = nxt;
            }
        }
        uint4 *S = reinterpret_cast<uint4 *>(A.summ) + 3ull * W.id;
        S[0] = sel_pack(v[0], A.g, bx, by, bz);
        if (nvar == 3) {
            S[1] = sel_pack(v[1], A.g, bx, by, bz);
            S[2] = sel_pack(v[2], A.g, bx, by, bz);
        }
    } else {
        float I = 0.0f, comp = 0.0f, csum = 0.0f;
        for (int t0 = 0; t0 < W.ns; t0 += 16) {
            uint32_t w = W.word(t0);
            const int n = min(16, W.ns - t0);
            for (int t = 0; t < n; t++, w >>= 2) {
                const int a = (int)(w & 3u);
                const int nxt = cur + W.pst(a);
                const float4 gv = F[nxt];
                kahan_add(I, comp, W.h(a) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z)));
                if (METHOD == OMNI3D_METHOD_WEIGHTED) csum += __fdiv_rn(gv.w, 1.0e4f);
                gl = gv;
                cur = nxt;
            }
        }
        if (METHOD == OMNI3D_METHOD_WEIGHTED)
            reinterpret_cast<float4 *>(A.summ)[W.id] = make_float4(I, csum, (float)W.ns, 0.0f);
        else
            reinterpret_cast<float *>(A.summ)[W.id] = I;
    }
}

// B2: contributions of one segment into the brick accumulators.
template <int METHOD>
__device__ __forceinline__ void b2_segment(const BrickArgs &A, const float4 *F, float2 *acc, const uint4 &ra,
                                           const uint4 &rb, int bx, int by, int bz)
{
    SegWalk W;
    W.init(A.g, ra, rb);
    const float thr = A.g.thr;
    int cur = W.cur, acur = W.acur;
    float4 gl = F[cur];
    if (METHOD == OMNI3D_METHOD_PLAIN) {
        const float pe = __ldg(A.p + W.entry);
        float I = reinterpret_cast<const float *>(A.carry)[W.id], comp = 0.0f;
        if (W.first_entry) {
            atomicAdd(&acc[acur].x, pe);
            atomicAdd(&acc[acur].y, 1.0f);
        }
        for (int t0 = 0; t0 < W.ns; t0 += 16) {
            uint32_t w = W.word(t0);
            const int n = min(16, W.ns - t0);
            for (int t = 0; t < n; t++, w >>= 2) {
                const int a = (int)(w & 3u);
                cur += W.pst(a);
                acur += W.ast(a);
                const float4 gv = F[cur];
                kahan_add(I, comp, W.h(a) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z)));
                atomicAdd(&acc[acur].x, pe + I);
                atomicAdd(&acc[acur].y, 1.0f);
                gl = gv;
            }
        }
    } else if (METHOD == OMNI3D_METHOD_WEIGHTED) {
        const float pe = __ldg(A.p + W.entry);
        const float4 c = reinterpret_cast<const float4 *>(A.carry)[W.id];
        float I = c.x, comp = 0.0f, csum = c.y, nseg = c.z;
        for (int t0 = 0; t0 < W.ns; t0 += 16) {
            uint32_t w = W.word(t0);
            const int n = min(16, W.ns - t0);
            for (int t = 0; t < n; t++, w >>= 2) {
                const int a = (int)(w & 3u);
                cur += W.pst(a);
                acur += W.ast(a);
                const float4 gv = F[cur];
                kahan_add(I, comp, W.h(a) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z)));
                csum += __fdiv_rn(gv.w, 1.0e4f);
                nseg += 1.0f;
                if (csum != 0.0f) {
                    const float wc = __fdividef(nseg, csum);
                    atomicAdd(&acc[acur].x, (pe + I) * wc);
                    atomicAdd(&acc[acur].y, wc);
                }
                gl = gv;
            }
        }
    } else {  // selected method
        bool started, paused;
        float p0 = 0.0f, I = 0.0f, comp = 0.0f, csum = 0.0f, nseg = 0.0f;
        if (W.first_entry) {
            const float ce = gl.w;
            started = !(ce == 0.0f || ce > thr);
            paused = false;
            if (started) p0 = __ldg(A.p + W.entry);
        } else {
            const uint4 c = reinterpret_cast<const uint4 *>(A.carry)[W.id];
            const uint32_t mode = c.x & 3u;
            started = mode != kNotStarted;
            paused = mode == kPaused;
            nseg = (float)(c.x >> 2);
            if (started) p0 = __ldg(A.p + c.y);
            I = __uint_as_float(c.z);
            csum = __uint_as_float(c.w);
        }
        for (int t0 = 0; t0 < W.ns; t0 += 16) {
            uint32_t w = W.word(t0);
            const int n = min(16, W.ns - t0);
            for (int t = 0; t < n; t++, w >>= 2) {
                const int a = (int)(w & 3u);
                cur += W.pst(a);
                acur += W.ast(a);
                const float4 gv = F[cur];
                const float cn = gv.w;
                if (!started) {
                    bool ok = (a == 0) ? (cn != 0.0f && cn < thr) : (cn != 0.0f);
                    if (ok) {
                        p0 = __ldg(A.p + global_of(A.g, bx, by, bz, cur));
                        started = true;
                        I = 0.0f; comp = 0.0f; nseg = 0.0f; csum = 0.0f;
                    }
                } else {
                    const bool good = cn < thr && cn != 0.0f;
                    if (!paused && good) {
                        kahan_add(I, comp, W.h(a) *
                                               (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z)));
                        csum += cn * 1.0e-4f;
                        nseg += 1.0f;
                        const float wc = __fdividef(nseg, csum);
                        atomicAdd(&acc[acur].x, (p0 + I) * wc);
                        atomicAdd(&acc[acur].y, wc);
                    }
                    const bool enter_bad = (a == 0) ? ((!paused && cn >= thr) || cn == 0.0f) : (!paused && cn >= thr);
                    if (enter_bad) paused = true;
                    if (paused && good) {
                        p0 = __ldg(A.p + global_of(A.g, bx, by, bz, cur));
                        I = 0.0f; comp = 0.0f;
                        paused = false;
                        if (a != 2) { nseg = 0.0f; csum = 0.0f; }
                    }
                }
                gl = gv;
            }
        }
    }
}

// One pass over the bricks: PHASE 1 = summaries, PHASE 2 = accumulation.  Persistent CTAs
// take (brick, segment range) items from a counter; each item stages its brick by TMA.
template <int METHOD, int PHASE>
__global__ void __launch_bounds__(kThreads, 1) k_brick(const __grid_constant__ CUtensorMap fmap, BrickArgs A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // the TMA destination on a 128-byte boundary (the launch adds 128 bytes of slack)
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float4 *F = reinterpret_cast<float4 *>(smem);
    float2 *acc = reinterpret_cast<float2 *>(smem + kFieldBytes);
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_item;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    uint32_t parity = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(A.work, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= A.n_items) break;
        const uint4 it = A.items[item];
        const int bx = (int)(it.x % (uint32_t)A.nbx), by = (int)((it.x / (uint32_t)A.nbx) % (uint32_t)A.nby),
                  bz = (int)(it.x / ((uint32_t)A.nbx * (uint32_t)A.nby));
        if (threadIdx.x == 0) {
            mbar_expect_tx(&bar, kFieldBytes);
            tma_load_brick(F, &fmap, &bar, bx * kB - 1, by * kB - 1, bz * kB - 1);
        }
        if (PHASE == 2)
            for (int q = threadIdx.x; q < kB * kB * kB; q += blockDim.x) acc[q] = make_float2(0.0f, 0.0f);
        const bool ok = mbar_wait(&bar, parity);
        parity ^= 1u;
        if (!__syncthreads_and(ok)) {
            // the copy did not arrive: report, wait (bounded) for it to land, and stop
            if (threadIdx.x == 0) {
                atomicExch(A.err, 1);
                mbar_wait(&bar, parity ^ 1u);
            }
            return;
        }
        for (uint32_t s = it.y + threadIdx.x; s < it.z; s += blockDim.x) {
            const uint4 ra = __ldg(A.rec + 2ull * s), rb = __ldg(A.rec + 2ull * s + 1);
            if (PHASE == 1) b1_segment<METHOD>(A, F, ra, rb, bx, by, bz);
            else b2_segment<METHOD>(A, F, acc, ra, rb, bx, by, bz);
        }
        __syncthreads();
        if (PHASE == 2) {
            for (int q = threadIdx.x; q < kB * kB * kB; q += blockDim.x) {
                const float2 v = acc[q];
                if (v.x == 0.0f && v.y == 0.0f) continue;
                const int x = bx * kB + (q & 15), y = by * kB + ((q >> 4) & 15), z = bz * kB + (q >> 8);
                if (x >= A.g.X || y >= A.g.Y || z >= A.g.Z) continue;
                atomicAdd(A.pncnt + (x + (long long)y * A.g.X + (long long)z * A.g.XY), v);
            }
        }
        fence_proxy_async();  // generic reads of F before the next copy overwrites it
        __syncthreads();
    }
}

// L: compose the summaries of each line's segments in line order into carry-in states.
template <int METHOD>
__global__ void __launch_bounds__(256) k_line_carry(long long n_lines, const uint32_t *__restrict__ line_seg,
                                                   const void *__restrict__ summ, void *carry)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    const uint32_t s0 = line_seg[li], s1 = line_seg[li + 1];
    if (METHOD == OMNI3D_METHOD_PLAIN) {
        const float *S = reinterpret_cast<const float *>(summ);
        float *Cy = reinterpret_cast<float *>(carry);
        float I = 0.0f, comp = 0.0f;
        for (uint32_t s = s0; s < s1; s++) {
            Cy[s] = I;
            kahan_add(I, comp, __ldg(S + s));
        }
    } else if (METHOD == OMNI3D_METHOD_WEIGHTED) {
        const float4 *S = reinterpret_cast<const float4 *>(summ);
        float4 *Cy = reinterpret_cast<float4 *>(carry);
        float I = 0.0f, comp = 0.0f, csum = 0.0f, nseg = 0.0f;
        for (uint32_t s = s0; s < s1; s++) {
            Cy[s] = make_float4(I, csum, nseg, 0.0f);
            const float4 d = __ldg(S + s);
            kahan_add(I, comp, d.x);
            csum += d.y;
            nseg += d.z;
        }
    } else {
        const uint4 *S = reinterpret_cast<const uint4 *>(summ);
        uint4 *Cy = reinterpret_cast<uint4 *>(carry);
        uint32_t mode = kNotStarted, start = 0, nseg = 0;
        float I = 0.0f, comp = 0.0f, csum = 0.0f;
        for (uint32_t s = s0; s < s1; s++) {
            Cy[s] = make_uint4(mode | (nseg << 2), start, __float_as_uint(I), __float_as_uint(csum));
            const uint4 v = __ldg(S + 3ull * s + (s == s0 ? 0u : mode));
            const uint32_t f = v.x;
            if (s != s0 && mode == kNotStarted && (f & 3u) == kNotStarted) continue;  // still not started
            if ((f >> 2) & 1u) {  // (re)started inside the segment
                start = v.y;
                I = __uint_as_float(v.z);
                comp = 0.0f;
            } else {
                kahan_add(I, comp, __uint_as_float(v.z));
            }
            if ((f >> 3) & 1u) {
                csum = __uint_as_float(v.w);
                nseg = f >> 4;
            } else {
                csum += __uint_as_float(v.w);
                nseg += f >> 4;
            }
            mode = f & 3u;
        }
    }
}

// The brick passes implement the three accumulations; the fixed-boundary variants use
// their base method's on their own staircases.  -1: not available (minimum-curl walks
// change with every field, so their segments cannot be cached).
int brick_method(int method)
{
    switch (method_accum(method)) {
    case kAccPlain: return OMNI3D_METHOD_PLAIN;
    case kAccSelect: return OMNI3D_METHOD_SELECT;
    case kAccWeighted: return OMNI3D_METHOD_WEIGHTED;
    default: return -1;
    }
}

size_t summary_bytes(int method)
{
    return method == OMNI3D_METHOD_SELECT ? 48 : (method == OMNI3D_METHOD_WEIGHTED ? 16 : 4);
}
size_t carry_bytes(int method) { return method == OMNI3D_METHOD_PLAIN ? 4 : 16; }

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

template <int METHOD, int PHASE>
cudaError_t launch_brick(const CUtensorMap &map, const BrickArgs &A, int grid, cudaStream_t st)
{
    const int smem = kFieldBytes + (PHASE == 2 ? kAccBytes : 0) + 128;
    cudaError_t e = cudaFuncSetAttribute(k_brick<METHOD, PHASE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_brick<METHOD, PHASE><<<grid, kThreads, smem, st>>>(map, A);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

}  // namespace

void free_bricks(Bricks *B)
{
    cudaFree(B->rec); cudaFree(B->brick_off); cudaFree(B->line_seg); cudaFree(B->items); cudaFree(B->work);
    cudaFree(B->summ); cudaFree(B->carry);
    *B = Bricks();
}

cudaError_t build_bricks(const Geometry &geo, Bricks *B, cudaStream_t st, std::string *err)
{
    auto fail = [&](cudaError_t e, const char *what) {
        if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
        return e;
    };
    if (B->built) return cudaSuccess;
    const Grid &g = geo.grid;
    B->nbx = (g.X + kB - 1) / kB;
    B->nby = (g.Y + kB - 1) / kB;
    B->nbz = (g.Z + kB - 1) / kB;
    const long long nb = (long long)B->nbx * B->nby * B->nbz;
    B->n_bricks = nb;
    const long long nl = geo.n_lines;
    if (nl == 0) { B->built = true; return cudaSuccess; }
    if (!tensor_map_encoder()) {
        if (err) *err = "cuTensorMapEncodeTiled is not available from the driver";
        return cudaErrorNotSupported;
    }
    cudaError_t e;
    const long long nkeys = nb * kLenKeys;
    uint32_t *kcount = nullptr, *koff = nullptr, *lnseg = nullptr, *tmp = nullptr;
    auto cleanup = [&]() { cudaFree(kcount); cudaFree(koff); cudaFree(lnseg); cudaFree(tmp); };
    if ((e = cudaMalloc(&kcount, sizeof(uint32_t) * (size_t)nkeys)) != cudaSuccess ||
        (e = cudaMalloc(&koff, sizeof(uint32_t) * (size_t)nkeys)) != cudaSuccess ||
        (e = cudaMalloc(&lnseg, sizeof(uint32_t) * (size_t)(nl + 1))) != cudaSuccess ||
        (e = cudaMalloc(&B->brick_off, sizeof(uint32_t) * (size_t)(nb + 1))) != cudaSuccess ||
        (e = cudaMalloc(&B->line_seg, sizeof(uint32_t) * (size_t)(nl + 1))) != cudaSuccess ||
        (e = cudaMalloc(&tmp, sizeof(uint32_t) * scan_tmp_elems(nl))) != cudaSuccess) {
        cleanup();
        return fail(e, "brick segment counts");
    }
    const unsigned lblocks = (unsigned)((nl + 255) / 256);
    cudaMemsetAsync(kcount, 0, sizeof(uint32_t) * (size_t)nkeys, st);
    k_seg_count<<<lblocks, 256, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc, nl, B->nbx, B->nby, kcount, lnseg);
    OM_COUNT_LAUNCH();
    if ((e = cudaGetLastError()) != cudaSuccess) { cleanup(); return fail(e, "k_seg_count"); }
    if ((e = exclusive_scan_u32(lnseg, B->line_seg, nl, tmp, st)) != cudaSuccess) {
        cleanup();
        return fail(e, "segment scan");
    }
    // offsets of the (brick, length) keys on the host; the totals are checked in 64 bits
    // because segment ids are 32-bit
    std::vector<uint32_t> hk((size_t)nkeys);
    if ((e = cudaMemcpyAsync(hk.data(), kcount, sizeof(uint32_t) * (size_t)nkeys, cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        cleanup();
        return fail(e, "segment counts");
    }
    std::vector<uint32_t> hoff((size_t)nb + 1);
    unsigned long long total = 0;
    for (long long q = 0; q < nkeys; q++) {
        if (q % kLenKeys == 0) hoff[(size_t)(q / kLenKeys)] = (uint32_t)total;
        const uint32_t c = hk[(size_t)q];
        hk[(size_t)q] = (uint32_t)total;
        total += c;
        if (total >= (1ull << 32)) {
            cleanup();
            if (err) *err = "more than 2^32 line segments";
            return cudaErrorNotSupported;
        }
    }
    hoff[(size_t)nb] = (uint32_t)total;
    B->n_segs = (long long)total;
    if ((e = cudaMemcpyAsync(koff, hk.data(), sizeof(uint32_t) * (size_t)nkeys, cudaMemcpyHostToDevice, st)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(B->brick_off, hoff.data(), sizeof(uint32_t) * (size_t)(nb + 1), cudaMemcpyHostToDevice,
                             st)) != cudaSuccess) {
        cleanup();
        return fail(e, "segment offsets");
    }
    if ((e = cudaMalloc(&B->rec, 32 * (size_t)std::max(total, 1ull))) != cudaSuccess) {
        cleanup();
        return fail(e, "segment records");
    }
    SegOut O;
    O.rec = B->rec;
    O.key_off = koff;
    O.cursor = kcount;
    O.line_seg = B->line_seg;
    O.nbx = B->nbx;
    O.nby = B->nby;
    cudaMemsetAsync(kcount, 0, sizeof(uint32_t) * (size_t)nkeys, st);
    k_seg_fill<<<lblocks, 256, 0, st>>>(g, geo.d_lines, geo.d_gbase, geo.d_desc, nl, O);
    OM_COUNT_LAUNCH();
    if ((e = cudaGetLastError()) != cudaSuccess) { cleanup(); return fail(e, "k_seg_fill"); }
    // work items: a brick, or a slice of a large brick, so that every SM has several
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned long long chunk = std::max(4096ull, total / (unsigned long long)(8 * sms) + 1);
    std::vector<uint4> items;
    for (long long b = 0; b < nb; b++) {
        const uint32_t lo = hoff[(size_t)b], hi = hoff[(size_t)b + 1];
        for (unsigned long long s = lo; s < hi; s += chunk)
            items.push_back(make_uint4((uint32_t)b, (uint32_t)s, (uint32_t)std::min<unsigned long long>(hi, s + chunk), 0));
    }
    B->n_items = (uint32_t)items.size();
    B->grid = (int)std::min<long long>((long long)items.size(), sms);
    if ((e = cudaMalloc(&B->items, sizeof(uint4) * std::max<size_t>(items.size(), 1))) != cudaSuccess ||
        (e = cudaMalloc(&B->work, sizeof(uint32_t) * 2)) != cudaSuccess) {
        cleanup();
        return fail(e, "work items");
    }
    if (!items.empty() &&
        (e = cudaMemcpyAsync(B->items, items.data(), sizeof(uint4) * items.size(), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess) {
        cleanup();
        return fail(e, "work items");
    }
    e = cudaStreamSynchronize(st);
    cleanup();
    if (e != cudaSuccess) return fail(e, "segment fill");
    B->built = true;
    return cudaSuccess;
}

cudaError_t brick_prepare(const Geometry &geo, Bricks *B, const Field &f, int method, cudaStream_t st,
                          std::string *err)
{
    auto fail = [&](cudaError_t e, const char *what) {
        if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
        return e;
    };
    if (!B->built) return fail(cudaErrorInvalidValue, "bricks not built");
    if (!f.f32) return fail(cudaErrorInvalidValue, "brick engine needs the FP32 field");
    method = brick_method(method);
    if (method < 0) return fail(cudaErrorNotSupported, "the brick engine does not take minimum-curl walks");
    const Grid &g = geo.grid;
    // tensor map of the float4 field: dims (4 floats, X, Y, Z), box (4, 18, 18, 18)
    if (B->map_for != f.f32) {
        cuuint64_t dims[4] = {4, (cuuint64_t)g.X, (cuuint64_t)g.Y, (cuuint64_t)g.Z};
        cuuint64_t strides[3] = {16, 16ull * (cuuint64_t)g.X, 16ull * (cuuint64_t)g.XY};
        cuuint32_t box[4] = {4, kP, kP, kP};
        cuuint32_t estr[4] = {1, 1, 1, 1};
        CUresult r = tensor_map_encoder()(reinterpret_cast<CUtensorMap *>(B->map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                                          f.f32, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(cudaErrorInvalidValue, "cuTensorMapEncodeTiled");
        B->map_for = f.f32;
    }
    const size_t need_s = summary_bytes(method) * (size_t)std::max(B->n_segs, 1LL);
    const size_t need_c = carry_bytes(method) * (size_t)std::max(B->n_segs, 1LL);
    cudaError_t e;
    if (need_s > B->summ_cap) {
        cudaFree(B->summ);
        B->summ = nullptr;
        B->summ_cap = 0;
        if ((e = cudaMalloc(&B->summ, need_s)) != cudaSuccess) return fail(e, "segment summaries");
        B->summ_cap = need_s;
    }
    if (need_c > B->carry_cap) {
        cudaFree(B->carry);
        B->carry = nullptr;
        B->carry_cap = 0;
        if ((e = cudaMalloc(&B->carry, need_c)) != cudaSuccess) return fail(e, "segment carries");
        B->carry_cap = need_c;
    }
    if (B->n_items == 0) return cudaSuccess;
    BrickArgs A{};
    A.g = g;
    A.nbx = B->nbx; A.nby = B->nby; A.nbz = B->nbz;
    A.rec = B->rec;
    A.items = B->items;
    A.n_items = B->n_items;
    A.work = B->work;
    A.err = reinterpret_cast<int *>(B->work + 1);
    A.summ = B->summ;
    if ((e = cudaMemsetAsync(B->work, 0, sizeof(uint32_t) * 2, st)) != cudaSuccess) return fail(e, "work counter");
    const CUtensorMap &map = *reinterpret_cast<const CUtensorMap *>(B->map);
    if (method == OMNI3D_METHOD_SELECT) e = launch_brick<OMNI3D_METHOD_SELECT, 1>(map, A, B->grid, st);
    else if (method == OMNI3D_METHOD_WEIGHTED) e = launch_brick<OMNI3D_METHOD_WEIGHTED, 1>(map, A, B->grid, st);
    else e = launch_brick<OMNI3D_METHOD_PLAIN, 1>(map, A, B->grid, st);
    if (e != cudaSuccess) return fail(e, "brick summaries");
    const unsigned lblocks = (unsigned)((geo.n_lines + 255) / 256);
    if (method == OMNI3D_METHOD_SELECT)
        k_line_carry<OMNI3D_METHOD_SELECT><<<lblocks, 256, 0, st>>>(geo.n_lines, B->line_seg, B->summ, B->carry);
    else if (method == OMNI3D_METHOD_WEIGHTED)
        k_line_carry<OMNI3D_METHOD_WEIGHTED><<<lblocks, 256, 0, st>>>(geo.n_lines, B->line_seg, B->summ, B->carry);
    else
        k_line_carry<OMNI3D_METHOD_PLAIN><<<lblocks, 256, 0, st>>>(geo.n_lines, B->line_seg, B->summ, B->carry);
    OM_COUNT_LAUNCH();
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "line carries");
    B->prepared_method = method;
    return cudaSuccess;
}

cudaError_t brick_sweep(const Geometry &geo, Bricks *B, int method, const float *p, float2 *pncnt, cudaStream_t st)
{
    method = brick_method(method);
    if (!B->built || B->prepared_method != method || !p || !pncnt || (B->n_segs > 0 && (!B->summ || !B->carry)))
        return cudaErrorInvalidValue;
    if (B->n_items == 0) return cudaSuccess;
    BrickArgs A{};
    A.g = geo.grid;
    A.nbx = B->nbx; A.nby = B->nby; A.nbz = B->nbz;
    A.rec = B->rec;
    A.items = B->items;
    A.n_items = B->n_items;
    A.work = B->work;
    A.err = reinterpret_cast<int *>(B->work + 1);
    A.carry = B->carry;
    A.p = p;
    A.pncnt = pncnt;
    cudaError_t e = cudaMemsetAsync(B->work, 0, sizeof(uint32_t), st);  // the error word is kept
    if (e != cudaSuccess) return e;
    const CUtensorMap &map = *reinterpret_cast<const CUtensorMap *>(B->map);
    if (method == OMNI3D_METHOD_SELECT) return launch_brick<OMNI3D_METHOD_SELECT, 2>(map, A, B->grid, st);
    if (method == OMNI3D_METHOD_WEIGHTED) return launch_brick<OMNI3D_METHOD_WEIGHTED, 2>(map, A, B->grid, st);
    return launch_brick<OMNI3D_METHOD_PLAIN, 2>(map, A, B->grid, st);
}

cudaError_t brick_error(const Bricks &B, int *flag, cudaStream_t st)
{
    *flag = 0;
    if (!B.work) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(flag, B.work + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

}  // namespace omni3d
