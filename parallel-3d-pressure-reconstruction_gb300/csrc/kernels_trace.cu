// Line tracing: every (direction, lattice point) pair -> line records -> staircase step
// descriptors.  Replaces the per-thread line setup at the top of the reference's omni
// kernels (K:6153-6206) and the walk of bodyIntegralInner (K:1762-1861), done once per
// geometry instead of once per line per iteration.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "geometry.cuh"
#include "omni3d_internal.h"

namespace omni3d {

namespace {

constexpr int kTraceBlock = 256;
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;  // items per thread
constexpr long long kScanTile = (long long)kScanBlock * kScanItems;

// Candidate order: (group of `gsize` neighbouring directions, tile of 32 lattice points,
// direction within the group, point within the tile).  A tile is 2^tw_log2 lattice columns
// wide and 32 / 2^tw_log2 rows high (8 x 4 by default).  A warp then holds the 32 lines of
// one direction through a compact patch of its lattice plane, a bundle whose staircases
// share voxels and 32-byte sectors along the whole walk (a 32 x 1 row of the lattice
// spreads over 32 lines' worth of width and shares far fewer), and a block of warps holds
// the same patch of several nearly parallel directions, which walk through the same voxels
// at the same time.  Tiles are visited in Z order within super-tiles of up to 32 x 32 tiles,
// the super-tiles row by row, so the lines in flight at any moment (about a thousand tiles'
// worth) cover a compact patch of the lattice plane rather than a long strip: at 512^3 their
// L2 footprints overlap more (final sweep 953 -> 868 ms; 256^3 unchanged).  On lattices of
// fewer than 32 tiles a side the super-tile shrinks to the smallest power of two that covers
// the tiles, so that few of its slots are empty.
constexpr int kSuperLog2Max = 5;  // super-tile side in tiles: at most 32
struct CandOrder {
    long long ng2;    // lattice points per direction
    long long su;     // super-tiles across the lattice plane
    long long nblk;   // tile slots per direction (super-tiles x side^2; slots outside the lattice are empty)
    int tw_log2;      // log2 of the tile width (2, 3 or 4)
    int s_log2;       // log2 of the super-tile side in tiles (0..kSuperLog2Max)
    int gsize;        // directions per group
    int nv;
};

// Super-tile side (log2) for a lattice of tu x tv tiles: the smallest power of two that
// covers both, at most 2^kSuperLog2Max.
inline int super_log2(long long tu, long long tv)
{
    int s = 0;
    while (s < kSuperLog2Max && (1LL << s) < std::max(tu, tv)) s++;
    return s;
}

// Even bits of x, packed (the column of a Z-order index).
__device__ __forceinline__ uint32_t z_compact(uint32_t x)
{
    x &= 0x55555555u;
    x = (x ^ (x >> 1)) & 0x33333333u;
    x = (x ^ (x >> 2)) & 0x0f0f0f0fu;
    x = (x ^ (x >> 4)) & 0x00ff00ffu;
    x = (x ^ (x >> 8)) & 0x0000ffffu;
    return x;
}

__device__ __forceinline__ bool trace_candidate(const Grid &g, const DirEntry *dirs, const CandOrder &co,
                                                long long c, int in[3], int out[3], float o[3],
                                                int *dir)
{
    const long long per_block = (long long)co.gsize * 32;
    const long long per_group = co.nblk * per_block;
    long long grp = c / per_group;
    long long r = c - grp * per_group;
    long long blk = r / per_block;
    r -= blk * per_block;
    int d = (int)(grp * co.gsize + r / 32);
    const long long sup = blk >> (2 * co.s_log2);
    const uint32_t z = (uint32_t)(blk & ((1LL << (2 * co.s_log2)) - 1));
    const long long tx = (sup % co.su) * (1LL << co.s_log2) + z_compact(z);
    const long long ty = (sup / co.su) * (1LL << co.s_log2) + z_compact(z >> 1);
    const long long u = tx * (1LL << co.tw_log2) + (r & ((1LL << co.tw_log2) - 1));
    const long long v = ty * (32LL >> co.tw_log2) + ((r & 31) >> co.tw_log2);
    *dir = d;
    if (d >= co.nv || u >= g.ng || v >= g.ng) return false;
    const long long pt = u + v * g.ng;  // lattice point: column u, row v
    DirEntry D = dirs[d];
    om_line_offset(pt, g.ng, g.ls, D, o[0], o[1], o[2]);
    om_cross2point(g, o[0], o[1], o[2], D.k1, D.k2, D.k3, D.cas, in, out);
    return om_line_valid(g, in, out);
}

// Pass 1: number of valid lines per block of candidates.
__global__ void __launch_bounds__(kTraceBlock) k_trace_count(Grid g, const DirEntry *dirs,
                                                             long long ncand, CandOrder co,
                                                             uint32_t *blk_cnt)
{
    __shared__ uint32_t warp_cnt[kTraceBlock / 32];
    long long c = (long long)blockIdx.x * kTraceBlock + threadIdx.x;
    bool valid = false;
    if (c < ncand) {
        int in[3], out[3], d;
        float o[3];
        valid = trace_candidate(g, dirs, co, c, in, out, o, &d);
    }
    unsigned b = __ballot_sync(0xffffffffu, valid);
    if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < kTraceBlock / 32; w++) s += warp_cnt[w];
        blk_cnt[blockIdx.x] = s;
    }
}

// Pass 2: write the valid lines of each block at its offset, in candidate order.
__global__ void __launch_bounds__(kTraceBlock) k_trace_emit(Grid g, const DirEntry *dirs,
                                                            long long ncand, CandOrder co,
                                                            const uint32_t *blk_off,
                                                            LineRec *lines, float4 *off)
{
    __shared__ uint32_t warp_cnt[kTraceBlock / 32];
    long long c = (long long)blockIdx.x * kTraceBlock + threadIdx.x;
    bool valid = false;
    int in[3], out[3], d = 0;
    float o[3];
    if (c < ncand) valid = trace_candidate(g, dirs, co, c, in, out, o, &d);
    unsigned b = __ballot_sync(0xffffffffu, valid);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_cnt[warp] = __popc(b);
    __syncthreads();
    if (!valid) return;
    uint32_t base = blk_off[blockIdx.x];
    for (int w = 0; w < warp; w++) base += warp_cnt[w];
    base += __popc(b & ((1u << lane) - 1u));
    LineRec r;
    r.e = (uint32_t)(in[0] + (long long)in[1] * g.X + (long long)in[2] * g.XY);
    r.x = (uint32_t)(out[0] + (long long)out[1] * g.X + (long long)out[2] * g.XY);
    r.dir = d;
    r.m = abs(out[0] - in[0]) + abs(out[1] - in[1]) + abs(out[2] - in[2]);
    lines[base] = r;
    off[base] = make_float4(o[0], o[1], o[2], 0.0f);
}

// Words per lane of every group of 32 lines: ceil(max steps / 16).
__global__ void k_group_words(const LineRec *lines, long long n_lines, long long n_groups,
                              uint32_t *gw)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((li >> 5) >= n_groups) return;  // whole warps only (blockDim is a multiple of 32)
    int m = li < n_lines ? lines[li].m : 0;
    int mx = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) gw[li >> 5] = (uint32_t)((mx + 15) >> 4);
}

// Walk every line once (K:1762-1861) and store its staircase, 2 bits per step.  RULE is
// the walk rule of OmWalker::step; rule 3 reads `curl`.  The full path length
// |di| + |dj| + |dk| bounds every walk (each step moves one axis toward the exit), so a
// re-walk with another field fits the words reserved for the line.  counters[0] counts
// walks that stopped early under rule 0 (the reference's "Wrong Point" error; under the
// other rules stopping early is their design), counters[1] the voxel visits.
template <int RULE>
__global__ void __launch_bounds__(256) k_walk(Grid g, const DirEntry *dirs, LineRec *lines,
                                              const float4 *off, const uint32_t *gbase,
                                              uint32_t *desc, long long n_lines,
                                              unsigned long long *counters, const float *curl)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned mask = __ballot_sync(0xffffffffu, li < n_lines);
    if (li >= n_lines) return;  // the tail of the last warp only
    LineRec r = lines[li];
    float4 o = off[li];
    DirEntry D = dirs[r.dir];
    int ie = (int)(r.e % g.X), je = (int)((r.e / g.X) % g.Y), ke = (int)(r.e / g.XY);
    int ix = (int)(r.x % g.X), jx = (int)((r.x / g.X) % g.Y), kx = (int)(r.x / g.XY);
    OmWalker w;
    w.init(g, o.x, o.y, o.z, D.k1, D.k2, D.k3, ie, je, ke, ix, jx, kx);
    uint32_t *dp = desc + 32ull * gbase[li >> 5] + (li & 31);
    uint32_t word = 0;
    int s = 0;
    const int m = abs(ix - ie) + abs(jx - je) + abs(kx - ke);
    for (; s < m; s++) {
        int a = w.step<RULE>(curl, g.X, g.XY, g.V);
        if (a < 0) break;
        word |= (uint32_t)a << (2 * (s & 15));
        if ((s & 15) == 15) { dp[32 * (s >> 4)] = word; word = 0; }
    }
    if (s & 15) dp[32 * (s >> 4)] = word;
    if (s != r.m) lines[li].m = s;  // the reference keeps the contributions of the steps taken
    if (s != m && RULE == 0) atomicAdd(&counters[0], 1ull);
    // voxel-direction updates: entry + one per step
    unsigned u = __reduce_add_sync(mask, (unsigned)(s + 1));
    if ((threadIdx.x & 31) == (__ffs(mask) - 1)) atomicAdd(&counters[1], (unsigned long long)u);
}

// Number of lines through every voxel (entry included): a geometry-only bound on the
// contributions any voxel can receive in one sweep.
__global__ void __launch_bounds__(256) k_lines_through(Grid g, const LineRec *__restrict__ lines,
                                                       const uint32_t *__restrict__ gbase,
                                                       const uint32_t *__restrict__ desc, long long n_lines,
                                                       uint32_t *cnt)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    int ie = (int)(r.e % (uint32_t)g.X), je = (int)((r.e / (uint32_t)g.X) % (uint32_t)g.Y),
        ke = (int)(r.e / (uint32_t)g.XY);
    int ix = (int)(r.x % (uint32_t)g.X), jx = (int)((r.x / (uint32_t)g.X) % (uint32_t)g.Y),
        kx = (int)(r.x / (uint32_t)g.XY);
    const int d0 = ix > ie ? 1 : -1, d1 = (jx > je ? 1 : -1) * g.X, d2 = (kx > ke ? 1 : -1) * (int)g.XY;
    long long v = r.e;
    atomicAdd(cnt + v, 1u);
    const uint32_t *dp = desc + 32ull * gbase[li >> 5] + (li & 31);
    for (int s0 = 0; s0 < r.m; s0 += 16) {
        uint32_t w = __ldg(dp + 32 * (s0 >> 4));
        int n = min(16, r.m - s0);
        for (int t = 0; t < n; t++, w >>= 2) {
            int a = (int)(w & 3u);
            v += a == 0 ? d0 : (a == 1 ? d1 : d2);
            atomicAdd(cnt + v, 1u);
        }
    }
}

// ---------------------------------------------------------------- scan
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *sh, T *total)
{
    // sh: kScanBlock / 32 + 1 entries
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T s = lane < kScanBlock / 32 ? sh[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanBlock / 32) sh[lane] = s;
    }
    __syncthreads();
    T warp_excl = warp ? sh[warp - 1] : T(0);
    if (total) *total = sh[kScanBlock / 32 - 1];
    __syncthreads();
    return warp_excl + x - v;
}

template <typename T>
__global__ void __launch_bounds__(kScanBlock) k_scan_reduce(const T *in, long long n, T *part)
{
    __shared__ T sh[kScanBlock / 32 + 1];
    long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
        if (base + i < n) s += in[base + i];
    T tot;
    block_exclusive_scan<T>(s, sh, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Scan of the partial sums in one block (sequential over tiles of kScanBlock items).
template <typename T>
__global__ void __launch_bounds__(kScanBlock) k_scan_partials(T *part, long long np)
{
    __shared__ T sh[kScanBlock / 32 + 1];
    T carry = 0;
    for (long long t0 = 0; t0 < np; t0 += kScanBlock) {
        long long i = t0 + threadIdx.x;
        T v = i < np ? part[i] : T(0);
        T tot;
        T ex = block_exclusive_scan<T>(v, sh, &tot);
        if (i < np) part[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) part[np] = carry;
}

template <typename T>
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(const T *in, long long n, const T *part,
                                                           T *out)
{
    __shared__ T sh[kScanBlock / 32 + 1];
    long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    T v[kScanItems];
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = base + i < n ? in[base + i] : T(0);
        s += v[i];
    }
    T ex = block_exclusive_scan<T>(s, sh, nullptr) + part[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = part[gridDim.x];
}

template <typename T>
cudaError_t exclusive_scan(const T *in, T *out, long long n, T *tmp, cudaStream_t st)
{
    long long nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) {
        return cudaMemsetAsync(out, 0, sizeof(T), st);
    }
    k_scan_reduce<T><<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, tmp);
    OM_COUNT_LAUNCH();
    k_scan_partials<T><<<1, kScanBlock, 0, st>>>(tmp, nb);
    OM_COUNT_LAUNCH();
    k_scan_apply<T><<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, tmp, out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

}  // namespace

size_t scan_tmp_elems(long long n) { return (size_t)((n + kScanTile - 1) / kScanTile) + 2; }

cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, long long n, uint32_t *tmp,
                               cudaStream_t st)
{
    return exclusive_scan<uint32_t>(in, out, n, tmp, st);
}
cudaError_t exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, long long n,
                               unsigned long long *tmp, cudaStream_t st)
{
    return exclusive_scan<unsigned long long>(in, out, n, tmp, st);
}

#define OM_TRY(x)                                                         \
    do {                                                                  \
        cudaError_t e_ = (x);                                             \
        if (e_ != cudaSuccess) {                                          \
            if (err) *err = std::string(#x) + ": " + cudaGetErrorString(e_); \
            return e_;                                                    \
        }                                                                 \
    } while (0)

namespace {
// A device temporary freed when the guard goes out of scope (any return path).
struct TmpBuf {
    void *p = nullptr;
    template <typename T>
    cudaError_t alloc(T **out, size_t elems)
    {
        cudaError_t e = cudaMalloc(&p, sizeof(T) * std::max<size_t>(elems, 1));
        *out = e == cudaSuccess ? static_cast<T *>(p) : nullptr;
        return e;
    }
    ~TmpBuf() { cudaFree(p); }
};
}  // namespace

cudaError_t ensure_lines_through(Geometry *g, cudaStream_t st)
{
    if (g->d_lines_through) return cudaSuccess;
    cudaError_t e = cudaMalloc(&g->d_lines_through, sizeof(uint32_t) * (size_t)std::max(g->grid.V, 1LL));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(g->d_lines_through, 0, sizeof(uint32_t) * (size_t)g->grid.V, st);
    if (e != cudaSuccess || g->n_lines == 0) return e;
    k_lines_through<<<(unsigned)((g->n_lines + 255) / 256), 256, 0, st>>>(g->grid, g->d_lines, g->d_gbase, g->d_desc,
                                                                          g->n_lines, g->d_lines_through);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

namespace {
__global__ void k_max_u32(long long n, const uint32_t *__restrict__ x, unsigned *out)
{
    unsigned m = 0u;
    const long long nthr = ((n + 31) / 32) * 32;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nthr; i += (long long)gridDim.x * blockDim.x)
        if (i < n) m = max(m, x[i]);
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}
}  // namespace

cudaError_t max_lines_through(Geometry *g, cudaStream_t st, unsigned *out)
{
    if (!g->d_lines_through) g->max_through = 0;
    if (g->max_through) {
        *out = g->max_through;
        return cudaSuccess;
    }
    cudaError_t e = ensure_lines_through(g, st);
    if (e != cudaSuccess) return e;
    TmpBuf tb;
    unsigned *d = nullptr;
    if ((e = tb.alloc(&d, 1)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(d, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
    const long long V = g->grid.V;
    long long blocks = std::min<long long>((V + 255) / 256, 152LL * 64);
    k_max_u32<<<(unsigned)std::max<long long>(blocks, 1), 256, 0, st>>>(V, g->d_lines_through, d);
    OM_COUNT_LAUNCH();
    unsigned h = 0;
    if ((e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
    g->max_through = h;
    *out = h;
    return cudaSuccess;
}

void free_geometry(Geometry *g)
{
    cudaFree(g->d_lines_through);
    g->d_lines_through = nullptr;
    g->max_through = 0;
    cudaFree(g->d_counters);
    g->d_counters = nullptr;
    cudaFree(g->d_off);
    cudaFree(g->d_lines);
    cudaFree(g->d_gbase);
    cudaFree(g->d_desc);
    g->d_off = nullptr;
    g->d_lines = nullptr;
    g->d_gbase = nullptr;
    g->d_desc = nullptr;
    g->n_lines = g->n_groups = g->n_words = g->n_units = g->walk_errors = 0;
}

cudaError_t build_geometry(Geometry *g, cudaStream_t st, std::string *err)
{
    const Grid &G = g->grid;
    CandOrder co;
    co.ng2 = (long long)G.ng * G.ng;
    co.tw_log2 = g->tile_width == 4 ? 2 : (g->tile_width == 16 ? 4 : 3);
    const long long tw = 1LL << co.tw_log2, th = 32LL >> co.tw_log2;
    const long long tu = (G.ng + tw - 1) / tw, tv = (G.ng + th - 1) / th;
    co.s_log2 = super_log2(tu, tv);
    const long long side = 1LL << co.s_log2;
    co.su = (tu + side - 1) / side;
    co.nblk = co.su * ((tv + side - 1) / side) * side * side;
    co.gsize = std::max(1, std::min(g->dir_group, g->nv));
    co.nv = g->nv;
    long long ngroups = (g->nv + co.gsize - 1) / co.gsize;
    long long ncand = ngroups * co.nblk * co.gsize * 32;
    long long nblk = (ncand + kTraceBlock - 1) / kTraceBlock;
    if (nblk > 0x7fffffffLL) {
        if (err) *err = "too many lattice candidates";
        return cudaErrorInvalidValue;
    }
    // temporaries of the build, freed on every exit
    TmpBuf tb_blk, tb_tmp, tb_gw, tb_gtmp;
    uint32_t *blk = nullptr, *tmp = nullptr;
    OM_TRY(tb_blk.alloc(&blk, (size_t)(2 * nblk + 1)));
    OM_TRY(tb_tmp.alloc(&tmp, scan_tmp_elems(nblk)));
    uint32_t *blk_off = blk + nblk;
    k_trace_count<<<(unsigned)nblk, kTraceBlock, 0, st>>>(G, g->d_dirs, ncand, co, blk);
    OM_COUNT_LAUNCH();
    OM_TRY(cudaGetLastError());
    OM_TRY(exclusive_scan_u32(blk, blk_off, nblk, tmp, st));
    uint32_t total = 0;
    OM_TRY(cudaMemcpyAsync(&total, blk_off + nblk, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    OM_TRY(cudaStreamSynchronize(st));
    g->n_lines = total;
    g->n_groups = (total + 31) / 32;
    if (total == 0) {
        g->n_words = 0;
        g->n_units = 0;
        return cudaSuccess;
    }
    OM_TRY(cudaMalloc(&g->d_lines, sizeof(LineRec) * (size_t)total));
    OM_TRY(cudaMalloc(&g->d_off, sizeof(float4) * (size_t)total));
    k_trace_emit<<<(unsigned)nblk, kTraceBlock, 0, st>>>(G, g->d_dirs, ncand, co, blk_off, g->d_lines,
                                                         g->d_off);
    OM_COUNT_LAUNCH();
    OM_TRY(cudaGetLastError());

    // words per group -> prefix offsets
    uint32_t *gw = nullptr, *gtmp = nullptr;
    OM_TRY(tb_gw.alloc(&gw, (size_t)g->n_groups));
    OM_TRY(cudaMalloc(&g->d_gbase, sizeof(uint32_t) * (size_t)(g->n_groups + 1)));
    OM_TRY(tb_gtmp.alloc(&gtmp, scan_tmp_elems(g->n_groups)));
    long long nthr = g->n_groups * 32;
    k_group_words<<<(unsigned)((nthr + 255) / 256), 256, 0, st>>>(g->d_lines, g->n_lines, g->n_groups, gw);
    OM_COUNT_LAUNCH();
    OM_TRY(cudaGetLastError());
    OM_TRY(exclusive_scan_u32(gw, g->d_gbase, g->n_groups, gtmp, st));
    uint32_t words_per_lane_total = 0;
    OM_TRY(cudaMemcpyAsync(&words_per_lane_total, g->d_gbase + g->n_groups, sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, st));
    OM_TRY(cudaStreamSynchronize(st));
    g->n_words = 32LL * words_per_lane_total;
    OM_TRY(cudaMalloc(&g->d_desc, sizeof(uint32_t) * (size_t)std::max(g->n_words, 1LL)));

    OM_TRY(cudaMalloc(&g->d_counters, 2 * sizeof(unsigned long long)));
    // the minimum-curl rule needs a field: its geometry starts from the nearest-candidate
    // walk and is re-walked per field (rewalk_min_curl)
    return run_walk(g, g->walk_rule == 3 ? 0 : g->walk_rule, nullptr, st);
}

cudaError_t run_walk(Geometry *g, int rule, const float *curl, cudaStream_t st)
{
    if (g->n_lines == 0) return cudaSuccess;
    if (!g->d_counters || !g->d_lines || !g->d_desc || (rule == 3 && !curl)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(g->d_counters, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((g->n_lines + 255) / 256);
    const Grid &G = g->grid;
    switch (rule) {
    case 1: k_walk<1><<<blocks, 256, 0, st>>>(G, g->d_dirs, g->d_lines, g->d_off, g->d_gbase, g->d_desc, g->n_lines,
                                              g->d_counters, curl); break;
    case 2: k_walk<2><<<blocks, 256, 0, st>>>(G, g->d_dirs, g->d_lines, g->d_off, g->d_gbase, g->d_desc, g->n_lines,
                                              g->d_counters, curl); break;
    case 3: k_walk<3><<<blocks, 256, 0, st>>>(G, g->d_dirs, g->d_lines, g->d_off, g->d_gbase, g->d_desc, g->n_lines,
                                              g->d_counters, curl); break;
    default: k_walk<0><<<blocks, 256, 0, st>>>(G, g->d_dirs, g->d_lines, g->d_off, g->d_gbase, g->d_desc, g->n_lines,
                                               g->d_counters, curl); break;
    }
    OM_COUNT_LAUNCH();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    unsigned long long herr[2] = {0, 0};
    if ((e = cudaMemcpyAsync(herr, g->d_counters, sizeof(herr), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
    g->walk_errors = (long long)herr[0];
    g->n_units = (long long)herr[1];
    // anything derived from the staircases is stale
    cudaFree(g->d_lines_through);
    g->d_lines_through = nullptr;
    g->max_through = 0;
    g->walk_generation++;
    return cudaSuccess;
}

}  // namespace omni3d
