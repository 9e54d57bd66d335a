// Omni sweep over the traced lines: the accumulation half of bodyIntegralInner
// (K:1743-1863), bodyIntegralInnerWeighted (K:1993-2135) and bodyIntegralInnerSelect
// (K:2280-2537), the normalisation
// devidecountInner (K:6746-6759), the curl indicator (K:8352-8378) and the gauge.
//
// One thread walks one line by decoding its 2-bit staircase; a warp holds 32 neighbouring
// lines of one direction, whose step words are interleaved so that every word load is one
// coalesced 128-byte transaction.  The gradient and curl of each visited voxel are one
// 16-byte (FP32) or 8-byte (BF16) gather; contributions go to an interleaved (pn, count) pair with
// one vector reduction (red.global.add.v2.f32) per visited voxel.  The trapezoid prefix
// integral along the line is a compensated (Kahan) FP32 sum.
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

#include "fixed.cuh"
#include "omni3d_internal.h"
#include "walk.cuh"

namespace omni3d {

// Steps whose gathers a walk issues together (walk.cuh); the batched kernels run 4 CTAs of
// 256 threads per SM (64 registers: the batch's gathers stay in registers).  CTAs of 128 or
// 64 threads changed nothing (73.7 and 73.9 against 73.8 ms at 256^3 / 642 directions): the
// full sweep is bound by its scattered reductions.
constexpr int kWalkBatch = 4;
constexpr int kSweepThreads = 256, kSweepBlocks = 4;  // threads per CTA, CTAs per SM

namespace {

__device__ __forceinline__ float bf_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

// (ax, ay, az, curl) of voxel v from either storage.
template <bool BF16>
__device__ __forceinline__ float4 load_grad(const float4 *f32, const uint2 *b16, long long v)
{
    if (BF16) {
        uint2 u = __ldg(b16 + v);
        return make_float4(bf_lo(u.x), bf_hi(u.x), bf_lo(u.y), bf_hi(u.y));
    } else {
        return __ldg(f32 + v);
    }
}

__device__ __forceinline__ float sel3(int a, float x, float y, float z)
{
    return a == 0 ? x : (a == 1 ? y : z);
}

// Per-line constants of the accumulation walk.
struct LineWalk {
    uint32_t v;           // current voxel
    int d0, d1, d2;       // signed strides of a step along x, y, z
    float h0, h1, h2;     // -rho * sign * spacing / 2 per axis (K:1816, 1825, 1834)
    int m;
    const uint32_t *dp;   // this lane's first step word

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
        // the reference forms -rho*s*dl in float and halves it in double (exact)
        h0 = __fmul_rn(-g.rho * (float)si, g.dx) * 0.5f;
        h1 = __fmul_rn(-g.rho * (float)sj, g.dy) * 0.5f;
        h2 = __fmul_rn(-g.rho * (float)sk, g.dz) * 0.5f;
        v = r.e;
        m = r.m;
        dp = desc + 32ull * gbase[li >> 5] + (li & 31);
    }
};

// Contributions into the (pn, count) accumulators: one FP32 vector reduction, (the FP64
// defect-correction sweep) two FP64 reductions, each a native L2 atomic, or (the
// bit-reproducible mode) two 64-bit fixed-point additions with the scales fs.
struct FixScale {
    double pn = 0.0, cnt = 0.0;
};
template <typename ACC>
__device__ __forceinline__ FixScale load_fix(const double *fix)
{
    FixScale f;
    if (std::is_same<ACC, Fix2>::value && fix) {
        f.pn = fix[kFixPn];
        f.cnt = fix[kFixCnt];
    }
    return f;
}
__device__ __forceinline__ void acc_add(const FixScale &, float2 *a, float x, float y)
{
    atomicAdd(a, make_float2(x, y));
}
__device__ __forceinline__ void acc_add(const FixScale &, double2 *a, float x, float y)
{
    atomicAdd(&a->x, (double)x);
    atomicAdd(&a->y, (double)y);
}
__device__ __forceinline__ void acc_add(const FixScale &fs, Fix2 *a, float x, float y)
{
    fix_add(&a->pn, x, fs.pn);
    fix_add(&a->cnt, y, fs.cnt);
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// Plain method: every voxel of the line, the entry included, receives p[entry] + I(v).
// SELF = false leaves the entry out (the minimum-curl plain variant, K:2797-2936).
template <bool BF16, bool SELF, typename ACC>
__global__ void __launch_bounds__(kSweepThreads, kSweepBlocks)
k_sweep_plain(Grid g, const LineRec *__restrict__ lines,
              const uint32_t *__restrict__ gbase,
              const uint32_t *__restrict__ desc, long long n_lines,
              const float4 *__restrict__ f32,
              const uint2 *__restrict__ b16,
              const float *__restrict__ p, ACC *pncnt,
              const double *__restrict__ fix)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    LineWalk L;
    L.init(g, r, gbase, desc, li);
    const FixScale fs = load_fix<ACC>(fix);
    const float pe = __ldg(p + r.e);
    if (SELF) acc_add(fs, pncnt + r.e, pe, 1.0f);
    float4 gl = load_grad<BF16>(f32, b16, L.v);
    float I = 0.0f, comp = 0.0f;
    walk_steps<kWalkBatch, BF16 ? kGradBF16 : kGradF32, false>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, b16, nullptr, [&](int a, uint32_t v, const float4 &gv, uint32_t) {
            float term = sel3(a, L.h0, L.h1, L.h2) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z));
            kahan_add(I, comp, term);
            acc_add(fs, pncnt + v, pe + I, 1.0f);
            gl = gv;
        });
}

// Weighted method (K:1993-2135): the entry receives nothing; step s of the line (s = 1..m)
// adds w_s (p[entry] + I_s) and w_s, w_s = s / sum_{t<=s} curl_t/1e4, once that sum is
// nonzero.  Each curl/1e4 term is the reference's correctly rounded float division, so the
// "sum != 0" decision (all curls so far zero) is the reference's.
template <bool BF16, typename ACC>
__global__ void __launch_bounds__(kSweepThreads, kSweepBlocks)
k_sweep_weighted(Grid g, const LineRec *__restrict__ lines,
                 const uint32_t *__restrict__ gbase,
                 const uint32_t *__restrict__ desc, long long n_lines,
                 const float4 *__restrict__ f32,
                 const uint2 *__restrict__ b16,
                 const float *__restrict__ curl,
                 const float *__restrict__ p, ACC *pncnt,
                 const double *__restrict__ fix)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    LineWalk L;
    L.init(g, r, gbase, desc, li);
    const FixScale fs = load_fix<ACC>(fix);
    const float pe = __ldg(p + r.e);
    float4 gl = load_grad<BF16>(f32, b16, L.v);
    float I = 0.0f, comp = 0.0f, csum = 0.0f, nseg = 0.0f;
    walk_steps<kWalkBatch, BF16 ? kGradBF16 : kGradF32, false>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, b16, nullptr, [&](int a, uint32_t v, const float4 &gv, uint32_t) {
            float cn = gv.w;
            float term = sel3(a, L.h0, L.h1, L.h2) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z));
            kahan_add(I, comp, term);
            csum += __fdiv_rn(cn, 1.0e4f);
            nseg += 1.0f;
            if (csum != 0.0f) {
                float wc = __fdividef(nseg, csum);
                acc_add(fs, pncnt + v, (pe + I) * wc, wc);
            }
            gl = gv;
        });
}

// Weighted method with raw curl sums (the minimum-curl variant, K:2937-3085): the sum starts
// at the entry's curl and the entry receives (p[entry], 1) / C; step s adds its curl (not
// divided by 1e4) and contributes w (p[entry] + I), w = (s + 1) / C, with no test for a zero
// sum: a zero sum gives infinities, as in the reference.
template <bool BF16, typename ACC>
__global__ void __launch_bounds__(kSweepThreads, kSweepBlocks)
k_sweep_weighted_raw(Grid g, const LineRec *__restrict__ lines,
                     const uint32_t *__restrict__ gbase,
                     const uint32_t *__restrict__ desc, long long n_lines,
                     const float4 *__restrict__ f32,
                     const uint2 *__restrict__ b16,
                     const float *__restrict__ curl,
                     const float *__restrict__ p, ACC *pncnt,
                     const double *__restrict__ fix)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    LineWalk L;
    L.init(g, r, gbase, desc, li);
    const FixScale fs = load_fix<ACC>(fix);
    const float pe = __ldg(p + r.e);
    float4 gl = load_grad<BF16>(f32, b16, L.v);
    float csum = gl.w, nseg = 1.0f;
    {
        const float w0 = __frcp_rn(csum);
        acc_add(fs, pncnt + L.v, pe * w0, w0);
    }
    float I = 0.0f, comp = 0.0f;
    walk_steps<kWalkBatch, BF16 ? kGradBF16 : kGradF32, false>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, b16, nullptr, [&](int a, uint32_t v, const float4 &gv, uint32_t) {
            float cn = gv.w;
            kahan_add(I, comp, sel3(a, L.h0, L.h1, L.h2) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z)));
            csum += cn;
            nseg += 1.0f;
            const float wc = __fdividef(nseg, csum);
            acc_add(fs, pncnt + v, (pe + I) * wc, wc);
            gl = gv;
        });
}

// Selected method (K:2280-2537), state machine and asymmetries included: the entry is a
// segment start when 0 < curl <= thr; before the first start an x step needs
// 0 < curl < thr, a y/z step only curl != 0; a bad voxel pauses the segment (an x step
// also pauses on curl == 0, a y/z step walks through it without adding that step's
// increment); a good voxel after a pause restarts the segment at that voxel; the z
// branch keeps the running curl/count sums on restart.
template <bool BF16, typename ACC>
__global__ void __launch_bounds__(kSweepThreads, kSweepBlocks)
k_sweep_select(Grid g, const LineRec *__restrict__ lines,
               const uint32_t *__restrict__ gbase,
               const uint32_t *__restrict__ desc, long long n_lines,
               const float4 *__restrict__ f32,
               const uint2 *__restrict__ b16,
               const float *__restrict__ curl,
               const float *__restrict__ p, ACC *pncnt,
               const double *__restrict__ fix)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    LineWalk L;
    L.init(g, r, gbase, desc, li);
    const FixScale fs = load_fix<ACC>(fix);
    const float thr = g.thr;
    float4 gl = load_grad<BF16>(f32, b16, L.v);
    float ce = gl.w;
    bool started = !(ce == 0.0f || ce > thr);
    bool paused = false;
    float p0 = started ? __ldg(p + L.v) : 0.0f;
    float I = 0.0f, comp = 0.0f, csum = 0.0f, nseg = 0.0f;
    walk_steps<kWalkBatch, BF16 ? kGradBF16 : kGradF32, false>(
        L.v, L.d0, L.d1, L.d2, L.m, L.dp, f32, b16, nullptr, [&](int a, uint32_t v, const float4 &gv, uint32_t) {
            const float cn = gv.w;
            if (!started) {
                bool ok = (a == 0) ? (cn != 0.0f && cn < thr) : (cn != 0.0f);
                if (ok) {
                    p0 = __ldg(p + v);
                    started = true;
                    I = 0.0f; comp = 0.0f; nseg = 0.0f; csum = 0.0f;
                }
            } else {
                bool good = cn < thr && cn != 0.0f;
                if (!paused && good) {
                    float term = sel3(a, L.h0, L.h1, L.h2) * (sel3(a, gv.x, gv.y, gv.z) + sel3(a, gl.x, gl.y, gl.z));
                    kahan_add(I, comp, term);
                    // weight n / sum(curl / 1e4) of the reference (K:2390-2392), as one fast
                    // division (within 2 ulp) instead of its two correctly rounded ones: the
                    // weights only scale averages, and the FP64-oracle bars hold (the 256^3
                    // solve took 127.9 against 130.5 ms with a correctly rounded reciprocal)
                    csum += cn * 1.0e-4f;
                    nseg += 1.0f;
                    float wc = __fdividef(nseg, csum);
                    acc_add(fs, pncnt + v, (p0 + I) * wc, wc);
                }
                bool enter_bad = (a == 0) ? ((!paused && cn >= thr) || cn == 0.0f) : (!paused && cn >= thr);
                if (enter_bad) paused = true;
                if (paused && good) {
                    p0 = __ldg(p + v);
                    I = 0.0f; comp = 0.0f;
                    paused = false;
                    if (a != 2) { nseg = 0.0f; csum = 0.0f; }
                }
            }
            gl = gv;
        });
}

__global__ void k_normalize(long long V, const float2 *__restrict__ pncnt, const float *__restrict__ p_keep,
                            float *p_out, float *cnt_out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        float2 a = pncnt[v];
        float pk = p_keep ? p_keep[v] : 0.0f;
        if (p_out) p_out[v] = a.y > 0.0f ? __fdiv_rn(a.x, a.y) : pk;
        if (cnt_out) cnt_out[v] = a.y;
    }
}

__global__ void k_accum_split(long long V, const float2 *__restrict__ acc, float *pn, float *cnt)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        float2 a = acc[v];
        pn[v] += a.x;
        cnt[v] += a.y;
    }
}

__global__ void k_init_accum(long long V, const float *__restrict__ p_init, int seed, float2 *pncnt)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x)
        pncnt[v] = make_float2(seed && p_init ? p_init[v] : 0.0f, 0.0f);
}

__device__ __forceinline__ uint32_t to_bf16(float x)
{
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
}

// BF16 pattern of a curl value.  Round to nearest even, except that a nonzero curl never
// rounds to zero and, for a thresholded method (g.curl_map), every decision of the selected
// method is kept: the kernels then compare against the BF16 stand-in g.thr of the threshold
// g.thr_src (its truncation), and a positive curl below g.thr_src maps below g.thr, one equal
// to it maps to g.thr, one above it maps above g.thr (positive BF16 patterns order like their
// values).  The decisions (curl == 0, curl < thr, curl > thr) are then those of the FP32 curl.
__device__ __forceinline__ uint32_t curl_bf16(float c, const Grid &g)
{
    if (c == 0.0f) return __float_as_uint(c) >> 16;  // +0 and -0 stay as they are
    uint32_t v = to_bf16(c);
    if ((v & 0x7fffu) == 0u) v |= 1u;  // no underflow to zero
    if (g.curl_map && c > 0.0f && g.thr_src > 0.0f) {
        const uint32_t t = __float_as_uint(g.thr) >> 16;
        if (c < g.thr_src) {
            if (v >= t) v = t - 1u;
        } else if (c == g.thr_src) {
            v = t;
        } else if (v <= t) {
            v = t + 1u;
        }
    }
    return v;
}

// The packed field: float4 (ax, ay, az, curl) and, for BF16 storage, the 8-byte record
// {ax | ay << 16, az | curl << 16} of round-to-nearest-even BF16 values (the curl by
// curl_bf16).  With BF16 storage the FP32 entry holds the stored values as floats, and
// curl_out (which may be the curl array itself) the stored curl: every pass then sees the
// same field, the full sweeps gathering the 8-byte records and the anchor operator's filling
// pass, which is bound by instruction issue rather than by its gathers, the float4 entries
// (nothing to unpack: 1.8 ms of its 50.9 ms at 256^3 / 642 directions).
__global__ void k_pack(Grid g, const float *__restrict__ ax, const float *__restrict__ ay,
                       const float *__restrict__ az, const float *curl, float4 *f32, uint2 *b16, float *curl_out)
{
    const long long V = g.V;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        float x = ax[v], y = ay[v], z = az[v];
        float c = curl ? curl[v] : 0.0f;
        if (b16) {
            const uint32_t bx = to_bf16(x), by = to_bf16(y), bz = to_bf16(z), cb = curl_bf16(c, g);
            b16[v] = make_uint2(bx | (by << 16), bz | (cb << 16));
            x = __uint_as_float(bx << 16);
            y = __uint_as_float(by << 16);
            z = __uint_as_float(bz << 16);
            c = __uint_as_float(cb << 16);
            if (curl_out) curl_out[v] = c;
        }
        f32[v] = make_float4(x, y, z, c);
    }
}

// |curl a| x mask with the reference's stencil and evaluation order (K:8352-8378).
__global__ void k_curl(Grid g, const float *__restrict__ au, const float *__restrict__ av,
                       const float *__restrict__ aw, const float *__restrict__ mask, float *out)
{
    const long long X = g.X, Y = g.Y, Z = g.Z, XY = g.XY;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.V;
         v += (long long)gridDim.x * blockDim.x) {
        long long i = v % X, j = (v / X) % Y, k = v / XY;
        long long i0 = i - 1 >= 0 ? i - 1 : i, j0 = j - 1 >= 0 ? j - 1 : j, k0 = k - 1 >= 0 ? k - 1 : k;
        long long ie = i + 1 <= X - 1 ? i + 1 : i, je = j + 1 <= Y - 1 ? j + 1 : j, ke = k + 1 <= Z - 1 ? k + 1 : k;
        float dj = (float)(je - j0), dk = (float)(ke - k0), di = (float)(ie - i0);
        float cx = __fdiv_rn(__fdiv_rn(__fsub_rn(aw[i + je * X + k * XY], aw[i + j0 * X + k * XY]), dj), g.dy);
        cx = __fadd_rn(cx, __fdiv_rn(__fdiv_rn(-__fsub_rn(av[i + j * X + ke * XY], av[i + j * X + k0 * XY]), dk), g.dz));
        float cy = __fdiv_rn(__fdiv_rn(-__fsub_rn(aw[ie + j * X + k * XY], aw[i0 + j * X + k * XY]), di), g.dx);
        cy = __fadd_rn(cy, __fdiv_rn(__fdiv_rn(__fsub_rn(au[i + j * X + ke * XY], au[i + j * X + k0 * XY]), dk), g.dz));
        float cz = __fdiv_rn(__fdiv_rn(__fsub_rn(av[ie + j * X + k * XY], av[i0 + j * X + k * XY]), di), g.dx);
        cz = __fadd_rn(cz, __fdiv_rn(__fdiv_rn(-__fsub_rn(au[i + je * X + k * XY], au[i + j0 * X + k * XY]), dj), g.dy));
        float s = __fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz));
        out[v] = __fmul_rn(__fsqrt_rn(s), mask ? mask[v] : 1.0f);
    }
}

// Deterministic FP64 sums: fixed grid, per-block partials, one block adds them in order.
constexpr int kRedBlocks = 256, kRedThreads = 256;

__device__ __forceinline__ double block_sum(double x, double *sh)
{
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
    __syncthreads();
    return s;
}

__global__ void k_masked_sum(long long V, const float *__restrict__ p, const float *__restrict__ cnt,
                             double *part)
{
    __shared__ double sh[32];
    double s = 0.0, n = 0.0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        if (cnt[v] > 0.0f) { s += (double)p[v]; n += 1.0; }
    }
    double bs = block_sum(s, sh);
    double bn = block_sum(n, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = bs; part[2 * blockIdx.x + 1] = bn; }
}

__global__ void k_finish_sums(const double *part, int nblk, int width, double *out)
{
    if (threadIdx.x < width) {
        double s = 0.0;
        for (int b = 0; b < nblk; b++) s += part[width * b + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

// p -= sums[0] / sums[1] (the mean, or the reference value with sums[1] = 1).
__global__ void k_shift(long long V, const double *sums, float *p)
{
    const double sub = sums[1] > 0 ? sums[0] / sums[1] : 0.0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x)
        p[v] = (float)((double)p[v] - sub);
}

__global__ void k_read_point(const float *p, long long ref, double *out) { out[0] = (double)p[ref]; out[1] = 1.0; }

// One wavefront of the centre integration (initialIntegration.cpp:9-407): every voxel at L1
// distance L = a + b + c from the centre (X/2, Y/2, Z/2), thread (a, b) taking the up to
// eight voxels (+-a, +-b, +-c).  A voxel's value is the mean over its off-centre axes, in
// x, y, z order, of (the neighbour one step nearer the centre, at distance L - 1) + or -
// rho * 0.5 * (a[voxel] + a[neighbour]) * spacing, + on the low side of the centre; FP64
// with explicit rounding in the reference's C evaluation order.
__global__ void k_centre_level(Grid g, int L, const float *__restrict__ au, const float *__restrict__ av,
                               const float *__restrict__ aw, int stride, double *pn)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long w1 = (long long)L + 1;
    if (t >= w1 * w1) return;
    const int a = (int)(t / w1), b = (int)(t % w1);
    if (a + b > L) return;
    const int c = L - a - b;
    const int cx = g.X / 2, cy = g.Y / 2, cz = g.Z / 2;
    const double rho = (double)g.rho, dx = (double)g.dx, dy = (double)g.dy, dz = (double)g.dz;
    for (int o = 0; o < 8; o++) {
        const int sx = (o & 1) ? 1 : -1, sy = (o & 2) ? 1 : -1, sz = (o & 4) ? 1 : -1;
        if ((a == 0 && sx > 0) || (b == 0 && sy > 0) || (c == 0 && sz > 0)) continue;  // each voxel once
        const int i = cx + sx * a, j = cy + sy * b, k = cz + sz * c;
        if (i < 0 || i >= g.X || j < 0 || j >= g.Y || k < 0 || k >= g.Z) continue;
        const long long ind = i + (long long)j * g.X + (long long)k * g.XY;
        double v = 0.0;
        int n = 0;
        if (a) {
            const long long nb = ind - sx;
            const double tr = __dmul_rn(__dmul_rn(__dmul_rn(0.5, __dadd_rn((double)au[ind * stride], (double)au[nb * stride])), dx), rho);
            v = sx < 0 ? __dadd_rn(pn[nb], tr) : __dsub_rn(pn[nb], tr);
            n = 1;
        }
        if (b) {
            const long long nb = ind - (long long)sy * g.X;
            const double tr = __dmul_rn(__dmul_rn(__dmul_rn(0.5, __dadd_rn((double)av[ind * stride], (double)av[nb * stride])), dy), rho);
            const double w = sy < 0 ? __dadd_rn(pn[nb], tr) : __dsub_rn(pn[nb], tr);
            v = n ? __dadd_rn(v, w) : w;
            n++;
        }
        if (c) {
            const long long nb = ind - (long long)sz * g.XY;
            const double tr = __dmul_rn(__dmul_rn(__dmul_rn(0.5, __dadd_rn((double)aw[ind * stride], (double)aw[nb * stride])), dz), rho);
            const double w = sz < 0 ? __dadd_rn(pn[nb], tr) : __dsub_rn(pn[nb], tr);
            v = n ? __dadd_rn(v, w) : w;
            n++;
        }
        pn[ind] = n == 1 ? v : __ddiv_rn(v, n == 2 ? 2.0 : 3.0);
    }
}

__global__ void k_to_float(long long V, const double *__restrict__ in, float *out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        out[v] = (float)in[v];
}

unsigned grid_for(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 64) b = 152LL * 64;
    if (b < 1) b = 1;
    return (unsigned)b;
}

template <typename ACC>
cudaError_t sweep_full_t(const Geometry &geo, const Field &f, int method, bool bf16, const float *p, ACC *pncnt,
                         cudaStream_t st, const double *fix = nullptr)
{
    if (geo.n_lines == 0) return cudaSuccess;
    // every pointer the kernels dereference must be set: refuse to launch otherwise
    if (!geo.d_lines || !geo.d_gbase || !geo.d_desc || !p || !pncnt || (bf16 ? !f.bf16 : !f.f32) ||
        (method_uses_curl(method) && !f.curl))
        return cudaErrorInvalidValue;
    unsigned blocks = (unsigned)((geo.n_lines + kSweepThreads - 1) / kSweepThreads);
    const int acc = method_accum(method);
    if (acc == kAccWeighted) {
        if (bf16)
            k_sweep_weighted<true, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                           geo.n_lines, f.f32, f.bf16, f.curl, p, pncnt, fix);
        else
            k_sweep_weighted<false, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                            geo.n_lines, f.f32, f.bf16, f.curl, p, pncnt, fix);
        OM_COUNT_LAUNCH();
    } else if (acc == kAccWeightedRawCurl) {
        if (bf16)
            k_sweep_weighted_raw<true, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                               geo.n_lines, f.f32, f.bf16, f.curl, p, pncnt, fix);
        else
            k_sweep_weighted_raw<false, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                                geo.n_lines, f.f32, f.bf16, f.curl, p, pncnt, fix);
        OM_COUNT_LAUNCH();
    } else if (acc == kAccSelect) {
        if (bf16)
            k_sweep_select<true, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines,
                                                         f.f32, f.bf16, f.curl, p, pncnt, fix);
        else
            k_sweep_select<false, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines,
                                                          f.f32, f.bf16, f.curl, p, pncnt, fix);
        OM_COUNT_LAUNCH();
    } else if (acc == kAccPlainNoEntry) {
        if (bf16)
            k_sweep_plain<true, false, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                               geo.n_lines, f.f32, f.bf16, p, pncnt, fix);
        else
            k_sweep_plain<false, false, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                                geo.n_lines, f.f32, f.bf16, p, pncnt, fix);
        OM_COUNT_LAUNCH();
    } else {
        if (bf16)
            k_sweep_plain<true, true, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                              geo.n_lines, f.f32, f.bf16, p, pncnt, fix);
        else
            k_sweep_plain<false, true, ACC><<<blocks, kSweepThreads, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc,
                                                               geo.n_lines, f.f32, f.bf16, p, pncnt, fix);
        OM_COUNT_LAUNCH();
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t sweep_full(const Geometry &geo, const Field &f, int method, bool bf16, const float *p, float2 *pncnt,
                       cudaStream_t st)
{
    return sweep_full_t(geo, f, method, bf16, p, pncnt, st);
}

cudaError_t sweep_full64(const Geometry &geo, const Field &f, int method, bool bf16, const float *p, double2 *pncnt,
                         cudaStream_t st)
{
    return sweep_full_t(geo, f, method, bf16, p, pncnt, st);
}

cudaError_t sweep_full_fix(const Geometry &geo, const Field &f, int method, bool bf16, const float *p, Fix2 *pncnt,
                           const double *scale, cudaStream_t st)
{
    if (!scale) return cudaErrorInvalidValue;
    return sweep_full_t(geo, f, method, bf16, p, pncnt, st, scale);
}

namespace {

__global__ void k_init_accum64(long long V, const float *__restrict__ p_init, int seed, double2 *pncnt)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x)
        pncnt[v] = make_double2(seed && p_init ? (double)p_init[v] : 0.0, 0.0);
}

__global__ void k_normalize64(long long V, const double2 *__restrict__ pncnt, const float *__restrict__ p_keep,
                              float *p_out, float *cnt_out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        const double2 a = pncnt[v];
        const float pk = p_keep ? p_keep[v] : 0.0f;
        if (p_out) p_out[v] = a.y > 0.0 ? (float)(a.x / a.y) : pk;
        if (cnt_out) cnt_out[v] = (float)a.y;
    }
}

}  // namespace

cudaError_t init_accum64(long long V, const float *p_init, bool seed, double2 *pncnt, cudaStream_t st)
{
    k_init_accum64<<<grid_for(V), 256, 0, st>>>(V, p_init, seed ? 1 : 0, pncnt);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t normalize64(long long V, const double2 *pncnt, const float *p_keep, float *p_out, float *cnt_out,
                        cudaStream_t st)
{
    k_normalize64<<<grid_for(V), 256, 0, st>>>(V, pncnt, p_keep, p_out, cnt_out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t normalize(long long V, const float2 *pncnt, const float *p_keep, float *p_out, float *cnt_out,
                      cudaStream_t st)
{
    k_normalize<<<grid_for(V), 256, 0, st>>>(V, pncnt, p_keep, p_out, cnt_out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t accum_split(long long V, const float2 *acc, float *pn, float *cnt, cudaStream_t st)
{
    k_accum_split<<<grid_for(V), 256, 0, st>>>(V, acc, pn, cnt);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t init_accum(long long V, const float *p_init, bool seed, float2 *pncnt, cudaStream_t st)
{
    k_init_accum<<<grid_for(V), 256, 0, st>>>(V, p_init, seed ? 1 : 0, pncnt);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t pack_field(const Grid &g, const float *ax, const float *ay, const float *az, const float *curl,
                       Field *f, bool make_bf16, cudaStream_t st, float *curl_rounded)
{
    k_pack<<<grid_for(g.V), 256, 0, st>>>(g, ax, ay, az, curl, f->f32, make_bf16 ? f->bf16 : nullptr,
                                          make_bf16 ? curl_rounded : nullptr);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

namespace {
__global__ void k_field_curl(long long V, const float4 *__restrict__ f32, float *out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        out[v] = f32[v].w;
}
}  // namespace

cudaError_t field_curl(long long V, const float4 *f32, float *out, cudaStream_t st)
{
    k_field_curl<<<grid_for(V), 256, 0, st>>>(V, f32, out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t curl_field(const Grid &g, const float *ax, const float *ay, const float *az, const float *mask,
                       float *out, cudaStream_t st)
{
    k_curl<<<grid_for(g.V), 256, 0, st>>>(g, ax, ay, az, mask, out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t apply_gauge(long long V, int gauge, long long ref, const float *cnt, float *p, double *scratch,
                        cudaStream_t st)
{
    if (gauge == OMNI3D_GAUGE_NONE) return cudaSuccess;
    if (gauge == OMNI3D_GAUGE_MEAN) {
        k_masked_sum<<<kRedBlocks, kRedThreads, 0, st>>>(V, p, cnt, scratch + 2);
        OM_COUNT_LAUNCH();
        k_finish_sums<<<1, 32, 0, st>>>(scratch + 2, kRedBlocks, 2, scratch);
        OM_COUNT_LAUNCH();
    } else {
        k_read_point<<<1, 1, 0, st>>>(p, ref, scratch);
        OM_COUNT_LAUNCH();
    }
    k_shift<<<grid_for(V), 256, 0, st>>>(V, scratch, p);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

size_t gauge_scratch_doubles() { return 2 + 2 * kRedBlocks; }

cudaError_t centre_integration(const Grid &g, const float *ax, const float *ay, const float *az, int stride,
                               double pref, double *scratch, float *out, cudaStream_t st)
{
    if (!ax || !ay || !az || !scratch || !out) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(double) * (size_t)g.V, st);
    if (e != cudaSuccess) return e;
    // voxel 0 takes pref first, as in the reference; its own wavefront overwrites it
    if ((e = cudaMemcpyAsync(scratch, &pref, sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;  // pref is a host stack value
    const int cx = g.X / 2, cy = g.Y / 2, cz = g.Z / 2;
    const int lmax = std::max(cx, g.X - 1 - cx) + std::max(cy, g.Y - 1 - cy) + std::max(cz, g.Z - 1 - cz);
    for (int L = 1; L <= lmax; L++) {
        const long long n = ((long long)L + 1) * ((long long)L + 1);
        k_centre_level<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, L, ax, ay, az, stride, scratch);
        OM_COUNT_LAUNCH();
    }
    k_to_float<<<grid_for(g.V), 256, 0, st>>>(g.V, scratch, out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

}  // namespace omni3d
