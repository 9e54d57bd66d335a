// Scales, bounds, initialisation and normalisation of the bit-reproducible mode (fixed.cuh).
#include <cfloat>

#include "fixed.cuh"
#include "omni3d_internal.h"

namespace omni3d {

namespace {

unsigned grid_for(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 64) b = 152LL * 64;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// The warp's maximum of non-negative floats by their bits (order-preserving for x >= 0).
__device__ __forceinline__ unsigned warp_max_bits(unsigned b)
{
    return __reduce_max_sync(0xffffffffu, b);
}
__device__ __forceinline__ unsigned warp_min_bits(unsigned b)
{
    return __reduce_min_sync(0xffffffffu, b);
}

// bits[kBitsA] = max |component|, bits[kBitsC] = least nonzero |curl| (+inf when none)
__global__ void k_field_bounds(long long V, const float4 *__restrict__ f32, unsigned *bits)
{
    unsigned amax = 0u, cmin = 0x7f800000u;
    const long long nthr = ((V + 31) / 32) * 32;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nthr;
         v += (long long)gridDim.x * blockDim.x) {
        if (v < V) {
            const float4 q = f32[v];
            amax = max(amax, __float_as_uint(fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fabsf(q.z))));
            const float c = fabsf(q.w);
            if (c != 0.0f) cmin = min(cmin, __float_as_uint(c));
        }
    }
    amax = warp_max_bits(amax);
    cmin = warp_min_bits(cmin);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(bits + kBitsA, amax);
        atomicMin(bits + kBitsC, cmin);
    }
}

// bits[slot] = max |x| over n values
__global__ void k_absmax(long long n, const float *__restrict__ x, unsigned *bits, int slot)
{
    unsigned m = 0u;
    const long long nthr = ((n + 31) / 32) * 32;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nthr;
         i += (long long)gridDim.x * blockDim.x)
        if (i < n) m = max(m, __float_as_uint(fabsf(x[i])));
    m = warp_max_bits(m);
    if ((threadIdx.x & 31) == 0) atomicMax(bits + slot, m);
}

// 2^(62 - e) for a bound B < 2^e; 0 when B is not finite (no scale can hold the sum).
__device__ __forceinline__ double scale_for(double B)
{
    if (!(B <= DBL_MAX)) return 0.0;
    if (B <= 0.0) return 1.0;
    int e = 0;
    frexp(B, &e);
    return ldexp(1.0, 62 - e);
}

struct Bounds {
    double imax, wmax;
};

__device__ __forceinline__ Bounds bounds(const unsigned *bits, int acc, double hmax, double path)
{
    const double amax = (double)__uint_as_float(bits[kBitsA]);
    const double cmin = (double)__uint_as_float(bits[kBitsC]);
    Bounds b;
    b.imax = 4.0 * hmax * amax * path;  // a factor of two for BF16 storage's rounding of a
    if (acc == kAccPlain || acc == kAccPlainNoEntry) b.wmax = 1.0;
    else if (acc == kAccSelect) b.wmax = 1.0e4 / cmin;
    else if (acc == kAccWeighted) b.wmax = path * 1.0e4 / cmin;
    else b.wmax = (path + 1.0) / cmin;
    b.wmax *= 2.0;  // the FP32 rounding of the weights
    return b;
}

// mode 0: the operator rows' (b, c); 1: the row sums of an iteration; 2: a full sweep
__global__ void k_scales(int mode, unsigned *bits, double *scale, int acc, double lmax, double hmax, double path,
                         const int *stop)
{
    if (stop && *stop) return;
    const Bounds b = bounds(bits, acc, hmax, path);
    if (mode == 0) {
        scale[kFixB] = scale_for(lmax * b.wmax * b.imax);
        scale[kFixC] = scale_for(lmax * b.wmax);
    } else if (mode == 1) {
        const double pmax = (double)__uint_as_float(bits[kBitsRow]);
        scale[kFixRow] = scale_for(lmax * b.wmax * pmax);
        bits[kBitsRow] = 0u;  // ready for the next iteration's maximum
    } else {
        const double pmax = (double)__uint_as_float(bits[kBitsVol]);
        scale[kFixPn] = scale_for((lmax * b.wmax + 1.0) * (pmax + b.imax));
        scale[kFixCnt] = scale_for(lmax * b.wmax);
        bits[kBitsVol] = 0u;
    }
}

__global__ void k_absmax_gated(long long n, const float *__restrict__ x, unsigned *bits, int slot, const int *stop)
{
    if (stop && *stop) return;
    unsigned m = 0u;
    const long long nthr = ((n + 31) / 32) * 32;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nthr;
         i += (long long)gridDim.x * blockDim.x)
        if (i < n) m = max(m, __float_as_uint(fabsf(x[i])));
    m = warp_max_bits(m);
    if ((threadIdx.x & 31) == 0) atomicMax(bits + slot, m);
}

__global__ void k_rows_to_float(long long n, const long long *__restrict__ bc64, const double *__restrict__ scale,
                                float2 *bc, int keep_c)
{
    const double sb = scale[kFixB], sc = scale[kFixC];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float b = (float)((double)bc64[2 * i] / sb);
        if (keep_c) bc[i].x = b;
        else bc[i] = make_float2(b, (float)((double)bc64[2 * i + 1] / sc));
    }
}

__global__ void k_init_fix(long long V, const float *__restrict__ p_init, int seed, const double *__restrict__ scale,
                           Fix2 *acc)
{
    const double sp = scale[kFixPn];
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        acc[v] = Fix2{seed && p_init ? (long long)fix_term(p_init[v], sp) : 0LL, 0LL};
}

__global__ void k_normalize_fix(long long V, const Fix2 *__restrict__ acc, const double *__restrict__ scale,
                                const float *__restrict__ p_keep, float *p_out, float *cnt_out)
{
    const double sp = scale[kFixPn], sc = scale[kFixCnt];
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        const Fix2 a = acc[v];
        const double c = (double)a.cnt / sc;
        const float pk = p_keep ? p_keep[v] : 0.0f;
        if (p_out) p_out[v] = c > 0.0 ? (float)(((double)a.pn / sp) / c) : pk;
        if (cnt_out) cnt_out[v] = (float)c;
    }
}

}  // namespace

cudaError_t fix_field_bounds(long long V, const float4 *f32, const Fixed &fx, cudaStream_t st)
{
    const unsigned init[kBitsSlots] = {0u, 0x7f800000u, 0u, 0u};
    cudaError_t e = cudaMemcpyAsync(fx.bits, init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    k_field_bounds<<<grid_for(V), 256, 0, st>>>(V, f32, fx.bits);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t fix_fill_scales(const Fixed &fx, cudaStream_t st)
{
    k_scales<<<1, 1, 0, st>>>(0, fx.bits, fx.scale, fx.acc, fx.lmax, fx.hmax, fx.path, nullptr);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t fix_row_scale(long long n, const float *pa, const Fixed &fx, cudaStream_t st, const int *stop)
{
    k_absmax_gated<<<grid_for(n), 256, 0, st>>>(n, pa, fx.bits, kBitsRow, stop);
    OM_COUNT_LAUNCH();
    k_scales<<<1, 1, 0, st>>>(1, fx.bits, fx.scale, fx.acc, fx.lmax, fx.hmax, fx.path, stop);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t fix_sweep_scales(long long V, const float *vol, const Fixed &fx, cudaStream_t st)
{
    k_absmax<<<grid_for(V), 256, 0, st>>>(V, vol, fx.bits, kBitsVol);
    OM_COUNT_LAUNCH();
    k_scales<<<1, 1, 0, st>>>(2, fx.bits, fx.scale, fx.acc, fx.lmax, fx.hmax, fx.path, nullptr);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t fix_rows_to_float(long long n, const Fixed &fx, float2 *bc, bool keep_c, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_rows_to_float<<<grid_for(n), 256, 0, st>>>(n, fx.bc64, fx.scale, bc, keep_c ? 1 : 0);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t init_accum_fix(long long V, const float *p_init, bool seed, const Fixed &fx, Fix2 *acc, cudaStream_t st)
{
    k_init_fix<<<grid_for(V), 256, 0, st>>>(V, p_init, seed ? 1 : 0, fx.scale, acc);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

cudaError_t normalize_fix(long long V, const Fix2 *acc, const Fixed &fx, const float *p_keep, float *p_out,
                          float *cnt_out, cudaStream_t st)
{
    k_normalize_fix<<<grid_for(V), 256, 0, st>>>(V, acc, fx.scale, p_keep, p_out, cnt_out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

}  // namespace omni3d
