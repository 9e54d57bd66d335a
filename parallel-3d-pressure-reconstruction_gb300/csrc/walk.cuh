// Batched walk along one line's staircase, shared by the sweep and anchor kernels.
//
// A line's voxel addresses follow from its 2-bit steps alone, not from the values loaded
// along it.  The walk therefore decodes a batch of B steps, issues the B gradient gathers
// (and, with AUX, B loads of a 32-bit word per voxel from `aux`, e.g. an anchor bitmap
// indexed by voxel >> 5) before using any of them, and only then hands the steps in order
// to f(axis, voxel, gradient, aux word).  Without the batch each step's gather waits for the
// previous step's arithmetic, and a warp walking 32 lines spends most of its time waiting
// on L2 latency.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace omni3d {

__device__ __forceinline__ float4 load_grad_f32(const float4 *f32, long long v) { return __ldg(f32 + v); }

// (ax, ay, az, curl) from the 8-byte BF16 record {ax | ay << 16, az | curl << 16}: one
// 8-byte gather per voxel.  The curl's sign bit (bit 31 of the second word) is the anchor
// flag that the filling pass sets on the anchor voxels (curl is a magnitude, so the bit is
// otherwise clear).
__device__ __forceinline__ float4 load_grad_b16(const uint2 *b16, long long v)
{
    const uint2 u = __ldg(b16 + v);
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                       __uint_as_float(u.y & 0xffff0000u));
}

// Which gradient a walk gathers per step.
enum WalkGrad { kNoGrad = 0, kGradF32 = 1, kGradBF16 = 2 };

// v: the line's current voxel (advanced to its last voxel; voxel indices are below 2^32,
// and a negative stride wraps modulo 2^32 to the right index); d0..d2: signed strides of a step
// along x, y, z; m: steps; dp: the lane's first step word (words 32 apart).
template <int B, int GRAD, bool AUX, typename F>
__device__ __forceinline__ void walk_steps(uint32_t &v, int d0, int d1, int d2, int m, const uint32_t *dp,
                                           const float4 *f32, const uint2 *b16, const uint32_t *aux, F &&f)
{
    for (int s0 = 0; s0 < m; s0 += 16) {
        uint32_t w = __ldg(dp + 32 * (s0 >> 4));
        const int n = min(16, m - s0);
        for (int t0 = 0; t0 < n; t0 += B) {
            int ax[B];
            uint32_t vv[B];
            float4 g[B];
            uint32_t xw[B];
#pragma unroll
            for (int q = 0; q < B; q++) {
                ax[q] = (int)(w & 3u);
                w >>= 2;
                if (t0 + q < n) {
                    v += (uint32_t)(ax[q] == 0 ? d0 : (ax[q] == 1 ? d1 : d2));
                    vv[q] = v;
                    if (GRAD == kGradF32) g[q] = load_grad_f32(f32, v);
                    else if (GRAD == kGradBF16) g[q] = load_grad_b16(b16, v);
                    else g[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (AUX) xw[q] = __ldg(aux + (v >> 5));
                }
            }
#pragma unroll
            for (int q = 0; q < B; q++)
                if (t0 + q < n) f(ax[q], vv[q], g[q], AUX ? xw[q] : 0u);
        }
    }
}

}  // namespace omni3d
