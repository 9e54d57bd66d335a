// 64-bit fixed-point sums of the bit-reproducible mode (params.deterministic).
//
// The default sums are FP32 atomics (voxel accumulators, operator rows' (b, c)) and operator
// rows whose entries land in the order the atomics hand out their slots, so their last bits
// depend on the order in which the GPU schedules the lines.  In the bit-reproducible mode
// every such sum is taken in 64-bit two's-complement fixed point instead: each term x is
// rounded once to round(x * s) with a power-of-two scale s, and integer addition is exact
// and order-independent, so every run gives the same bits.  The scale of each sum is set on
// the device from a bound B of its magnitude (s = 2^(62 - e) with B < 2^e, so no sum can
// overflow), and the bounds follow from the field: every contribution to a voxel is
// w (p(start) + I) with |I| <= 2 max|h| max|a| (X + Y + Z) along a staircase, a voxel
// receives at most one contribution per line through it, and w is at most 1 (plain
// methods), 1e4 / (least nonzero curl) (selected), (X + Y + Z) 1e4 / (least nonzero curl)
// (weighted) or (X + Y + Z + 1) / (least nonzero curl) (weighted, raw curl sums); a factor
// of two covers the FP32 rounding of w.  With B at most about 2^62 / s, a term is resolved to
// B * 2^-62, far below the FP32 rounding of the default sums.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace omni3d {

// Scales in Fixed::scale: voxel pn, voxel count, row b, row c, operator row sums.
enum FixSlot { kFixPn = 0, kFixCnt = 1, kFixB = 2, kFixC = 3, kFixRow = 4, kFixSlots = 5 };
// Float bits in Fixed::bits: max |a|, least nonzero |curl|, max |p| of the operator values,
// max |p| of the volume a full sweep reads.
enum FixBits { kBitsA = 0, kBitsC = 1, kBitsRow = 2, kBitsVol = 3, kBitsSlots = 4 };

// Fixed-point accumulator pair of one voxel.
struct Fix2 {
    long long pn, cnt;
};

__device__ __forceinline__ unsigned long long fix_term(float x, double s)
{
    return (unsigned long long)__double2ll_rn((double)x * s);
}

__device__ __forceinline__ void fix_add(long long *a, float x, double s)
{
    atomicAdd(reinterpret_cast<unsigned long long *>(a), fix_term(x, s));
}

}  // namespace omni3d
