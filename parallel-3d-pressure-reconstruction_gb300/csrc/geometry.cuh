// Device line geometry, bit-exact with the reference's FP32 host evaluation.
//
// Which voxels a line visits is decided by FP32 comparisons in the reference (cross2point,
// K:663-1113, and the nearest-candidate walk, K:1762-1861).  Every float operation below
// is an explicitly rounded intrinsic, so nvcc cannot contract a multiply and an add into
// an FMA and change a rounding; the order of operations is the reference's left-to-right
// C evaluation.
#pragma once

#include "omni3d_internal.h"

namespace omni3d {

#define OM_MUL __fmul_rn
#define OM_ADD __fadd_rn
#define OM_SUB __fsub_rn
#define OM_DIV __fdiv_rn

// floor(f + 0.5) with the addition exact, as the reference evaluates it in double (K:703).
__device__ __forceinline__ int om_round_half(float f)
{
    float fl = floorf(f);
    return (int)fl + (OM_SUB(f, fl) >= 0.5f ? 1 : 0);
}

// Centred offset of lattice point pt of a direction (K:6171-6194).  The reference forms
// (row - (ng-1)/2) * spacing in double and rounds to float; the difference is an exact
// half-integer in float, so one rounded float product gives the same value.
__device__ __forceinline__ void om_line_offset(long long pt, int ng, float ls, const DirEntry &D,
                                               float &x, float &y, float &z)
{
    int row = (int)(pt / ng);
    int col = (int)(pt - (long long)row * ng);
    float h = 0.5f * (float)(ng - 1);
    float xp = OM_MUL(OM_SUB((float)row, h), ls);
    float yp = OM_MUL(OM_SUB((float)col, h), ls);
    float t = OM_MUL(xp, D.ct);
    x = OM_SUB(OM_MUL(t, D.cp), OM_MUL(yp, D.sp));
    y = OM_ADD(OM_MUL(t, D.sp), OM_MUL(yp, D.cp));
    z = OM_MUL(-xp, D.st);
}

// cross2point (K:663-1113).  `cases` has bit c-1 set when the direction satisfies the
// test of case c (evaluated once per direction on the host); a case whose offset test
// fails falls through to the next, as in the reference.  in/out keep the sentinel
// (X, Y, Z) when no intersection is recorded.
__device__ __forceinline__ void om_cross2point(const Grid &g, float x, float y, float z,
                                               float k1, float k2, float k3, int cases,
                                               int in[3], int out[3])
{
    const float cx = g.cx, cy = g.cy, cz = g.cz;
    const int X = g.X, Y = g.Y, Z = g.Z;
    in[0] = X; in[1] = Y; in[2] = Z;
    out[0] = X; out[1] = Y; out[2] = Z;
    float r;
    int t;
    if ((cases & 1) && x > -cx && x < cx) {  // case 1: k1 == 0
        float z1, z2, y3, y4;
        r = OM_DIV(OM_SUB(-cy, y), k2); z1 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(cy, y), k2); z2 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(-cz, z), k3); y3 = OM_ADD(y, OM_MUL(k2, r));
        r = OM_DIV(OM_SUB(cz, z), k3); y4 = OM_ADD(y, OM_MUL(k2, r));
        bool flag = false;
        int ic = om_round_half(OM_ADD(x, cx));
        if (z1 <= cz && z1 >= -cz) { in[0] = ic; in[1] = 0; in[2] = om_round_half(OM_ADD(z1, cz)); flag = true; }
        if (z2 <= cz && z2 >= -cz) {
            int *o = flag ? out : in;
            o[0] = ic; o[1] = Y - 1; o[2] = om_round_half(OM_ADD(z2, cz)); flag = true;
        }
        if (y3 <= cy && y3 >= -cy) {
            int *o = flag ? out : in;
            o[0] = ic; o[1] = om_round_half(OM_ADD(y3, cy)); o[2] = 0; flag = true;
        }
        if (y4 <= cy && y4 >= -cy) {
            int *o = flag ? out : in;
            o[0] = ic; o[1] = om_round_half(OM_ADD(y4, cy)); o[2] = Z - 1;
        }
        if (flag) {
            if (OM_ADD(OM_MUL((float)(out[1] - in[1]), k2), OM_MUL((float)(out[2] - in[2]), k3)) < 0) {
                t = in[1]; in[1] = out[1]; out[1] = t;
                t = in[2]; in[2] = out[2]; out[2] = t;
            }
        }
        return;
    }
    if ((cases & 2) && y > -cy && y < cy) {  // case 2: k2 == 0
        float z1, z2, x3, x4;
        r = OM_DIV(OM_SUB(-cx, x), k1); z1 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(cx, x), k1); z2 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(-cz, z), k3); x3 = OM_ADD(x, OM_MUL(k1, r));
        r = OM_DIV(OM_SUB(cz, z), k3); x4 = OM_ADD(x, OM_MUL(k1, r));
        bool flag = false;
        int jc = om_round_half(OM_ADD(y, cy));
        if (z1 <= cz && z1 >= -cz) { in[0] = 0; in[1] = jc; in[2] = om_round_half(OM_ADD(z1, cz)); flag = true; }
        if (z2 <= cz && z2 >= -cz) {
            int *o = flag ? out : in;
            o[0] = X - 1; o[1] = jc; o[2] = om_round_half(OM_ADD(z2, cz)); flag = true;
        }
        if (x3 <= cx && x3 >= -cx) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x3, cx)); o[1] = jc; o[2] = 0; flag = true;
        }
        if (x4 <= cx && x4 >= -cx) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x4, cx)); o[1] = jc; o[2] = Z - 1; flag = true;
        }
        if (flag) {
            if (OM_ADD(OM_MUL((float)(out[0] - in[0]), k1), OM_MUL((float)(out[2] - in[2]), k3)) < 0) {
                t = in[0]; in[0] = out[0]; out[0] = t;
                t = in[2]; in[2] = out[2]; out[2] = t;
            }
        }
        return;
    }
    if ((cases & 4) && z > -cz && z < cz) {  // case 3: k3 == 0 (z where y is meant, K:854-855)
        float y1, y2, x3, x4;
        r = OM_DIV(OM_SUB(-cx, x), k1); y1 = OM_ADD(y, OM_MUL(k2, r));
        r = OM_DIV(OM_SUB(cx, x), k1); y2 = OM_ADD(y, OM_MUL(k2, r));
        r = OM_DIV(OM_SUB(-cy, z), k2); x3 = OM_ADD(x, OM_MUL(k1, r));
        r = OM_DIV(OM_SUB(cy, z), k2); x4 = OM_ADD(x, OM_MUL(k1, r));
        bool flag = false;
        int kc = om_round_half(OM_ADD(z, cz));
        if (y1 <= cy && y1 >= -cy) { in[0] = 0; in[1] = om_round_half(OM_ADD(y1, cy)); in[2] = kc; flag = true; }
        if (y2 <= cy && y2 >= -cy) {
            int *o = flag ? out : in;
            o[0] = X - 1; o[1] = om_round_half(OM_ADD(y2, cy)); o[2] = kc; flag = true;
        }
        if (x3 <= cx && x3 >= -cx) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x3, cx)); o[1] = 0; o[2] = kc; flag = true;
        }
        if (x4 <= cx && x4 >= -cx) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x4, cx)); o[1] = Y - 1; o[2] = kc; flag = true;
        }
        if (flag) {
            if (OM_ADD(OM_MUL((float)(out[0] - in[0]), k1), OM_MUL((float)(out[1] - in[1]), k2)) < 0) {
                t = in[0]; in[0] = out[0]; out[0] = t;
                t = in[1]; in[1] = out[1]; out[1] = t;
            }
        }
        return;
    }
    if ((cases & 8) && x < cx && x > -cx && y < cy && y > -cy) {  // case 4: along z
        in[0] = out[0] = om_round_half(OM_ADD(x, cx));
        in[1] = out[1] = om_round_half(OM_ADD(y, cy));
        if (k3 > 0) { in[2] = 0; out[2] = Z - 1; } else { in[2] = Z - 1; out[2] = 0; }
        return;
    }
    if ((cases & 16) && x > -cx && x < cx && z > -cz && z < cz) {  // case 5: along y
        in[0] = out[0] = om_round_half(OM_ADD(x, cx));
        in[2] = out[2] = om_round_half(OM_ADD(z, cz));
        if (k2 > 0) { out[1] = Y - 1; in[1] = 0; } else { in[1] = Y - 1; out[1] = 0; }
        return;
    }
    if (cases & 32) {  // case 6: along x; reports success even on a miss (K:989)
        if (y > -cy && y < cy && z > -cz && z < cz) {
            in[1] = out[1] = om_round_half(OM_ADD(y, cy));
            in[2] = out[2] = om_round_half(OM_ADD(z, cz));
            if (k1 > 0) { out[0] = X - 1; in[0] = 0; } else { in[0] = X - 1; out[0] = 0; }
        }
        return;
    }
    if (cases & 64) {  // case 7: general direction, six face intersections
        float y1, z1, y2, z2, x3, z3, x4, z4, x5, y5, x6, y6;
        r = OM_DIV(OM_SUB(-cx, x), k1); y1 = OM_ADD(y, OM_MUL(k2, r)); z1 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(cx, x), k1); y2 = OM_ADD(y, OM_MUL(k2, r)); z2 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(-cy, y), k2); x3 = OM_ADD(x, OM_MUL(k1, r)); z3 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(cy, y), k2); x4 = OM_ADD(x, OM_MUL(k1, r)); z4 = OM_ADD(z, OM_MUL(k3, r));
        r = OM_DIV(OM_SUB(-cz, z), k3); x5 = OM_ADD(x, OM_MUL(k1, r)); y5 = OM_ADD(y, OM_MUL(k2, r));
        r = OM_DIV(OM_SUB(cz, z), k3); x6 = OM_ADD(x, OM_MUL(k1, r)); y6 = OM_ADD(y, OM_MUL(k2, r));
        bool flag = false;
        if (y1 <= cy && y1 >= -cy && z1 <= cz && z1 >= -cz) {
            in[0] = 0; in[1] = om_round_half(OM_ADD(y1, cy)); in[2] = om_round_half(OM_ADD(z1, cz)); flag = true;
        }
        if (y2 <= cy && y2 >= -cy && z2 <= cz && z2 >= -cz) {
            int *o = flag ? out : in;
            o[0] = X - 1; o[1] = om_round_half(OM_ADD(y2, cy)); o[2] = om_round_half(OM_ADD(z2, cz)); flag = true;
        }
        if (x3 <= cx && x3 >= -cx && z3 <= cz && z3 >= -cz) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x3, cx)); o[1] = 0; o[2] = om_round_half(OM_ADD(z3, cz)); flag = true;
        }
        if (x4 <= cx && x4 >= -cx && z4 <= cz && z4 >= -cz) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x4, cx)); o[1] = Y - 1; o[2] = om_round_half(OM_ADD(z4, cz)); flag = true;
        }
        if (x5 <= cx && x5 >= -cx && y5 <= cy && y5 >= -cy) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x5, cx)); o[1] = om_round_half(OM_ADD(y5, cy)); o[2] = 0; flag = true;
        }
        if (x6 <= cx && x6 >= -cx && y6 <= cy && y6 >= -cy) {
            int *o = flag ? out : in;
            o[0] = om_round_half(OM_ADD(x6, cx)); o[1] = om_round_half(OM_ADD(y6, cy)); o[2] = Z - 1; flag = true;
        }
        float dot = OM_ADD(OM_ADD(OM_MUL((float)(out[0] - in[0]), k1), OM_MUL((float)(out[1] - in[1]), k2)),
                           OM_MUL((float)(out[2] - in[2]), k3));
        if (dot < 0) {
            t = in[0]; in[0] = out[0]; out[0] = t;
            t = in[1]; in[1] = out[1]; out[1] = t;
            t = in[2]; in[2] = out[2]; out[2] = t;
        }
        return;
    }
}

// Acceptance test of the caller (K:6202-6206): both voxels inside and distinct.
__device__ __forceinline__ bool om_line_valid(const Grid &g, const int in[3], const int out[3])
{
    bool inside = in[0] >= 0 && in[0] < g.X && in[1] >= 0 && in[1] < g.Y && in[2] >= 0 && in[2] < g.Z &&
                  out[0] >= 0 && out[0] < g.X && out[1] >= 0 && out[1] < g.Y && out[2] >= 0 && out[2] < g.Z;
    return inside && !(in[0] == out[0] && in[1] == out[1] && in[2] == out[2]);
}

// sqrt_rn(a) <= sqrt_rn(b) and sqrt_rn(a) < sqrt_rn(b) without computing the square roots
// unless a and b are within 2^-21 of each other (two correctly rounded square roots can
// only be equal when a / b < (1 + 2^-23)^2).  NaN compares false, as in the reference.
__device__ __forceinline__ bool om_sqrt_le(float a, float b)
{
    if (a <= b) return true;
    if (!(OM_SUB(a, b) <= OM_MUL(b, 4.76837158203125e-7f))) return false;
    return __fsqrt_rn(a) == __fsqrt_rn(b);
}
__device__ __forceinline__ bool om_sqrt_lt(float a, float b)
{
    if (!(a < b)) return false;
    if (!(OM_SUB(b, a) <= OM_MUL(a, 4.76837158203125e-7f))) return true;
    return __fsqrt_rn(a) != __fsqrt_rn(b);
}

// Squared distance of candidate voxel (ci, cj, ck) from the line at parameter r
// (K:1800-1810).
__device__ __forceinline__ float om_dist2(float x, float y, float z, float k1, float k2, float k3,
                                          float r, float ci, float cj, float ck)
{
    float a = OM_SUB(OM_ADD(x, OM_MUL(k1, r)), ci);
    float b = OM_SUB(OM_ADD(y, OM_MUL(k2, r)), cj);
    float c = OM_SUB(OM_ADD(z, OM_MUL(k3, r)), ck);
    return OM_ADD(OM_ADD(OM_MUL(a, a), OM_MUL(b, b)), OM_MUL(c, c));
}

// Walker state of one line (K:1745-1761).
struct OmWalker {
    float x, y, z, k1, k2, k3, xk1, yk2, zk3;
    int il, jl, kl, io, jo, ko;

    __device__ __forceinline__ void init(const Grid &g, float ox, float oy, float oz, float d1,
                                         float d2, float d3, int ie, int je, int ke, int ix,
                                         int jx, int kx)
    {
        x = OM_ADD(ox, g.cx); y = OM_ADD(oy, g.cy); z = OM_ADD(oz, g.cz);
        il = ie; jl = je; kl = ke; io = ix; jo = jx; ko = kx;
        float dot = OM_ADD(OM_ADD(OM_MUL(d1, (float)(ix - ie)), OM_MUL(d2, (float)(jx - je))),
                           OM_MUL(d3, (float)(kx - ke)));
        if (dot < 0) { d1 = -d1; d2 = -d2; d3 = -d3; }
        k1 = d1; k2 = d2; k3 = d3;
        xk1 = OM_MUL(x, k1); yk2 = OM_MUL(k2, y); zk3 = OM_MUL(k3, z);
    }

    // One step of the walk.  Returns the axis moved along (0, 1, 2) or -1 when no candidate
    // qualifies (the reference's loop ends there).  RULE:
    //   0  nearest candidate to the line, ties x, y, z (K:1762-1840);
    //   1  as 0, but no y step into j = 0 (bodyIntegralInnerWeightedFixedBC, K:2227);
    //   2  nearest candidate, ties y, x, z; no y step into j = 0 and no x or z step on
    //      j = 0 (bodyIntegralInnerSelectFixedBC, K:2628, 2675, 2722);
    //   3  the candidate with the smallest curl, read at the candidate's linear index when
    //      that index lies inside the volume and 1e10 otherwise, ties x, y, z
    //      (bodyIntegralInner(Weighted)MiniCurl, K:2869-2883).  The far candidate of an axis
    //      already at its exit coordinate (60000 cells away) may land inside the volume at an
    //      unrelated voxel, as in the reference; its coordinate test still rejects it.
    template <int RULE>
    __device__ __forceinline__ int step(const float *curl, int X, long long XY, long long V)
    {
        int i1 = il < io ? il + 1 : (il == io ? il - 60000 : il - 1);
        int j2 = jl < jo ? jl + 1 : (jl == jo ? jl - 60000 : jl - 1);
        int k3n = kl < ko ? kl + 1 : (kl == ko ? kl - 60000 : kl - 1);
        if (RULE == 3) {
            const long long q1 = (long long)i1 + (long long)jl * X + (long long)kl * XY;
            const long long q2 = (long long)il + (long long)j2 * X + (long long)kl * XY;
            const long long q3 = (long long)il + (long long)jl * X + (long long)k3n * XY;
            const float c1 = (q1 >= 0 && q1 < V) ? __ldg(curl + q1) : 1e10f;
            const float c2 = (q2 >= 0 && q2 < V) ? __ldg(curl + q2) : 1e10f;
            const float c3 = (q3 >= 0 && q3 < V) ? __ldg(curl + q3) : 1e10f;
            if (il != io && c1 <= c2 && c1 <= c3) { il = i1; return 0; }
            if (jl != jo && c2 < c1 && c2 <= c3) { jl = j2; return 1; }
            if (kl != ko && c3 < c1 && c3 < c2) { kl = k3n; return 2; }
            return -1;
        }
        float fil = (float)il, fjl = (float)jl, fkl = (float)kl;
        float fi1 = (float)i1, fj2 = (float)j2, fk3 = (float)k3n;
        float k2jl = OM_MUL(k2, fjl), k3kl = OM_MUL(k3, fkl);
        float A = OM_SUB(OM_MUL(k1, fil), xk1);
        float r1 = OM_SUB(OM_ADD(OM_SUB(OM_ADD(OM_SUB(OM_MUL(k1, fi1), xk1), k2jl), yk2), k3kl), zk3);
        float r2 = OM_SUB(OM_ADD(OM_SUB(OM_ADD(A, OM_MUL(k2, fj2)), yk2), k3kl), zk3);
        float r3 = OM_SUB(OM_ADD(OM_SUB(OM_ADD(A, k2jl), yk2), OM_MUL(k3, fk3)), zk3);
        float q1 = om_dist2(x, y, z, k1, k2, k3, r1, fi1, fjl, fkl);
        float q2 = om_dist2(x, y, z, k1, k2, k3, r2, fil, fj2, fkl);
        float q3 = om_dist2(x, y, z, k1, k2, k3, r3, fil, fjl, fk3);
        // the candidate toward the exit is always inside; the far (-60000) one never is
        if (RULE == 2) {
            if (il != io && jl != 0 && om_sqrt_lt(q1, q2) && om_sqrt_le(q1, q3)) { il = i1; return 0; }
            if (jl != jo && j2 != 0 && om_sqrt_le(q2, q1) && om_sqrt_le(q2, q3)) { jl = j2; return 1; }
            if (kl != ko && jl != 0 && om_sqrt_lt(q3, q1) && om_sqrt_lt(q3, q2)) { kl = k3n; return 2; }
            return -1;
        }
        if (il != io && om_sqrt_le(q1, q2) && om_sqrt_le(q1, q3)) { il = i1; return 0; }
        if (jl != jo && (RULE != 1 || j2 != 0) && om_sqrt_lt(q2, q1) && om_sqrt_le(q2, q3)) { jl = j2; return 1; }
        if (kl != ko && om_sqrt_lt(q3, q1) && om_sqrt_lt(q3, q2)) { kl = k3n; return 2; }
        return -1;
    }
};

}  // namespace omni3d
