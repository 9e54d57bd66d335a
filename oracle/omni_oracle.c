/*
 * CPU oracle for the Omni3D parallel-line omni-directional pressure integration.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the reference
 * algorithm (Omni3D_8.0/Omni3D_8.0/kernel.cu, "K" below).  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may load it,
 * and only as the checker or the timed CPU baseline.  The product library never
 * links or calls it.
 *
 * Parity pin: every function here is checked bit-for-bit against the reference's own
 * functions (cross2point, bodyIntegralInner, bodyIntegralInnerSelect, calIndex,
 * calCurlofMaterialAccCPU, omni3dparallellinesESInnerCPU + devidecountInnerCPU)
 * compiled from the reference sources by oracle/build_ref.sh into oracle/_ref/.
 *
 * Arithmetic rules copied from the reference's C semantics (they decide which voxels a
 * line visits, so they are reproduced exactly):
 *   - all geometry is FP32 with every operation rounded separately (compile with
 *     -ffp-contract=off, no -ffast-math);
 *   - floor(f + 0.5) is evaluated in double ("0.5" is a double literal, K:703);
 *   - the "zero" threshold 1e-7 is a double (K:23);
 *   - the trapezoid increment is formed in double and added to a float accumulator
 *     ("0.5" promotes the product, K:1816), i.e. pint = (float)((double)pint + term).
 *
 * Two accumulation precisions share one discrete geometry:
 *   - "f32": the reference's float arithmetic reproduced exactly (sequential order);
 *   - "f64": the same voxel paths, with every sum and weight in double.  This is the
 *     FP64 oracle of the same discrete method.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_ZERO 1e-7                               /* K:23 */
#define ORC_PI 3.1415926535897932384626433832795    /* K:24 */

/* ------------------------------------------------------------------------------------ */
/* geometry                                                                               */
/* ------------------------------------------------------------------------------------ */

/* Number of lattice points per row.  GPU kernel form (K:6159-6167): largest dimension
 * times 1.732 divided by the line spacing, in double, truncated.  The CPU twin (K:8286)
 * omits the division by the spacing; geom_cpu_twin selects it. */
int orc_nogrid(long X, long Y, long Z, float ls, int geom_cpu_twin)
{
    int ng = (int)X;
    if (ng < Y) ng = (int)Y;
    if (ng < Z) ng = (int)Z;
    if (geom_cpu_twin) return (int)(ng * 1.732);
    return (int)(ng * 1.732 / (double)ls);
}

/* Per-direction rotation coefficients (K:6178-6191 with libm sinf/cosf in place of the
 * fast intrinsics, as the CPU twin K:8296-8302 does).  out = {cos th, sin th, cos ph,
 * sin ph}.  With the pole guard (GPU form) sin th == 0 gives ph = 0; without it (CPU
 * twin) the division by zero propagates NaN exactly as the reference's CPU path does. */
void orc_dir_coeffs(float k1, float k2, float k3, int geom_cpu_twin, float out[4])
{
    float theta = acosf(k3);
    float st = sinf(theta);
    float phi = 0.0f;
    if (geom_cpu_twin || st != 0.0f) {
        phi = asinf(k2 / st);
        if (k1 / st < 0) phi = (float)(-phi + ORC_PI);
    }
    out[0] = cosf(theta);
    out[1] = st;
    out[2] = cosf(phi);
    out[3] = sinf(phi);
}

/* Line offset of lattice point `point` (K:6171-6194). */
void orc_line_offset(int point, int ng, float ls, const float c[4], float xyz[3])
{
    float xp = (float)(((double)(float)(point / ng) - 0.5 * (ng - 1)) * (double)ls);
    float yp = (float)(((double)(float)(point - point / ng * ng) - 0.5 * (ng - 1)) * (double)ls);
    float t = xp * c[0];
    xyz[0] = t * c[2] - yp * c[3];
    xyz[1] = t * c[3] + yp * c[2];
    xyz[2] = -xp * c[1];
}

static inline int rnd_half(float f) { return (int)floor((double)f + 0.5); }

/* Entry / exit voxels of the line through (x,y,z) with direction k, following K:663-1113
 * case by case, including its quirks: case 3 uses z where y is meant (K:854-855); in
 * case 6 the function reports success even when the offset misses (K:989), leaving the
 * sentinel (X,Y,Z) in place.  Returns 1 if a case matched, 0 otherwise; in/out hold the
 * sentinel when nothing was found. */
int orc_cross2point(long X, long Y, long Z, float x, float y, float z, float k1, float k2,
                    float k3, int in[3], int out[3])
{
    float cx = (float)((X - 1) / 2.0), cy = (float)((Y - 1) / 2.0), cz = (float)((Z - 1) / 2.0);
    in[0] = (int)X; in[1] = (int)Y; in[2] = (int)Z;
    out[0] = (int)X; out[1] = (int)Y; out[2] = (int)Z;
    int flag, t;
    float r;
    if (k1 == 0 && k2 != 0 && k3 != 0) {                 /* case 1, K:672 */
        if (x > -cx && x < cx) {
            float y1, z1, y2, z2, z3, y3, z4, y4;
            r = (-cy - y) / k2; y1 = -cy; z1 = z + k3 * r;
            r = (cy - y) / k2; y2 = cy; z2 = z + k3 * r;
            r = (-cz - z) / k3; z3 = -cz; y3 = y + k2 * r;
            r = (cz - z) / k3; z4 = cz; y4 = y + k2 * r;
            (void)y1; (void)y2; (void)z3; (void)z4;
            flag = 0;
            if (z1 <= cz && z1 >= -cz && flag == 0) {
                if (flag == 0) { in[0] = rnd_half(x + cx); in[1] = 0; in[2] = rnd_half(z1 + cz); }
                flag = 1;
            }
            if (z2 <= cz && z2 >= -cz) {
                if (flag == 0) { in[0] = rnd_half(x + cx); in[1] = (int)Y - 1; in[2] = rnd_half(z2 + cz); }
                else { out[0] = rnd_half(x + cx); out[1] = (int)Y - 1; out[2] = rnd_half(z2 + cz); }
                flag = 1;
            }
            if (y3 <= cy && y3 >= -cy) {
                if (flag == 0) { in[0] = rnd_half(x + cx); in[1] = rnd_half(y3 + cy); in[2] = 0; }
                else { out[0] = rnd_half(x + cx); out[1] = rnd_half(y3 + cy); out[2] = 0; }
                flag = 1;
            }
            if (y4 <= cy && y4 >= -cy) {
                if (flag == 0) { in[0] = rnd_half(x + cx); in[1] = rnd_half(y4 + cy); in[2] = (int)Z - 1; }
                else { out[0] = rnd_half(x + cx); out[1] = rnd_half(y4 + cy); out[2] = (int)Z - 1; }
            }
            if (flag != 0) {
                if ((float)(out[1] - in[1]) * k2 + (float)(out[2] - in[2]) * k3 < 0) {
                    t = in[1]; in[1] = out[1]; out[1] = t;
                    t = in[2]; in[2] = out[2]; out[2] = t;
                }
            }
            return 1;
        }
    }
    if (k1 != 0 && k2 == 0 && k3 != 0) {                 /* case 2, K:759 */
        if (y > -cy && y < cy) {
            float z1, z2, x3, x4;
            r = (-cx - x) / k1; z1 = z + k3 * r;
            r = (cx - x) / k1; z2 = z + k3 * r;
            r = (-cz - z) / k3; x3 = x + k1 * r;
            r = (cz - z) / k3; x4 = x + k1 * r;
            flag = 0;
            if (z1 <= cz && z1 >= -cz) {
                if (flag == 0) { in[0] = 0; in[1] = rnd_half(y + cy); in[2] = rnd_half(z1 + cz); }
                else { out[0] = 0; out[1] = rnd_half(y + cy); out[2] = rnd_half(z1 + cz); }
                flag = 1;
            }
            if (z2 <= cz && z2 >= -cz) {
                if (flag == 0) { in[0] = (int)X - 1; in[1] = rnd_half(y + cy); in[2] = rnd_half(z2 + cz); }
                else { out[0] = (int)X - 1; out[1] = rnd_half(y + cy); out[2] = rnd_half(z2 + cz); }
                flag = 1;
            }
            if (x3 <= cx && x3 >= -cx) {
                if (flag == 0) { in[0] = rnd_half(x3 + cx); in[1] = rnd_half(y + cy); in[2] = 0; }
                else { out[0] = rnd_half(x3 + cx); out[1] = rnd_half(y + cy); out[2] = 0; }
                flag = 1;
            }
            if (x4 <= cx && x4 >= -cx) {
                if (flag == 0) { in[0] = rnd_half(x4 + cx); in[1] = rnd_half(y + cy); in[2] = (int)Z - 1; }
                else { out[0] = rnd_half(x4 + cx); out[1] = rnd_half(y + cy); out[2] = (int)Z - 1; }
                flag = 1;
            }
            if (flag != 0) {
                if ((float)(out[0] - in[0]) * k1 + (float)(out[2] - in[2]) * k3 < 0) {
                    t = in[0]; in[0] = out[0]; out[0] = t;
                    t = in[2]; in[2] = out[2]; out[2] = t;
                }
            }
            return 1;
        }
    }
    if (k1 != 0 && k2 != 0 && k3 == 0) {                 /* case 3, K:847 */
        if (z > -cz && z < cz) {
            float y1, y2, x3, x4;
            r = (-cx - x) / k1; y1 = y + k2 * r;
            r = (cx - x) / k1; y2 = y + k2 * r;
            r = (-cy - z) / k2; x3 = x + k1 * r;          /* z for y: K:854 */
            r = (cy - z) / k2; x4 = x + k1 * r;           /* K:855 */
            flag = 0;
            if (y1 <= cy && y1 >= -cy) {
                if (flag == 0) { in[0] = 0; in[1] = rnd_half(y1 + cy); in[2] = rnd_half(z + cz); }
                else { out[0] = 0; out[1] = rnd_half(y1 + cy); out[2] = rnd_half(z + cz); }
                flag = 1;
            }
            if (y2 <= cy && y2 >= -cy) {
                if (flag == 0) { in[0] = (int)X - 1; in[1] = rnd_half(y2 + cy); in[2] = rnd_half(z + cz); }
                else { out[0] = (int)X - 1; out[1] = rnd_half(y2 + cy); out[2] = rnd_half(z + cz); }
                flag = 1;
            }
            if (x3 <= cx && x3 >= -cx) {
                if (flag == 0) { in[0] = rnd_half(x3 + cx); in[1] = 0; in[2] = rnd_half(z + cz); }
                else { out[0] = rnd_half(x3 + cx); out[1] = 0; out[2] = rnd_half(z + cz); }
                flag = 1;
            }
            if (x4 <= cx && x4 >= -cx) {
                if (flag == 0) { in[0] = rnd_half(x4 + cx); in[1] = (int)Y - 1; in[2] = rnd_half(z + cz); }
                else { out[0] = rnd_half(x4 + cx); out[1] = (int)Y - 1; out[2] = rnd_half(z + cz); }
                flag = 1;
            }
            if (flag != 0) {
                if ((float)(out[0] - in[0]) * k1 + (float)(out[1] - in[1]) * k2 < 0) {
                    t = in[0]; in[0] = out[0]; out[0] = t;
                    t = in[1]; in[1] = out[1]; out[1] = t;
                }
            }
            return 1;
        }
    }
    if ((double)fabsf(k1) < ORC_ZERO && (double)fabsf(k2) < ORC_ZERO && (double)fabsf(k3) >= ORC_ZERO) { /* case 4 */
        if (x < cx && x > -cx && y < cy && y > -cy) {
            in[0] = rnd_half(x + cx); out[0] = in[0];
            in[1] = rnd_half(y + cy); out[1] = in[1];
            if (k3 > 0) { in[2] = 0; out[2] = (int)Z - 1; }
            else { in[2] = (int)Z - 1; out[2] = 0; }
            return 1;
        }
    }
    if ((double)fabsf(k1) < ORC_ZERO && (double)fabsf(k2) >= ORC_ZERO && (double)fabsf(k3) < ORC_ZERO) { /* case 5 */
        if (x > -cx && x < cx && z > -cz && z < cz) {
            in[0] = rnd_half(x + cx); out[0] = in[0];
            in[2] = rnd_half(z + cz); out[2] = in[2];
            if (k2 > 0) { out[1] = (int)Y - 1; in[1] = 0; }
            else { in[1] = (int)Y - 1; out[1] = 0; }
            return 1;
        }
    }
    if ((double)fabsf(k1) >= ORC_ZERO && (double)fabsf(k2) < ORC_ZERO && (double)fabsf(k3) < ORC_ZERO) { /* case 6 */
        if (y > -cy && y < cy && z > -cz && z < cz) {
            in[1] = rnd_half(y + cy); out[1] = in[1];
            in[2] = rnd_half(z + cz); out[2] = in[2];
            if (k1 > 0) { out[0] = (int)X - 1; in[0] = 0; }
            else { in[0] = (int)X - 1; out[0] = 0; }
        }
        return 1;                                          /* K:989 */
    }
    if ((double)fabsf(k1) >= ORC_ZERO && (double)fabsf(k2) >= ORC_ZERO && (double)fabsf(k3) >= ORC_ZERO) { /* case 7 */
        float x1v, y1v, z1v, x2v, y2v, z2v, x3v, y3v, z3v, x4v, y4v, z4v, x5v, y5v, z5v, x6v, y6v, z6v;
        r = (-cx - x) / k1; x1v = -cx; y1v = y + k2 * r; z1v = z + k3 * r;
        r = (cx - x) / k1; x2v = cx; y2v = y + k2 * r; z2v = z + k3 * r;
        r = (-cy - y) / k2; x3v = x + k1 * r; y3v = -cy; z3v = z + k3 * r;
        r = (cy - y) / k2; x4v = x + k1 * r; y4v = cy; z4v = z + k3 * r;
        r = (-cz - z) / k3; x5v = x + k1 * r; y5v = y + k2 * r; z5v = -cz;
        r = (cz - z) / k3; x6v = x + k1 * r; y6v = y + k2 * r; z6v = cz;
        (void)x1v; (void)x2v; (void)y3v; (void)y4v; (void)z5v; (void)z6v;
        flag = 0;
        if (y1v <= cy && y1v >= -cy && z1v <= cz && z1v >= -cz) {
            if (flag == 0) { in[0] = 0; in[1] = rnd_half(y1v + cy); in[2] = rnd_half(z1v + cz); }
            else { out[0] = 0; out[1] = rnd_half(y1v + cy); out[2] = rnd_half(z1v + cz); }
            flag = 1;
        }
        if (y2v <= cy && y2v >= -cy && z2v <= cz && z2v >= -cz) {
            if (flag == 0) { in[0] = (int)X - 1; in[1] = rnd_half(y2v + cy); in[2] = rnd_half(z2v + cz); }
            else { out[0] = (int)X - 1; out[1] = rnd_half(y2v + cy); out[2] = rnd_half(z2v + cz); }
            flag = 1;
        }
        if (x3v <= cx && x3v >= -cx && z3v <= cz && z3v >= -cz) {
            if (flag == 0) { in[0] = rnd_half(x3v + cx); in[1] = 0; in[2] = rnd_half(z3v + cz); }
            else { out[0] = rnd_half(x3v + cx); out[1] = 0; out[2] = rnd_half(z3v + cz); }
            flag = 1;
        }
        if (x4v <= cx && x4v >= -cx && z4v <= cz && z4v >= -cz) {
            if (flag == 0) { in[0] = rnd_half(x4v + cx); in[1] = (int)Y - 1; in[2] = rnd_half(z4v + cz); }
            else { out[0] = rnd_half(x4v + cx); out[1] = (int)Y - 1; out[2] = rnd_half(z4v + cz); }
            flag = 1;
        }
        if (x5v <= cx && x5v >= -cx && y5v <= cy && y5v >= -cy) {
            if (flag == 0) { in[0] = rnd_half(x5v + cx); in[1] = rnd_half(y5v + cy); in[2] = 0; }
            else { out[0] = rnd_half(x5v + cx); out[1] = rnd_half(y5v + cy); out[2] = 0; }
            flag = 1;
        }
        if (x6v <= cx && x6v >= -cx && y6v <= cy && y6v >= -cy) {
            if (flag == 0) { in[0] = rnd_half(x6v + cx); in[1] = rnd_half(y6v + cy); in[2] = (int)Z - 1; }
            else { out[0] = rnd_half(x6v + cx); out[1] = rnd_half(y6v + cy); out[2] = (int)Z - 1; }
            flag = 1;
        }
        if ((float)(out[0] - in[0]) * k1 + (float)(out[1] - in[1]) * k2 + (float)(out[2] - in[2]) * k3 < 0) {
            t = in[0]; in[0] = out[0]; out[0] = t;
            t = in[1]; in[1] = out[1]; out[1] = t;
            t = in[2]; in[2] = out[2]; out[2] = t;
        }
        return 1;
    }
    return 0;
}

/* Caller-side acceptance test (K:6202-6206): both voxels inside the box and distinct
 * boundary indices.  The boundary index (K:8171-8212) is a bijection on boundary voxels
 * (checked against the reference's calIndex by the oracle tests), so "distinct index"
 * is "distinct voxel". */
int orc_line_valid(long X, long Y, long Z, const int in[3], const int out[3])
{
    if (!(in[0] >= 0 && in[0] < X && in[1] >= 0 && in[1] < Y && in[2] >= 0 && in[2] < Z &&
          out[0] >= 0 && out[0] < X && out[1] >= 0 && out[1] < Y && out[2] >= 0 && out[2] < Z))
        return 0;
    return !(in[0] == out[0] && in[1] == out[1] && in[2] == out[2]);
}

/* Greedy staircase walk of K:1762-1861: from the entry voxel, step along the axis whose
 * next voxel centre is nearest the line (ties x, then y, then z), until the exit voxel is
 * reached.  Writes one axis code (0,1,2) per step and returns the number of steps, or
 * -(steps+1) if no candidate qualified ("Error! Wrong Point Found!", K:1841).
 * rule selects the variant walks of the reference:
 *   0  the nearest-candidate rule above;
 *   1  bodyIntegralInnerWeightedFixedBC (K:2227): as 0, but a y step may not enter j = 0;
 *   2  bodyIntegralInnerSelectFixedBC (K:2628, 2675, 2722): ties y, then x, then z; no y
 *      step into j = 0 and no x or z step on j = 0;
 *   3  bodyIntegralInner(Weighted)MiniCurl (K:2869-2883, 3010-3024): the candidate with the
 *      smallest curl, read at the candidate's linear index when that index is inside the
 *      volume and 1e10 otherwise (the far candidate of an axis already at its exit
 *      coordinate can land inside the volume at an unrelated voxel), ties x, y, z.
 * A walk that stops early keeps the steps taken (the reference's loop ends there). */
int orc_walk_rule(long X, long Y, long Z, const int in[3], const int out[3], float x, float y,
                  float z, float k1, float k2, float k3, int rule, const float *curl,
                  signed char *axes, int cap)
{
    float cx = (float)((X - 1) / 2.0), cy = (float)((Y - 1) / 2.0), cz = (float)((Z - 1) / 2.0);
    x = x + cx; y = y + cy; z = z + cz;
    long il = in[0], jl = in[1], kl = in[2];
    long io = out[0], jo = out[1], ko = out[2];
    if (k1 * (float)(out[0] - in[0]) + k2 * (float)(out[1] - in[1]) + k3 * (float)(out[2] - in[2]) < 0) {
        k1 = -k1; k2 = -k2; k3 = -k3;
    }
    int n = 0;
    do {
        long i1 = il < io ? il + 1 : (il == io ? il - 60000 : il - 1);
        long j2 = jl < jo ? jl + 1 : (jl == jo ? jl - 60000 : jl - 1);
        long k3n = kl < ko ? kl + 1 : (kl == ko ? kl - 60000 : kl - 1);
        float r, xt, yt, zt, d1, d2, d3, a, b, c;
        if (rule == 3) {
            const long V = X * Y * Z;
            const long q1 = i1 + jl * X + kl * X * Y, q2 = il + j2 * X + kl * X * Y, q3 = il + jl * X + k3n * X * Y;
            d1 = (q1 >= 0 && q1 < V) ? curl[q1] : 1e10f;
            d2 = (q2 >= 0 && q2 < V) ? curl[q2] : 1e10f;
            d3 = (q3 >= 0 && q3 < V) ? curl[q3] : 1e10f;
        } else {
            r = k1 * (float)i1 - x * k1 + k2 * (float)jl - k2 * y + k3 * (float)kl - k3 * z;
            xt = x + k1 * r; yt = y + k2 * r; zt = z + k3 * r;
            a = xt - (float)i1; b = yt - (float)jl; c = zt - (float)kl;
            d1 = sqrtf(a * a + b * b + c * c);
            r = k1 * (float)il - x * k1 + k2 * (float)j2 - k2 * y + k3 * (float)kl - k3 * z;
            xt = x + k1 * r; yt = y + k2 * r; zt = z + k3 * r;
            a = xt - (float)il; b = yt - (float)j2; c = zt - (float)kl;
            d2 = sqrtf(a * a + b * b + c * c);
            r = k1 * (float)il - x * k1 + k2 * (float)jl - k2 * y + k3 * (float)k3n - k3 * z;
            xt = x + k1 * r; yt = y + k2 * r; zt = z + k3 * r;
            a = xt - (float)il; b = yt - (float)jl; c = zt - (float)k3n;
            d3 = sqrtf(a * a + b * b + c * c);
        }
        int moved = 0, tx, ty, tz;
        if (rule == 2) {
            tx = d1 < d2 && d1 <= d3 && i1 >= 0 && i1 < X && jl != 0;
            ty = d2 <= d1 && d2 <= d3 && j2 > 0 && j2 < Y;
            tz = d3 < d1 && d3 < d2 && k3n >= 0 && k3n < Z && jl != 0;
        } else {
            tx = d1 <= d2 && d1 <= d3 && i1 >= 0 && i1 < X;
            ty = d2 < d1 && d2 <= d3 && j2 >= (rule == 1 ? 1 : 0) && j2 < Y;
            tz = d3 < d1 && d3 < d2 && k3n >= 0 && k3n < Z;
        }
        if (tx) { if (n < cap) axes[n] = 0; n++; il = i1; moved = 1; }
        if (ty) { if (n < cap) axes[n] = 1; n++; jl = j2; moved = 1; }
        if (tz) { if (n < cap) axes[n] = 2; n++; kl = k3n; moved = 1; }
        if (!moved) return -(n + 1);
    } while ((double)(labs(il - io) + labs(jl - jo) + labs(kl - ko)) > 1e-5);
    return n;
}

int orc_walk(long X, long Y, long Z, const int in[3], const int out[3], float x, float y,
             float z, float k1, float k2, float k3, signed char *axes, int cap)
{
    return orc_walk_rule(X, Y, Z, in, out, x, y, z, k1, k2, k3, 0, NULL, axes, cap);
}

/* ------------------------------------------------------------------------------------ */
/* accumulation along one line                                                            */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    long X, Y, Z;
    float dx, dy, dz, rho, thr;
} orc_grid;

/* Sign of each axis step along a line: +1 toward a larger exit index, -1 otherwise. */
static inline void axis_signs(const int in[3], const int out[3], int sg[3])
{
    for (int a = 0; a < 3; a++) sg[a] = out[a] > in[a] ? 1 : -1;
}

/* Plain method along one line (K:1743-1863).  REAL = float reproduces the reference's
 * arithmetic bit for bit; REAL = double is the FP64 oracle.  self = 0 drops the entry's own
 * contribution, as bodyIntegralInnerMiniCurl does (K:2814). */
#define DEFINE_LINE_PLAIN(SUFFIX, REAL, EXACT)                                                  \
    static void line_plain_##SUFFIX(const orc_grid *g, const int in[3], const int out[3],      \
                                    const signed char *ax, int n, const float *au,              \
                                    const float *av, const float *aw, const REAL *p, REAL *pn,  \
                                    REAL *cnt, int self)                                        \
    {                                                                                           \
        long X = g->X, XY = g->X * g->Y;                                                        \
        int sg[3];                                                                              \
        axis_signs(in, out, sg);                                                                \
        long e = in[0] + in[1] * X + in[2] * XY;                                                \
        long last = e;                                                                          \
        const long stride[3] = {1, X, XY};                                                      \
        const float *comp[3] = {au, av, aw};                                                    \
        const float dl[3] = {g->dx, g->dy, g->dz};                                              \
        REAL pint = 0;                                                                          \
        if (self) {                                                                             \
            pn[e] += p[e];                                                                      \
            cnt[e] += 1;                                                                        \
        }                                                                                       \
        for (int s = 0; s < n; s++) {                                                           \
            int a = ax[s];                                                                      \
            long nx = last + sg[a] * stride[a];                                                 \
            if (EXACT) {                                                                        \
                float h = (-g->rho * (float)sg[a]) * dl[a];                                     \
                float as = comp[a][nx] + comp[a][last];                                         \
                pint = (REAL)((double)pint + ((double)h * 0.5) * (double)as);                  \
                pn[nx] += (REAL)(p[e] + pint);                                                  \
            } else {                                                                            \
                double term = -(double)g->rho * (double)sg[a] * (double)dl[a] * 0.5 *          \
                              ((double)comp[a][nx] + (double)comp[a][last]);                    \
                pint += (REAL)term;                                                             \
                pn[nx] += p[e] + pint;                                                          \
            }                                                                                   \
            cnt[nx] += 1;                                                                       \
            last = nx;                                                                          \
        }                                                                                       \
    }
DEFINE_LINE_PLAIN(f32, float, 1)
DEFINE_LINE_PLAIN(f64, double, 0)

/* Selected method along one line (K:2280-2537), including its asymmetries:
 *   - the entry counts as a segment start when 0 < curl <= thr (K:2301);
 *   - before the first start, an x step needs 0 < curl < thr but y/z steps only curl != 0
 *     (K:2376, 2422, 2468);
 *   - entering a bad voxel pauses the segment; an x step also pauses on curl == 0 through
 *     the operator precedence of K:2394, a y/z step does not (K:2440, 2486) -- it walks
 *     through the zero voxel without adding that step's increment;
 *   - a good voxel after a pause restarts the segment with p0 = p[voxel], I = 0; the z
 *     branch keeps the running curl/count sums (K:2497-2506);
 *   - contributions: pn += (p0+I)/C*n, count += 1/C*n with C = sum(curl/1e4), n = steps. */
#define DEFINE_LINE_SELECT(SUFFIX, REAL, EXACT)                                                  \
    static void line_select_##SUFFIX(const orc_grid *g, const int in[3], const int out[3],      \
                                     const signed char *ax, int n, const float *au,              \
                                     const float *av, const float *aw, const float *curl,        \
                                     const REAL *p, REAL *pn, REAL *cnt)                         \
    {                                                                                            \
        long X = g->X, XY = g->X * g->Y;                                                         \
        int sg[3];                                                                               \
        axis_signs(in, out, sg);                                                                 \
        long e = in[0] + in[1] * X + in[2] * XY;                                                 \
        long last = e;                                                                           \
        const long stride[3] = {1, X, XY};                                                       \
        const float *comp[3] = {au, av, aw};                                                     \
        const float dl[3] = {g->dx, g->dy, g->dz};                                               \
        const float thr = g->thr;                                                                \
        REAL pint = 0, ctmp = 0, ntmp = 0, p0 = 0;                                               \
        int started, outz = 0;                                                                   \
        if (curl[e] == 0 || curl[e] > thr) started = 0;                                          \
        else { p0 = p[e]; started = 1; ctmp = 0; ntmp = 0; }                                     \
        for (int s = 0; s < n; s++) {                                                            \
            int a = ax[s];                                                                       \
            long nx = last + sg[a] * stride[a];                                                  \
            float cn = curl[nx];                                                                 \
            if (!started) {                                                                      \
                int ok = (a == 0) ? (cn != 0 && cn < thr) : (cn != 0);                           \
                if (ok) { p0 = p[nx]; started = 1; pint = 0; ntmp = 0; ctmp = 0; }               \
            } else {                                                                             \
                int good = (cn < thr && cn != 0);                                                \
                if (outz == 0 && good) {                                                         \
                    if (EXACT) {                                                                 \
                        float h = (-g->rho * (float)sg[a]) * dl[a];                              \
                        float as = comp[a][nx] + comp[a][last];                                  \
                        pint = (REAL)((double)pint + ((double)h * 0.5) * (double)as);           \
                        ctmp += (REAL)(cn / 10000);                                              \
                    } else {                                                                     \
                        pint += -(double)g->rho * (double)sg[a] * (double)dl[a] * 0.5 *        \
                                ((double)comp[a][nx] + (double)comp[a][last]);                   \
                        ctmp += (double)cn / 10000.0;                                            \
                    }                                                                            \
                    ntmp += 1;                                                                   \
                    pn[nx] += (p0 + pint) * 1 / ctmp * ntmp;                                     \
                    cnt[nx] += 1 / ctmp * ntmp;                                                  \
                }                                                                                \
                int enter_bad = (a == 0) ? ((outz == 0 && cn >= thr) || cn == 0)                 \
                                         : (outz == 0 && cn >= thr);                             \
                if (enter_bad) outz = 1;                                                         \
                if (outz == 1 && good) {                                                         \
                    p0 = p[nx]; pint = 0; outz = 0;                                              \
                    if (a != 2) { ntmp = 0; ctmp = 0; }                                          \
                }                                                                                \
            }                                                                                    \
            last = nx;                                                                           \
        }                                                                                        \
    }
DEFINE_LINE_SELECT(f32, float, 1)
DEFINE_LINE_SELECT(f64, double, 0)

/* Weighted method along one line (K:1993-2135): the plain walk from the entry (no
 * contribution to the entry itself), every step adds its increment, and a step's voxel
 * receives (p0 + I)/C*n in pn and 1/C*n in count while C = sum(curl/1e4) != 0. */
#define DEFINE_LINE_WEIGHTED(SUFFIX, REAL, EXACT)                                                 \
    static void line_weighted_##SUFFIX(const orc_grid *g, const int in[3], const int out[3],     \
                                       const signed char *ax, int n, const float *au,             \
                                       const float *av, const float *aw, const float *curl,       \
                                       const REAL *p, REAL *pn, REAL *cnt)                        \
    {                                                                                             \
        long X = g->X, XY = g->X * g->Y;                                                          \
        int sg[3];                                                                                \
        axis_signs(in, out, sg);                                                                  \
        long e = in[0] + in[1] * X + in[2] * XY;                                                  \
        long last = e;                                                                            \
        const long stride[3] = {1, X, XY};                                                        \
        const float *comp[3] = {au, av, aw};                                                      \
        const float dl[3] = {g->dx, g->dy, g->dz};                                                \
        REAL pint = 0, ctmp = 0, ntmp = 0;                                                        \
        for (int s = 0; s < n; s++) {                                                             \
            int a = ax[s];                                                                        \
            long nx = last + sg[a] * stride[a];                                                   \
            if (EXACT) {                                                                          \
                float h = (-g->rho * (float)sg[a]) * dl[a];                                       \
                float as = comp[a][nx] + comp[a][last];                                           \
                pint = (REAL)((double)pint + ((double)h * 0.5) * (double)as);                    \
                ctmp += (REAL)(curl[nx] / 10000);                                                 \
            } else {                                                                              \
                pint += -(double)g->rho * (double)sg[a] * (double)dl[a] * 0.5 *                  \
                        ((double)comp[a][nx] + (double)comp[a][last]);                            \
                ctmp += (double)curl[nx] / 10000.0;                                               \
            }                                                                                     \
            ntmp += 1;                                                                            \
            if (ctmp != 0) {                                                                      \
                pn[nx] += (p[e] + pint) * 1 / ctmp * ntmp;                                        \
                cnt[nx] += 1 / ctmp * ntmp;                                                       \
            }                                                                                     \
            last = nx;                                                                            \
        }                                                                                         \
    }
DEFINE_LINE_WEIGHTED(f32, float, 1)
DEFINE_LINE_WEIGHTED(f64, double, 0)

/* Weighted method on the minimum-curl walk (bodyIntegralInnerWeightedMiniCurl, K:2937-3085):
 * the weight sum starts at the entry's curl, unscaled, and the entry receives p0/C*1; every
 * step adds its curl (not divided by 1e4) and contributes (p0 + I)/C*n, with no test for a
 * zero sum (a zero sum gives the reference's infinities). */
#define DEFINE_LINE_WEIGHTED_MC(SUFFIX, REAL, EXACT)                                              \
    static void line_weighted_mc_##SUFFIX(const orc_grid *g, const int in[3], const int out[3], \
                                          const signed char *ax, int n, const float *au,         \
                                          const float *av, const float *aw, const float *curl,   \
                                          const REAL *p, REAL *pn, REAL *cnt)                    \
    {                                                                                             \
        long X = g->X, XY = g->X * g->Y;                                                          \
        int sg[3];                                                                                \
        axis_signs(in, out, sg);                                                                  \
        long e = in[0] + in[1] * X + in[2] * XY;                                                  \
        long last = e;                                                                            \
        const long stride[3] = {1, X, XY};                                                        \
        const float *comp[3] = {au, av, aw};                                                      \
        const float dl[3] = {g->dx, g->dy, g->dz};                                                \
        REAL pint = 0, ctmp = (REAL)curl[e], ntmp = 1;                                            \
        pn[e] += p[e] * 1 / ctmp * ntmp;                                                          \
        cnt[e] += 1 / ctmp * ntmp;                                                                \
        for (int s = 0; s < n; s++) {                                                             \
            int a = ax[s];                                                                        \
            long nx = last + sg[a] * stride[a];                                                   \
            if (EXACT) {                                                                          \
                float h = (-g->rho * (float)sg[a]) * dl[a];                                       \
                float as = comp[a][nx] + comp[a][last];                                           \
                pint = (REAL)((double)pint + ((double)h * 0.5) * (double)as);                    \
            } else {                                                                              \
                pint += -(double)g->rho * (double)sg[a] * (double)dl[a] * 0.5 *                  \
                        ((double)comp[a][nx] + (double)comp[a][last]);                            \
            }                                                                                     \
            ctmp += (REAL)curl[nx];                                                               \
            ntmp += 1;                                                                            \
            pn[nx] += (p[e] + pint) * 1 / ctmp * ntmp;                                            \
            cnt[nx] += 1 / ctmp * ntmp;                                                           \
            last = nx;                                                                            \
        }                                                                                         \
    }
DEFINE_LINE_WEIGHTED_MC(f32, float, 1)
DEFINE_LINE_WEIGHTED_MC(f64, double, 0)

/* ------------------------------------------------------------------------------------ */
/* full sweep, normalisation, iteration                                                   */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    long X, Y, Z;
    float dx, dy, dz, rho, ls, thr;
    int nv;
    const float *k1, *k2, *k3;
    int mode;          /* 0 plain, 1 select, 2 weighted, 3 weighted fixed-BC, 4 select
                          fixed-BC, 5 minimum-curl plain, 6 minimum-curl weighted */
    int geom_cpu_twin; /* 1: CPU-twin geometry (no pole guard, NoGrid without spacing) */
} orc_problem;

/* Walk rule of each mode (see orc_walk_rule). */
static int orc_mode_walk_rule(int mode)
{
    switch (mode) {
    case 3: return 1;
    case 4: return 2;
    case 5:
    case 6: return 3;
    default: return 0;
    }
}

static long max_path(long X, long Y, long Z) { return X + Y + Z + 4; }

/* Walk every (direction, lattice point) pair in the reference's CPU order (K:8288-8290)
 * over the directions [d0, d1), accumulating into pn / cnt. Returns the number of lines
 * that hit the "Wrong Point" branch. */
#define DEFINE_SWEEP(SUFFIX, REAL)                                                                \
    static long sweep_range_##SUFFIX(const orc_problem *P, int d0, int d1, const float *au,       \
                                     const float *av, const float *aw, const float *curl,          \
                                     const REAL *p, REAL *pn, REAL *cnt)                           \
    {                                                                                              \
        orc_grid g = {P->X, P->Y, P->Z, P->dx, P->dy, P->dz, P->rho, P->thr};                      \
        int ng = orc_nogrid(P->X, P->Y, P->Z, P->ls, P->geom_cpu_twin);                            \
        long cap = max_path(P->X, P->Y, P->Z);                                                     \
        signed char *ax = (signed char *)malloc((size_t)cap);                                      \
        long errors = 0;                                                                           \
        for (int d = d0; d < d1; d++) {                                                            \
            float c[4];                                                                            \
            orc_dir_coeffs(P->k1[d], P->k2[d], P->k3[d], P->geom_cpu_twin, c);                     \
            for (int pt = 0; pt < ng * ng; pt++) {                                                 \
                float xyz[3];                                                                      \
                int in[3], out[3];                                                                 \
                orc_line_offset(pt, ng, P->ls, c, xyz);                                            \
                orc_cross2point(P->X, P->Y, P->Z, xyz[0], xyz[1], xyz[2], P->k1[d], P->k2[d],      \
                                P->k3[d], in, out);                                                \
                if (!orc_line_valid(P->X, P->Y, P->Z, in, out)) continue;                          \
                const int rule = orc_mode_walk_rule(P->mode);                                      \
                int n = orc_walk_rule(P->X, P->Y, P->Z, in, out, xyz[0], xyz[1], xyz[2], P->k1[d], \
                                      P->k2[d], P->k3[d], rule, curl, ax, (int)cap);               \
                if (n < 0) { if (rule == 0) errors++; n = -n - 1; }                                \
                if (P->mode == 0 || P->mode == 5)                                                  \
                    line_plain_##SUFFIX(&g, in, out, ax, n, au, av, aw, p, pn, cnt, P->mode == 0); \
                else if (P->mode == 2 || P->mode == 3)                                             \
                    line_weighted_##SUFFIX(&g, in, out, ax, n, au, av, aw, curl, p, pn, cnt);      \
                else if (P->mode == 6)                                                             \
                    line_weighted_mc_##SUFFIX(&g, in, out, ax, n, au, av, aw, curl, p, pn, cnt);   \
                else                                                                               \
                    line_select_##SUFFIX(&g, in, out, ax, n, au, av, aw, curl, p, pn, cnt);        \
            }                                                                                      \
        }                                                                                          \
        free(ax);                                                                                  \
        return errors;                                                                             \
    }
DEFINE_SWEEP(f32, float)
DEFINE_SWEEP(f64, double)

/* Sweep all directions.  nthreads > 1 splits the directions into contiguous blocks with
 * private accumulators that are added in block order, which changes only the order of
 * floating-point sums. */
#define DEFINE_SWEEP_ALL(SUFFIX, REAL)                                                            \
    long orc_sweep_##SUFFIX(const orc_problem *P, const float *au, const float *av,               \
                            const float *aw, const float *curl, const REAL *p, REAL *pn,          \
                            REAL *cnt, int nthreads)                                              \
    {                                                                                             \
        long V = P->X * P->Y * P->Z;                                                              \
        if (nthreads <= 1)                                                                        \
            return sweep_range_##SUFFIX(P, 0, P->nv, au, av, aw, curl, p, pn, cnt);               \
        REAL *pp = (REAL *)calloc((size_t)V * 2 * (size_t)nthreads, sizeof(REAL));                \
        long errors = 0;                                                                          \
        _Pragma("omp parallel for num_threads(nthreads) reduction(+ : errors) schedule(static, 1)") \
        for (int t = 0; t < nthreads; t++) {                                                      \
            int d0 = (int)((long)P->nv * t / nthreads), d1 = (int)((long)P->nv * (t + 1) / nthreads); \
            REAL *mypn = pp + (size_t)V * 2 * t, *mycnt = mypn + V;                               \
            errors += sweep_range_##SUFFIX(P, d0, d1, au, av, aw, curl, p, mypn, mycnt);          \
        }                                                                                         \
        for (int t = 0; t < nthreads; t++) {                                                      \
            REAL *mypn = pp + (size_t)V * 2 * t, *mycnt = mypn + V;                               \
            for (long v = 0; v < V; v++) { pn[v] += mypn[v]; cnt[v] += mycnt[v]; }               \
        }                                                                                         \
        free(pp);                                                                                 \
        return errors;                                                                            \
    }
DEFINE_SWEEP_ALL(f32, float)
DEFINE_SWEEP_ALL(f64, double)

/* Normalisation.  gpu_form = 1: devidecountInner (K:6746-6759), count > 0, pn reset.
 * gpu_form = 0: devidecountInnerCPU (K:8340-8351), count > 1, pn reset only there. */
#define DEFINE_DIVIDE(SUFFIX, REAL)                                                               \
    void orc_divide_##SUFFIX(long V, REAL *p, REAL *pn, const REAL *cnt, int gpu_form)            \
    {                                                                                             \
        for (long v = 0; v < V; v++) {                                                            \
            if (gpu_form ? cnt[v] > 0 : cnt[v] > 1) {                                             \
                pn[v] = pn[v] / cnt[v];                                                           \
                p[v] = pn[v];                                                                     \
                pn[v] = 0;                                                                        \
            }                                                                                     \
        }                                                                                         \
    }
DEFINE_DIVIDE(f32, float)
DEFINE_DIVIDE(f64, double)

/* The iteration of main() (K:8794-8863): p = pn = p_init, then niter times
 * {count = 0; sweep; divide}.  Returns p and the last iteration's count. */
#define DEFINE_SOLVE(SUFFIX, REAL)                                                                \
    long orc_solve_##SUFFIX(const orc_problem *P, const float *au, const float *av,               \
                            const float *aw, const float *curl, const float *p_init, int niter,   \
                            REAL *p, REAL *cnt, int nthreads)                                     \
    {                                                                                             \
        long V = P->X * P->Y * P->Z, errors = 0;                                                  \
        REAL *pn = (REAL *)malloc(sizeof(REAL) * (size_t)V);                                      \
        for (long v = 0; v < V; v++) { p[v] = (REAL)p_init[v]; pn[v] = (REAL)p_init[v]; cnt[v] = 0; } \
        for (int it = 0; it < niter; it++) {                                                      \
            memset(cnt, 0, sizeof(REAL) * (size_t)V);                                             \
            errors += orc_sweep_##SUFFIX(P, au, av, aw, curl, p, pn, cnt, nthreads);              \
            orc_divide_##SUFFIX(V, p, pn, cnt, 1);                                                \
        }                                                                                         \
        free(pn);                                                                                 \
        return errors;                                                                            \
    }
DEFINE_SOLVE(f32, float)
DEFINE_SOLVE(f64, double)

/* ------------------------------------------------------------------------------------ */
/* the same iteration with the line geometry traced and walked once                      */
/* ------------------------------------------------------------------------------------ */

/* orc_solve_f64 re-traces and re-walks every line in every sweep, as the reference does.
 * For fixed points at the full grid sizes of the benchmark (hundreds of iterations of a
 * direction subset) the lines are traced once here -- the same cross2point, validity test
 * and walk per (direction, lattice point) -- and only the accumulation (the f64 line
 * functions above, unchanged) runs per iteration.  Lines are processed in (direction,
 * lattice point) order, split into nthreads contiguous blocks of about equal step count
 * with private accumulators added in block order.  With tol > 0 the iteration stops after
 * the first iteration whose mean-gauged relative change over the voxels with count > 0,
 * sqrt(sum (d - mean d)^2 / sum (p - mean p)^2) with d = p_new - p_old, is below tol.
 * The iterates after the iteration counts save_at[0..nsave) (ascending) are copied to
 * saves + j * V.  Returns the number of lines that hit the reference's "Wrong Point" branch. */
typedef struct {
    int in[3], out[3];
    int n;
    long off;  /* first step in the step array */
} orc_cline;

typedef struct {
    orc_cline *lines;
    long nl, capl;
    signed char *steps;
    long ns, caps;
    long errors;
} orc_clist;

static void clist_push(orc_clist *L, const int in[3], const int out[3], const signed char *ax, int n)
{
    if (L->nl == L->capl) {
        L->capl = L->capl ? 2 * L->capl : 1024;
        L->lines = (orc_cline *)realloc(L->lines, sizeof(orc_cline) * (size_t)L->capl);
    }
    if (L->ns + n > L->caps) {
        while (L->ns + n > L->caps) L->caps = L->caps ? 2 * L->caps : 65536;
        L->steps = (signed char *)realloc(L->steps, (size_t)L->caps);
    }
    orc_cline *c = &L->lines[L->nl++];
    memcpy(c->in, in, sizeof(c->in));
    memcpy(c->out, out, sizeof(c->out));
    c->n = n;
    c->off = L->ns;
    memcpy(L->steps + L->ns, ax, (size_t)n);
    L->ns += n;
}

/* The traced lines of one problem, kept between sweeps (orc_cache_*). */
typedef struct {
    orc_problem P;
    orc_cline *lines;
    signed char *steps;
    long nl, ns, errors;
    long *bound;     /* nthreads + 1 line offsets of about equal work */
    int nthreads;
    double *pp;      /* per-thread private accumulators, 2 V each */
} orc_cache;

void *orc_cache_build(const orc_problem *P, const float *curl, int nthreads)
{
    const int ng = orc_nogrid(P->X, P->Y, P->Z, P->ls, P->geom_cpu_twin);
    const int rule = orc_mode_walk_rule(P->mode);
    const long cap = max_path(P->X, P->Y, P->Z);
    if (nthreads < 1) nthreads = 1;
    orc_clist *per_dir = (orc_clist *)calloc((size_t)P->nv, sizeof(orc_clist));
    /* trace and walk once, one direction per task */
    _Pragma("omp parallel for num_threads(nthreads) schedule(dynamic, 1)")
    for (int d = 0; d < P->nv; d++) {
        signed char *ax = (signed char *)malloc((size_t)cap);
        float c[4];
        orc_dir_coeffs(P->k1[d], P->k2[d], P->k3[d], P->geom_cpu_twin, c);
        for (int pt = 0; pt < ng * ng; pt++) {
            float xyz[3];
            int in[3], out[3];
            orc_line_offset(pt, ng, P->ls, c, xyz);
            orc_cross2point(P->X, P->Y, P->Z, xyz[0], xyz[1], xyz[2], P->k1[d], P->k2[d], P->k3[d], in, out);
            if (!orc_line_valid(P->X, P->Y, P->Z, in, out)) continue;
            int n = orc_walk_rule(P->X, P->Y, P->Z, in, out, xyz[0], xyz[1], xyz[2], P->k1[d], P->k2[d], P->k3[d],
                                  rule, curl, ax, (int)cap);
            if (n < 0) {
                if (rule == 0) per_dir[d].errors++;
                n = -n - 1;
            }
            clist_push(&per_dir[d], in, out, ax, n);
        }
        free(ax);
    }
    orc_cache *h = (orc_cache *)calloc(1, sizeof(orc_cache));
    h->P = *P;
    h->nthreads = nthreads;
    /* concatenate in direction order */
    for (int d = 0; d < P->nv; d++) {
        h->nl += per_dir[d].nl;
        h->ns += per_dir[d].ns;
        h->errors += per_dir[d].errors;
    }
    h->lines = (orc_cline *)malloc(sizeof(orc_cline) * (size_t)(h->nl > 0 ? h->nl : 1));
    h->steps = (signed char *)malloc((size_t)(h->ns > 0 ? h->ns : 1));
    for (long d = 0, l0 = 0, s0 = 0; d < P->nv; d++) {
        for (long i = 0; i < per_dir[d].nl; i++) {
            h->lines[l0 + i] = per_dir[d].lines[i];
            h->lines[l0 + i].off += s0;
        }
        memcpy(h->steps + s0, per_dir[d].steps, (size_t)per_dir[d].ns);
        l0 += per_dir[d].nl;
        s0 += per_dir[d].ns;
        free(per_dir[d].lines);
        free(per_dir[d].steps);
    }
    free(per_dir);
    /* thread blocks of about equal work (steps + 1 per line) */
    h->bound = (long *)malloc(sizeof(long) * (size_t)(nthreads + 1));
    long total = h->ns + h->nl, acc = 0, li = 0;
    h->bound[0] = 0;
    for (int t = 1; t < nthreads; t++) {
        long target = total * t / nthreads;
        while (li < h->nl && acc < target) acc += h->lines[li++].n + 1;
        h->bound[t] = li;
    }
    h->bound[nthreads] = h->nl;
    const long V = P->X * P->Y * P->Z;
    h->pp = (double *)malloc(sizeof(double) * (size_t)V * 2 * (size_t)nthreads);
    return h;
}

long orc_cache_errors(const void *hv) { return ((const orc_cache *)hv)->errors; }

void orc_cache_free(void *hv)
{
    orc_cache *h = (orc_cache *)hv;
    if (!h) return;
    free(h->lines);
    free(h->steps);
    free(h->bound);
    free(h->pp);
    free(h);
}

/* One FP64 sweep of the traced lines from p: pn += contributions, cnt += weights (the
 * threads' private sums added in block order). */
void orc_cache_sweep_f64(void *hv, const float *au, const float *av, const float *aw, const float *curl,
                         const double *p, double *pn, double *cnt)
{
    orc_cache *h = (orc_cache *)hv;
    const orc_problem *P = &h->P;
    const long V = P->X * P->Y * P->Z;
    const int nthreads = h->nthreads;
    orc_grid g = {P->X, P->Y, P->Z, P->dx, P->dy, P->dz, P->rho, P->thr};
    _Pragma("omp parallel for num_threads(nthreads) schedule(static, 1)")
    for (int t = 0; t < nthreads; t++) {
        double *mypn = h->pp + (size_t)V * 2 * t, *mycnt = mypn + V;
        memset(mypn, 0, sizeof(double) * 2 * (size_t)V);
        for (long i = h->bound[t]; i < h->bound[t + 1]; i++) {
            const orc_cline *c = &h->lines[i];
            const signed char *ax = h->steps + c->off;
            if (P->mode == 0 || P->mode == 5)
                line_plain_f64(&g, c->in, c->out, ax, c->n, au, av, aw, p, mypn, mycnt, P->mode == 0);
            else if (P->mode == 2 || P->mode == 3)
                line_weighted_f64(&g, c->in, c->out, ax, c->n, au, av, aw, curl, p, mypn, mycnt);
            else if (P->mode == 6)
                line_weighted_mc_f64(&g, c->in, c->out, ax, c->n, au, av, aw, curl, p, mypn, mycnt);
            else
                line_select_f64(&g, c->in, c->out, ax, c->n, au, av, aw, curl, p, mypn, mycnt);
        }
    }
    for (int t = 0; t < nthreads; t++) {
        const double *mypn = h->pp + (size_t)V * 2 * t, *mycnt = mypn + V;
        for (long v = 0; v < V; v++) { pn[v] += mypn[v]; cnt[v] += mycnt[v]; }
    }
}

long orc_solve_cached_f64(const orc_problem *P, const float *au, const float *av, const float *aw,
                          const float *curl, const float *p_init, int niter, double tol, double *p,
                          double *cnt, int nthreads, int *iters_out, double *rel_out, const int *save_at,
                          int nsave, double *saves)
{
    const long V = P->X * P->Y * P->Z;
    void *h = orc_cache_build(P, curl, nthreads);
    const long errors = orc_cache_errors(h);
    double *pn = (double *)malloc(sizeof(double) * (size_t)V);
    double *pold = (double *)malloc(sizeof(double) * (size_t)V);
    for (long v = 0; v < V; v++) { p[v] = (double)p_init[v]; pn[v] = (double)p_init[v]; cnt[v] = 0; }
    int it = 0;
    double rel = 0.0;
    for (it = 0; it < niter;) {
        memcpy(pold, p, sizeof(double) * (size_t)V);
        memset(cnt, 0, sizeof(double) * (size_t)V);
        orc_cache_sweep_f64(h, au, av, aw, curl, p, pn, cnt);
        orc_divide_f64(V, p, pn, cnt, 1);
        it++;
        for (int j = 0; j < nsave; j++)
            if (save_at[j] == it) memcpy(saves + (size_t)j * V, p, sizeof(double) * (size_t)V);
        /* mean-gauged relative change */
        double sd = 0, sp = 0, m = 0;
        for (long v = 0; v < V; v++)
            if (cnt[v] > 0) { sd += p[v] - pold[v]; sp += p[v]; m += 1; }
        double md = m > 0 ? sd / m : 0, mp = m > 0 ? sp / m : 0, a = 0, b = 0;
        for (long v = 0; v < V; v++)
            if (cnt[v] > 0) {
                double dd = p[v] - pold[v] - md, q = p[v] - mp;
                a += dd * dd;
                b += q * q;
            }
        rel = b > 0 ? sqrt(a / b) : 0.0;
        if (tol > 0 && rel < tol) break;
    }
    if (iters_out) *iters_out = it;
    if (rel_out) *rel_out = rel;
    orc_cache_free(h);
    free(pn);
    free(pold);
    return errors;
}

/* ------------------------------------------------------------------------------------ */
/* helpers exposed for the tests                                                          */
/* ------------------------------------------------------------------------------------ */

/* Line table of one direction: for every lattice point, valid flag, entry, exit and the
 * walk length (or -1 for invalid points). */
long orc_trace_direction(long X, long Y, long Z, float ls, float k1, float k2, float k3,
                         int geom_cpu_twin, int *valid, int *inout, int *nsteps, float *xyz)
{
    int ng = orc_nogrid(X, Y, Z, ls, geom_cpu_twin);
    float c[4];
    orc_dir_coeffs(k1, k2, k3, geom_cpu_twin, c);
    long cap = max_path(X, Y, Z), nvalid = 0;
    signed char *ax = (signed char *)malloc((size_t)cap);
    for (int pt = 0; pt < ng * ng; pt++) {
        int in[3], out[3];
        float o[3];
        orc_line_offset(pt, ng, ls, c, o);
        orc_cross2point(X, Y, Z, o[0], o[1], o[2], k1, k2, k3, in, out);
        int ok = orc_line_valid(X, Y, Z, in, out);
        valid[pt] = ok;
        for (int a = 0; a < 3; a++) { inout[6 * pt + a] = in[a]; inout[6 * pt + 3 + a] = out[a]; xyz[3 * pt + a] = o[a]; }
        nsteps[pt] = ok ? orc_walk(X, Y, Z, in, out, o[0], o[1], o[2], k1, k2, k3, ax, (int)cap) : -1;
        nvalid += ok;
    }
    free(ax);
    return nvalid;
}

/* Boundary numbering of calIndex (K:8171-8212): writes index[v] for boundary voxels and
 * leaves the rest untouched. */
void orc_calindex(long X, long Y, long Z, long *index)
{
    long n = X * Y * 2 + (Z - 2) * Y * 2 + (X - 2) * (Z - 2) * 2;
    for (long no = n - 1; no >= 0; no--) {
        long io = 0, jo = 0, ko = 0;
        long a = X * Y, b = a + Y * (Z - 1), c = b + (X - 1) * Y, d = c + (X - 1) * (Z - 2),
             e = d + (Y - 1) * (Z - 2);
        if (no <= a - 1) { ko = 0; jo = no / X; io = no - X * jo; }
        if (no > a - 1 && no <= b - 1) { io = X - 1; jo = (no - a) / (Z - 1); ko = no - a - jo * (Z - 1) + 1; }
        if (no > b - 1 && no <= c - 1) { ko = Z - 1; jo = (no - b) / (X - 1); io = no - b - jo * (X - 1); io = X - 2 - io; }
        if (no > c - 1 && no <= d - 1) { jo = 0; ko = (no - c) / (X - 1); io = no - c - ko * (X - 1); io = X - 2 - io; ko = ko + 1; }
        if (no > d - 1 && no <= e - 1) { io = 0; jo = (no - d) / (Z - 2); ko = no - d - jo * (Z - 2); ko = Z - 2 - ko; jo = jo + 1; }
        if (no > e - 1) { jo = Y - 1; ko = (no - e) / (X - 2); io = no - e - ko * (X - 2); ko = Z - 2 - ko; io = io + 1; }
        index[io + jo * X + ko * X * Y] = no;
    }
}

/* |curl a| times the mask (K:8352-8378): central differences inside, one-sided at the
 * faces, FP32 as in the reference. */
void orc_curl(long X, long Y, long Z, float dx, float dy, float dz, const float *au,
              const float *av, const float *aw, const float *mask, float *curl)
{
    for (long k = 0; k < Z; k++)
        for (long j = 0; j < Y; j++)
            for (long i = 0; i < X; i++) {
                long i0 = i - 1 >= 0 ? i - 1 : i, j0 = j - 1 >= 0 ? j - 1 : j, k0 = k - 1 >= 0 ? k - 1 : k;
                long ie = i + 1 <= X - 1 ? i + 1 : i, je = j + 1 <= Y - 1 ? j + 1 : j, ke = k + 1 <= Z - 1 ? k + 1 : k;
                long XY = X * Y;
                float cxv = (aw[i + je * X + k * XY] - aw[i + j0 * X + k * XY]) / (float)(je - j0) / dy;
                cxv += -(av[i + j * X + ke * XY] - av[i + j * X + k0 * XY]) / (float)(ke - k0) / dz;
                float cyv = -(aw[ie + j * X + k * XY] - aw[i0 + j * X + k * XY]) / (float)(ie - i0) / dx;
                cyv += (au[i + j * X + ke * XY] - au[i + j * X + k0 * XY]) / (float)(ke - k0) / dz;
                float czv = (av[ie + j * X + k * XY] - av[i0 + j * X + k * XY]) / (float)(ie - i0) / dx;
                czv += -(au[i + je * X + k * XY] - au[i + j0 * X + k * XY]) / (float)(je - j0) / dy;
                curl[i + j * X + k * XY] = sqrtf(cxv * cxv + cyv * cyv + czv * czv) * mask[i + j * X + k * XY];
            }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------------ */
/* FP64 adjoint of the plain iteration                                                    */
/* ------------------------------------------------------------------------------------ */

/* Visit every valid line of the plain method (same geometry as the sweep): the callback
 * receives the line's voxels v_0 (entry) .. v_n and the per-step axis and trapezoid
 * coefficient h_t = -rho * sign * dl / 2. */
typedef void (*orc_line_fn)(void *ud, const long *vox, const signed char *ax, const double *h, int n);

static void for_each_line(const orc_problem *P, orc_line_fn fn, void *ud)
{
    int ng = orc_nogrid(P->X, P->Y, P->Z, P->ls, P->geom_cpu_twin);
    long cap = max_path(P->X, P->Y, P->Z);
    signed char *ax = (signed char *)malloc((size_t)cap);
    long *vox = (long *)malloc(sizeof(long) * (size_t)(cap + 1));
    double *h = (double *)malloc(sizeof(double) * (size_t)cap);
    const long stride[3] = {1, P->X, P->X * P->Y};
    const float dl[3] = {P->dx, P->dy, P->dz};
    for (int d = 0; d < P->nv; d++) {
        float c[4];
        orc_dir_coeffs(P->k1[d], P->k2[d], P->k3[d], P->geom_cpu_twin, c);
        for (int pt = 0; pt < ng * ng; pt++) {
            float xyz[3];
            int in[3], out[3], sg[3];
            orc_line_offset(pt, ng, P->ls, c, xyz);
            orc_cross2point(P->X, P->Y, P->Z, xyz[0], xyz[1], xyz[2], P->k1[d], P->k2[d], P->k3[d], in, out);
            if (!orc_line_valid(P->X, P->Y, P->Z, in, out)) continue;
            int n = orc_walk(P->X, P->Y, P->Z, in, out, xyz[0], xyz[1], xyz[2], P->k1[d], P->k2[d], P->k3[d], ax,
                             (int)cap);
            if (n < 0) n = -n - 1;
            axis_signs(in, out, sg);
            vox[0] = in[0] + in[1] * P->X + in[2] * P->X * P->Y;
            for (int s = 0; s < n; s++) {
                int a = ax[s];
                vox[s + 1] = vox[s] + sg[a] * stride[a];
                h[s] = -(double)P->rho * (double)sg[a] * (double)dl[a] * 0.5;
            }
            fn(ud, vox, ax, h, n);
        }
    }
    free(ax);
    free(vox);
    free(h);
}

typedef struct {
    const double *mu;   /* per voxel */
    double *lam;        /* per voxel: gathered to line entries */
    double *cnt;
    double *ga[3];
} adj_ud;

static void cb_count(void *ud, const long *vox, const signed char *ax, const double *h, int n)
{
    adj_ud *U = (adj_ud *)ud;
    (void)ax; (void)h;
    for (int s = 0; s <= n; s++) U->cnt[vox[s]] += 1.0;
}

static void cb_gather(void *ud, const long *vox, const signed char *ax, const double *h, int n)
{
    adj_ud *U = (adj_ud *)ud;
    (void)ax; (void)h;
    double t = 0.0;
    for (int s = 0; s <= n; s++) t += U->mu[vox[s]];
    U->lam[vox[0]] += t;
}

static void cb_grad(void *ud, const long *vox, const signed char *ax, const double *h, int n)
{
    adj_ud *U = (adj_ud *)ud;
    double R = 0.0;
    for (int s = 1; s <= n; s++) R += U->mu[vox[s]];
    for (int t = 1; t <= n; t++) {
        int a = ax[t - 1];
        U->ga[a][vox[t]] += h[t - 1] * R;
        U->ga[a][vox[t - 1]] += h[t - 1] * R;
        R -= U->mu[vox[t]];
    }
}

/* Gradient of <g, p_K> with respect to (au, av, aw) for the plain iteration of orc_solve
 * (p = pn = p_init, niter x {sweep, divide where count > 0}), in FP64: the transpose of
 * p_k(v) = (sum over lines through v of p_{k-1}(entry) + I(v)) / c(v), kept p where c = 0.
 * The seeding of the first sweep with p_init does not depend on the gradient field. */
void orc_adjoint_f64(const orc_problem *P, int niter, const double *g, double *gau, double *gav, double *gaw)
{
    long V = P->X * P->Y * P->Z;
    double *cnt = (double *)calloc((size_t)V, sizeof(double));
    double *lam = (double *)malloc(sizeof(double) * (size_t)V);
    double *nxt = (double *)malloc(sizeof(double) * (size_t)V);
    double *mu = (double *)malloc(sizeof(double) * (size_t)V);
    double *macc = (double *)calloc((size_t)V, sizeof(double));
    adj_ud U;
    memset(&U, 0, sizeof(U));
    U.cnt = cnt;
    for_each_line(P, cb_count, &U);
    memcpy(lam, g, sizeof(double) * (size_t)V);
    for (int k = niter; k >= 1; k--) {
        for (long v = 0; v < V; v++) {
            mu[v] = cnt[v] > 0 ? lam[v] / cnt[v] : 0.0;
            macc[v] += mu[v];
            nxt[v] = cnt[v] > 0 ? 0.0 : lam[v];
        }
        if (k > 1) {
            U.mu = mu;
            U.lam = nxt;
            for_each_line(P, cb_gather, &U);
            memcpy(lam, nxt, sizeof(double) * (size_t)V);
        }
    }
    memset(gau, 0, sizeof(double) * (size_t)V);
    memset(gav, 0, sizeof(double) * (size_t)V);
    memset(gaw, 0, sizeof(double) * (size_t)V);
    U.mu = macc;
    U.ga[0] = gau;
    U.ga[1] = gav;
    U.ga[2] = gaw;
    for_each_line(P, cb_grad, &U);
    free(cnt);
    free(lam);
    free(nxt);
    free(mu);
    free(macc);
}

/* ------------------------------------------------------------------------------------ */
/* initial guess by integration outward from the centre (initialIntegration.cpp:9-407)   */
/* ------------------------------------------------------------------------------------ */

/* The eight octant sweeps of initialIntegration.cpp in its order (No.1-No.8): from the
 * centre voxel (X/2, Y/2, Z/2) outward, each voxel takes the mean over its off-centre axes,
 * in x, y, z order, of (the neighbour one step nearer the centre) + or - rho * 0.5 *
 * (a[voxel] + a[neighbour]) * spacing (+ when the voxel lies on the low side of the
 * centre along that axis).  The centre keeps its initial value; p[0] = pref is written
 * first (initialIntegration.cpp:12-13) and then overwritten by the first octant.
 * Double precision throughout, as the reference. */
void orc_centre_integration(long X, long Y, long Z, double dx, double dy, double dz, double rho,
                            const double *au, const double *av, const double *aw, double pref,
                            double *p)
{
    const long XY = X * Y;
    const long cx = X / 2, cy = Y / 2, cz = Z / 2;
    memset(p, 0, sizeof(double) * (size_t)(X * Y * Z));
    p[0] = pref;
    const int order[8][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {-1, 1, 1},  {1, 1, 1}};
    for (int o = 0; o < 8; o++) {
        const int sx = order[o][0], sy = order[o][1], sz = order[o][2];
        for (long k = cz; k >= 0 && k < Z; k += sz)
            for (long j = cy; j >= 0 && j < Y; j += sy)
                for (long i = cx; i >= 0 && i < X; i += sx) {
                    const long ind = i + j * X + k * XY;
                    int n = 0;
                    double v = 0.0;
                    if (i != cx) {
                        const long nb = ind - sx;
                        const double t = 0.5 * (au[ind] + au[nb]) * dx * rho;
                        v = sx < 0 ? p[nb] + t : p[nb] - t;
                        n++;
                    }
                    if (j != cy) {
                        const long nb = ind - sy * X;
                        const double t = 0.5 * (av[ind] + av[nb]) * dy * rho;
                        const double w = sy < 0 ? p[nb] + t : p[nb] - t;
                        v = n ? v + w : w;
                        n++;
                    }
                    if (k != cz) {
                        const long nb = ind - sz * XY;
                        const double t = 0.5 * (aw[ind] + aw[nb]) * dz * rho;
                        const double w = sz < 0 ? p[nb] + t : p[nb] - t;
                        v = n ? v + w : w;
                        n++;
                    }
                    if (n == 0) continue;  /* the centre */
                    p[ind] = n == 1 ? v : (n == 2 ? v / 2.0 : v / 3.0);
                }
    }
}

/* ------------------------------------------------------------------------------------ */
/* the reference's CPU Poisson baseline (sor3D.cpp) restated, for counting its iterations */
/* ------------------------------------------------------------------------------------ */

/* sor3D.cpp:9-1588 with its BCScheme all zero and its weights weight1 = weight2 = 0
 * (sor3D.cpp:5-7) is a weighted Jacobi iteration with omega = 0.8 on the Neumann Laplacian:
 * every voxel takes pn = (sum of its in-box axis neighbours + RHS) / (number of them) --
 * 6 inside, 5 on a face, 4 on an edge, 3 at a corner, the neighbours added in the order
 * i-1, i+1, j-1, j+1, k-1, k+1 -- then pn = p + 0.8 * (pn - p) (sor3D.cpp:739).  Each loop of
 * sor3D runs two such steps (a forward and a backward pass, sor3D.cpp:790-1575), so it
 * always takes an even number of steps.  This restatement runs the same steps with OpenMP;
 * it exists to count how many steps the reference needs at sizes where running the
 * reference itself to that point takes hours (the reference's own seconds per step are
 * timed separately). */
static void jacobi_step_f64(long X, long Y, long Z, const double *rhs, const double *p, double *pn,
                            int nthreads)
{
    const long XY = X * Y;
    _Pragma("omp parallel for num_threads(nthreads) schedule(static)")
    for (long k = 0; k < Z; k++)
        for (long j = 0; j < Y; j++)
            for (long i = 0; i < X; i++) {
                const long v = i + j * X + k * XY;
                double s = 0.0;
                int n = 0, first = 1;
#define ORC_NB(cond, off)                         \
    if (cond) {                                   \
        s = first ? p[v + (off)] : s + p[v + (off)]; \
        first = 0;                                \
        n++;                                      \
    }
                ORC_NB(i > 0, -1)
                ORC_NB(i < X - 1, 1)
                ORC_NB(j > 0, -X)
                ORC_NB(j < Y - 1, X)
                ORC_NB(k > 0, -XY)
                ORC_NB(k < Z - 1, XY)
#undef ORC_NB
                s += rhs[v];
                s = s / (double)n;
                pn[v] = p[v] + 0.8 * (s - p[v]);
            }
}

/* Mean-gauged relative L2 distance of p from ref (ref already mean-free). */
static double gauged_rel_f64(long V, const double *p, const double *ref, int nthreads)
{
    double sp = 0.0;
    _Pragma("omp parallel for num_threads(nthreads) reduction(+ : sp)")
    for (long v = 0; v < V; v++) sp += p[v];
    const double mp = sp / (double)V;
    double a = 0.0, b = 0.0;
    _Pragma("omp parallel for num_threads(nthreads) reduction(+ : a, b)")
    for (long v = 0; v < V; v++) {
        const double d = p[v] - mp - ref[v];
        a += d * d;
        b += ref[v] * ref[v];
    }
    return b > 0 ? sqrt(a / b) : 0.0;
}

/* nsteps steps of the restated iteration from p (in place). */
void orc_sor_steps_f64(long X, long Y, long Z, const double *rhs, double *p, long nsteps, int nthreads)
{
    const long V = X * Y * Z;
    double *pn = (double *)malloc(sizeof(double) * (size_t)V);
    for (long s = 0; s < nsteps; s++) {
        jacobi_step_f64(X, Y, Z, rhs, p, pn, nthreads);
        memcpy(p, pn, sizeof(double) * (size_t)V);
    }
    free(pn);
}

/* The converged (mean-free) solution of the restated iteration by conjugate gradients:
 * its fixed point solves A p = rhs - c * d, where A is the Neumann Laplacian (A p)_v =
 * d_v p_v - sum of in-box neighbours, d_v the neighbour count, and c = sum(rhs) / sum(d)
 * (the part of rhs along the constant mode, which only shifts the iterate's mean).
 * Stops when ||r|| <= tol * ||b||; returns the CG iterations. */
long orc_sor_converged_f64(long X, long Y, long Z, const double *rhs, double tol, long max_iter, double *p,
                           int nthreads)
{
    const long V = X * Y * Z, XY = X * Y;
    double *b = (double *)malloc(sizeof(double) * (size_t)V);
    double *r = (double *)malloc(sizeof(double) * (size_t)V);
    double *d = (double *)malloc(sizeof(double) * (size_t)V);
    double *q = (double *)malloc(sizeof(double) * (size_t)V);
    double *nb = (double *)malloc(sizeof(double) * (size_t)V);
    double srhs = 0.0, sd = 0.0;
    for (long v = 0; v < V; v++) {
        long i = v % X, j = (v / X) % Y, k = v / XY;
        nb[v] = (double)((i > 0) + (i < X - 1) + (j > 0) + (j < Y - 1) + (k > 0) + (k < Z - 1));
        srhs += rhs[v];
        sd += nb[v];
    }
    const double c = srhs / sd;
    double bb = 0.0;
    for (long v = 0; v < V; v++) {
        b[v] = rhs[v] - c * nb[v];
        p[v] = 0.0;
        r[v] = b[v];
        d[v] = r[v];
        bb += b[v] * b[v];
    }
    double rr = bb;
    long it = 0;
    while (it < max_iter && rr > tol * tol * bb) {
        double dq = 0.0;
        _Pragma("omp parallel for num_threads(nthreads) reduction(+ : dq) schedule(static)")
        for (long k = 0; k < Z; k++)
            for (long j = 0; j < Y; j++)
                for (long i = 0; i < X; i++) {
                    const long v = i + j * X + k * XY;
                    double s = nb[v] * d[v];
                    if (i > 0) s -= d[v - 1];
                    if (i < X - 1) s -= d[v + 1];
                    if (j > 0) s -= d[v - X];
                    if (j < Y - 1) s -= d[v + X];
                    if (k > 0) s -= d[v - XY];
                    if (k < Z - 1) s -= d[v + XY];
                    q[v] = s;
                    dq += d[v] * s;
                }
        const double alpha = rr / dq;
        double rr2 = 0.0;
        _Pragma("omp parallel for num_threads(nthreads) reduction(+ : rr2)")
        for (long v = 0; v < V; v++) {
            p[v] += alpha * d[v];
            r[v] -= alpha * q[v];
            rr2 += r[v] * r[v];
        }
        const double beta = rr2 / rr;
        rr = rr2;
        _Pragma("omp parallel for num_threads(nthreads)")
        for (long v = 0; v < V; v++) d[v] = r[v] + beta * d[v];
        it++;
    }
    double sp = 0.0;
    for (long v = 0; v < V; v++) sp += p[v];
    for (long v = 0; v < V; v++) p[v] -= sp / (double)V;
    free(b);
    free(r);
    free(d);
    free(q);
    free(nb);
    return it;
}

/* Steps of the restated iteration from p = 0 until the mean-gauged relative L2 distance
 * from ref (mean-free, e.g. orc_sor_converged_f64) is at most target, counted in sor3D's
 * pairs (the result is even); the distance is checked every `check` pairs and the last
 * interval is bisected by re-running from its start.  Returns -1 when max_steps pass. */
long orc_sor_steps_to_f64(long X, long Y, long Z, const double *rhs, const double *ref, double target, long max_steps,
                          long check, int nthreads, double *err_out)
{
    const long V = X * Y * Z;
    double *a = (double *)calloc((size_t)V, sizeof(double));
    double *b = (double *)malloc(sizeof(double) * (size_t)V);
    double *keep = (double *)malloc(sizeof(double) * (size_t)V);
    if (check < 1) check = 1;
    long steps = 0, found = -1;
    double err = gauged_rel_f64(V, a, ref, nthreads);
    while (steps < max_steps && err > target) {
        memcpy(keep, a, sizeof(double) * (size_t)V);
        const long s0 = steps;
        for (long c = 0; c < check; c++) {  /* one pair: a -> b -> a */
            jacobi_step_f64(X, Y, Z, rhs, a, b, nthreads);
            jacobi_step_f64(X, Y, Z, rhs, b, a, nthreads);
        }
        steps += 2 * check;
        err = gauged_rel_f64(V, a, ref, nthreads);
        if (err <= target) {  /* the first even step count in (s0, steps] that meets target */
            memcpy(a, keep, sizeof(double) * (size_t)V);
            long s = s0;
            double e = 0.0;
            do {
                jacobi_step_f64(X, Y, Z, rhs, a, b, nthreads);
                jacobi_step_f64(X, Y, Z, rhs, b, a, nthreads);
                s += 2;
                e = gauged_rel_f64(V, a, ref, nthreads);
            } while (e > target && s < steps);
            found = s;
            err = e;
        }
    }
    if (err_out) *err_out = err;
    free(a);
    free(b);
    free(keep);
    return found;
}

/* ------------------------------------------------------------------------------------ */
/* FP64 adjoint of every accumulation mode, curl held fixed                               */
/* ------------------------------------------------------------------------------------ */

/* With the curl field held fixed, every mode's iteration is affine in the gradient field:
 * a line's walk, its segments (the selected method's starts, pauses and restarts), its
 * weights and the steps whose trapezoid increments enter its integral depend on the curl
 * alone.  line_program_f64 records that structure for one line, in the FP64 line functions'
 * arithmetic (line_plain / line_select / line_weighted / line_weighted_mc above), for the
 * entry (index 0) and every step s = 1..n:
 *   vox[s]   the voxel;  seg[s] the segment the step belongs to (-1: none yet);
 *   term[s]  1 when the step's increment h * (a(v_s) + a(v_{s-1})) enters the integral;
 *   w[s]     the weight of the contribution w * (p(start) + I) made to vox[s] (0: none);
 * and start[j], the voxel whose value segment j reads.  Returns the number of segments. */
static int line_program_f64(const orc_grid *g, int mode, const int in[3], const int out[3], const signed char *ax,
                            int n, const float *curl, long *vox, int *seg, unsigned char *term, double *w,
                            long *start)
{
    const long X = g->X, XY = g->X * g->Y;
    int sg[3];
    axis_signs(in, out, sg);
    const long stride[3] = {1, X, XY};
    vox[0] = in[0] + in[1] * X + in[2] * XY;
    for (int s = 1; s <= n; s++) vox[s] = vox[s - 1] + sg[ax[s - 1]] * stride[ax[s - 1]];
    memset(term, 0, (size_t)n + 1);
    for (int s = 0; s <= n; s++) { w[s] = 0.0; seg[s] = -1; }
    const long e = vox[0];
    int nseg = 0;
    if (mode == 0 || mode == 5) {  /* plain: one segment from the entry, unit weights */
        start[nseg++] = e;
        for (int s = 0; s <= n; s++) { seg[s] = 0; term[s] = s > 0; w[s] = (s > 0 || mode == 0) ? 1.0 : 0.0; }
        return nseg;
    }
    if (mode == 2 || mode == 3 || mode == 6) {  /* weighted: one segment from the entry */
        start[nseg++] = e;
        double ctmp = mode == 6 ? (double)curl[e] : 0.0, ntmp = mode == 6 ? 1.0 : 0.0;
        seg[0] = 0;
        if (mode == 6) w[0] = 1 / ctmp * ntmp;
        for (int s = 1; s <= n; s++) {
            seg[s] = 0;
            term[s] = 1;
            ctmp += mode == 6 ? (double)curl[vox[s]] : (double)curl[vox[s]] / 10000.0;
            ntmp += 1;
            if (mode == 6 || ctmp != 0) w[s] = 1 / ctmp * ntmp;
        }
        return nseg;
    }
    /* selected (modes 1 and 4): the state machine of line_select */
    const float thr = g->thr;
    double ctmp = 0, ntmp = 0;
    int started = 0, outz = 0, cur = -1;
    if (!(curl[e] == 0 || curl[e] > thr)) { started = 1; cur = nseg; start[nseg++] = e; }
    seg[0] = cur;
    for (int s = 1; s <= n; s++) {
        const int a = ax[s - 1];
        const float cn = curl[vox[s]];
        if (!started) {
            int ok = (a == 0) ? (cn != 0 && cn < thr) : (cn != 0);
            if (ok) { started = 1; cur = nseg; start[nseg++] = vox[s]; ntmp = 0; ctmp = 0; }
        } else {
            int good = (cn < thr && cn != 0);
            if (outz == 0 && good) {
                ctmp += (double)cn / 10000.0;
                ntmp += 1;
                term[s] = 1;
                w[s] = 1 / ctmp * ntmp;
            }
            int enter_bad = (a == 0) ? ((outz == 0 && cn >= thr) || cn == 0) : (outz == 0 && cn >= thr);
            if (enter_bad) outz = 1;
            if (outz == 1 && good) {
                cur = nseg;
                start[nseg++] = vox[s];
                outz = 0;
                if (a != 2) { ntmp = 0; ctmp = 0; }
            }
        }
        seg[s] = cur;
    }
    return nseg;
}

/* Gradient of <g, p_niter> with respect to (au, av, aw) for the iteration of orc_solve
 * (p = pn = p_init, niter x {sweep, p = pn / count where count > 0}) of any mode, with curl
 * held fixed, in FP64 on the full voxel set (no anchor operator):
 *   p_k(v) = (sum over contributions c to v of w_c (p_{k-1}(start_c) + I_c) + seeding)
 *            / C(v)  where C(v) = sum w_c > 0, else p_{k-1}(v);
 * backwards: mu_k = lambda_k / C, dL/dI_c += w_c mu_k(v_c), lambda_{k-1}(start_c) +=
 * w_c mu_k(v_c) (+ lambda_k where C = 0); then along each segment the suffix sums R_t of
 * dL/dI over the contributions at or after step t multiply the step's trapezoid coefficient
 * and go to both voxels of the step.  The seeding by p_init does not depend on the field. */
void orc_adjoint_modes_f64(const orc_problem *P, const float *curl, int niter, const double *g, double *gau,
                           double *gav, double *gaw)
{
    const long V = P->X * P->Y * P->Z;
    orc_cache *h = (orc_cache *)orc_cache_build(P, curl, 1);
    orc_grid gr = {P->X, P->Y, P->Z, P->dx, P->dy, P->dz, P->rho, P->thr};
    const long cap = max_path(P->X, P->Y, P->Z) + 2;
    long *vox = (long *)malloc(sizeof(long) * (size_t)cap), *start = (long *)malloc(sizeof(long) * (size_t)cap);
    int *seg = (int *)malloc(sizeof(int) * (size_t)cap);
    unsigned char *term = (unsigned char *)malloc((size_t)cap);
    double *w = (double *)malloc(sizeof(double) * (size_t)cap);
    /* pass 1: the contributions (voxel, start voxel, weight) in line order, and C */
    long nc = 0, capc = 1 << 20;
    long *cv = (long *)malloc(sizeof(long) * (size_t)capc), *cs = (long *)malloc(sizeof(long) * (size_t)capc);
    double *cw = (double *)malloc(sizeof(double) * (size_t)capc);
    double *C = (double *)calloc((size_t)V, sizeof(double));
    for (long i = 0; i < h->nl; i++) {
        const orc_cline *c = &h->lines[i];
        line_program_f64(&gr, P->mode, c->in, c->out, h->steps + c->off, c->n, curl, vox, seg, term, w, start);
        for (int s = 0; s <= c->n; s++) {
            if (w[s] == 0.0) continue;
            if (nc == capc) {
                capc *= 2;
                cv = (long *)realloc(cv, sizeof(long) * (size_t)capc);
                cs = (long *)realloc(cs, sizeof(long) * (size_t)capc);
                cw = (double *)realloc(cw, sizeof(double) * (size_t)capc);
            }
            cv[nc] = vox[s];
            cs[nc] = start[seg[s]];
            cw[nc] = w[s];
            C[vox[s]] += w[s];
            nc++;
        }
    }
    /* the iterations backwards */
    double *dI = (double *)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
    double *lam = (double *)malloc(sizeof(double) * (size_t)V), *nxt = (double *)malloc(sizeof(double) * (size_t)V);
    double *mu = (double *)malloc(sizeof(double) * (size_t)V);
    memcpy(lam, g, sizeof(double) * (size_t)V);
    for (int k = niter; k >= 1; k--) {
        for (long v = 0; v < V; v++) {
            mu[v] = C[v] > 0 ? lam[v] / C[v] : 0.0;
            nxt[v] = C[v] > 0 ? 0.0 : lam[v];
        }
        for (long j = 0; j < nc; j++) {
            const double t = cw[j] * mu[cv[j]];
            dI[j] += t;
            nxt[cs[j]] += t;
        }
        memcpy(lam, nxt, sizeof(double) * (size_t)V);
    }
    /* pass 2: suffix sums along each segment, scattered to the two voxels of each step */
    memset(gau, 0, sizeof(double) * (size_t)V);
    memset(gav, 0, sizeof(double) * (size_t)V);
    memset(gaw, 0, sizeof(double) * (size_t)V);
    double *ga[3] = {gau, gav, gaw};
    const float dl[3] = {P->dx, P->dy, P->dz};
    long j0 = 0;
    for (long i = 0; i < h->nl; i++) {
        const orc_cline *c = &h->lines[i];
        const signed char *ax = h->steps + c->off;
        line_program_f64(&gr, P->mode, c->in, c->out, ax, c->n, curl, vox, seg, term, w, start);
        int sgn[3];
        axis_signs(c->in, c->out, sgn);
        long nline = 0;
        for (int s = 0; s <= c->n; s++) nline += w[s] != 0.0;
        long j = j0 + nline;  /* contributions of this line: [j0, j0 + nline) in step order */
        double R = 0.0;
        for (int s = c->n; s >= 1; s--) {
            if (s < c->n && seg[s] != seg[s + 1]) R = 0.0;
            if (w[s] != 0.0) R += dI[--j];
            if (term[s]) {
                const int a = ax[s - 1];
                const double hc = -(double)P->rho * (double)sgn[a] * (double)dl[a] * 0.5;
                ga[a][vox[s]] += hc * R;
                ga[a][vox[s - 1]] += hc * R;
            }
        }
        j0 += nline;
    }
    orc_cache_free(h);
    free(vox); free(start); free(seg); free(term); free(w);
    free(cv); free(cs); free(cw); free(C); free(dI); free(lam); free(nxt); free(mu);
}
