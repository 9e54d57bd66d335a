// Driver around the reference's own CPU functions (staged by oracle/build_ref.sh).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/ to pin the oracle, and by bench.py as the
// timed reference CPU baseline.  Nothing in the product links it.
//
// The reference's CPU iteration (omni3dparallellinesESInnerCPU, kernel.cu:8271-8327)
// differs from its GPU kernel (kernel.cu:6151-6215) in the lattice size (no division by
// the line spacing) and in the missing sin(theta) == 0 guard.  ref_sweep() therefore
// drives the reference's cross2point / bodyIntegralInner / bodyIntegralInnerSelect over
// every (direction, lattice point) pair with the GPU kernel's geometry, evaluated with
// libm sinf/cosf; ref_cpu_twin_solve() runs the reference's own CPU loop unchanged.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <streambuf>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

// reference functions (kernel.cu, sor3D.cpp, calRHS.cpp)
bool cross2point(long Xsize, long Ysize, long Zsize, int *iin, int *jin, int *kin, float xin,
                 float yin, float zin, float k1, float k2, float k3, int *iout, int *jout,
                 int *kout);
float bodyIntegralInner(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin, int iout,
                        int jout, int kout, float x, float y, float z, float k1, float k2,
                        float k3, float deltx, float delty, float deltz, float density,
                        float *DuDt, float *DvDt, float *DwDt, float *p, float *pn,
                        float *pcountinner);
float bodyIntegralInnerSelect(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin,
                              int iout, int jout, int kout, float x, float y, float z, float k1,
                              float k2, float k3, float deltx, float delty, float deltz,
                              float density, float *DuDt, float *DvDt, float *DwDt, float *p,
                              float *pn, float *curl, float *pcountinner, float threshold);
float bodyIntegralInnerWeighted(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin,
                                int iout, int jout, int kout, float x, float y, float z, float k1,
                                float k2, float k3, float deltx, float delty, float deltz,
                                float density, float *DuDt, float *DvDt, float *DwDt, float *curl,
                                float *p, float *pn, float *pcountinner);
float bodyIntegralInnerWeightedFixedBC(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin,
                                int iout, int jout, int kout, float x, float y, float z, float k1,
                                float k2, float k3, float deltx, float delty, float deltz,
                                float density, float *DuDt, float *DvDt, float *DwDt, float *curl,
                                float *p, float *pn, float *pcountinner);
float bodyIntegralInnerMiniCurl(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin,
                                int iout, int jout, int kout, float x, float y, float z, float k1,
                                float k2, float k3, float deltx, float delty, float deltz,
                                float density, float *DuDt, float *DvDt, float *DwDt, float *curl,
                                float *p, float *pn, float *pcountinner);
float bodyIntegralInnerWeightedMiniCurl(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin,
                                int iout, int jout, int kout, float x, float y, float z, float k1,
                                float k2, float k3, float deltx, float delty, float deltz,
                                float density, float *DuDt, float *DvDt, float *DwDt, float *curl,
                                float *p, float *pn, float *pcountinner);
float bodyIntegralInnerSelectFixedBC(long Xsize, long Ysize, long Zsize, int iin, int jin, int kin,
                              int iout, int jout, int kout, float x, float y, float z, float k1,
                              float k2, float k3, float deltx, float delty, float deltz,
                              float density, float *DuDt, float *DvDt, float *DwDt, float *p,
                              float *pn, float *curl, float *pcountinner, float threshold);
extern "C" void initialIntegration(long Xsize, long Ysize, long Zsize, double deltx, double delty, double deltz,
                                   double density, double *DuDt, double *DvDt, double *DwDt, double pref,
                                   double *p, double *pn, double *pBC);
void calIndex(long *index, long Xsize, long Ysize, long Zsize);
void omni3dparallellinesESInnerCPU(long Xsize, long Ysize, long Zsize, int NoAngles,
                                   float linespacing, float *k1_d, float *k2_d, float *k3_d,
                                   long *index, float deltx, float delty, float deltz,
                                   float density, float *DuDt, float *DvDt, float *DwDt, float *p,
                                   float *pn, float *pcountinner);
void devidecountInnerCPU(long Xsize, long Ysize, long Zsize, float *p, float *pn,
                         float *pcountinner);
void calCurlofMaterialAccCPU(long Xsize, long Ysize, long Zsize, float deltx, float delty,
                             float deltz, float *DuDt, float *DvDt, float *DwDt, float *curl,
                             float *mask);
extern "C" void sor3D(int Xsize, int Ysize, int Zsize, int NoItr, int *BCScheme, double *x,
                      double *y, double *z, double *p, double *pn, double *RHS, double eps);
extern "C" void calRHS(int Xsize, int Ysize, int Zsize, double deltx, double delty,
                       double deltz, double density, double *DuDt, double *DvDt, double *DwDt,
                       double *RHS);

namespace {

struct Problem {
    long X, Y, Z;
    float dx, dy, dz, rho, ls, thr;
    int nv;
    const float *k1, *k2, *k3;
    int mode;  // 0 plain, 1 select, 2 weighted, 3 weighted fixed-BC, 4 select fixed-BC,
               // 5 minimum-curl plain, 6 minimum-curl weighted
};

// Geometry of the GPU kernel (kernel.cu:6159-6194) with libm trigonometry.
int nogrid(const Problem &P)
{
    long ng = P.X;
    if (ng < P.Y) ng = P.Y;
    if (ng < P.Z) ng = P.Z;
    return (int)(ng * 1.732 / (double)P.ls);
}

long long sweep_range(const Problem &P, int d0, int d1, long *index, float *au, float *av, float *aw,
                      float *curl, float *p, float *pn, float *cnt)
{
    int ng = nogrid(P);
    long long units = 0;
    for (int angle = d0; angle < d1; angle++) {
        float k1 = P.k1[angle], k2 = P.k2[angle], k3 = P.k3[angle];
        float theta = acosf(k3);
        float st = sinf(theta);
        float phi = 0;
        if (st != 0) {
            phi = asinf(k2 / st);
            if (k1 / st < 0) phi = -phi + 3.1415926535897932384626433832795;
        }
        for (int point = 0; point < ng * ng; point++) {
            float xprime = (float(point / ng) - 0.5 * (ng - 1)) * P.ls;
            float yprime = (float(point - point / ng * ng) - 0.5 * (ng - 1)) * P.ls;
            float x = xprime * cosf(theta) * cosf(phi) - yprime * sinf(phi);
            float y = xprime * cosf(theta) * sinf(phi) + yprime * cosf(phi);
            float z = -xprime * sinf(theta);
            int iin, jin, kin, iout, jout, kout;
            cross2point(P.X, P.Y, P.Z, &iin, &jin, &kin, x, y, z, k1, k2, k3, &iout, &jout, &kout);
            if (iin >= 0 && iin < P.X && jin >= 0 && jin < P.Y && kin >= 0 && kin < P.Z &&
                iout >= 0 && iout < P.X && jout >= 0 && jout < P.Y && kout >= 0 && kout < P.Z) {
                long nin = index[iin + jin * P.X + kin * P.X * P.Y];
                long nout = index[iout + jout * P.X + kout * P.X * P.Y];
                if (nin != nout) {
                    units += std::abs(iout - iin) + std::abs(jout - jin) + std::abs(kout - kin) + 1;
                    if (P.mode == 0)
                        bodyIntegralInner(P.X, P.Y, P.Z, iin, jin, kin, iout, jout, kout, x, y, z,
                                          k1, k2, k3, P.dx, P.dy, P.dz, P.rho, au, av, aw, p, pn,
                                          cnt);
                    else if (P.mode == 2)
                        bodyIntegralInnerWeighted(P.X, P.Y, P.Z, iin, jin, kin, iout, jout, kout, x,
                                                  y, z, k1, k2, k3, P.dx, P.dy, P.dz, P.rho, au, av,
                                                  aw, curl, p, pn, cnt);
                    else if (P.mode == 3)
                        bodyIntegralInnerWeightedFixedBC(P.X, P.Y, P.Z, iin, jin, kin, iout, jout, kout,
                                                         x, y, z, k1, k2, k3, P.dx, P.dy, P.dz, P.rho,
                                                         au, av, aw, curl, p, pn, cnt);
                    else if (P.mode == 4)
                        bodyIntegralInnerSelectFixedBC(P.X, P.Y, P.Z, iin, jin, kin, iout, jout, kout,
                                                       x, y, z, k1, k2, k3, P.dx, P.dy, P.dz, P.rho, au,
                                                       av, aw, p, pn, curl, cnt, P.thr);
                    else if (P.mode == 5)
                        bodyIntegralInnerMiniCurl(P.X, P.Y, P.Z, iin, jin, kin, iout, jout, kout, x,
                                                  y, z, k1, k2, k3, P.dx, P.dy, P.dz, P.rho, au, av,
                                                  aw, curl, p, pn, cnt);
                    else if (P.mode == 6)
                        bodyIntegralInnerWeightedMiniCurl(P.X, P.Y, P.Z, iin, jin, kin, iout, jout,
                                                          kout, x, y, z, k1, k2, k3, P.dx, P.dy, P.dz,
                                                          P.rho, au, av, aw, curl, p, pn, cnt);
                    else
                        bodyIntegralInnerSelect(P.X, P.Y, P.Z, iin, jin, kin, iout, jout, kout, x,
                                                y, z, k1, k2, k3, P.dx, P.dy, P.dz, P.rho, au, av,
                                                aw, p, pn, curl, cnt, P.thr);
                }
            }
        }
    }
    return units;
}

struct NullBuf : std::streambuf {
    int overflow(int c) override { return c; }
};

}  // namespace

extern "C" {

void ref_calindex(long X, long Y, long Z, long *index) { calIndex(index, X, Y, Z); }

int ref_cross2point(long X, long Y, long Z, float x, float y, float z, float k1, float k2,
                    float k3, int *inout)
{
    return cross2point(X, Y, Z, inout + 0, inout + 1, inout + 2, x, y, z, k1, k2, k3, inout + 3,
                       inout + 4, inout + 5) ? 1 : 0;
}

// One full-coverage sweep (every direction, every lattice point) over [0, nv).  With
// nthreads > 1 the directions are split into contiguous blocks with private accumulators
// that are added in block order.  Returns the voxel-direction updates performed.
long long ref_sweep(long X, long Y, long Z, float dx, float dy, float dz, float rho, float ls,
               float thr, int nv, const float *k1, const float *k2, const float *k3, int mode,
               float *au, float *av, float *aw, float *curl, float *p, float *pn, float *cnt,
               int nthreads)
{
    Problem P{X, Y, Z, dx, dy, dz, rho, ls, thr, nv, k1, k2, k3, mode};
    long V = X * Y * Z;
    std::vector<long> index((size_t)V, -1);
    calIndex(index.data(), X, Y, Z);
    if (nthreads <= 1) return sweep_range(P, 0, nv, index.data(), au, av, aw, curl, p, pn, cnt);
    std::vector<float> priv((size_t)V * 2 * nthreads, 0.0f);
    long long units = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static, 1) reduction(+ : units)
    for (int t = 0; t < nthreads; t++) {
        int d0 = (int)((long)nv * t / nthreads), d1 = (int)((long)nv * (t + 1) / nthreads);
        float *mypn = priv.data() + (size_t)V * 2 * t, *mycnt = mypn + V;
        units += sweep_range(P, d0, d1, index.data(), au, av, aw, curl, p, mypn, mycnt);
    }
    for (int t = 0; t < nthreads; t++) {
        const float *mypn = priv.data() + (size_t)V * 2 * t, *mycnt = mypn + V;
        for (long v = 0; v < V; v++) { pn[v] += mypn[v]; cnt[v] += mycnt[v]; }
    }
    return units;
}

// Sweep of the directions [d0, d1) only (a bounded sample for timing), single thread per
// call; callers run several calls in parallel through nthreads in ref_sweep.
void ref_sweep_dirs(long X, long Y, long Z, float dx, float dy, float dz, float rho, float ls,
                    float thr, int d0, int d1, const float *k1, const float *k2,
                    const float *k3, int mode, float *au, float *av, float *aw, float *curl,
                    float *p, float *pn, float *cnt)
{
    Problem P{X, Y, Z, dx, dy, dz, rho, ls, thr, d1, k1, k2, k3, mode};
    long V = X * Y * Z;
    std::vector<long> index((size_t)V, -1);
    calIndex(index.data(), X, Y, Z);
    sweep_range(P, d0, d1, index.data(), au, av, aw, curl, p, pn, cnt);
}

// The iteration of the reference main() (kernel.cu:8794-8863) with full coverage:
// p = pn = p_init, then niter x {count = 0; sweep; p = pn / count where count > 0}.
void ref_solve(long X, long Y, long Z, float dx, float dy, float dz, float rho, float ls,
               float thr, int nv, const float *k1, const float *k2, const float *k3, int mode,
               float *au, float *av, float *aw, float *curl, const float *p_init, int niter,
               float *p, float *cnt, int nthreads)
{
    long V = X * Y * Z;
    std::vector<float> pn(p_init, p_init + V);
    memcpy(p, p_init, sizeof(float) * (size_t)V);
    for (int it = 0; it < niter; it++) {
        memset(cnt, 0, sizeof(float) * (size_t)V);
        ref_sweep(X, Y, Z, dx, dy, dz, rho, ls, thr, nv, k1, k2, k3, mode, au, av, aw, curl, p,
                  pn.data(), cnt, nthreads);
        for (long v = 0; v < V; v++) {  // devidecountInner, kernel.cu:6746-6759
            if (cnt[v] > 0) {
                pn[v] = pn[v] / cnt[v];
                p[v] = pn[v];
                pn[v] = 0;
            }
        }
    }
}

// The reference's own CPU loop, unchanged: omni3dparallellinesESInnerCPU followed by
// devidecountInnerCPU, niter times, starting from p = pn = p_init.
void ref_cpu_twin_solve(long X, long Y, long Z, float dx, float dy, float dz, float rho,
                        float ls, int nv, float *k1, float *k2, float *k3, float *au, float *av,
                        float *aw, const float *p_init, int niter, float *p, float *cnt)
{
    long V = X * Y * Z;
    std::vector<long> index((size_t)V, -1);
    calIndex(index.data(), X, Y, Z);
    std::vector<float> pn(p_init, p_init + V);
    memcpy(p, p_init, sizeof(float) * (size_t)V);
    for (int it = 0; it < niter; it++) {
        memset(cnt, 0, sizeof(float) * (size_t)V);
        omni3dparallellinesESInnerCPU(X, Y, Z, nv, ls, k1, k2, k3, index.data(), dx, dy, dz, rho,
                                      au, av, aw, p, pn.data(), cnt);
        devidecountInnerCPU(X, Y, Z, p, pn.data(), cnt);
    }
}

void ref_curl(long X, long Y, long Z, float dx, float dy, float dz, float *au, float *av,
              float *aw, float *mask, float *curl)
{
    calCurlofMaterialAccCPU(X, Y, Z, dx, dy, dz, au, av, aw, curl, mask);
}

// The reference's CPU Poisson baseline: RHS from calRHS, then sor3D (weighted Jacobi,
// omega = 0.8, forward/backward sweeps) for at most niter double sweeps or until the mean
// |residual| drops below eps.  Its per-iteration console output is discarded.
void ref_sor(int X, int Y, int Z, double dx, double dy, double dz, double rho, double *au,
             double *av, double *aw, int niter, double eps, double *p)
{
    long V = (long)X * Y * Z;
    std::vector<double> rhs((size_t)V, 0.0), pn((size_t)V, 0.0), xs((size_t)V, 0.0);
    calRHS(X, Y, Z, dx, dy, dz, rho, au, av, aw, rhs.data());
    int bc[6] = {0, 0, 0, 0, 0, 0};
    NullBuf nb;
    std::streambuf *old = std::cout.rdbuf(&nb);
    sor3D(X, Y, Z, niter, bc, xs.data(), xs.data(), xs.data(), p, pn.data(), rhs.data(), eps);
    std::cout.rdbuf(old);
}

void ref_calrhs(int X, int Y, int Z, double dx, double dy, double dz, double rho, double *au,
                double *av, double *aw, double *rhs)
{
    calRHS(X, Y, Z, dx, dy, dz, rho, au, av, aw, rhs);
}

int ref_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"

// initialIntegration.cpp on zeroed p / pn buffers (the reference leaves them to the caller).
extern "C" void ref_initial_integration(long X, long Y, long Z, double dx, double dy, double dz, double rho,
                                        double *au, double *av, double *aw, double pref, double *p)
{
    std::vector<double> pn((size_t)(X * Y * Z), 0.0), bc((size_t)(X * Y * Z), 0.0);
    std::fill(p, p + X * Y * Z, 0.0);
    initialIntegration(X, Y, Z, dx, dy, dz, rho, au, av, aw, pref, p, pn.data(), bc.data());
}
