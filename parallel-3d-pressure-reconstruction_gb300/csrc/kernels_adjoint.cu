// Adjoint of a solve: the gradient of <g, p_K> with respect to the gradient field
// (ax, ay, az), for every method, with the curl field held fixed.  No stored iterates are
// needed: with the curl fixed, a line's walk, segments, weights and the steps whose
// increments enter its integral depend on the curl alone, so the K-iteration map is affine
// in the field,
//     q_k = D^-1 (b + M q_{k-1} + seeding)        on the anchors, k = 1 .. K-1,
//     p(v) = (B(v) + S(v; q_{K-1}) + seeding) / c(v)  on every voxel with c(v) > 0,
// where a voxel v receives from every contribution c of a segment through it the weight
// w_c times (q(start_c) + I_c): B(v) = sum w_c I_c, S(v; q) = sum w_c q(start_c), c = sum w_c,
// b = B and M the weighted links on the anchors.  Its transpose is
//     mu = g / c;  lambda_{K-1} = S^T mu  (each segment's sum of w mu, sent to its start);
//     for k = K-1 .. 1:  acc += D^-1 lambda_k;  lambda_{k-1} = M^T D^-1 lambda_k (+ lambda_k
//                        where c = 0);
//     dL/dB = mu + acc on the anchors;
//     dL/da: along every segment, the suffix sum R_t of w dL/dB over the contributions at or
//     after step t multiplies the trapezoid coefficient h_t of every step whose increment
//     enters the integral, and is scattered to the two voxels of that step
//     (I_c = sum over those steps t <= c of h_t (a(v_t) + a(v_{t-1})) along the step's axis).
// The selected method (K:2280-2537), the weighted ones (K:1993-2135, 2937-3085) and the
// plain ones (K:1743-1863, 2797-2936) differ only in the line program below.  The curl of
// a voxel is read from .w of the packed FP32 field of the solve (the stored curl for BF16
// storage).  The derivative through the curl (its weights and segment decisions, which
// are piecewise constant in it) is not included.
#include <algorithm>
#include <utility>

#include "omni3d_internal.h"

namespace omni3d {

namespace {

struct AdjWalk {
    long long v;
    int d0, d1, d2;
    float h0, h1, h2;
    int m;
    const uint32_t *dp;
    __device__ __forceinline__ void init(const Grid &g, const LineRec &r, const uint32_t *gbase, const uint32_t *desc,
                                         long long li)
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

// The per-line program of a method's accumulation (the forward kernels' state machines and
// weight arithmetic): init() at the entry gives the entry's contribution weight and whether
// a segment starts there; step() for each step gives the contribution weight w (0: none),
// whether the step's increment enters the integral, and whether a new segment starts at the
// step's voxel.
template <int ACC>
struct LineProg {
    bool started = true, paused = false;
    float csum = 0.0f, nseg = 0.0f;
    __device__ __forceinline__ void init(float ce, float thr, float &w, bool &seg)
    {
        w = 0.0f;
        seg = true;
        if (ACC == kAccPlain) w = 1.0f;
        if (ACC == kAccWeightedRawCurl) {
            csum = ce;
            nseg = 1.0f;
            w = __frcp_rn(csum);
        }
        if (ACC == kAccSelect) {
            started = !(ce == 0.0f || ce > thr);
            seg = started;
        }
    }
    __device__ __forceinline__ void step(int a, float cn, float thr, float &w, bool &term, bool &restart)
    {
        w = 0.0f;
        term = false;
        restart = false;
        if (ACC == kAccPlain || ACC == kAccPlainNoEntry) {
            w = 1.0f;
            term = true;
        } else if (ACC == kAccWeighted) {
            term = true;
            csum += __fdiv_rn(cn, 1.0e4f);
            nseg += 1.0f;
            if (csum != 0.0f) w = __fdividef(nseg, csum);
        } else if (ACC == kAccWeightedRawCurl) {
            term = true;
            csum += cn;
            nseg += 1.0f;
            w = __fdividef(nseg, csum);
        } else {  // selected
            if (!started) {
                const bool ok = (a == 0) ? (cn != 0.0f && cn < thr) : (cn != 0.0f);
                if (ok) {
                    started = true;
                    restart = true;
                    nseg = 0.0f;
                    csum = 0.0f;
                }
            } else {
                const bool good = cn < thr && cn != 0.0f;
                if (!paused && good) {
                    term = true;
                    csum += cn * 1.0e-4f;
                    nseg += 1.0f;
                    w = __fdividef(nseg, csum);
                }
                const bool enter_bad = (a == 0) ? ((!paused && cn >= thr) || cn == 0.0f) : (!paused && cn >= thr);
                if (enter_bad) paused = true;
                if (paused && good) {
                    restart = true;
                    paused = false;
                    if (a != 2) {
                        nseg = 0.0f;
                        csum = 0.0f;
                    }
                }
            }
        }
    }
};

// Step decoder over a line's staircase (2-bit steps, lane-interleaved words).
struct StepCursor {
    const uint32_t *dp;
    uint32_t word;
    int s, m;
    long long v;
    __device__ __forceinline__ bool next(const AdjWalk &L, int &a, long long &prev)
    {
        if (s >= m) return false;
        if ((s & 15) == 0) word = __ldg(dp + 32 * (s >> 4));
        a = (int)(word & 3u);
        word >>= 2;
        prev = v;
        v += a == 0 ? L.d0 : (a == 1 ? L.d1 : L.d2);
        s++;
        return true;
    }
};

__device__ __forceinline__ float curl_at(const float4 *f32, long long v) { return __ldg(&f32[v].w); }

// mu = g / c where c > 0, else 0
__global__ void k_adj_mu(long long V, const float *g, const float *cnt, float *mu)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        mu[v] = cnt[v] > 0.0f ? __fdiv_rn(g[v], cnt[v]) : 0.0f;
}

// lambda[id(start)] += sum of w mu over each segment (S^T mu)
template <int ACC>
__global__ void __launch_bounds__(256) k_adj_gather(Grid g, const LineRec *__restrict__ lines,
                                                    const uint32_t *__restrict__ gbase,
                                                    const uint32_t *__restrict__ desc, long long n_lines,
                                                    const float4 *__restrict__ f32, const float *__restrict__ mu,
                                                    const int32_t *__restrict__ id, float *lam)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    AdjWalk L;
    L.init(g, r, gbase, desc, li);
    LineProg<ACC> P;
    float w;
    bool seg;
    P.init(curl_at(f32, L.v), g.thr, w, seg);
    long long start = seg ? L.v : -1;
    float t = w != 0.0f ? w * __ldg(mu + L.v) : 0.0f;
    StepCursor c{L.dp, 0u, 0, L.m, L.v};
    int a;
    long long prev;
    while (c.next(L, a, prev)) {
        bool term, restart;
        P.step(a, curl_at(f32, c.v), g.thr, w, term, restart);
        if (restart) {
            if (start >= 0 && t != 0.0f) {
                const int row = __ldg(id + start);
                if (row >= 0) atomicAdd(lam + row, t);
            }
            start = c.v;
            t = 0.0f;
        }
        if (w != 0.0f) t += w * __ldg(mu + c.v);
    }
    if (start >= 0 && t != 0.0f) {
        const int row = __ldg(id + start);
        if (row >= 0) atomicAdd(lam + row, t);
    }
}

// The sum of w dB over the contributions of the segment that follows the cursor's position
// (up to the next segment start or the end of the line), without moving the cursor.
template <int ACC>
__device__ __forceinline__ float segment_total(const Grid &g, const AdjWalk &L, StepCursor c, LineProg<ACC> P,
                                               const float4 *f32, const float *dB)
{
    float T = 0.0f;
    int a;
    long long prev;
    while (c.next(L, a, prev)) {
        float w;
        bool term, restart;
        P.step(a, curl_at(f32, c.v), g.thr, w, term, restart);
        if (restart) break;
        if (w != 0.0f) T += w * __ldg(dB + c.v);
    }
    return T;
}

// dL/da along every segment: suffix sums R_t of w dB times the trapezoid coefficients
template <int ACC>
__global__ void __launch_bounds__(256) k_adj_grad(Grid g, const LineRec *__restrict__ lines,
                                                  const uint32_t *__restrict__ gbase,
                                                  const uint32_t *__restrict__ desc, long long n_lines,
                                                  const float4 *__restrict__ f32, const float *__restrict__ dB,
                                                  float *gx, float *gy, float *gz)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    AdjWalk L;
    L.init(g, r, gbase, desc, li);
    LineProg<ACC> P;
    float w;
    bool seg;
    P.init(curl_at(f32, L.v), g.thr, w, seg);
    StepCursor c{L.dp, 0u, 0, L.m, L.v};
    float R = seg ? segment_total<ACC>(g, L, c, P, f32, dB) : 0.0f;
    int a;
    long long prev;
    while (c.next(L, a, prev)) {
        bool term, restart;
        P.step(a, curl_at(f32, c.v), g.thr, w, term, restart);
        if (restart) R = segment_total<ACC>(g, L, c, P, f32, dB);  // the new segment's contributions
        if (term) {
            const float val = (a == 0 ? L.h0 : (a == 1 ? L.h1 : L.h2)) * R;
            float *ga = a == 0 ? gx : (a == 1 ? gy : gz);
            atomicAdd(ga + c.v, val);
            atomicAdd(ga + prev, val);
        }
        if (w != 0.0f) R -= w * __ldg(dB + c.v);
    }
}

// Column and weight of operator entry j: unit-weight operators store the column alone,
// weighted ones (column, weight bits).
__device__ __forceinline__ uint32_t entry_col(const uint32_t *col, const uint2 *cw, unsigned long long j)
{
    return col ? col[j] : cw[j].x;
}
__device__ __forceinline__ float entry_w(const uint2 *cw, unsigned long long j)
{
    return cw ? __uint_as_float(cw[j].y) : 1.0f;
}

// transposed operator: count entries per column
__global__ void k_adj_tcount(long long n, const unsigned long long *rowptr, const uint32_t *rowlen,
                             const uint32_t *col, const uint2 *cw, uint32_t *tcnt)
{
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    unsigned long long j0 = rowptr[row], j1 = j0 + rowlen[row];
    for (unsigned long long j = j0 + lane; j < j1; j += 32) atomicAdd(tcnt + entry_col(col, cw, j), 1u);
}

__global__ void k_adj_tfill(long long n, const unsigned long long *rowptr, const uint32_t *rowlen, const uint32_t *col,
                            const uint2 *cw, const unsigned long long *tptr, uint32_t *tcur, uint32_t *trow, float *tw)
{
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    unsigned long long j0 = rowptr[row], j1 = j0 + rowlen[row];
    for (unsigned long long j = j0 + lane; j < j1; j += 32) {
        const uint32_t c = entry_col(col, cw, j);
        const unsigned long long pos = tptr[c] + atomicAdd(tcur + c, 1u);
        trow[pos] = (uint32_t)row;
        if (tw) tw[pos] = entry_w(cw, j);
    }
}

__global__ void k_u32_to_u64(long long n, const uint32_t *in, unsigned long long *out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i];
}

// acc += lambda / c (c > 0)
__global__ void k_adj_accum(long long n, const float *lam, const float2 *bc, float *acc)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float c = bc[i].y;
        if (c > 0.0f) acc[i] += __fdiv_rn(lam[i], c);
    }
}

// next = M^T D^-1 lambda (+ lambda where c = 0), a warp per column of M (tw: the entries'
// weights, null for unit weights)
__global__ void __launch_bounds__(256) k_adj_spmvT(long long n, const unsigned long long *__restrict__ tptr,
                                                   const uint32_t *__restrict__ trow, const float *__restrict__ tw,
                                                   const float *__restrict__ lam, const float2 *__restrict__ bc,
                                                   float *__restrict__ next)
{
    long long a = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (a >= n) return;
    unsigned long long j0 = tptr[a], j1 = tptr[a + 1];
    float s = 0.0f;
    for (unsigned long long j = j0 + lane; j < j1; j += 32) {
        uint32_t r = __ldg(trow + j);
        float cr = __ldg(&bc[r].y);
        if (cr > 0.0f) s += (tw ? __ldg(tw + j) : 1.0f) * __fdiv_rn(__ldg(lam + r), cr);
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) next[a] = s + (bc[a].y > 0.0f ? 0.0f : lam[a]);
}

// dB[vox[a]] += acc[a]
__global__ void k_adj_add_anchor(long long n, const uint32_t *vox, const float *acc, float *dB)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dB[vox[i]] += acc[i];
}

// Transpose of the gauge applied to the output: G = I - 1 w^T with w = [count > 0] / n_c
// (mean) or the unit vector at ref (point), so G^T g = g - w * sum(g).
constexpr int kRB = 256;
__global__ void k_sum_g(long long V, const float *g, const float *cnt, double *part)
{
    __shared__ double sh[2][32];
    double s = 0.0, n = 0.0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        s += (double)g[v];
        n += cnt[v] > 0.0f ? 1.0 : 0.0;
    }
    for (int o = 16; o; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        n += __shfl_down_sync(0xffffffffu, n, o);
    }
    if ((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = s; sh[1][threadIdx.x >> 5] = n; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a += sh[0][w]; b += sh[1][w]; }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

__global__ void k_gauge_T(long long V, const float *g, const float *cnt, const double *part, int nblk, int gauge,
                          long long ref, float *out)
{
    double S = 0.0, N = 0.0;
    for (int b = 0; b < nblk; b++) { S += part[2 * b]; N += part[2 * b + 1]; }
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        double x = (double)g[v];
        if (gauge == OMNI3D_GAUGE_MEAN && cnt[v] > 0.0f && N > 0) x -= S / N;
        if (gauge == OMNI3D_GAUGE_POINT && v == ref) x -= S;
        out[v] = (float)x;
    }
}

unsigned grid_for(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 64) b = 152LL * 64;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace

cudaError_t gauge_transpose(long long V, int gauge, long long ref, const float *g, const float *cnt, float *out,
                            double *part, cudaStream_t st)
{
    if (gauge == OMNI3D_GAUGE_NONE)
        return cudaMemcpyAsync(out, g, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st);
    k_sum_g<<<kRB, 256, 0, st>>>(V, g, cnt, part);
    OM_COUNT_LAUNCH();
    k_gauge_T<<<grid_for(V), 256, 0, st>>>(V, g, cnt, part, kRB, gauge, ref, out);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

size_t gauge_transpose_scratch_doubles() { return 2 * kRB; }

void adjoint_free(AdjointBuffers *B)
{
    cudaFree(B->tptr);
    cudaFree(B->trow);
    cudaFree(B->tw);
    cudaFree(B->tmp);
    cudaFree(B->mu);
    cudaFree(B->lam);
    cudaFree(B->nxt);
    cudaFree(B->acc);
    *B = AdjointBuffers();
}

#define ADJ_TRY(x)                               \
    do {                                         \
        cudaError_t e_ = (x);                    \
        if (e_ != cudaSuccess) return e_;        \
    } while (0)

template <int ACC>
void launch_adj_lines(const Geometry &geo, bool gather, const float4 *f32, const float *in, const int32_t *id,
                      float *lam, float *gx, float *gy, float *gz, cudaStream_t st)
{
    const unsigned lblocks = (unsigned)((geo.n_lines + 255) / 256);
    if (gather)
        k_adj_gather<ACC><<<lblocks, 256, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines, f32, in,
                                                   id, lam);
    else
        k_adj_grad<ACC><<<lblocks, 256, 0, st>>>(geo.grid, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines, f32, in,
                                                 gx, gy, gz);
    OM_COUNT_LAUNCH();
}

void adj_lines(int acc, const Geometry &geo, bool gather, const float4 *f32, const float *in, const int32_t *id,
               float *lam, float *gx, float *gy, float *gz, cudaStream_t st)
{
    switch (acc) {
    case kAccSelect: launch_adj_lines<kAccSelect>(geo, gather, f32, in, id, lam, gx, gy, gz, st); break;
    case kAccWeighted: launch_adj_lines<kAccWeighted>(geo, gather, f32, in, id, lam, gx, gy, gz, st); break;
    case kAccPlainNoEntry: launch_adj_lines<kAccPlainNoEntry>(geo, gather, f32, in, id, lam, gx, gy, gz, st); break;
    case kAccWeightedRawCurl: launch_adj_lines<kAccWeightedRawCurl>(geo, gather, f32, in, id, lam, gx, gy, gz, st); break;
    default: launch_adj_lines<kAccPlain>(geo, gather, f32, in, id, lam, gx, gy, gz, st); break;
    }
}

cudaError_t adjoint_solve(const Geometry &geo, const Anchor &A, AdjointBuffers *B, int K, int method, const float4 *f32,
                          const float *g, const float *cnt, float *gx, float *gy, float *gz, cudaStream_t st)
{
    if (!f32 || !A.id || !A.bc || !A.vox || !A.rowptr || !A.rowlen || (A.unit_weights ? !A.col : !A.cw))
        return cudaErrorInvalidValue;
    const int acc = method_accum(method);
    const long long V = geo.grid.V, n = A.n;
    ADJ_TRY(cudaMemsetAsync(gx, 0, sizeof(float) * (size_t)V, st));
    ADJ_TRY(cudaMemsetAsync(gy, 0, sizeof(float) * (size_t)V, st));
    ADJ_TRY(cudaMemsetAsync(gz, 0, sizeof(float) * (size_t)V, st));
    if (K <= 0 || geo.n_lines == 0) return cudaSuccess;
    if (!B->mu) ADJ_TRY(cudaMalloc(&B->mu, sizeof(float) * (size_t)V));
    if (!B->lam) {
        ADJ_TRY(cudaMalloc(&B->lam, sizeof(float) * (size_t)std::max(n, 1LL)));
        ADJ_TRY(cudaMalloc(&B->nxt, sizeof(float) * (size_t)std::max(n, 1LL)));
        ADJ_TRY(cudaMalloc(&B->acc, sizeof(float) * (size_t)std::max(n, 1LL)));
    }
    // transposed operator (once per operator)
    if (!B->tptr) {
        uint32_t *tcnt = nullptr;
        unsigned long long *t64 = nullptr, *tmp = nullptr;
        ADJ_TRY(cudaMalloc(&tcnt, sizeof(uint32_t) * (size_t)std::max(n, 1LL)));
        ADJ_TRY(cudaMalloc(&t64, sizeof(unsigned long long) * (size_t)std::max(n, 1LL)));
        ADJ_TRY(cudaMalloc(&tmp, sizeof(unsigned long long) * scan_tmp_elems(n)));
        ADJ_TRY(cudaMalloc(&B->tptr, sizeof(unsigned long long) * (size_t)(n + 1)));
        ADJ_TRY(cudaMemsetAsync(tcnt, 0, sizeof(uint32_t) * (size_t)std::max(n, 1LL), st));
        long long threads = n * 32;
        const uint32_t *col = A.unit_weights ? A.col : nullptr;
        const uint2 *cw = A.unit_weights ? nullptr : A.cw;
        k_adj_tcount<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, A.rowptr, A.rowlen, col, cw, tcnt);
        OM_COUNT_LAUNCH();
        k_u32_to_u64<<<grid_for(n), 256, 0, st>>>(n, tcnt, t64);
        OM_COUNT_LAUNCH();
        ADJ_TRY(exclusive_scan_u64(t64, B->tptr, n, tmp, st));
        unsigned long long tn = 0;
        ADJ_TRY(cudaMemcpyAsync(&tn, B->tptr + n, sizeof(tn), cudaMemcpyDeviceToHost, st));
        ADJ_TRY(cudaStreamSynchronize(st));
        ADJ_TRY(cudaMalloc(&B->trow, sizeof(uint32_t) * (size_t)std::max(tn, 1ULL)));
        if (!A.unit_weights) ADJ_TRY(cudaMalloc(&B->tw, sizeof(float) * (size_t)std::max(tn, 1ULL)));
        ADJ_TRY(cudaMemsetAsync(tcnt, 0, sizeof(uint32_t) * (size_t)std::max(n, 1LL), st));
        k_adj_tfill<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, A.rowptr, A.rowlen, col, cw, B->tptr, tcnt,
                                                                       B->trow, B->tw);
        OM_COUNT_LAUNCH();
        ADJ_TRY(cudaGetLastError());
        ADJ_TRY(cudaStreamSynchronize(st));
        cudaFree(tcnt);
        cudaFree(t64);
        cudaFree(tmp);
    }
    // mu = g / c; lambda_{K-1} = S^T mu
    k_adj_mu<<<grid_for(V), 256, 0, st>>>(V, g, cnt, B->mu);
    OM_COUNT_LAUNCH();
    ADJ_TRY(cudaMemsetAsync(B->lam, 0, sizeof(float) * (size_t)std::max(n, 1LL), st));
    ADJ_TRY(cudaMemsetAsync(B->acc, 0, sizeof(float) * (size_t)std::max(n, 1LL), st));
    adj_lines(acc, geo, true, f32, B->mu, A.id, B->lam, nullptr, nullptr, nullptr, st);
    // anchor iterations, backwards
    long long threads = n * 32;
    for (int k = K - 1; k >= 1; k--) {
        k_adj_accum<<<grid_for(n), 256, 0, st>>>(n, B->lam, A.bc, B->acc);
        OM_COUNT_LAUNCH();
        if (k > 1) {
            k_adj_spmvT<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, B->tptr, B->trow, B->tw, B->lam, A.bc,
                                                                           B->nxt);
            OM_COUNT_LAUNCH();
            std::swap(B->lam, B->nxt);
        }
    }
    // dL/dB = mu + acc on the anchors, then the line scatter
    k_adj_add_anchor<<<grid_for(n), 256, 0, st>>>(n, A.vox, B->acc, B->mu);
    OM_COUNT_LAUNCH();
    adj_lines(acc, geo, false, f32, B->mu, nullptr, nullptr, gx, gy, gz, st);
    return cudaGetLastError();
}

}  // namespace omni3d
