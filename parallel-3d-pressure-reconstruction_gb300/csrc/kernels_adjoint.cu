// Adjoint of the plain-method solve: the gradient of <g, p_K> with respect to the gradient
// field (ax, ay, az).  No stored iterates are needed: with the plain method the K-iteration
// map is affine in the field,
//     q_k = D^-1 (b + M q_{k-1} + seeding)        on the anchors, k = 1 .. K-1,
//     p(v) = (B(v) + S(v; q_{K-1}) + seeding) / c(v)  on every voxel with c(v) > 0,
// where B(v) = sum over lines through v of the prefix trapezoid integral I(v), b = B on
// the anchors, S(v; q) = sum over lines through v of q(entry).  Its transpose is
//     mu = g / c;  lambda_{K-1} = S^T mu  (each line's sum of mu, sent to its entry);
//     for k = K-1 .. 1:  acc += D^-1 lambda_k;  lambda_{k-1} = M^T D^-1 lambda_k (+ lambda_k
//                        where c = 0);
//     dL/dB = mu + acc on the anchors;
//     dL/da: along every line, the suffix sum R_t of dL/dB over the steps t..n multiplies
//     the trapezoid coefficient h_t, and is scattered to the two voxels of step t
//     (I(v_s) = sum_{t <= s} h_t (a(v_t) + a(v_{t-1})) along the step's axis).
// Lines are walked forwards twice (total, then suffix sums), from the same step descriptors
// as the sweep.
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

// mu = g / c where c > 0, else 0
__global__ void k_adj_mu(long long V, const float *g, const float *cnt, float *mu)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        mu[v] = cnt[v] > 0.0f ? __fdiv_rn(g[v], cnt[v]) : 0.0f;
}

// lambda[id(entry)] += sum of mu over the line (entry included)
__global__ void __launch_bounds__(256) k_adj_gather(Grid g, const LineRec *__restrict__ lines,
                                                    const uint32_t *__restrict__ gbase,
                                                    const uint32_t *__restrict__ desc, long long n_lines,
                                                    const float *__restrict__ mu, const int32_t *__restrict__ id,
                                                    float *lam)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    AdjWalk L;
    L.init(g, r, gbase, desc, li);
    float t = __ldg(mu + L.v);
    for (int s0 = 0; s0 < L.m; s0 += 16) {
        uint32_t w = __ldg(L.dp + 32 * (s0 >> 4));
        int n = min(16, L.m - s0);
        for (int k = 0; k < n; k++, w >>= 2) {
            int a = (int)(w & 3u);
            L.v += a == 0 ? L.d0 : (a == 1 ? L.d1 : L.d2);
            t += __ldg(mu + L.v);
        }
    }
    atomicAdd(lam + __ldg(id + r.e), t);
}

// dL/da along every line: suffix sums of dL/dB times the trapezoid coefficients
__global__ void __launch_bounds__(256) k_adj_grad(Grid g, const LineRec *__restrict__ lines,
                                                  const uint32_t *__restrict__ gbase,
                                                  const uint32_t *__restrict__ desc, long long n_lines,
                                                  const float *__restrict__ dB, float *gx, float *gy, float *gz)
{
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n_lines) return;
    LineRec r = lines[li];
    AdjWalk L;
    L.init(g, r, gbase, desc, li);
    // total over the steps 1..m
    float R = 0.0f;
    long long v = L.v;
    for (int s0 = 0; s0 < L.m; s0 += 16) {
        uint32_t w = __ldg(L.dp + 32 * (s0 >> 4));
        int n = min(16, L.m - s0);
        for (int k = 0; k < n; k++, w >>= 2) {
            int a = (int)(w & 3u);
            v += a == 0 ? L.d0 : (a == 1 ? L.d1 : L.d2);
            R += __ldg(dB + v);
        }
    }
    // scatter
    v = L.v;
    for (int s0 = 0; s0 < L.m; s0 += 16) {
        uint32_t w = __ldg(L.dp + 32 * (s0 >> 4));
        int n = min(16, L.m - s0);
        for (int k = 0; k < n; k++, w >>= 2) {
            int a = (int)(w & 3u);
            long long prev = v;
            v += a == 0 ? L.d0 : (a == 1 ? L.d1 : L.d2);
            float val = (a == 0 ? L.h0 : (a == 1 ? L.h1 : L.h2)) * R;
            float *ga = a == 0 ? gx : (a == 1 ? gy : gz);
            atomicAdd(ga + v, val);
            atomicAdd(ga + prev, val);
            R -= __ldg(dB + v);
        }
    }
}

// transposed operator: count entries per column
__global__ void k_adj_tcount(long long n, const unsigned long long *rowptr, const uint32_t *rowlen,
                             const uint32_t *col, uint32_t *tcnt)
{
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    unsigned long long j0 = rowptr[row], j1 = j0 + rowlen[row];
    for (unsigned long long j = j0 + lane; j < j1; j += 32) atomicAdd(tcnt + col[j], 1u);
}

__global__ void k_adj_tfill(long long n, const unsigned long long *rowptr, const uint32_t *rowlen, const uint32_t *col,
                            const unsigned long long *tptr, uint32_t *tcur, uint32_t *trow)
{
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    unsigned long long j0 = rowptr[row], j1 = j0 + rowlen[row];
    for (unsigned long long j = j0 + lane; j < j1; j += 32) {
        uint32_t c = col[j];
        trow[tptr[c] + atomicAdd(tcur + c, 1u)] = (uint32_t)row;
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

// next = M^T D^-1 lambda (+ lambda where c = 0), a warp per column of M
__global__ void __launch_bounds__(256) k_adj_spmvT(long long n, const unsigned long long *__restrict__ tptr,
                                                   const uint32_t *__restrict__ trow, const float *__restrict__ lam,
                                                   const float2 *__restrict__ bc, float *__restrict__ next)
{
    long long a = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (a >= n) return;
    unsigned long long j0 = tptr[a], j1 = tptr[a + 1];
    float s = 0.0f;
    for (unsigned long long j = j0 + lane; j < j1; j += 32) {
        uint32_t r = __ldg(trow + j);
        float cr = __ldg(&bc[r].y);
        if (cr > 0.0f) s += __fdiv_rn(__ldg(lam + r), cr);
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

cudaError_t adjoint_plain(const Geometry &geo, const Anchor &A, AdjointBuffers *B, int K, const float *g,
                          const float *cnt, float *gx, float *gy, float *gz, cudaStream_t st)
{
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
        k_adj_tcount<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, A.rowptr, A.rowlen, A.col, tcnt);
        OM_COUNT_LAUNCH();
        k_u32_to_u64<<<grid_for(n), 256, 0, st>>>(n, tcnt, t64);
        OM_COUNT_LAUNCH();
        ADJ_TRY(exclusive_scan_u64(t64, B->tptr, n, tmp, st));
        unsigned long long tn = 0;
        ADJ_TRY(cudaMemcpyAsync(&tn, B->tptr + n, sizeof(tn), cudaMemcpyDeviceToHost, st));
        ADJ_TRY(cudaStreamSynchronize(st));
        ADJ_TRY(cudaMalloc(&B->trow, sizeof(uint32_t) * (size_t)std::max(tn, 1ULL)));
        ADJ_TRY(cudaMemsetAsync(tcnt, 0, sizeof(uint32_t) * (size_t)std::max(n, 1LL), st));
        k_adj_tfill<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, A.rowptr, A.rowlen, A.col, B->tptr, tcnt,
                                                                       B->trow);
        OM_COUNT_LAUNCH();
        ADJ_TRY(cudaGetLastError());
        ADJ_TRY(cudaStreamSynchronize(st));
        cudaFree(tcnt);
        cudaFree(t64);
        cudaFree(tmp);
    }
    const Grid &gr = geo.grid;
    unsigned lblocks = (unsigned)((geo.n_lines + 255) / 256);
    // mu = g / c; lambda_{K-1} = S^T mu
    k_adj_mu<<<grid_for(V), 256, 0, st>>>(V, g, cnt, B->mu);
    OM_COUNT_LAUNCH();
    ADJ_TRY(cudaMemsetAsync(B->lam, 0, sizeof(float) * (size_t)std::max(n, 1LL), st));
    ADJ_TRY(cudaMemsetAsync(B->acc, 0, sizeof(float) * (size_t)std::max(n, 1LL), st));
    k_adj_gather<<<lblocks, 256, 0, st>>>(gr, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines, B->mu, A.id, B->lam);
    OM_COUNT_LAUNCH();
    // anchor iterations, backwards
    long long threads = n * 32;
    for (int k = K - 1; k >= 1; k--) {
        k_adj_accum<<<grid_for(n), 256, 0, st>>>(n, B->lam, A.bc, B->acc);
        OM_COUNT_LAUNCH();
        if (k > 1) {
            k_adj_spmvT<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, B->tptr, B->trow, B->lam, A.bc, B->nxt);
            OM_COUNT_LAUNCH();
            std::swap(B->lam, B->nxt);
        }
    }
    // dL/dB = mu + acc on the anchors, then the line scatter
    k_adj_add_anchor<<<grid_for(n), 256, 0, st>>>(n, A.vox, B->acc, B->mu);
    OM_COUNT_LAUNCH();
    k_adj_grad<<<lblocks, 256, 0, st>>>(gr, geo.d_lines, geo.d_gbase, geo.d_desc, geo.n_lines, B->mu, gx, gy, gz);
    OM_COUNT_LAUNCH();
    return cudaGetLastError();
}

}  // namespace omni3d
