// C ABI of libomni3d_gb300: solver contexts, the per-snapshot solve and the diagnostics.
// The per-file block of the reference main() (K:8794-8863) becomes omni3d_solve(); the
// per-direction setup of its kernels (K:6175-6191) is evaluated once per direction here on
// the host and uploaded as a table.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <utility>
#include <vector>

#include "fixed.cuh"
#include "omni3d_internal.h"

using namespace omni3d;

namespace {

thread_local std::string g_error;

struct DeviceBuf {
    void *p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= n) return cudaSuccess;
        cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) n = bytes;
        return e;
    }
    void release()
    {
        cudaFree(p);
        p = nullptr;
        n = 0;
    }
    template <typename T>
    T *as() const { return reinterpret_cast<T *>(p); }
};

}  // namespace

namespace omni3d {
unsigned long long g_kernel_launches = 0;
void set_global_error(const std::string &msg) { g_error = msg; }
}  // namespace omni3d

struct omni3d_ctx {
    omni3d_params prm{};
    std::vector<float> dirs;
    std::vector<DirEntry> table;
    Geometry geo;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::string err;
    double ms_geometry = 0.0;
    // per-solve buffers
    DeviceBuf in_ax, in_ay, in_az, in_aux, in_pinit;  // staging of host inputs
    DeviceBuf f32, b16, curl;
    DeviceBuf pvol_a, pvol_b, pout, cnt, pncnt, scratch, flags;
    Anchor anc;
    bool anc_cached = false;  // plain method: operator structure built for this geometry
    bool anc_last = false;    // the operator in anc is that of the last solve's field and method
    DeviceBuf centre;         // FP64 scratch of the centre integration
    DeviceBuf pncnt64;        // FP64 accumulators of the sweep_fp64 sweeps (or the fixed-point ones)
    Fixed fix;                // bit-reproducible mode: scales and bounds (params.deterministic)
    DeviceBuf fix_mem;        // its kFixSlots scales and kBitsSlots bits
    Bricks bricks;            // brick segments of the geometry (built on first use)
    bool bricks_failed = false;
    std::string bricks_why;
    AdjointBuffers adj;
    DeviceBuf adj_g, adj_out;  // staging of the adjoint's host arguments
    int last_iterations = -1;  // iterations of the last solve (-1: no solve yet)
    int last_method = -1;
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // tolerance-driven anchor iterations run as graph-captured chunks (see iterate_chunk)
    cudaGraphExec_t iter_exec = nullptr;
    std::vector<const void *> iter_key;  // what the captured chunk baked in
    unsigned long long iter_launches = 0; // kernels per chunk
    DeviceBuf iter_buf;                   // the chunk's stop word and per-step relative changes
};

namespace {

int fail(omni3d_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    g_error = msg;
    return code;
}

int cuda_fail(omni3d_ctx *ctx, cudaError_t e, const char *what)
{
    return fail(ctx, e == cudaErrorMemoryAllocation ? OMNI3D_ERR_NOMEM : OMNI3D_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(ctx, x)                                          \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #x); \
    } while (0)

// Rotation coefficients of one direction (K:6175-6191; libm in place of the intrinsics)
// and the cross2point branches its components select (K:672, 759, 847, 936, 955, 974,
// 992; "zero" is the double 1e-7, K:23).
DirEntry make_dir(float k1, float k2, float k3)
{
    DirEntry D{};
    float theta = acosf(k3);
    float st = sinf(theta);
    float phi = 0.0f;
    if (st != 0.0f) {
        phi = asinf(k2 / st);
        if (k1 / st < 0) phi = (float)(-phi + 3.1415926535897932384626433832795);
    }
    D.ct = cosf(theta);
    D.st = st;
    D.cp = cosf(phi);
    D.sp = sinf(phi);
    D.k1 = k1;
    D.k2 = k2;
    D.k3 = k3;
    const double z = 1e-7;
    double a1 = std::fabs((double)k1), a2 = std::fabs((double)k2), a3 = std::fabs((double)k3);
    int c = 0;
    if (k1 == 0 && k2 != 0 && k3 != 0) c |= 1;
    if (k1 != 0 && k2 == 0 && k3 != 0) c |= 2;
    if (k1 != 0 && k2 != 0 && k3 == 0) c |= 4;
    if (a1 < z && a2 < z && a3 >= z) c |= 8;
    if (a1 < z && a2 >= z && a3 < z) c |= 16;
    if (a1 >= z && a2 < z && a3 < z) c |= 32;
    if (a1 >= z && a2 >= z && a3 >= z) c |= 64;
    D.cas = c;
    return D;
}

// Processing order of the directions: serpentine bands of polar angle, each band ordered
// by azimuth, so that consecutive directions are neighbours on the sphere.  Lines are
// traced and swept in this order; the few directions in flight at a time then sweep nearly
// coincident sheets of the volume and share the gradient and accumulator lines in L2.
std::vector<int> sphere_order(const std::vector<float> &dirs)
{
    const int n = (int)(dirs.size() / 3);
    const double PI = 3.14159265358979323846;
    int nb = std::max(1, (int)std::lround(std::sqrt(n / 2.0)));
    std::vector<std::pair<std::pair<int, double>, int>> key;
    key.reserve(n);
    for (int d = 0; d < n; d++) {
        double k1 = dirs[3 * d], k2 = dirs[3 * d + 1], k3 = dirs[3 * d + 2];
        double r = std::sqrt(k1 * k1 + k2 * k2 + k3 * k3);
        double th = std::acos(std::max(-1.0, std::min(1.0, r > 0 ? k3 / r : 1.0)));
        double ph = std::atan2(k2, k1);
        int b = std::min(nb - 1, (int)(th / PI * nb));
        key.push_back({{b, (b & 1) ? -ph : ph}, d});
    }
    std::sort(key.begin(), key.end());
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = key[i].second;
    return order;
}

int check_params(const omni3d_params *p, std::string *why)
{
    if (!p) { *why = "params is NULL"; return OMNI3D_ERR_ARG; }
    if (p->nx < 2 || p->ny < 2 || p->nz < 2) { *why = "grid dimensions must be >= 2"; return OMNI3D_ERR_ARG; }
    long long V = (long long)p->nx * p->ny * p->nz;
    if (V >= (1LL << 32) || (long long)p->nx * p->ny >= (1LL << 31)) {
        *why = "grid too large: voxel indices are 32-bit";
        return OMNI3D_ERR_RANGE;
    }
    if (!(p->line_spacing > 0.0f) || !std::isfinite(p->line_spacing)) { *why = "line_spacing must be > 0"; return OMNI3D_ERR_ARG; }
    if (p->n_dirs <= 0 || !p->dirs) { *why = "no directions"; return OMNI3D_ERR_ARG; }
    if (p->max_iter < 0) { *why = "max_iter must be >= 0"; return OMNI3D_ERR_ARG; }
    if (p->method < OMNI3D_METHOD_PLAIN || p->method > OMNI3D_METHOD_WEIGHTED_MINI_CURL) {
        *why = "unknown method";
        return OMNI3D_ERR_ARG;
    }
    if (p->solver != OMNI3D_SOLVER_ANCHOR && p->solver != OMNI3D_SOLVER_SWEEP) { *why = "unknown solver"; return OMNI3D_ERR_ARG; }
    if (p->grad_storage != OMNI3D_GRAD_F32 && p->grad_storage != OMNI3D_GRAD_BF16) { *why = "unknown grad_storage"; return OMNI3D_ERR_ARG; }
    if (p->gauge < OMNI3D_GAUGE_NONE || p->gauge > OMNI3D_GAUGE_MEAN) { *why = "unknown gauge"; return OMNI3D_ERR_ARG; }
    if (p->gauge == OMNI3D_GAUGE_POINT &&
        (p->ref_i < 0 || p->ref_i >= p->nx || p->ref_j < 0 || p->ref_j >= p->ny || p->ref_k < 0 || p->ref_k >= p->nz)) {
        *why = "reference voxel outside the grid";
        return OMNI3D_ERR_ARG;
    }
    if (!(p->tol >= 0.0)) { *why = "tol must be >= 0"; return OMNI3D_ERR_ARG; }
    if (p->grad_storage == OMNI3D_GRAD_BF16 && method_accum(p->method) == kAccSelect && p->threshold > 0.0f &&
        p->threshold < 1.17549435e-38f) {
        *why = "BF16 storage needs a threshold of 0 or at least 1.2e-38 (FP32's normal range)";
        return OMNI3D_ERR_ARG;
    }
    if (p->anchor_max_links < 0) { *why = "anchor_max_links must be >= 0"; return OMNI3D_ERR_ARG; }
    if (p->engine < OMNI3D_ENGINE_AUTO || p->engine > OMNI3D_ENGINE_BRICKS) { *why = "unknown engine"; return OMNI3D_ERR_ARG; }
    if (p->sweep_fp64 != 0 && p->sweep_fp64 != 1) { *why = "sweep_fp64 must be 0 or 1"; return OMNI3D_ERR_ARG; }
    if (p->initial_guess != OMNI3D_INIT_ZERO && p->initial_guess != OMNI3D_INIT_CENTRE) {
        *why = "unknown initial_guess";
        return OMNI3D_ERR_ARG;
    }
    if (p->tile_width != 0 && p->tile_width != 4 && p->tile_width != 8 && p->tile_width != 16) {
        *why = "tile_width must be 0, 4, 8 or 16";
        return OMNI3D_ERR_ARG;
    }
    if (p->dir_group < 0 || p->dir_group > 32) { *why = "dir_group must be 0..32"; return OMNI3D_ERR_ARG; }
    if (p->autotune != 0 && p->autotune != 1) { *why = "autotune must be 0 or 1"; return OMNI3D_ERR_ARG; }
    if (p->deterministic != 0 && p->deterministic != 1) { *why = "deterministic must be 0 or 1"; return OMNI3D_ERR_ARG; }
    if (p->deterministic && p->engine == OMNI3D_ENGINE_BRICKS) {
        *why = "the brick engine's shared-memory sums are not bit-reproducible (deterministic needs the line engine)";
        return OMNI3D_ERR_ARG;
    }
    double ng = std::max(std::max(p->nx, p->ny), p->nz) * 1.732 / (double)p->line_spacing;
    if (ng * ng * (double)p->n_dirs / 256.0 > 2.0e9) { *why = "too many lines (lattice x directions)"; return OMNI3D_ERR_RANGE; }
    return OMNI3D_OK;
}

float ms_between(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// Upload (host) or adopt (device) one input volume.
int stage(omni3d_ctx *ctx, const float *src, bool dev, DeviceBuf &buf, long long V, const float **out)
{
    if (!src) { *out = nullptr; return OMNI3D_OK; }
    if (dev) { *out = src; return OMNI3D_OK; }
    CK(ctx, buf.ensure(sizeof(float) * (size_t)V));
    CK(ctx, cudaMemcpyAsync(buf.p, src, sizeof(float) * (size_t)V, cudaMemcpyHostToDevice, ctx->st));
    *out = buf.as<float>();
    return OMNI3D_OK;
}

// Build the device field (float4 ax, ay, az, curl; optional bf16 copy; curl array).
int prepare_field(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az, const float *curl,
                  const float *mask, bool dev, Field *F)
{
    const Grid &g = ctx->geo.grid;
    const long long V = g.V;
    const float *dax, *day, *daz, *daux;
    int rc;
    if ((rc = stage(ctx, ax, dev, ctx->in_ax, V, &dax))) return rc;
    if ((rc = stage(ctx, ay, dev, ctx->in_ay, V, &day))) return rc;
    if ((rc = stage(ctx, az, dev, ctx->in_az, V, &daz))) return rc;
    const float *dcurl = nullptr;
    if (method_uses_curl(ctx->prm.method)) {
        if (curl) {
            if ((rc = stage(ctx, curl, dev, ctx->in_aux, V, &daux))) return rc;
            dcurl = daux;
        } else {
            if ((rc = stage(ctx, mask, dev, ctx->in_aux, V, &daux))) return rc;
            CK(ctx, ctx->curl.ensure(sizeof(float) * (size_t)V));
            CK(ctx, curl_field(g, dax, day, daz, daux, ctx->curl.as<float>(), ctx->st));
            dcurl = ctx->curl.as<float>();
        }
    }
    const bool bf16 = ctx->prm.grad_storage == OMNI3D_GRAD_BF16;
    CK(ctx, ctx->f32.ensure(sizeof(float4) * (size_t)V));
    F->f32 = ctx->f32.as<float4>();
    float *rounded = nullptr;  // BF16 storage: every curl decision sees the rounded curl
    if (bf16) {
        CK(ctx, ctx->b16.ensure(sizeof(uint2) * (size_t)V));
        F->bf16 = ctx->b16.as<uint2>();
        if (dcurl) {
            CK(ctx, ctx->curl.ensure(sizeof(float) * (size_t)V));
            rounded = ctx->curl.as<float>();
        }
    }
    F->curl = rounded ? rounded : const_cast<float *>(dcurl);
    CK(ctx, pack_field(g, dax, day, daz, dcurl, F, bf16, ctx->st, rounded));
    return OMNI3D_OK;
}

// The sweep engine of a solve on ctx: bricks when asked for (FP32 storage, the segments
// built), else lines; automatic selection takes lines, the faster engine as measured.
// *rc is set when bricks were required but are unavailable.
int choose_engine(omni3d_ctx *ctx, bool bf16, int *rc)
{
    const int want = ctx->prm.engine;
    *rc = OMNI3D_OK;
    if (want == OMNI3D_ENGINE_LINES || want == OMNI3D_ENGINE_AUTO) return OMNI3D_ENGINE_LINES;
    if (bf16) {
        if (want == OMNI3D_ENGINE_BRICKS)
            *rc = fail(ctx, OMNI3D_ERR_STATE, "the brick engine needs FP32 gradient storage");
        return OMNI3D_ENGINE_LINES;
    }
    if (ctx->geo.walk_rule == 3) {
        *rc = fail(ctx, OMNI3D_ERR_STATE, "the brick engine does not take minimum-curl walks (they change per field)");
        return OMNI3D_ENGINE_LINES;
    }
    if (!ctx->bricks.built && !ctx->bricks_failed) {
        std::string why;
        cudaError_t e = build_bricks(ctx->geo, &ctx->bricks, ctx->st, &why);
        if (e != cudaSuccess) {
            cudaGetLastError();
            free_bricks(&ctx->bricks);
            ctx->bricks_failed = true;
            ctx->bricks_why = why;
        }
    }
    if (ctx->bricks.built) return OMNI3D_ENGINE_BRICKS;
    if (want == OMNI3D_ENGINE_BRICKS) *rc = fail(ctx, OMNI3D_ERR_STATE, "brick engine unavailable: " + ctx->bricks_why);
    return OMNI3D_ENGINE_LINES;
}

// Per-field brick passes (B1 + L) when the engine is bricks.  Automatic selection falls back
// to lines when the per-segment buffers do not fit in device memory.
int engine_prepare(omni3d_ctx *ctx, int *engine, const Field &F, int method)
{
    if (*engine != OMNI3D_ENGINE_BRICKS) return OMNI3D_OK;
    std::string why;
    cudaError_t e = brick_prepare(ctx->geo, &ctx->bricks, F, method, ctx->st, &why);
    if (e == cudaSuccess) return OMNI3D_OK;
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation && ctx->prm.engine == OMNI3D_ENGINE_AUTO) {
        *engine = OMNI3D_ENGINE_LINES;
        return OMNI3D_OK;
    }
    return fail(ctx, e == cudaErrorMemoryAllocation ? OMNI3D_ERR_NOMEM : OMNI3D_ERR_CUDA, "brick passes: " + why);
}

// One full sweep with the chosen engine.
cudaError_t engine_sweep(omni3d_ctx *ctx, int engine, const Field &F, int method, bool bf16, const float *p,
                         float2 *acc, cudaStream_t st)
{
    if (engine == OMNI3D_ENGINE_BRICKS) return brick_sweep(ctx->geo, &ctx->bricks, method, p, acc, st);
    return sweep_full(ctx->geo, F, method, bf16, p, acc, st);
}

// The brick passes' error flag (a TMA wait that gave up) as a status.
int engine_check(omni3d_ctx *ctx, int engine)
{
    if (engine != OMNI3D_ENGINE_BRICKS) return OMNI3D_OK;
    int flag = 0;
    CK(ctx, brick_error(ctx->bricks, &flag, ctx->st));
    if (flag) return fail(ctx, OMNI3D_ERR_CUDA, "brick pass: a shared-memory staging copy did not complete");
    return OMNI3D_OK;
}

// True when ctx can run the fully asynchronous solve: plain method, anchor solver with its
// operator already built for this geometry, a fixed iteration count, buffers allocated.
bool prepared_for_graph(const omni3d_ctx *ctx)
{
    const omni3d_params &P = ctx->prm;
    return P.method == OMNI3D_METHOD_PLAIN && P.solver == OMNI3D_SOLVER_ANCHOR && P.tol == 0.0 && ctx->anc_cached &&
           ctx->f32.p && ctx->in_pinit.p && ctx->pncnt.p && ctx->pout.p && ctx->cnt.p && ctx->pvol_a.p &&
           ctx->scratch.p && (P.grad_storage != OMNI3D_GRAD_BF16 || ctx->b16.p);
}

// The solve of omni3d_solve for a prepared context, issued on `st` with no host
// synchronisation and no allocation, so that it can be captured into a CUDA graph.
// Inputs are device pointers; p_init may be null (zero).
cudaError_t enqueue_prepared(omni3d_ctx *ctx, const float *dax, const float *day, const float *daz,
                             const float *dpinit, float *p_out, float *count_out, cudaStream_t st)
{
    const omni3d_params &P = ctx->prm;
    const Grid &g = ctx->geo.grid;
    const long long V = g.V;
    const bool bf16 = P.grad_storage == OMNI3D_GRAD_BF16;
    const long long ref = (long long)P.ref_i + (long long)P.ref_j * g.X + (long long)P.ref_k * g.XY;
    Field F;
    F.f32 = ctx->f32.as<float4>();
    F.bf16 = bf16 ? ctx->b16.as<uint2>() : nullptr;
    cudaError_t e = pack_field(g, dax, day, daz, nullptr, &F, bf16, st);
    if (e != cudaSuccess) return e;
    if (!dpinit) {
        if ((e = cudaMemsetAsync(ctx->in_pinit.p, 0, sizeof(float) * (size_t)V, st)) != cudaSuccess) return e;
        dpinit = ctx->in_pinit.as<float>();
    }
    Anchor &A = ctx->anc;
    if ((e = anchor_refresh_rhs(ctx->geo, F, &A, st)) != cudaSuccess) return e;
    if ((e = anchor_gather(A, dpinit, A.pa, st)) != cudaSuccess) return e;
    const int K = P.max_iter;
    const bool seed = P.seed_first_iteration != 0;
    float *pc = A.pa, *pn = A.pb;
    for (int it = 1; it <= K - 1; it++) {
        if ((e = anchor_step(A, dpinit, seed && it == 1, P.gauge, -1, pc, pn, nullptr, st)) != cudaSuccess) return e;
        std::swap(pc, pn);
    }
    float2 *acc = ctx->pncnt.as<float2>();
    float *vol = ctx->pvol_a.as<float>(), *dout = ctx->pout.as<float>(), *dcnt = ctx->cnt.as<float>();
    if (K == 0) {
        if ((e = cudaMemcpyAsync(dout, dpinit, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st))) return e;
        if ((e = cudaMemsetAsync(dcnt, 0, sizeof(float) * (size_t)V, st))) return e;
    } else {
        if ((e = cudaMemcpyAsync(vol, dpinit, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st))) return e;
        if ((e = anchor_scatter(A, pc, vol, st))) return e;
        if ((e = init_accum(V, dpinit, seed && K == 1, acc, st))) return e;
        if ((e = sweep_full(ctx->geo, F, P.method, bf16, vol, acc, st))) return e;
        if ((e = normalize(V, acc, dpinit, dout, dcnt, st))) return e;
    }
    if ((e = apply_gauge(V, P.gauge, ref, dcnt, dout, ctx->scratch.as<double>() + 4, st))) return e;
    if (p_out && (e = cudaMemcpyAsync(p_out, dout, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st))) return e;
    if (count_out && (e = cudaMemcpyAsync(count_out, dcnt, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st)))
        return e;
    return cudaSuccess;
}

}  // namespace

struct omni3d_batch {
    std::vector<omni3d_ctx *> ctx;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<const void *> key;  // pointers the captured graph reads and writes
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<cudaEvent_t> join;
    long long launches_per_graph = 0;
    std::string err;
};

extern "C" {

void omni3d_default_params(omni3d_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->nx = p->ny = p->nz = 64;             // K:8532-8534
    p->dx = p->dy = p->dz = 0.006135923151543f;  // K:8533-8535
    p->density = 1.0f;                      // K:8511
    p->line_spacing = 1.0f;
    p->max_iter = 100;                      // K:8526
    p->threshold = 0.0f;
    p->method = OMNI3D_METHOD_PLAIN;
    p->solver = OMNI3D_SOLVER_ANCHOR;
    p->grad_storage = OMNI3D_GRAD_F32;
    p->tol = 0.0;
    p->gauge = OMNI3D_GAUGE_NONE;
    p->seed_first_iteration = 1;
    p->device = 0;
}

const char *omni3d_last_error(const omni3d_ctx *ctx) { return ctx ? ctx->err.c_str() : g_error.c_str(); }
const char *omni3d_global_error(void) { return g_error.c_str(); }

namespace {

// Line-order tuning (params.autotune).  The line order decides which voxels the lanes of a
// warp, and the warps of a block, touch at the same time, so the best tile width and
// direction group depend on the grid and the direction set.  Each candidate pair is built
// and timed with one plain sweep of a zero field (the sweep's cost depends on where its
// gathers and reductions land, not on the values); the fastest pair is kept for the process,
// per device and size class.
struct TuneKey {
    int device, size_class, nv, rule;
    uint32_t ls_bits;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(device, size_class, nv, rule, ls_bits) <
               std::tie(o.device, o.size_class, o.nv, o.rule, o.ls_bits);
    }
};
std::mutex g_tune_mutex;
std::map<TuneKey, std::pair<int, int>> g_tune_cache;

cudaError_t tune_line_order(omni3d_ctx *ctx, std::string *err)
{
    Geometry &geo = ctx->geo;
    const Grid &g = geo.grid;
    uint32_t ls_bits;
    std::memcpy(&ls_bits, &g.ls, sizeof(ls_bits));
    const int mx = std::max(std::max(g.X, g.Y), g.Z);
    const TuneKey key{ctx->prm.device, (mx + 31) / 32, geo.nv, geo.walk_rule, ls_bits};
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
        geo.tile_width = it->second.first;
        geo.dir_group = it->second.second;
        return cudaSuccess;
    }
    static const int kCand[][2] = {{8, 4}, {4, 4}, {16, 4}, {8, 2}, {8, 8}};
    float4 *field = nullptr;
    float *p = nullptr;
    float2 *acc = nullptr;
    const size_t V = (size_t)g.V;
    cudaError_t e = cudaMalloc(&field, sizeof(float4) * V);
    if (e == cudaSuccess) e = cudaMalloc(&p, sizeof(float) * V);
    if (e == cudaSuccess) e = cudaMalloc(&acc, sizeof(float2) * V);
    if (e == cudaSuccess) e = cudaMemsetAsync(field, 0, sizeof(float4) * V, ctx->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, sizeof(float) * V, ctx->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, sizeof(float2) * V, ctx->st);
    float best = 0.0f;
    int bt = 8, bg = 4;
    for (const auto &c : kCand) {
        if (e != cudaSuccess) break;
        geo.tile_width = c[0];
        geo.dir_group = c[1];
        if ((e = build_geometry(&geo, ctx->st, err)) != cudaSuccess) break;
        Field F;
        F.f32 = field;
        e = sweep_full(geo, F, OMNI3D_METHOD_PLAIN, false, p, acc, ctx->st);  // warm-up
        cudaEventRecord(ctx->ev[2], ctx->st);
        if (e == cudaSuccess) e = sweep_full(geo, F, OMNI3D_METHOD_PLAIN, false, p, acc, ctx->st);
        cudaEventRecord(ctx->ev[3], ctx->st);
        if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev[3]);
        const float ms = ms_between(ctx->ev[2], ctx->ev[3]);
        free_geometry(&geo);
        if (e == cudaSuccess && (best == 0.0f || ms < best)) {
            best = ms;
            bt = c[0];
            bg = c[1];
        }
    }
    cudaFree(field);
    cudaFree(p);
    cudaFree(acc);
    if (e != cudaSuccess) return e;
    geo.tile_width = bt;
    geo.dir_group = bg;
    g_tune_cache[key] = {bt, bg};
    return cudaSuccess;
}

}  // namespace

int omni3d_create(const omni3d_params *params, omni3d_ctx **out)
{
    if (!out) return fail(nullptr, OMNI3D_ERR_ARG, "out is NULL");
    *out = nullptr;
    std::string why;
    int rc = check_params(params, &why);
    if (rc) return fail(nullptr, rc, why);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, OMNI3D_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (params->device < 0 || params->device >= ndev) return fail(nullptr, OMNI3D_ERR_ARG, "device ordinal out of range");
    e = cudaSetDevice(params->device);
    if (e != cudaSuccess) return fail(nullptr, OMNI3D_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));

    omni3d_ctx *ctx = new omni3d_ctx();
    ctx->prm = *params;
    ctx->dirs.assign(params->dirs, params->dirs + 3 * (size_t)params->n_dirs);
    ctx->prm.dirs = ctx->dirs.data();
    for (int d : sphere_order(ctx->dirs)) {
        ctx->table.push_back(make_dir(ctx->dirs[3 * d], ctx->dirs[3 * d + 1], ctx->dirs[3 * d + 2]));
        ctx->table.back().orig = d;
    }

    Grid &g = ctx->geo.grid;
    g.X = params->nx;
    g.Y = params->ny;
    g.Z = params->nz;
    g.XY = (long long)g.X * g.Y;
    g.V = g.XY * g.Z;
    g.cx = (float)((g.X - 1) / 2.0);
    g.cy = (float)((g.Y - 1) / 2.0);
    g.cz = (float)((g.Z - 1) / 2.0);
    g.dx = params->dx;
    g.dy = params->dy;
    g.dz = params->dz;
    g.rho = params->density;
    g.ls = params->line_spacing;
    g.thr_src = params->threshold;
    g.thr = params->threshold;
    if (params->grad_storage == OMNI3D_GRAD_BF16 && method_accum(params->method) == kAccSelect) {
        // BF16 storage: the kernels compare the stored curl against the threshold's BF16
        // truncation, and k_pack maps every curl to the same side of it (curl_bf16)
        uint32_t b;
        std::memcpy(&b, &params->threshold, sizeof(b));
        b &= 0xffff0000u;
        std::memcpy(&g.thr, &b, sizeof(b));
        g.curl_map = 1;
    }
    int mx = std::max(std::max(g.X, g.Y), g.Z);
    g.ng = (int)(mx * 1.732 / (double)params->line_spacing);  // K:6167
    ctx->geo.nv = params->n_dirs;
    ctx->geo.walk_rule = method_walk_rule(params->method);

    auto bail = [&](cudaError_t ce, const char *what) {
        int r = cuda_fail(ctx, ce, what);
        g_error = ctx->err;
        omni3d_destroy(ctx);
        return r;
    };
    if ((e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
    ctx->own_stream = true;
    for (auto &ev : ctx->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaMalloc(&ctx->geo.d_dirs, sizeof(DirEntry) * ctx->table.size())) != cudaSuccess) return bail(e, "cudaMalloc dirs");
    if ((e = cudaMemcpyAsync(ctx->geo.d_dirs, ctx->table.data(), sizeof(DirEntry) * ctx->table.size(),
                             cudaMemcpyHostToDevice, ctx->st)) != cudaSuccess)
        return bail(e, "upload dirs");
    ctx->geo.tile_width = params->tile_width ? params->tile_width : 8;
    // Direction groups: up to 2^24 voxels, 32 directions walked through each lattice patch
    // together share the filling pass's gathers in L1 and L2 (256^3 / 642 directions: 124.8
    // against 127.2 ms per solve with groups of 4; 192^3: 53.5 against 55.1 ms); on larger
    // grids the final sweep's footprint outgrows the L2 and groups of 4 win (320^3: 256.7
    // against 260.9 ms with 16; 512^3: 1385 against 1551 ms with 32).
    ctx->geo.dir_group = params->dir_group ? params->dir_group : (ctx->geo.grid.V <= (1LL << 24) ? 32 : 4);
    std::string gerr;
    if (params->autotune && (e = tune_line_order(ctx, &gerr)) != cudaSuccess) {
        ctx->err = "line-order tuning: " + (gerr.empty() ? std::string(cudaGetErrorString(e)) : gerr);
        g_error = ctx->err;
        int r = e == cudaErrorMemoryAllocation ? OMNI3D_ERR_NOMEM : OMNI3D_ERR_CUDA;
        omni3d_destroy(ctx);
        return r;
    }
    cudaEventRecord(ctx->ev[0], ctx->st);
    e = build_geometry(&ctx->geo, ctx->st, &gerr);
    if (e != cudaSuccess) {
        ctx->err = "line tracing: " + gerr;
        g_error = ctx->err;
        int r = e == cudaErrorMemoryAllocation ? OMNI3D_ERR_NOMEM : OMNI3D_ERR_CUDA;
        omni3d_destroy(ctx);
        return r;
    }
    cudaEventRecord(ctx->ev[1], ctx->st);
    cudaEventSynchronize(ctx->ev[1]);
    ctx->ms_geometry = ms_between(ctx->ev[0], ctx->ev[1]);
    *out = ctx;
    return OMNI3D_OK;
}

int omni3d_destroy(omni3d_ctx *ctx)
{
    if (!ctx) return OMNI3D_OK;
    cudaSetDevice(ctx->prm.device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    free_geometry(&ctx->geo);
    cudaFree(ctx->geo.d_dirs);
    anchor_free(&ctx->anc);
    cudaFree(ctx->fix.bc64);
    ctx->fix_mem.release();
    free_bricks(&ctx->bricks);
    adjoint_free(&ctx->adj);
    ctx->adj_g.release();
    ctx->adj_out.release();
    for (DeviceBuf *b : {&ctx->in_ax, &ctx->in_ay, &ctx->in_az, &ctx->in_aux, &ctx->in_pinit, &ctx->f32, &ctx->b16,
                         &ctx->curl, &ctx->pvol_a, &ctx->pvol_b, &ctx->pout, &ctx->cnt, &ctx->pncnt, &ctx->scratch,
                         &ctx->flags, &ctx->centre, &ctx->pncnt64})
        b->release();
    if (ctx->iter_exec) cudaGraphExecDestroy(ctx->iter_exec);
    ctx->iter_buf.release();
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->own_stream && ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return OMNI3D_OK;
}

int omni3d_set_stream(omni3d_ctx *ctx, void *stream)
{
    if (!ctx) return fail(nullptr, OMNI3D_ERR_ARG, "ctx is NULL");
    cudaStreamSynchronize(ctx->st);
    if (ctx->own_stream) cudaStreamDestroy(ctx->st);
    ctx->st = (cudaStream_t)stream;
    ctx->own_stream = false;
    return OMNI3D_OK;
}

int omni3d_geometry_info(omni3d_ctx *ctx, long long *n_lines, long long *n_units, long long *walk_errors)
{
    if (!ctx) return fail(nullptr, OMNI3D_ERR_ARG, "ctx is NULL");
    if (n_lines) *n_lines = ctx->geo.n_lines;
    if (n_units) *n_units = ctx->geo.n_units;
    if (walk_errors) *walk_errors = ctx->geo.walk_errors;
    return OMNI3D_OK;
}

int omni3d_line_table(omni3d_ctx *ctx, int32_t *rows, long long n_max)
{
    if (!ctx || !rows || n_max < 0) return fail(ctx, OMNI3D_ERR_ARG, "bad arguments");
    long long n = std::min(n_max, ctx->geo.n_lines);
    if (n == 0) return OMNI3D_OK;
    cudaSetDevice(ctx->prm.device);
    CK(ctx, cudaMemcpyAsync(rows, ctx->geo.d_lines, sizeof(LineRec) * (size_t)n, cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaStreamSynchronize(ctx->st));
    for (long long i = 0; i < n; i++) rows[4 * i + 2] = ctx->table[rows[4 * i + 2]].orig;
    return OMNI3D_OK;
}

int omni3d_line_steps(omni3d_ctx *ctx, long long line, int8_t *axes, int cap)
{
    if (!ctx || !axes || line < 0 || line >= ctx->geo.n_lines) return fail(ctx, OMNI3D_ERR_ARG, "bad arguments");
    cudaSetDevice(ctx->prm.device);
    LineRec r;
    uint32_t gb;
    CK(ctx, cudaMemcpyAsync(&r, ctx->geo.d_lines + line, sizeof(r), cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaMemcpyAsync(&gb, ctx->geo.d_gbase + (line >> 5), sizeof(gb), cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaStreamSynchronize(ctx->st));
    if (r.m > cap) return fail(ctx, OMNI3D_ERR_RANGE, "cap smaller than the line's step count");
    int nw = (r.m + 15) / 16;
    std::vector<uint32_t> words((size_t)std::max(nw, 1));
    for (int w = 0; w < nw; w++)
        CK(ctx, cudaMemcpyAsync(&words[w], ctx->geo.d_desc + 32ull * gb + 32ull * w + (line & 31), sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaStreamSynchronize(ctx->st));
    for (int s = 0; s < r.m; s++) axes[s] = (int8_t)((words[s >> 4] >> (2 * (s & 15))) & 3u);
    return r.m;
}

int omni3d_gauge(omni3d_ctx *ctx, float *p, const float *count, long long n, int gauge, long long ref,
                 int device_ptrs)
{
    if (!ctx || !p) return fail(ctx, OMNI3D_ERR_ARG, "NULL argument");
    const long long V = ctx->geo.grid.V;
    if (n != V) return fail(ctx, OMNI3D_ERR_ARG, "n differs from the context's voxel count");
    if (gauge < OMNI3D_GAUGE_NONE || gauge > OMNI3D_GAUGE_MEAN) return fail(ctx, OMNI3D_ERR_ARG, "unknown gauge");
    if (gauge == OMNI3D_GAUGE_POINT && (ref < 0 || ref >= V)) return fail(ctx, OMNI3D_ERR_ARG, "ref outside the grid");
    if (gauge == OMNI3D_GAUGE_MEAN && !count) return fail(ctx, OMNI3D_ERR_ARG, "the mean gauge needs count");
    cudaSetDevice(ctx->prm.device);
    const bool dev = device_ptrs != 0;
    float *dp = p;
    const float *dc = count;
    if (!dev) {
        CK(ctx, ctx->pout.ensure(sizeof(float) * (size_t)V));
        dp = ctx->pout.as<float>();
        CK(ctx, cudaMemcpyAsync(dp, p, sizeof(float) * (size_t)V, cudaMemcpyHostToDevice, ctx->st));
        if (count) {
            int rc = stage(ctx, count, false, ctx->in_aux, V, &dc);
            if (rc) return rc;
        }
    }
    CK(ctx, ctx->scratch.ensure(sizeof(double) * std::max(change_scratch_doubles(), gauge_scratch_doubles()) + 64));
    CK(ctx, apply_gauge(V, gauge, ref, dc, dp, ctx->scratch.as<double>() + 4, ctx->st));
    if (!dev) CK(ctx, cudaMemcpyAsync(p, dp, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaStreamSynchronize(ctx->st));
    return OMNI3D_OK;
}

int omni3d_curl(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az, const float *mask, float *curl_out,
                int device_ptrs)
{
    if (!ctx || !ax || !ay || !az || !curl_out) return fail(ctx, OMNI3D_ERR_ARG, "NULL argument");
    cudaSetDevice(ctx->prm.device);
    const long long V = ctx->geo.grid.V;
    const bool dev = device_ptrs != 0;
    const float *dax, *day, *daz, *dmask;
    int rc;
    if ((rc = stage(ctx, ax, dev, ctx->in_ax, V, &dax))) return rc;
    if ((rc = stage(ctx, ay, dev, ctx->in_ay, V, &day))) return rc;
    if ((rc = stage(ctx, az, dev, ctx->in_az, V, &daz))) return rc;
    if ((rc = stage(ctx, mask, dev, ctx->in_aux, V, &dmask))) return rc;
    float *dout = curl_out;
    if (!dev) {
        CK(ctx, ctx->curl.ensure(sizeof(float) * (size_t)V));
        dout = ctx->curl.as<float>();
    }
    CK(ctx, curl_field(ctx->geo.grid, dax, day, daz, dmask, dout, ctx->st));
    if (!dev) CK(ctx, cudaMemcpyAsync(curl_out, dout, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaStreamSynchronize(ctx->st));
    return OMNI3D_OK;
}

int omni3d_centre_integration(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az, double pref,
                              float *p_out, int device_ptrs)
{
    if (!ctx || !ax || !ay || !az || !p_out) return fail(ctx, OMNI3D_ERR_ARG, "NULL argument");
    cudaSetDevice(ctx->prm.device);
    const long long V = ctx->geo.grid.V;
    const bool dev = device_ptrs != 0;
    const float *dax, *day, *daz;
    int rc;
    if ((rc = stage(ctx, ax, dev, ctx->in_ax, V, &dax))) return rc;
    if ((rc = stage(ctx, ay, dev, ctx->in_ay, V, &day))) return rc;
    if ((rc = stage(ctx, az, dev, ctx->in_az, V, &daz))) return rc;
    CK(ctx, ctx->centre.ensure(sizeof(double) * (size_t)V));
    float *dout = p_out;
    if (!dev) {
        CK(ctx, ctx->pvol_a.ensure(sizeof(float) * (size_t)V));
        dout = ctx->pvol_a.as<float>();
    }
    CK(ctx, centre_integration(ctx->geo.grid, dax, day, daz, 1, pref, ctx->centre.as<double>(), dout, ctx->st));
    if (!dev) CK(ctx, cudaMemcpyAsync(p_out, dout, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, ctx->st));
    CK(ctx, cudaStreamSynchronize(ctx->st));
    return OMNI3D_OK;
}

int omni3d_sweep(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az, const float *curl, const float *p,
                 float *pn, float *count, int device_ptrs)
{
    if (!ctx || !ax || !ay || !az || !p || !pn || !count) return fail(ctx, OMNI3D_ERR_ARG, "NULL argument");
    if (method_uses_curl(ctx->prm.method) && !curl)
        return fail(ctx, OMNI3D_ERR_ARG, "the selected and weighted methods need curl");
    cudaSetDevice(ctx->prm.device);
    const long long V = ctx->geo.grid.V;
    const bool dev = device_ptrs != 0;
    Field F;
    int rc = prepare_field(ctx, ax, ay, az, curl, nullptr, dev, &F);
    if (rc) return rc;
    if (ctx->geo.walk_rule == 3) CK(ctx, run_walk(&ctx->geo, 3, F.curl, ctx->st));  // paths follow this field
    const float *dp;
    if ((rc = stage(ctx, p, dev, ctx->in_pinit, V, &dp))) return rc;
    CK(ctx, ctx->pncnt.ensure(sizeof(float2) * (size_t)V));
    float2 *acc = ctx->pncnt.as<float2>();
    const bool bf16 = ctx->prm.grad_storage == OMNI3D_GRAD_BF16;
    int engine = choose_engine(ctx, bf16, &rc);
    if (rc) return rc;
    if ((rc = engine_prepare(ctx, &engine, F, ctx->prm.method))) return rc;
    CK(ctx, init_accum(V, nullptr, false, acc, ctx->st));
    CK(ctx, engine_sweep(ctx, engine, F, ctx->prm.method, bf16, dp, acc, ctx->st));
    // add (pn, count) to the caller's arrays
    float *dpn = pn, *dcount = count;
    if (!dev) {
        CK(ctx, ctx->pvol_a.ensure(sizeof(float) * (size_t)V));
        CK(ctx, ctx->pvol_b.ensure(sizeof(float) * (size_t)V));
        dpn = ctx->pvol_a.as<float>();
        dcount = ctx->pvol_b.as<float>();
        CK(ctx, cudaMemcpyAsync(dpn, pn, sizeof(float) * (size_t)V, cudaMemcpyHostToDevice, ctx->st));
        CK(ctx, cudaMemcpyAsync(dcount, count, sizeof(float) * (size_t)V, cudaMemcpyHostToDevice, ctx->st));
    }
    CK(ctx, accum_split(V, acc, dpn, dcount, ctx->st));
    if (!dev) {
        CK(ctx, cudaMemcpyAsync(pn, dpn, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, ctx->st));
        CK(ctx, cudaMemcpyAsync(count, dcount, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, ctx->st));
    }
    CK(ctx, cudaStreamSynchronize(ctx->st));
    return engine_check(ctx, engine);
}

namespace {

// Tolerance-driven anchor iterations in CUDA-graph chunks.  Checking the relative change on
// the host after every step costs a stream synchronisation per iteration (about 70 us,
// several times the step itself on small grids).  A chunk of kIterChunk steps is captured
// once into a graph; each step is followed by a one-thread convergence test that sets a
// device stop word, and every later kernel of the chunk sees the word and returns.  The host
// synchronises once per chunk and learns from the word which step met the tolerance, so the
// iterate and the iteration count are those of the step-by-step loop.
constexpr int kIterChunk = 16;  // even: a chunk leaves the ping-pong buffers in place

cudaError_t iterate_chunk(omni3d_ctx *ctx, const Anchor &A, int gauge, long long ref_anchor, double tol, float *pc,
                          float *pn, double *red2, cudaStream_t st, int *j_out, double *rel_out, const Fixed *fx)
{
    cudaError_t e = ctx->iter_buf.ensure(sizeof(double) * (kIterChunk + 1));
    if (e != cudaSuccess) return e;
    int *stop = ctx->iter_buf.as<int>();
    double *rels = ctx->iter_buf.as<double>() + 1;
    uint64_t tol_bits;
    std::memcpy(&tol_bits, &tol, sizeof(tol_bits));
    const std::vector<const void *> key = {
        A.rowptr, A.rowlen, A.col, A.cw, A.bc, A.vox, A.red, reinterpret_cast<const void *>((uintptr_t)A.n),
        reinterpret_cast<const void *>((uintptr_t)A.unit_weights), pc, pn, red2,
        reinterpret_cast<const void *>((uintptr_t)gauge), reinterpret_cast<const void *>((intptr_t)ref_anchor),
        reinterpret_cast<const void *>((uintptr_t)tol_bits), stop, fx ? fx->scale : nullptr,
        fx ? fx->bits : nullptr};
    if (!ctx->iter_exec || ctx->iter_key != key) {
        if (ctx->iter_exec) cudaGraphExecDestroy(ctx->iter_exec);
        ctx->iter_exec = nullptr;
        const unsigned long long l0 = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
        if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
        cudaError_t ce = cudaMemsetAsync(stop, 0, sizeof(int), st);
        for (int j = 0; j < kIterChunk && ce == cudaSuccess; j++) {
            const float *from = (j % 2 == 0) ? pc : pn;
            float *to = (j % 2 == 0) ? pn : pc;
            ce = anchor_step(A, nullptr, false, gauge, ref_anchor, from, to, red2, st, stop, fx);
            if (ce == cudaSuccess) ce = converged_test_launch(red2, tol, j, stop, rels, st);
        }
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(st, &graph);
        const unsigned long long l1 = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
        __atomic_fetch_sub(&g_kernel_launches, l1 - l0, __ATOMIC_RELAXED);  // captured, not launched
        if (ce == cudaSuccess) ce = e;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&ctx->iter_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            ctx->iter_exec = nullptr;
            return ce;
        }
        ctx->iter_key = key;
        ctx->iter_launches = l1 - l0;
    }
    if ((e = cudaGraphLaunch(ctx->iter_exec, st)) != cudaSuccess) return e;
    __atomic_fetch_add(&g_kernel_launches, ctx->iter_launches, __ATOMIC_RELAXED);
    double h[kIterChunk + 1];
    if ((e = cudaMemcpyAsync(h, ctx->iter_buf.p, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
    int stopv = 0;
    std::memcpy(&stopv, &h[0], sizeof(stopv));
    *j_out = stopv - 1;
    *rel_out = h[1 + (stopv > 0 ? stopv - 1 : kIterChunk - 1)];
    return cudaSuccess;
}

}  // namespace

int omni3d_solve(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az, const float *curl,
                 const float *mask, const float *p_init, float *p_out, float *count_out, int device_ptrs,
                 omni3d_stats *stats)
{
    if (!ctx || !ax || !ay || !az || !p_out) return fail(ctx, OMNI3D_ERR_ARG, "NULL argument");
    cudaSetDevice(ctx->prm.device);
    const omni3d_params &P = ctx->prm;
    const Grid &g = ctx->geo.grid;
    const long long V = g.V;
    const bool dev = device_ptrs != 0;
    const bool bf16 = P.grad_storage == OMNI3D_GRAD_BF16;
    cudaStream_t st = ctx->st;
    long long ref = (long long)P.ref_i + (long long)P.ref_j * g.X + (long long)P.ref_k * g.XY;

    const unsigned long long launches0 = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
    cudaEventRecord(ctx->ev[0], st);
    Field F;
    int rc = prepare_field(ctx, ax, ay, az, curl, mask, dev, &F);
    if (rc) return rc;
    if (ctx->geo.walk_rule == 3 && P.max_iter > 0)
        CK(ctx, run_walk(&ctx->geo, 3, F.curl, st));  // minimum-curl paths follow this field
    int engine = OMNI3D_ENGINE_LINES;
    const bool det = P.deterministic != 0;  // bit-reproducible: fixed-point sums, line engine
    if (P.max_iter > 0 && (P.sweep_fp64 || det)) {
        if (P.engine == OMNI3D_ENGINE_BRICKS)
            return fail(ctx, OMNI3D_ERR_STATE, "the brick engine accumulates in FP32 only (sweep_fp64)");
    } else if (P.max_iter > 0) {
        engine = choose_engine(ctx, bf16, &rc);
        if (rc) return rc;
        if ((rc = engine_prepare(ctx, &engine, F, P.method))) return rc;
    }
    // initial pressure (zero when not given)
    const float *dpinit;
    if (p_init) {
        if ((rc = stage(ctx, p_init, dev, ctx->in_pinit, V, &dpinit))) return rc;
    } else {
        CK(ctx, ctx->in_pinit.ensure(sizeof(float) * (size_t)V));
        if (P.initial_guess == OMNI3D_INIT_CENTRE) {  // initialIntegration.cpp from the packed field
            CK(ctx, ctx->centre.ensure(sizeof(double) * (size_t)V));
            const float *f = reinterpret_cast<const float *>(F.f32);
            CK(ctx, centre_integration(g, f, f + 1, f + 2, 4, 0.0, ctx->centre.as<double>(), ctx->in_pinit.as<float>(),
                                       st));
        } else {
            CK(ctx, cudaMemsetAsync(ctx->in_pinit.p, 0, sizeof(float) * (size_t)V, st));
        }
        dpinit = ctx->in_pinit.as<float>();
    }
    CK(ctx, ctx->pncnt.ensure(sizeof(float2) * (size_t)V));
    CK(ctx, ctx->pout.ensure(sizeof(float) * (size_t)V));
    CK(ctx, ctx->cnt.ensure(sizeof(float) * (size_t)V));
    CK(ctx, ctx->pvol_a.ensure(sizeof(float) * (size_t)V));
    CK(ctx, ctx->scratch.ensure(sizeof(double) * std::max(change_scratch_doubles(), gauge_scratch_doubles()) + 64));
    float2 *acc = ctx->pncnt.as<float2>();
    float *dout = ctx->pout.as<float>(), *dcnt = ctx->cnt.as<float>();
    double *scratch = ctx->scratch.as<double>();
    double *red2 = scratch;  // 2 doubles, then the reduction scratch
    double *rscratch = scratch + 4;

    const int K = P.max_iter;
    const bool seed = P.seed_first_iteration != 0;
    int done = 0;
    double rel = 0.0;
    double hred[2];
    long long n_anchor = 0, n_links = 0;

    int solver = P.solver;
    Anchor &A = ctx->anc;
    long long ref_anchor = -1;
    ctx->anc_last = false;
    Fixed *fx = nullptr;
    if (det && K > 0) {  // the bounds of every fixed-point sum of this solve (kernels_fixed.cu)
        fx = &ctx->fix;
        CK(ctx, ctx->fix_mem.ensure(sizeof(double) * kFixSlots + sizeof(unsigned) * kBitsSlots));
        fx->scale = ctx->fix_mem.as<double>();
        fx->bits = reinterpret_cast<unsigned *>(fx->scale + kFixSlots);
        static const double ones[kFixSlots] = {1.0, 1.0, 1.0, 1.0, 1.0};  // scales this solve leaves unused
        CK(ctx, cudaMemcpyAsync(fx->scale, ones, sizeof(ones), cudaMemcpyHostToDevice, st));
        fx->acc = method_accum(P.method);
        fx->hmax = 0.5 * (double)P.density * (double)std::max(std::max(std::fabs(P.dx), std::fabs(P.dy)), std::fabs(P.dz));
        fx->path = (double)g.X + (double)g.Y + (double)g.Z;
        unsigned lmax = 0;
        CK(ctx, max_lines_through(&ctx->geo, st, &lmax));
        fx->lmax = (double)lmax;
        CK(ctx, fix_field_bounds(V, F.f32, *fx, st));
        CK(ctx, fix_fill_scales(*fx, st));
    }
    if (K > 0 && solver == OMNI3D_SOLVER_ANCHOR) {
        std::string aerr;
        cudaError_t e;
        if (P.method == OMNI3D_METHOD_PLAIN && ctx->anc_cached) {
            e = anchor_refresh_rhs(ctx->geo, F, &ctx->anc, st, fx);
            aerr = cudaGetErrorString(e);
        } else {
            ctx->anc_cached = false;
            long long max_links = P.anchor_max_links;
            if (max_links <= 0) {  // what 80 % of the free memory holds (column + weight)
                size_t fr = 0, tot = 0;
                cudaMemGetInfo(&fr, &tot);
                max_links = (long long)(0.8 * (double)fr / 8.0);
            }
            e = anchor_build(ctx->geo, F, P.method, P.gauge == OMNI3D_GAUGE_POINT ? ref : -1, max_links,
                             &ctx->anc, st, &aerr, fx);
            ctx->anc_cached = e == cudaSuccess && P.method == OMNI3D_METHOD_PLAIN;
            adjoint_free(&ctx->adj);
        }
        ctx->anc_last = e == cudaSuccess;
        if (e == cudaErrorNotSupported) {
            cudaGetLastError();
            solver = OMNI3D_SOLVER_SWEEP;  // operator not profitable: one sweep per iteration
        } else if (e != cudaSuccess) {
            return fail(ctx, e == cudaErrorMemoryAllocation ? OMNI3D_ERR_NOMEM : OMNI3D_ERR_CUDA,
                        "anchor operator: " + aerr);
        }
    }
    if (K == 0) {
        cudaEventRecord(ctx->ev[5], st);
        cudaEventRecord(ctx->ev[6], st);
        CK(ctx, cudaMemcpyAsync(dout, dpinit, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st));
        CK(ctx, cudaMemsetAsync(dcnt, 0, sizeof(float) * (size_t)V, st));
        cudaEventRecord(ctx->ev[1], st);
        cudaEventRecord(ctx->ev[2], st);
    } else if (solver == OMNI3D_SOLVER_SWEEP) {
        // the reference loop: NoItr x {sweep, devidecountInner}
        CK(ctx, ctx->pvol_b.ensure(sizeof(float) * (size_t)V));
        float *pc = ctx->pvol_a.as<float>(), *pn = ctx->pvol_b.as<float>();
        CK(ctx, cudaMemcpyAsync(pc, dpinit, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st));
        // the convergence test runs over the anchor voxels, as in the anchor solver
        uint8_t *amask = nullptr;
        if (P.tol > 0.0) {
            CK(ctx, ctx->flags.ensure((size_t)V + 64));
            amask = ctx->flags.as<uint8_t>();
            unsigned long long *cnt1 = reinterpret_cast<unsigned long long *>(amask + ((V + 7) / 8) * 8);
            CK(ctx, anchor_mark(ctx->geo, F, P.method, P.gauge == OMNI3D_GAUGE_POINT ? ref : -1, amask, cnt1,
                                st));
        }
        cudaEventRecord(ctx->ev[1], st);
        double2 *acc64 = nullptr;
        if (P.sweep_fp64 || det) {
            CK(ctx, ctx->pncnt64.ensure(sizeof(double2) * (size_t)V));
            acc64 = ctx->pncnt64.as<double2>();
        }
        for (int it = 1; it <= K; it++) {
            if (det) {  // exact fixed-point sums, normalised in FP64
                Fix2 *accf = reinterpret_cast<Fix2 *>(acc64);
                CK(ctx, fix_sweep_scales(V, pc, *fx, st));
                CK(ctx, init_accum_fix(V, dpinit, seed && it == 1, *fx, accf, st));
                cudaEventRecord(ctx->ev[5], st);
                CK(ctx, sweep_full_fix(ctx->geo, F, P.method, bf16, pc, accf, fx->scale, st));
                cudaEventRecord(ctx->ev[6], st);
                CK(ctx, normalize_fix(V, accf, *fx, pc, pn, dcnt, st));
            } else if (acc64) {
                CK(ctx, init_accum64(V, dpinit, seed && it == 1, acc64, st));
                cudaEventRecord(ctx->ev[5], st);
                CK(ctx, sweep_full64(ctx->geo, F, P.method, bf16, pc, acc64, st));
                cudaEventRecord(ctx->ev[6], st);
                CK(ctx, normalize64(V, acc64, pc, pn, dcnt, st));
            } else {
                CK(ctx, init_accum(V, dpinit, seed && it == 1, acc, st));
                cudaEventRecord(ctx->ev[5], st);
                CK(ctx, engine_sweep(ctx, engine, F, P.method, bf16, pc, acc, st));
                cudaEventRecord(ctx->ev[6], st);
                CK(ctx, normalize(V, acc, pc, pn, dcnt, st));
            }
            done = it;
            if (P.tol > 0.0) {
                CK(ctx, change_sums(V, pc, pn, P.gauge, P.gauge == OMNI3D_GAUGE_POINT ? ref : -1, rscratch, red2, st,
                                    amask));
                CK(ctx, cudaMemcpyAsync(hred, red2, sizeof(hred), cudaMemcpyDeviceToHost, st));
                CK(ctx, cudaStreamSynchronize(st));
                rel = hred[1] > 0 ? std::sqrt(hred[0] / hred[1]) : 0.0;
            }
            std::swap(pc, pn);
            if (P.tol > 0.0 && rel < P.tol) break;
        }
        cudaEventRecord(ctx->ev[2], st);
        CK(ctx, cudaMemcpyAsync(dout, pc, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st));
    } else {
        // anchor form: iterate the anchors, then one full sweep
        n_anchor = A.n;
        n_links = A.nnz;
        if (P.gauge == OMNI3D_GAUGE_POINT) {
            int32_t ra = -1;
            CK(ctx, cudaMemcpyAsync(&ra, A.id + ref, sizeof(ra), cudaMemcpyDeviceToHost, st));
            CK(ctx, cudaStreamSynchronize(st));
            ref_anchor = ra;
        }
        CK(ctx, anchor_gather(A, dpinit, A.pa, st));
        cudaEventRecord(ctx->ev[1], st);
        float *pc = A.pa, *pn = A.pb;
        int its = 0;
        for (int it = 1; it <= K - 1;) {
            if (P.tol > 0.0 && it > 1 && A.n > 0 && st != nullptr && K - it >= kIterChunk) {
                int j = -1;
                CK(ctx, iterate_chunk(ctx, A, P.gauge, ref_anchor, P.tol, pc, pn, red2, st, &j, &rel, fx));
                if (j >= 0) {  // step it + j met the tolerance; step j wrote pn when j is even
                    its = it + j;
                    if (j % 2 == 0) std::swap(pc, pn);
                    break;
                }
                its = it + kIterChunk - 1;
                it += kIterChunk;
                continue;
            }
            CK(ctx, anchor_step(A, dpinit, seed && it == 1, P.gauge, ref_anchor, pc, pn, P.tol > 0.0 ? red2 : nullptr, st,
                                nullptr, fx));
            its = it;
            std::swap(pc, pn);
            if (P.tol > 0.0) {
                CK(ctx, cudaMemcpyAsync(hred, red2, sizeof(hred), cudaMemcpyDeviceToHost, st));
                CK(ctx, cudaStreamSynchronize(st));
                rel = hred[1] > 0 ? std::sqrt(hred[0] / hred[1]) : 0.0;
                if (rel < P.tol) break;
            }
            it++;
        }
        cudaEventRecord(ctx->ev[2], st);
        float *vol = ctx->pvol_a.as<float>();
        CK(ctx, cudaMemcpyAsync(vol, dpinit, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st));
        CK(ctx, anchor_scatter(A, pc, vol, st));
        if (det) {  // bit-reproducible: exact fixed-point sums, normalised in FP64
            CK(ctx, ctx->pncnt64.ensure(sizeof(double2) * (size_t)V));
            Fix2 *accf = reinterpret_cast<Fix2 *>(ctx->pncnt64.p);
            CK(ctx, fix_sweep_scales(V, vol, *fx, st));
            CK(ctx, init_accum_fix(V, dpinit, seed && its == 0, *fx, accf, st));
            cudaEventRecord(ctx->ev[5], st);
            CK(ctx, sweep_full_fix(ctx->geo, F, P.method, bf16, vol, accf, fx->scale, st));
            cudaEventRecord(ctx->ev[6], st);
            CK(ctx, normalize_fix(V, accf, *fx, dpinit, dout, dcnt, st));
        } else if (P.sweep_fp64) {  // the defect-correction sweep: FP64 sums and normalisation
            CK(ctx, ctx->pncnt64.ensure(sizeof(double2) * (size_t)V));
            double2 *acc64 = ctx->pncnt64.as<double2>();
            CK(ctx, init_accum64(V, dpinit, seed && its == 0, acc64, st));
            cudaEventRecord(ctx->ev[5], st);
            CK(ctx, sweep_full64(ctx->geo, F, P.method, bf16, vol, acc64, st));
            cudaEventRecord(ctx->ev[6], st);
            CK(ctx, normalize64(V, acc64, dpinit, dout, dcnt, st));
        } else {
            CK(ctx, init_accum(V, dpinit, seed && its == 0, acc, st));
            cudaEventRecord(ctx->ev[5], st);
            CK(ctx, engine_sweep(ctx, engine, F, P.method, bf16, vol, acc, st));
            cudaEventRecord(ctx->ev[6], st);
            CK(ctx, normalize(V, acc, dpinit, dout, dcnt, st));
        }
        done = its + 1;
    }
    CK(ctx, apply_gauge(V, P.gauge, ref, dcnt, dout, rscratch, st));
    cudaEventRecord(ctx->ev[3], st);
    if (dev) {
        CK(ctx, cudaMemcpyAsync(p_out, dout, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st));
        if (count_out) CK(ctx, cudaMemcpyAsync(count_out, dcnt, sizeof(float) * (size_t)V, cudaMemcpyDeviceToDevice, st));
    } else {
        CK(ctx, cudaMemcpyAsync(p_out, dout, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, st));
        if (count_out) CK(ctx, cudaMemcpyAsync(count_out, dcnt, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, st));
    }
    cudaEventRecord(ctx->ev[4], st);
    CK(ctx, cudaStreamSynchronize(st));
    CK(ctx, cudaGetLastError());
    if ((rc = engine_check(ctx, engine))) return rc;
    if (fx) {  // a bound without a finite scale (a curl too close to zero): the sums were not held
        double sc[kFixSlots];
        CK(ctx, cudaMemcpy(sc, fx->scale, sizeof(sc), cudaMemcpyDeviceToHost));
        for (double x : sc)
            if (x == 0.0)
                return fail(ctx, OMNI3D_ERR_RANGE, "deterministic: a fixed-point bound is not finite (the least "
                                                   "nonzero curl is too small for the weights' bound)");
    }
    ctx->last_iterations = done;
    ctx->last_method = P.method;
    if (stats) {
        stats->iterations = done;
        stats->rel_change = rel;
        stats->n_lines = ctx->geo.n_lines;
        stats->n_units = ctx->geo.n_units;
        stats->walk_errors = ctx->geo.walk_errors;
        stats->n_anchors = n_anchor;
        stats->n_links = n_links;
        stats->ms_geometry = ctx->ms_geometry;
        stats->ms_setup = ms_between(ctx->ev[0], ctx->ev[1]);
        stats->ms_iterate = ms_between(ctx->ev[1], ctx->ev[2]);
        stats->ms_final = ms_between(ctx->ev[2], ctx->ev[3]);
        stats->ms_total = ms_between(ctx->ev[0], ctx->ev[4]);
        stats->ms_sweep = ms_between(ctx->ev[5], ctx->ev[6]);
        stats->kernel_launches = (long long)(__atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED) - launches0);
        stats->solver_used = solver;
        stats->engine_used = engine;
        stats->tile_width = ctx->geo.tile_width;
        stats->dir_group = ctx->geo.dir_group;
    }
    if (ctx->geo.walk_errors) return fail(ctx, OMNI3D_ERR_NUMERIC, "line walk hit the wrong-point branch");
    return OMNI3D_OK;
}

int omni3d_adjoint(omni3d_ctx *ctx, const float *grad_p, float *grad_ax, float *grad_ay, float *grad_az,
                   int device_ptrs)
{
    if (!ctx || !grad_p || !grad_ax || !grad_ay || !grad_az) return fail(ctx, OMNI3D_ERR_ARG, "NULL argument");
    if (ctx->last_iterations < 0) return fail(ctx, OMNI3D_ERR_STATE, "no solve to differentiate on this context");
    cudaSetDevice(ctx->prm.device);
    const omni3d_params &P = ctx->prm;
    const Grid &g = ctx->geo.grid;
    const long long V = g.V;
    const bool dev = device_ptrs != 0;
    cudaStream_t st = ctx->st;
    const long long ref = (long long)P.ref_i + (long long)P.ref_j * g.X + (long long)P.ref_k * g.XY;
    const bool plain = P.method == OMNI3D_METHOD_PLAIN;
    // the plain operator's structure and anchor counts depend on the geometry alone; the other
    // methods' weights depend on the curl, so their operator must be the last solve's
    if (plain ? !ctx->anc_cached : !ctx->anc_last) {  // the last solve ran the sweep form: build it now
        Field F;
        F.f32 = ctx->f32.as<float4>();
        F.bf16 = P.grad_storage == OMNI3D_GRAD_BF16 ? ctx->b16.as<uint2>() : nullptr;
        if (method_uses_curl(P.method)) {  // the curl the solve used, from the packed field
            CK(ctx, ctx->curl.ensure(sizeof(float) * (size_t)V));
            CK(ctx, field_curl(V, F.f32, ctx->curl.as<float>(), st));
            F.curl = ctx->curl.as<float>();
        }
        std::string aerr;
        cudaError_t e = anchor_build(ctx->geo, F, P.method, P.gauge == OMNI3D_GAUGE_POINT ? ref : -1,
                                     -1, &ctx->anc, st, &aerr);
        if (e != cudaSuccess) return fail(ctx, OMNI3D_ERR_CUDA, "anchor operator: " + aerr);
        ctx->anc_cached = plain;
        ctx->anc_last = true;
        adjoint_free(&ctx->adj);
    }
    const float *dg = grad_p;
    CK(ctx, ctx->adj_g.ensure(sizeof(float) * (size_t)V));
    if (!dev) {
        CK(ctx, ctx->adj_out.ensure(sizeof(float) * 3 * (size_t)V));
        CK(ctx, cudaMemcpyAsync(ctx->adj_out.p, grad_p, sizeof(float) * (size_t)V, cudaMemcpyHostToDevice, st));
        dg = ctx->adj_out.as<float>();
    }
    CK(ctx, ctx->scratch.ensure(sizeof(double) * std::max(change_scratch_doubles(),
                                                          std::max(gauge_scratch_doubles(),
                                                                   gauge_transpose_scratch_doubles())) + 64));
    float *gg = ctx->adj_g.as<float>();
    CK(ctx, gauge_transpose(V, P.gauge, ref, dg, ctx->cnt.as<float>(), gg, ctx->scratch.as<double>() + 4, st));
    float *gx = grad_ax, *gy = grad_ay, *gz = grad_az;
    if (!dev) {
        gx = ctx->adj_out.as<float>();
        gy = gx + V;
        gz = gy + V;
    }
    CK(ctx, adjoint_solve(ctx->geo, ctx->anc, &ctx->adj, ctx->last_iterations, P.method, ctx->f32.as<float4>(), gg,
                          ctx->cnt.as<float>(), gx, gy, gz, st));
    if (!dev) {
        CK(ctx, cudaMemcpyAsync(grad_ax, gx, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, st));
        CK(ctx, cudaMemcpyAsync(grad_ay, gy, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, st));
        CK(ctx, cudaMemcpyAsync(grad_az, gz, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, st));
    }
    CK(ctx, cudaStreamSynchronize(st));
    return OMNI3D_OK;
}

}  // extern "C"

// Context accessors for the translation units that do not see struct omni3d_ctx.
namespace omni3d {
const Geometry *context_geometry(const omni3d_ctx *ctx) { return &ctx->geo; }
const omni3d_params *context_params(const omni3d_ctx *ctx) { return &ctx->prm; }
cudaStream_t context_stream(const omni3d_ctx *ctx) { return ctx->st; }
void context_set_error(omni3d_ctx *ctx, const std::string &msg) { ctx->err = msg; }
}  // namespace omni3d

extern "C" {

// ------------------------------------------------------------------------- batches

int omni3d_batch_create(omni3d_ctx *const *ctxs, int n, omni3d_batch **out)
{
    if (!ctxs || n <= 0 || !out) return fail(nullptr, OMNI3D_ERR_ARG, "bad arguments");
    *out = nullptr;
    int dev = ctxs[0] ? ctxs[0]->prm.device : 0;
    for (int i = 0; i < n; i++) {
        if (!ctxs[i]) return fail(nullptr, OMNI3D_ERR_ARG, "NULL context in the batch");
        if (ctxs[i]->prm.device != dev) return fail(nullptr, OMNI3D_ERR_ARG, "contexts on different devices");
        for (int j = 0; j < i; j++)
            if (ctxs[j] == ctxs[i]) return fail(nullptr, OMNI3D_ERR_ARG, "a context appears twice in the batch");
    }
    cudaSetDevice(dev);
    omni3d_batch *b = new omni3d_batch();
    b->ctx.assign(ctxs, ctxs + n);
    b->device = dev;
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
    b->join.assign((size_t)n, nullptr);
    for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        omni3d_batch_destroy(b);
        return fail(nullptr, OMNI3D_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
    }
    *out = b;
    return OMNI3D_OK;
}

int omni3d_batch_destroy(omni3d_batch *b)
{
    if (!b) return OMNI3D_OK;
    cudaSetDevice(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (cudaEvent_t ev : b->join)
        if (ev) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return OMNI3D_OK;
}

const char *omni3d_batch_last_error(const omni3d_batch *b) { return b ? b->err.c_str() : g_error.c_str(); }

namespace {

// A member that the one-graph form can run: plain method, anchor solver, fixed iteration
// count (its solve has no host synchronisation once the cached operator exists).
bool graph_member(const omni3d_ctx *c)
{
    return c->prm.method == OMNI3D_METHOD_PLAIN && c->prm.solver == OMNI3D_SOLVER_ANCHOR && c->prm.tol == 0.0 &&
           !c->prm.deterministic;
}

// The concurrent form: every member solved by omni3d_solve on its own context stream, the
// members shared among a pool of host threads, so that one member's host synchronisations
// (operator sizes of the selected method, tolerance checks) hold up only its own thread
// while the others keep the GPU busy.  Returns the first failing member's status.
int batch_solve_concurrent(omni3d_batch *b, const float *const *ax, const float *const *ay, const float *const *az,
                           const float *const *mask, const float *const *p_init, float *const *p_out, float *const *count_out, int device_ptrs,
                           omni3d_stats *stats)
{
    const int n = (int)b->ctx.size();
    std::vector<omni3d_stats> st((size_t)n);
    std::vector<int> rc((size_t)n, OMNI3D_OK);
    std::atomic<int> next{0};
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
            rc[i] = omni3d_solve(b->ctx[i], ax[i], ay[i], az[i], nullptr, mask ? mask[i] : nullptr,
                                 p_init ? p_init[i] : nullptr, p_out[i],
                                 count_out ? count_out[i] : nullptr, device_ptrs, &st[i]);
        }
    };
    const int nthreads = std::max(1, std::min(n, 8));
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (int i = 0; i < n; i++)
        if (rc[i] != OMNI3D_OK) {
            b->err = "batch member " + std::to_string(i) + ": " + b->ctx[i]->err;
            g_error = b->err;
            return rc[i];
        }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->ms_total = ms;
        stats->solver_used = OMNI3D_SOLVER_ANCHOR;
        stats->engine_used = OMNI3D_ENGINE_LINES;
        stats->tile_width = b->ctx[0]->geo.tile_width;  // members may differ: the first's
        stats->dir_group = b->ctx[0]->geo.dir_group;
        for (int i = 0; i < n; i++) {
            const omni3d_stats &m = st[i];
            stats->iterations = std::max(stats->iterations, m.iterations);
            stats->rel_change = std::max(stats->rel_change, m.rel_change);
            stats->n_lines += m.n_lines;
            stats->n_units += m.n_units;
            stats->walk_errors += m.walk_errors;
            stats->n_anchors += m.n_anchors;
            stats->n_links += m.n_links;
            stats->ms_setup += m.ms_setup;
            stats->ms_iterate += m.ms_iterate;
            stats->ms_final += m.ms_final;
            stats->ms_sweep += m.ms_sweep;
            stats->kernel_launches += m.kernel_launches;
            if (m.solver_used == OMNI3D_SOLVER_SWEEP) stats->solver_used = OMNI3D_SOLVER_SWEEP;
            if (m.engine_used == OMNI3D_ENGINE_BRICKS) stats->engine_used = OMNI3D_ENGINE_BRICKS;
        }
    }
    return OMNI3D_OK;
}

}  // namespace

int omni3d_batch_solve(omni3d_batch *b, const float *const *ax, const float *const *ay, const float *const *az,
                       const float *const *mask, const float *const *p_init, float *const *p_out, float *const *count_out, int device_ptrs,
                       omni3d_stats *stats)
{
    auto bfail = [&](int code, const std::string &m) {
        if (b) b->err = m;
        g_error = m;
        return code;
    };
    if (!b || !ax || !ay || !az || !p_out) return bfail(OMNI3D_ERR_ARG, "NULL argument");
    cudaSetDevice(b->device);
    const int n = (int)b->ctx.size();
    for (int i = 0; i < n; i++)
        if (!ax[i] || !ay[i] || !az[i] || !p_out[i]) return bfail(OMNI3D_ERR_ARG, "NULL member argument");
    bool any_mask = false;
    for (int i = 0; mask && i < n; i++) any_mask = any_mask || mask[i] != nullptr;
    if (any_mask || !std::all_of(b->ctx.begin(), b->ctx.end(), graph_member))
        return batch_solve_concurrent(b, ax, ay, az, mask, p_init, p_out, count_out, device_ptrs, stats);
    const bool dev = device_ptrs != 0;
    // device-side inputs and outputs of every member
    std::vector<const float *> dax(n), day(n), daz(n), dp0(n);
    std::vector<float *> dout(n), dcnt(n);
    for (int i = 0; i < n; i++) {
        omni3d_ctx *c = b->ctx[i];
        if (!ax[i] || !ay[i] || !az[i] || !p_out[i]) return bfail(OMNI3D_ERR_ARG, "NULL member argument");
        // first use: a regular solve builds the context's cached operator and buffers
        if (!prepared_for_graph(c)) {
            int rc = omni3d_solve(c, ax[i], ay[i], az[i], nullptr, nullptr, p_init ? p_init[i] : nullptr, p_out[i],
                                  count_out ? count_out[i] : nullptr, device_ptrs, nullptr);
            if (rc) return bfail(rc, std::string("preparing batch member: ") + c->err);
            if (!prepared_for_graph(c)) return bfail(OMNI3D_ERR_STATE, "batch member could not be prepared");
        }
        const long long V = c->geo.grid.V;
        if (dev) {
            dax[i] = ax[i]; day[i] = ay[i]; daz[i] = az[i];
            dp0[i] = p_init ? p_init[i] : nullptr;
            dout[i] = p_out[i];
            dcnt[i] = count_out ? count_out[i] : nullptr;
        } else {
            // host buffers: copied outside the graph into the member's staging buffers
            const float *src[4] = {ax[i], ay[i], az[i], p_init ? p_init[i] : nullptr};
            DeviceBuf *stg[4] = {&c->in_ax, &c->in_ay, &c->in_az, &c->in_aux};
            const float *dst[4] = {nullptr, nullptr, nullptr, nullptr};
            for (int q = 0; q < 4; q++) {
                if (!src[q]) continue;
                if (stg[q]->ensure(sizeof(float) * (size_t)V) != cudaSuccess) return bfail(OMNI3D_ERR_NOMEM, "staging");
                dst[q] = stg[q]->as<float>();
            }
            dax[i] = dst[0]; day[i] = dst[1]; daz[i] = dst[2]; dp0[i] = dst[3];
            dout[i] = nullptr;  // results stay in the member's own output buffers
            dcnt[i] = nullptr;
        }
    }
    std::vector<const void *> key;
    for (int i = 0; i < n; i++) {
        key.insert(key.end(), {dax[i], day[i], daz[i], dp0[i], dout[i], dcnt[i]});
    }
    cudaError_t e;
    if (!dev) {
        for (int i = 0; i < n; i++) {
            omni3d_ctx *c = b->ctx[i];
            const size_t bytes = sizeof(float) * (size_t)c->geo.grid.V;
            const float *src[4] = {ax[i], ay[i], az[i], p_init ? p_init[i] : nullptr};
            const float *dst[4] = {dax[i], day[i], daz[i], dp0[i]};
            for (int q = 0; q < 4; q++)
                if (src[q] && (e = cudaMemcpyAsync((void *)dst[q], src[q], bytes, cudaMemcpyHostToDevice, b->st)))
                    return bfail(OMNI3D_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    if (!b->exec || key != b->key) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        // capture: fork every member onto its own stream, join back
        unsigned long long l0 = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
        if ((e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal)))
            return bfail(OMNI3D_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(e));
        cudaError_t ce = cudaEventRecord(b->fork, b->st);
        for (int i = 0; i < n && ce == cudaSuccess; i++) {
            omni3d_ctx *c = b->ctx[i];
            ce = cudaStreamWaitEvent(c->st, b->fork, 0);
            if (ce == cudaSuccess) ce = enqueue_prepared(c, dax[i], day[i], daz[i], dp0[i], dout[i], dcnt[i], c->st);
            if (ce == cudaSuccess) ce = cudaEventRecord(b->join[i], c->st);
            if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->st, b->join[i], 0);
        }
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(b->st, &graph);
        if (ce != cudaSuccess || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return bfail(OMNI3D_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce != cudaSuccess ? ce : e));
        }
        e = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e) return bfail(OMNI3D_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
        b->launches_per_graph = (long long)(__atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED) - l0);
        b->key = key;
    }
    cudaEventRecord(b->t0, b->st);
    if ((e = cudaGraphLaunch(b->exec, b->st))) return bfail(OMNI3D_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    cudaEventRecord(b->t1, b->st);
    if (!dev) {
        for (int i = 0; i < n; i++) {
            omni3d_ctx *c = b->ctx[i];
            const size_t bytes = sizeof(float) * (size_t)c->geo.grid.V;
            if ((e = cudaMemcpyAsync(p_out[i], c->pout.p, bytes, cudaMemcpyDeviceToHost, b->st)))
                return bfail(OMNI3D_ERR_CUDA, cudaGetErrorString(e));
            if (count_out && count_out[i] &&
                (e = cudaMemcpyAsync(count_out[i], c->cnt.p, bytes, cudaMemcpyDeviceToHost, b->st)))
                return bfail(OMNI3D_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    if ((e = cudaStreamSynchronize(b->st))) return bfail(OMNI3D_ERR_CUDA, cudaGetErrorString(e));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, b->t0, b->t1);
        stats->ms_total = ms;
        stats->kernel_launches = b->launches_per_graph;
        stats->solver_used = OMNI3D_SOLVER_ANCHOR;
        stats->engine_used = OMNI3D_ENGINE_LINES;
        stats->tile_width = b->ctx.empty() ? 0 : b->ctx[0]->geo.tile_width;  // members may differ: the first's
        stats->dir_group = b->ctx.empty() ? 0 : b->ctx[0]->geo.dir_group;
        for (omni3d_ctx *c : b->ctx) {
            stats->n_lines += c->geo.n_lines;
            stats->n_units += c->geo.n_units;
            stats->walk_errors += c->geo.walk_errors;
            stats->n_anchors += c->anc.n;
            stats->n_links += c->anc.nnz;
            stats->iterations = c->prm.max_iter;
        }
    }
    return OMNI3D_OK;
}

}  // extern "C"
