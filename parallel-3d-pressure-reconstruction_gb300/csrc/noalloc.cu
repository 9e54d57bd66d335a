// omni3d_sweep_noalloc: one omni sweep that allocates no device memory.
//
// omni3d_sweep packs the gradient into a float4 field and accumulates (pn, count) in a
// float2 volume, both in device buffers it allocates on first use.  Some callers cannot
// allocate at that point: a host framework that owns all device memory through its own
// pool and forbids driver allocations inside its step, a plugin loaded into an application
// whose memory budget is fixed up front, or a real-time pipeline that cannot afford
// cudaMalloc's implicit device synchronisation in its loop.  For them this variant keeps
// both scratch volumes in file-scope device arrays sized for at most
// OMNI3D_NOALLOC_MAX_VOXELS voxels (64^3: 4 MiB of field + 2 MiB of accumulator, held by
// every GPU that loads the library until the process exits).
//
// The host code below never passes the arrays' names to a kernel: in host code those
// names are host-side stand-ins, not device addresses.  The first call on a device looks
// up their device addresses with cudaGetSymbolAddress (with that device current) and keeps
// them for later calls; the caller's current device is restored before the call returns.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "omni3d_internal.h"

namespace {

constexpr long long kMaxVoxels = OMNI3D_NOALLOC_MAX_VOXELS;

// The scratch volumes, shared by every call on the same device.
static __device__ __align__(256) float4 g_noalloc_field[kMaxVoxels];
static __device__ __align__(256) float2 g_noalloc_accum[kMaxVoxels];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
float4 *g_field_addr[kMaxDevices] = {};
float2 *g_accum_addr[kMaxDevices] = {};

// Device addresses of the scratch arrays on `device` (the current device).
cudaError_t scratch_addresses(int device, float4 **field, float2 **accum)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_field_addr[device]) {
        void *f = nullptr, *a = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&f, g_noalloc_field);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&a, g_noalloc_accum);
        if (e != cudaSuccess) return e;
        g_field_addr[device] = static_cast<float4 *>(f);
        g_accum_addr[device] = static_cast<float2 *>(a);
    }
    *field = g_field_addr[device];
    *accum = g_accum_addr[device];
    return cudaSuccess;
}

// Makes `device` current for the guard's lifetime and restores the caller's device after.
struct DeviceScope {
    int prev = -1;
    cudaError_t enter(int device)
    {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) {
            prev = -1;
            return e;
        }
        return prev == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceScope()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

namespace omni3d {
void set_global_error(const std::string &msg);
// Context accessors (api.cu).
const Geometry *context_geometry(const omni3d_ctx *ctx);
const omni3d_params *context_params(const omni3d_ctx *ctx);
cudaStream_t context_stream(const omni3d_ctx *ctx);
void context_set_error(omni3d_ctx *ctx, const std::string &msg);
}  // namespace omni3d

extern "C" int omni3d_sweep_noalloc(omni3d_ctx *ctx, const float *ax, const float *ay, const float *az,
                                    const float *curl, const float *p, float *pn, float *count, void *stream)
{
    using namespace omni3d;
    auto fail = [&](int code, const std::string &m) {
        if (ctx) context_set_error(ctx, m);
        set_global_error(m);
        return code;
    };
    if (!ctx || !ax || !ay || !az || !p || !pn || !count) return fail(OMNI3D_ERR_ARG, "NULL argument");
    const omni3d_params *P = context_params(ctx);
    const Geometry *geo = context_geometry(ctx);
    if (method_uses_curl(P->method) && !curl)
        return fail(OMNI3D_ERR_ARG, "the selected and weighted methods need curl");
    if (P->grad_storage != OMNI3D_GRAD_F32)
        return fail(OMNI3D_ERR_STATE, "omni3d_sweep_noalloc supports FP32 gradient storage only");
    if (method_walk_rule(P->method) == 3)
        return fail(OMNI3D_ERR_STATE, "omni3d_sweep_noalloc does not re-walk the minimum-curl paths per field");
    if (geo->grid.V > kMaxVoxels)
        return fail(OMNI3D_ERR_RANGE, "omni3d_sweep_noalloc: " + std::to_string(geo->grid.V) +
                                          " voxels exceed its static scratch of OMNI3D_NOALLOC_MAX_VOXELS = " +
                                          std::to_string(kMaxVoxels));
    if (P->device < 0 || P->device >= kMaxDevices) return fail(OMNI3D_ERR_RANGE, "device ordinal too large");
    DeviceScope scope;
    cudaError_t e = scope.enter(P->device);
    float4 *field = nullptr;
    float2 *accum = nullptr;
    if (e == cudaSuccess) e = scratch_addresses(P->device, &field, &accum);
    if (e != cudaSuccess) return fail(OMNI3D_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : context_stream(ctx);
    const long long V = geo->grid.V;
    Field F;
    F.f32 = field;
    F.curl = const_cast<float *>(curl);
    if ((e = pack_field(geo->grid, ax, ay, az, curl, &F, false, st)) != cudaSuccess ||
        (e = init_accum(V, nullptr, false, accum, st)) != cudaSuccess ||  // the last call's sums are cleared
        (e = sweep_full(*geo, F, P->method, false, p, accum, st)) != cudaSuccess ||
        (e = accum_split(V, accum, pn, count, st)) != cudaSuccess)
        return fail(OMNI3D_ERR_CUDA, std::string("omni3d_sweep_noalloc: ") + cudaGetErrorString(e));
    return OMNI3D_OK;
}
