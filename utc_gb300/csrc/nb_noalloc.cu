// nb_noalloc.cu -- one fast FP32 step that allocates no memory.
//
// Who needs it: some callers cannot call cudaMalloc.  A host application
// whose memory manager reserves the GPU's memory up front and hands out
// sub-buffers itself cannot have a library allocate behind its back (the
// allocation fails, or it breaks the manager's accounting), and a
// latency-critical loop cannot afford the device-wide synchronisation that
// cudaMalloc and cudaFree may cause.  nb_step_f32_noalloc serves them: the
// caller passes its own input and output buffers, and the partial-force
// scratch the fast kernel needs lives in a fixed array compiled into this
// library instead of memory obtained at run time.
//
// The array: kNoAllocScratchFloat4 float4 = 16 MiB, a file-scope __device__
// array, so every GPU that loads this library holds it until the process
// exits.  It bounds the system size: n <= kNoAllocMaxBodies = 262,144.
//
// Host code never hands the array's name to a kernel: on the host that name
// is only a stand-in for the device symbol (using it as a pointer would fault,
// or on a GPU that can reach host memory silently use the wrong memory).  The
// array's device address belongs to a CUDA context, not to a device: the
// first call in each context looks it up with cudaGetSymbolAddress and caches
// it beside the context's unique ID (cuCtxGetId), one entry per device.  A
// call in another context on that device -- the primary context re-created
// after cudaDeviceReset, or a driver-API context the caller made current --
// sees a different ID and looks the address up again instead of using one
// that is no longer mapped.  The lookup should come before any stream capture
// in that context.
//
// All calls share the one array and it keeps what the last call wrote.
// Nothing in it has to start at zero: each call writes every scratch entry
// it later reads.  Calls whose kernels overlap on the GPU (for example on two
// streams at once) race on the array and corrupt each other's results;
// serialise them.
#include <cuda.h>

#include <mutex>

#include "nb_internal.cuh"

namespace {

constexpr size_t kNoAllocScratchFloat4 = size_t(1) << 20;  // 16 MiB
constexpr int kNoAllocMaxBodies = 262144;
constexpr int kNoAllocBlock = 128;  // launch shape: 128 threads x 8 bodies
constexpr int kNoAllocBpt = 8;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float4 g_noalloc_scratch[kNoAllocScratchFloat4];

struct ScratchAddress {
    unsigned long long ctx_id;  // cuCtxGetId of the context it was looked up in
    float4 *ptr;
};
std::mutex g_scratch_mu;
ScratchAddress g_scratch_addr[kMaxDevices] = {};

// The two driver calls, found through the runtime (the library does not link
// the driver library itself).  Resolved once, under g_scratch_mu.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int resolve_driver_calls()
{
    if (g_ctx_get_current && g_ctx_get_id) return NB_OK;
    void *f0 = nullptr, *f1 = nullptr;
    cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
    NB_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0));
    NB_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1));
    if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
        return nb::set_error(NB_ERR_CUDA, "nb_step_f32_noalloc: driver has no cuCtxGetCurrent/cuCtxGetId");
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
    return NB_OK;
}

// Unique ID of the calling thread's current CUDA context; 0 if none is
// current yet (the runtime binds one on its first call that needs it).
int current_context_id(unsigned long long *id)
{
    *id = 0;
    int st = resolve_driver_calls();
    if (st) return st;
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS)
        return nb::set_error(NB_ERR_CUDA, "nb_step_f32_noalloc: cuCtxGetCurrent failed");
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS)
        return nb::set_error(NB_ERR_CUDA, "nb_step_f32_noalloc: cuCtxGetId failed");
    return NB_OK;
}

// Device address of g_noalloc_scratch in the current context of device dev
// (looked up again whenever the context differs from the cached one).
int scratch_for_current_context(int dev, float4 **out)
{
    if (dev < 0 || dev >= kMaxDevices)
        return nb::set_error(NB_ERR_UNSUPPORTED, "nb_step_f32_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    unsigned long long id = 0;
    int st = current_context_id(&id);
    if (st) return st;
    ScratchAddress &a = g_scratch_addr[dev];
    if (id == 0 || !a.ptr || a.ctx_id != id) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return nb::cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        if (id == 0) {  // the lookup bound the runtime's context: cache under it
            st = current_context_id(&id);
            if (st) return st;
        }
        a.ctx_id = id;  // 0 still: not cached, looked up again next time
        a.ptr = static_cast<float4 *>(p);
    }
    *out = a.ptr;
    return NB_OK;
}

}  // namespace

extern "C" int nb_step_f32_noalloc(const float *pos_old, float *pos_new, float *vel, int n,
                                   float eps2, float damping, float dt, int kick, float G,
                                   void *stream)
{
    if (n < 0 || n > kNoAllocMaxBodies)
        return nb::set_error(NB_ERR_INVALID,
                             "nb_step_f32_noalloc: n must be in [0, 262144] (the fixed 16 MiB "
                             "scratch array holds the partial forces of at most 262,144 bodies)");
    if (kick != NB_KICK_REFERENCE && kick != NB_KICK_PHYSICAL)
        return nb::set_error(NB_ERR_INVALID, "nb_step_f32_noalloc: unknown kick mode");
    if (n == 0) return NB_OK;
    if (!pos_old || !pos_new || !vel)
        return nb::set_error(NB_ERR_INVALID, "nb_step_f32_noalloc: NULL buffer");
    if (pos_old == pos_new)
        return nb::set_error(NB_ERR_INVALID, "nb_step_f32_noalloc: pos_old and pos_new must differ");
    int dev = 0;
    NB_CUDA(cudaGetDevice(&dev));
    float4 *scratch = nullptr;
    int st = scratch_for_current_context(dev, &scratch);
    if (st) return st;
    nb::SkPlan plan;
    st = nb::fast_plan(n, kNoAllocBlock, kNoAllocBpt, 0, dev, &plan);
    if (st) return st;
    // keep slots * tbsize within the array: fewer persistent CTAs if needed
    const long long max_slots = (long long)(kNoAllocScratchFloat4 / (size_t)plan.tbsize);
    if (plan.ntb > max_slots)
        return nb::set_error(NB_ERR_INVALID, "nb_step_f32_noalloc: system too large for the scratch array");
    const long long grid_cap = max_slots - plan.ntb + 1;
    if (plan.grid > grid_cap) plan.grid = (int)grid_cap;
    plan.slots = plan.grid + plan.ntb - 1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = nb::fast_force(plan, reinterpret_cast<const float4 *>(pos_old), eps2, scratch, s);
    if (st) return st;
    return nb::fast_integrate(plan, reinterpret_cast<const float4 *>(pos_old),
                              reinterpret_cast<float4 *>(pos_new), reinterpret_cast<float4 *>(vel),
                              scratch, damping, dt, kick, G, nullptr, s);
}
