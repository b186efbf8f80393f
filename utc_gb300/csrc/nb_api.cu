// nb_api.cu -- the C ABI (include/nbody_gb300.h): contexts, state transfer,
// stepping and the task-style host run.
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "nb_internal.cuh"

namespace nb {

static thread_local std::string g_last_error;

int set_error(int status, const std::string &msg)
{
    g_last_error = msg;
    return status;
}

int cuda_error(cudaError_t e, const char *what)
{
    const int st = (e == cudaErrorMemoryAllocation) ? NB_ERR_OOM : NB_ERR_CUDA;
    return set_error(st, std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                             cudaGetErrorString(e) + ")");
}

}  // namespace nb

struct nb_ctx {
    nb_params p;
    int device = 0;
    size_t elem = 4;      // bytes of one value of the state type
    void *pos[2] = {nullptr, nullptr};
    void *vel = nullptr;
    int cur = 0;          // pos[cur] holds the current positions
    bool has_state = false;
    nb::SkPlan plan;
    float4 *partial = nullptr;
    void *stage_pos = nullptr;  // pinned staging (NB_MEM_PINNED run_host)
    void *stage_vel = nullptr;
    void *stage_out = nullptr;
    std::vector<cudaEvent_t> events;  // pool for nb_step_timed
};

using nb::set_error;

static size_t state_bytes(const nb_ctx *c) { return (size_t)c->p.n * 4 * c->elem; }

static int validate(const nb_params *p)
{
    if (!p) return set_error(NB_ERR_INVALID, "params is NULL");
    if (p->n < 0) return set_error(NB_ERR_INVALID, "n must be >= 0");
    if (p->precision != NB_F32 && p->precision != NB_F64 && p->precision != NB_F32_COMP)
        return set_error(NB_ERR_INVALID, "unknown precision");
    if (p->algo != NB_ALGO_FAST && p->algo != NB_ALGO_EXACT)
        return set_error(NB_ERR_INVALID, "unknown algo");
    if (p->kick != NB_KICK_REFERENCE && p->kick != NB_KICK_PHYSICAL)
        return set_error(NB_ERR_INVALID, "unknown kick mode");
    if (p->memtype < NB_MEM_PAGEABLE || p->memtype > NB_MEM_UNIFIED)
        return set_error(NB_ERR_INVALID, "unknown memtype");
    if (!std::isfinite(p->eps2) || !std::isfinite(p->damping) || !std::isfinite(p->dt) ||
        !std::isfinite(p->G))
        return set_error(NB_ERR_INVALID, "eps2, damping, dt and G must be finite");
    if (p->precision == NB_F64 && p->algo == NB_ALGO_FAST)
        return set_error(NB_ERR_UNSUPPORTED, "NB_F64 runs the exact algorithm only");
    if (p->precision == NB_F32_COMP)
        return set_error(NB_ERR_UNSUPPORTED, "NB_F32_COMP is not available in this build");
    return NB_OK;
}

static void free_ctx(nb_ctx *c)
{
    if (!c) return;
    cudaFree(c->pos[0]);
    cudaFree(c->pos[1]);
    cudaFree(c->vel);
    cudaFree(c->partial);
    cudaFreeHost(c->stage_pos);
    cudaFreeHost(c->stage_vel);
    cudaFreeHost(c->stage_out);
    for (cudaEvent_t e : c->events) cudaEventDestroy(e);
    delete c;
}

static int dalloc(nb_ctx *c, void **p, size_t bytes)
{
    if (bytes == 0) {
        *p = nullptr;
        return NB_OK;
    }
    cudaError_t e = c->p.memtype == NB_MEM_UNIFIED ? cudaMallocManaged(p, bytes)
                                                   : cudaMalloc(p, bytes);
    if (e != cudaSuccess) return nb::cuda_error(e, "state allocation");
    return NB_OK;
}

static bool uses_fast(const nb_ctx *c) { return c->p.precision == NB_F32 && c->p.algo == NB_ALGO_FAST; }

extern "C" {

void nb_params_default(nb_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->precision = NB_F32;
    p->algo = NB_ALGO_FAST;
    p->kick = NB_KICK_REFERENCE;
    p->eps2 = 0.00125;
    p->damping = 0.995;
    p->dt = 0.016;
    p->G = 1.0;
    p->memtype = NB_MEM_PAGEABLE;
}

int nb_abi_version(void) { return NB_ABI_VERSION; }

const char *nb_last_error(void) { return nb::g_last_error.c_str(); }

int nb_create(const nb_params *p, nb_ctx **out)
{
    if (!out) return set_error(NB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int st = validate(p);
    if (st) return st;
    nb_ctx *c = new nb_ctx();
    c->p = *p;
    c->elem = p->precision == NB_F64 ? 8 : 4;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) {
        delete c;
        return nb::cuda_error(e, "cudaGetDevice");
    }
    const size_t sb = state_bytes(c);
    if ((st = dalloc(c, &c->pos[0], sb)) || (st = dalloc(c, &c->pos[1], sb)) ||
        (st = dalloc(c, &c->vel, sb))) {
        free_ctx(c);
        return st;
    }
    if (uses_fast(c)) {
        st = nb::fast_plan(p->n, p->block, p->bpt, p->ctas_per_sm, c->device, &c->plan);
        if (st) {
            free_ctx(c);
            return st;
        }
        const size_t pb = (size_t)c->plan.slots * c->plan.tbsize * sizeof(float4);
        if (pb) {
            e = cudaMalloc((void **)&c->partial, pb);
            if (e != cudaSuccess) {
                free_ctx(c);
                return nb::cuda_error(e, "partial-sum scratch allocation");
            }
        }
    }
    *out = c;
    return NB_OK;
}

int nb_destroy(nb_ctx *c)
{
    if (!c) return NB_OK;
    cudaDeviceSynchronize();
    free_ctx(c);
    return NB_OK;
}

int nb_set_state(nb_ctx *c, const void *pos, const void *vel, int where, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    const size_t sb = state_bytes(c);
    if (sb && (!pos || !vel)) return set_error(NB_ERR_INVALID, "pos/vel is NULL");
    if (where != NB_HOST && where != NB_DEVICE) return set_error(NB_ERR_INVALID, "where");
    cudaStream_t s = (cudaStream_t)stream;
    c->cur = 0;
    if (sb) {
        NB_CUDA(cudaMemcpyAsync(c->pos[0], pos, sb, cudaMemcpyDefault, s));
        NB_CUDA(cudaMemcpyAsync(c->vel, vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    c->has_state = true;
    return NB_OK;
}

int nb_get_state(nb_ctx *c, void *pos, void *vel, int where, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (where != NB_HOST && where != NB_DEVICE) return set_error(NB_ERR_INVALID, "where");
    const size_t sb = state_bytes(c);
    cudaStream_t s = (cudaStream_t)stream;
    if (sb) {
        if (pos) NB_CUDA(cudaMemcpyAsync(pos, c->pos[c->cur], sb, cudaMemcpyDefault, s));
        if (vel) NB_CUDA(cudaMemcpyAsync(vel, c->vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    return NB_OK;
}

int nb_state_ptrs(nb_ctx *c, void **pos_dev, void **vel_dev)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (pos_dev) *pos_dev = c->pos[c->cur];
    if (vel_dev) *vel_dev = c->vel;
    return NB_OK;
}

// One step; when ev != nullptr, records ev[0] before the first kernel,
// ev[1] between the force and the integrate kernel and ev[2] at the end.
static int step_once(nb_ctx *c, cudaStream_t s, void *acc_out, cudaEvent_t *ev = nullptr)
{
    const nb_params &p = c->p;
    void *po = c->pos[c->cur], *pn = c->pos[c->cur ^ 1];
    int st;
    if (ev) NB_CUDA(cudaEventRecord(ev[0], s));
    if (p.precision == NB_F64) {
        st = nb::exact_step_f64(p.n, (const double4 *)po, (double4 *)pn, (double4 *)c->vel, p.eps2,
                                p.damping, p.dt, p.kick, p.G, (double4 *)acc_out, p.block, s);
    } else if (p.algo == NB_ALGO_EXACT) {
        st = nb::exact_step_f32(p.n, (const float4 *)po, (float4 *)pn, (float4 *)c->vel,
                                (float)p.eps2, (float)p.damping, (float)p.dt, p.kick, (float)p.G,
                                (float4 *)acc_out, p.block, s);
    } else {
        st = nb::fast_force(c->plan, (const float4 *)po, (float)p.eps2, c->partial, s);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[1], s));
        if (!st)
            st = nb::fast_integrate(c->plan, (const float4 *)po, (float4 *)pn, (float4 *)c->vel,
                                    c->partial, (float)p.damping, (float)p.dt, p.kick, (float)p.G,
                                    (float4 *)acc_out, s);
    }
    if (!st && ev) {
        if (!uses_fast(c)) NB_CUDA(cudaEventRecord(ev[1], s));
        NB_CUDA(cudaEventRecord(ev[2], s));
    }
    if (!st && !acc_out) c->cur ^= 1;
    return st;
}

int nb_step(nb_ctx *c, int steps, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    for (int i = 0; i < steps; ++i) {
        int st = step_once(c, (cudaStream_t)stream, nullptr);
        if (st) return st;
    }
    return NB_OK;
}

int nb_step_timed(nb_ctx *c, int steps, float *ms_force, float *ms_integrate, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!ms_force || !ms_integrate) return set_error(NB_ERR_INVALID, "ms outputs are NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t need = 3 * (size_t)steps;
    while (c->events.size() < need) {
        cudaEvent_t e;
        NB_CUDA(cudaEventCreate(&e));
        c->events.push_back(e);
    }
    for (int i = 0; i < steps; ++i) {
        int st = step_once(c, s, nullptr, &c->events[3 * (size_t)i]);
        if (st) return st;
    }
    NB_CUDA(cudaStreamSynchronize(s));
    float f = 0, g = 0, ms = 0;
    for (int i = 0; i < steps; ++i) {
        cudaEvent_t *e = &c->events[3 * (size_t)i];
        NB_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
        f += ms;
        NB_CUDA(cudaEventElapsedTime(&ms, e[1], e[2]));
        g += ms;
    }
    *ms_force += f;
    *ms_integrate += g;
    return NB_OK;
}

int nb_accel(nb_ctx *c, void *acc_dev, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (c->p.n == 0) return NB_OK;
    if (!acc_dev) return set_error(NB_ERR_INVALID, "acc_dev is NULL");
    return step_once(c, (cudaStream_t)stream, acc_dev);
}

int nb_launches_per_step(nb_ctx *c)
{
    if (!c) return -1;
    if (c->p.n == 0) return 0;
    return uses_fast(c) ? 2 : 1;
}

int nb_plan_info(nb_ctx *c, int *info5)
{
    if (!c || !info5) return set_error(NB_ERR_INVALID, "ctx/info is NULL");
    info5[0] = c->plan.block;
    info5[1] = c->plan.npair * 2;
    info5[2] = c->plan.grid;
    info5[3] = c->plan.tbsize;
    info5[4] = c->plan.slots;
    return NB_OK;
}

int nb_run_host(nb_ctx *c, const void *pos, const void *vel, int loops, int out_interval,
                void *outbuffer, double *timings, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (loops < 0) return set_error(NB_ERR_INVALID, "loops must be >= 0");
    if (out_interval <= 0) return set_error(NB_ERR_INVALID, "out_interval must be >= 1");
    const size_t sb = state_bytes(c);
    if (sb && (!pos || !vel)) return set_error(NB_ERR_INVALID, "pos/vel is NULL");
    if (sb && loops >= out_interval && !outbuffer)
        return set_error(NB_ERR_INVALID, "outbuffer is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const auto t_start = std::chrono::steady_clock::now();
    const bool pinned = c->p.memtype == NB_MEM_PINNED && sb > 0;
    if (pinned && !c->stage_pos) {
        NB_CUDA(cudaMallocHost(&c->stage_pos, sb));
        NB_CUDA(cudaMallocHost(&c->stage_vel, sb));
        NB_CUDA(cudaMallocHost(&c->stage_out, sb));
    }
    cudaEvent_t ev[4];
    for (int k = 0; k < 4; ++k) NB_CUDA(cudaEventCreate(&ev[k]));
    struct Guard {
        cudaEvent_t *e;
        ~Guard()
        {
            for (int k = 0; k < 4; ++k) cudaEventDestroy(e[k]);
        }
    } guard{ev};

    // copy in (GpuData::sync, body_task_sgpu.cu:63-68)
    double copyin = 0, kernel = 0, copyout = 0;
    float ms = 0;
    NB_CUDA(cudaEventRecord(ev[0], s));
    if (pinned) {
        std::memcpy(c->stage_pos, pos, sb);
        std::memcpy(c->stage_vel, vel, sb);
    }
    int st = nb_set_state(c, pinned ? c->stage_pos : pos, pinned ? c->stage_vel : vel,
                          NB_DEVICE, stream);
    if (st) return st;
    NB_CUDA(cudaEventRecord(ev[1], s));
    NB_CUDA(cudaEventSynchronize(ev[1]));
    NB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    copyin = ms * 1e-3;

    // step loop with frame copy-out every out_interval steps
    int done = 0;
    while (done < loops) {
        const int next_frame = (done / out_interval + 1) * out_interval;
        const int upto = next_frame < loops ? next_frame : loops;
        NB_CUDA(cudaEventRecord(ev[0], s));
        if ((st = nb_step(c, upto - done, stream))) return st;
        NB_CUDA(cudaEventRecord(ev[1], s));
        done = upto;
        if (done % out_interval == 0 && sb) {
            char *dst = (char *)outbuffer + (size_t)(done / out_interval - 1) * sb;
            NB_CUDA(cudaMemcpyAsync(pinned ? c->stage_out : dst, c->pos[c->cur], sb,
                                    cudaMemcpyDefault, s));
            NB_CUDA(cudaEventRecord(ev[2], s));
            NB_CUDA(cudaEventSynchronize(ev[2]));
            if (pinned) std::memcpy(dst, c->stage_out, sb);
            NB_CUDA(cudaEventElapsedTime(&ms, ev[1], ev[2]));
            copyout += ms * 1e-3;
        } else {
            NB_CUDA(cudaEventSynchronize(ev[1]));
        }
        NB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        kernel += ms * 1e-3;
    }
    NB_CUDA(cudaStreamSynchronize(s));
    const double total =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    if (timings) {
        timings[0] = total;
        timings[1] = kernel;
        timings[2] = copyin;
        timings[3] = copyout;
    }
    return NB_OK;
}

int nb_probe_fma_peak(int iters, int packed, double *flops, float *ms, void *stream)
{
    return nb::probe_fma(iters, packed, flops, ms, (cudaStream_t)stream);
}

}  // extern "C"
