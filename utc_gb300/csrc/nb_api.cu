// nb_api.cu -- the C ABI (include/nbody_gb300.h): contexts, state transfer,
// stepping and the task-style host run.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "nb_internal.cuh"

namespace nb {

static thread_local std::string g_last_error;

std::shared_mutex &capture_gate()
{
    static std::shared_mutex gate;
    return gate;
}

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

int create_recompute_stream(cudaStream_t *stream, cudaEvent_t ev_rec[2], cudaEvent_t *ev_go)
{
    cudaStream_t rs = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaError_t e = cudaStreamCreateWithFlags(&rs, cudaStreamNonBlocking);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (rs) cudaStreamDestroy(rs);
        return cuda_error(e, "adjoint recompute stream setup");
    }
    ev_rec[0] = ev[0];
    ev_rec[1] = ev[1];
    *ev_go = ev[2];
    *stream = rs;
    return NB_OK;
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
    std::vector<cudaEvent_t> events;  // pool for nb_step_timed and nb_run_host
    // frame output of nb_run_host: device snapshots copied to pinned staging
    // on their own stream while the next steps run
    cudaStream_t copy_stream = nullptr;
    void *snap[2] = {nullptr, nullptr};
    void *stage[2] = {nullptr, nullptr};
    cudaEvent_t ev_snap[2] = {nullptr, nullptr}, ev_c0[2] = {nullptr, nullptr},
                ev_c1[2] = {nullptr, nullptr};
    // NB_F32_COMP state (pos[0] holds the double4 positions, vel the FP32
    // velocity high parts)
    float4 *pos32 = nullptr;
    float4 *vel_lo = nullptr;
    double4 *tmpA = nullptr;  // host-format staging for set/get
    double4 *tmpB = nullptr;
    // energy pass: its own launch plan, per-body output and FP64 partials
    nb::SkPlan eplan;
    void *acc_tmp = nullptr;
    double *e_blocks = nullptr;
    double *e_out = nullptr;
    double4 *e_pos64 = nullptr;  // NB_F32 exact contexts: positions widened for the energy pass
    // symmetric algorithm: plan and its two partial arrays
    nb::SymPlan splan;
    float4 *sym_t = nullptr, *sym_s = nullptr;
    // banded plans: the per-body sums the fold kernel builds band by band
    // (float4, or double4 for FP64 state)
    void *sym_acc = nullptr;
    // float-float path for FP64 state: scaled three-float positions (3 n
    // float4) and the per-step scale record
    float4 *ff_split = nullptr;
    unsigned long long *ff_range = nullptr;
    // nb_step on a capturable stream replays a CUDA graph of kGraphSteps
    // steps (one per starting ping-pong buffer): small systems are otherwise
    // bound by the per-kernel launch cost
    cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
    // nb_step on the legacy default stream, which cannot be captured: the
    // steps run on this non-blocking stream instead, after an event recorded
    // on the caller's stream, and the caller's stream waits for a second one
    cudaStream_t side_stream = nullptr;
    cudaEvent_t side_ev[2] = {nullptr, nullptr};
    // shard of a multi-GPU target partition (nb_create_shard): this context
    // updates targets [shard_lo, shard_hi) of all n bodies; shard_count 1 is
    // a whole system
    int shard_rank = 0, shard_count = 1, shard_lo = 0, shard_hi = 0;
    // fixed-point source side: eps2 changed since its scale was recorded
    bool fx_dirty = false;
    // adjoint: checkpoints of the last nb_adj_forward and reverse-pass buffers
    struct Adj {
        int steps = 0, every = 0, nckpt = 0;
        int cap_ckpt = 0, cap_seg = 0;
        float4 *ckpt_pos = nullptr, *ckpt_vel = nullptr;  // [nckpt][n]
        float4 *seg_pos = nullptr;                        // [every + 1][n]
        float4 *seg_acc = nullptr;                        // [every][n]
        float4 *vel_tmp = nullptr, *lx = nullptr, *lv = nullptr, *gbuf = nullptr;
        float *gm = nullptr;
        float4 *partial = nullptr;
        nb::SkPlan plan;
        // symmetric contexts: symmetric VJP with its own layout
        bool sym = false;
        nb::SymPlan splan;
        float4 *sym_t = nullptr, *sym_s = nullptr;
        bool ready = false;
        // number of the recorded forward pass (nb_adj_forward counts from 1);
        // nb_adj_backward refuses any other
        unsigned long long generation = 0;
        // the forward pass left the last segment's states in seg_pos/seg_acc
        bool live_last = false;
        // second segment buffer: segment s-1 is recomputed on rstream while
        // the reverse pass runs through segment s on the caller's stream
        float4 *seg_pos2 = nullptr, *seg_acc2 = nullptr, *vel_tmp2 = nullptr;
        cudaStream_t rstream = nullptr;
        cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_go = nullptr;
    } adj;
};

using nb::set_error;

static size_t state_bytes(const nb_ctx *c) { return (size_t)c->p.n * 4 * c->elem; }

static int validate(const nb_params *p)
{
    if (!p) return set_error(NB_ERR_INVALID, "params is NULL");
    if (p->n < 0 || p->n > NB_MAX_BODIES)
        return set_error(NB_ERR_INVALID, "n must be in [0, 2^30]");
    if (p->precision != NB_F32 && p->precision != NB_F64 && p->precision != NB_F32_COMP)
        return set_error(NB_ERR_INVALID, "unknown precision");
    if (p->algo != NB_ALGO_FAST && p->algo != NB_ALGO_EXACT && p->algo != NB_ALGO_SYM &&
        p->algo != NB_ALGO_SYM_FP64)
        return set_error(NB_ERR_INVALID, "unknown algo");
    if (p->algo == NB_ALGO_SYM_FP64 && p->precision != NB_F64)
        return set_error(NB_ERR_UNSUPPORTED, "NB_ALGO_SYM_FP64 is for NB_F64 state");
    if (p->kick != NB_KICK_REFERENCE && p->kick != NB_KICK_PHYSICAL)
        return set_error(NB_ERR_INVALID, "unknown kick mode");
    if (p->memtype < NB_MEM_PAGEABLE || p->memtype > NB_MEM_UNIFIED)
        return set_error(NB_ERR_INVALID, "unknown memtype");
    if (p->source_side < NB_SOURCE_AUTO || p->source_side > NB_SOURCE_FIXED)
        return set_error(NB_ERR_INVALID, "unknown source_side");
    if (p->bands < 0 || p->bands == 1 || p->bands > nb::SymPlan::kMaxBands)
        return set_error(NB_ERR_INVALID, "bands is 0 (automatic) or 2..512");
    if (!std::isfinite(p->eps2) || !std::isfinite(p->damping) || !std::isfinite(p->dt) ||
        !std::isfinite(p->G))
        return set_error(NB_ERR_INVALID, "eps2, damping, dt and G must be finite");
    if (p->precision == NB_F64 && p->algo == NB_ALGO_FAST)
        return set_error(NB_ERR_UNSUPPORTED, "NB_F64 runs the exact or symmetric algorithm");
    if (p->precision == NB_F32_COMP && p->algo == NB_ALGO_EXACT)
        return set_error(NB_ERR_UNSUPPORTED,
                         "NB_F32_COMP runs the fast or symmetric (compensated) algorithms only");
    if (p->precision == NB_F32_COMP && p->memtype == NB_MEM_UNIFIED)
        return set_error(NB_ERR_UNSUPPORTED, "NB_F32_COMP keeps its state in device memory");
    return NB_OK;
}

static void free_ctx(nb_ctx *c)
{
    if (!c) return;
    for (auto &g : c->step_graph)
        if (g) nb::graph_exec_destroy(g);
    nb::dfree(c->pos[0]);
    nb::dfree(c->pos[1]);
    nb::dfree(c->vel);
    nb::dfree(c->partial);
    nb::hfree(c->stage_pos);
    nb::hfree(c->stage_vel);
    nb::hfree(c->stage_out);
    for (cudaEvent_t e : c->events) cudaEventDestroy(e);
    nb::dfree(c->pos32);
    nb::dfree(c->vel_lo);
    nb::dfree(c->tmpA);
    nb::dfree(c->tmpB);
    nb::dfree(c->acc_tmp);
    nb::dfree(c->e_blocks);
    nb::dfree(c->e_out);
    nb::dfree(c->e_pos64);
    nb::dfree(c->adj.ckpt_pos);
    nb::dfree(c->adj.ckpt_vel);
    nb::dfree(c->adj.seg_pos);
    nb::dfree(c->adj.seg_acc);
    nb::dfree(c->adj.vel_tmp);
    nb::dfree(c->adj.lx);
    nb::dfree(c->adj.lv);
    nb::dfree(c->adj.gbuf);
    nb::dfree(c->adj.gm);
    nb::dfree(c->adj.partial);
    nb::dfree(c->adj.sym_t);
    nb::dfree(c->adj.sym_s);
    nb::dfree(c->adj.seg_pos2);
    nb::dfree(c->adj.seg_acc2);
    nb::dfree(c->adj.vel_tmp2);
    if (c->adj.rstream) cudaStreamDestroy(c->adj.rstream);
    for (auto &e : c->adj.ev_rec)
        if (e) cudaEventDestroy(e);
    if (c->adj.ev_go) cudaEventDestroy(c->adj.ev_go);
    nb::dfree(c->sym_t);
    nb::dfree(c->sym_s);
    nb::dfree(c->sym_acc);
    nb::dfree(c->ff_split);
    nb::dfree(c->ff_range);
    for (int k = 0; k < 2; ++k) {
        nb::dfree(c->snap[k]);
        nb::hfree(c->stage[k]);
        if (c->ev_snap[k]) cudaEventDestroy(c->ev_snap[k]);
        if (c->ev_c0[k]) cudaEventDestroy(c->ev_c0[k]);
        if (c->ev_c1[k]) cudaEventDestroy(c->ev_c1[k]);
    }
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (cudaEvent_t e : c->side_ev)
        if (e) cudaEventDestroy(e);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    delete c;
}

static int dalloc(nb_ctx *c, void **p, size_t bytes)
{
    if (bytes == 0) {
        *p = nullptr;
        return NB_OK;
    }
    cudaError_t e = c->p.memtype == NB_MEM_UNIFIED ? nb::dmalloc_managed(p, bytes)
                                                   : nb::dmalloc(p, bytes);
    if (e != cudaSuccess) return nb::cuda_error(e, "state allocation");
    return NB_OK;
}

static bool uses_sym(const nb_ctx *c) { return c->p.precision == NB_F32 && c->p.algo == NB_ALGO_SYM; }
// compensated context stepping with the compensated symmetric kernel
static bool comp_sym(const nb_ctx *c) { return c->p.precision == NB_F32_COMP && c->p.algo == NB_ALGO_SYM; }
// FP64 context stepping with the FP64 symmetric kernel
static bool f64_sym(const nb_ctx *c)
{
    return c->p.precision == NB_F64 && (c->p.algo == NB_ALGO_SYM || c->p.algo == NB_ALGO_SYM_FP64);
}
// FP64 state stepped by the float-float symmetric kernel (NB_ALGO_SYM)
static bool ff_sym(const nb_ctx *c) { return c->p.precision == NB_F64 && c->p.algo == NB_ALGO_SYM; }
// the directed stream-K plan (c->plan) also serves the symmetric context's
// energy pass and adjoint
static bool uses_fast(const nb_ctx *c)
{
    return c->p.precision == NB_F32 && (c->p.algo == NB_ALGO_FAST || c->p.algo == NB_ALGO_SYM);
}
static bool is_comp(const nb_ctx *c) { return c->p.precision == NB_F32_COMP; }

static int dev_alloc(void **p, size_t bytes, const char *what)
{
    *p = nullptr;
    if (!bytes) return NB_OK;
    cudaError_t e = nb::dmalloc(p, bytes);
    if (e != cudaSuccess) return nb::cuda_error(e, what);
    return NB_OK;
}

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
    c->elem = (p->precision == NB_F64 || p->precision == NB_F32_COMP) ? 8 : 4;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) {
        delete c;
        return nb::cuda_error(e, "cudaGetDevice");
    }
    const size_t sb = state_bytes(c);
    const size_t n = (size_t)p->n;
    if (is_comp(c)) {
        if ((st = dev_alloc(&c->pos[0], n * sizeof(double4), "state allocation")) ||
            (st = dev_alloc(&c->vel, n * sizeof(float4), "state allocation")) ||
            (st = dev_alloc((void **)&c->pos32, n * sizeof(float4), "state allocation")) ||
            (st = dev_alloc((void **)&c->vel_lo, n * sizeof(float4), "state allocation")) ||
            (st = dev_alloc((void **)&c->tmpA, n * sizeof(double4), "staging allocation")) ||
            (st = dev_alloc((void **)&c->tmpB, n * sizeof(double4), "staging allocation"))) {
            free_ctx(c);
            return st;
        }
    } else if ((st = dalloc(c, &c->pos[0], sb)) || (st = dalloc(c, &c->pos[1], sb)) ||
               (st = dalloc(c, &c->vel, sb))) {
        free_ctx(c);
        return st;
    }
    if (p->precision == NB_F64 &&
        ((st = dev_alloc(&c->acc_tmp, n * sizeof(double4), "energy scratch allocation")) ||
         (st = dev_alloc((void **)&c->e_blocks, (size_t)(nb::energy_blocks(p->n) + 1) * 5 * sizeof(double),
                         "energy scratch allocation")) ||
         (st = dev_alloc((void **)&c->e_out, 8 * sizeof(double), "energy scratch allocation")))) {
        free_ctx(c);
        return st;
    }
    if (f64_sym(c) &&
        ((st = ff_sym(c) ? nb::symff_plan(p->n, p->block ? p->block / 32 : 0, p->bpt, c->device, &c->splan,
                                          p->bands)
                         : nb::sym64_plan(p->n, p->block ? p->block / 32 : 0, p->bpt, c->device, &c->splan)) ||
         (ff_sym(c) && (st = dev_alloc((void **)&c->ff_split, 3 * n * sizeof(float4), "split positions allocation"))) ||
         (ff_sym(c) && (st = dev_alloc((void **)&c->ff_range, 2 * sizeof(unsigned long long), "scale record allocation"))) ||
         (st = dev_alloc((void **)&c->sym_t, (size_t)c->splan.slots * c->splan.rb * sizeof(double4),
                         "symmetric scratch allocation")) ||
         (st = dev_alloc((void **)&c->sym_s, (size_t)c->splan.spart_size * sizeof(double4),
                         "symmetric source-side array (about N^2/(2 rb) entries; NB_ALGO_EXACT needs none)")) ||
         (c->splan.nbands > 1 &&
          (st = dev_alloc(&c->sym_acc, n * sizeof(double4), "per-body sums of the banded source side"))))) {
        free_ctx(c);
        return st;
    }
    if (uses_fast(c) || is_comp(c)) {
        const int flags = is_comp(c) ? nb::SK_COMP : 0;
        const bool own_shape = !(uses_sym(c) || comp_sym(c));
        const int block = (own_shape && p->block) ? p->block : (is_comp(c) ? 256 : 0);
        const int bpt = (own_shape && p->bpt) ? p->bpt : (is_comp(c) ? 4 : 0);
        st = nb::fast_plan(p->n, block, bpt, p->ctas_per_sm, c->device, &c->plan, flags);
        if (!st)
            st = nb::fast_plan(p->n, 256, is_comp(c) ? 4 : 8, 0, c->device, &c->eplan,
                               flags | nb::SK_PHI);
        if (st) {
            free_ctx(c);
            return st;
        }
        const size_t mult = is_comp(c) ? 2 : 1;
        size_t pb = mult * (size_t)c->plan.slots * c->plan.tbsize * sizeof(float4);
        const size_t pe = mult * (size_t)c->eplan.slots * c->eplan.tbsize * sizeof(float4);
        if (pe > pb) pb = pe;
        if (uses_sym(c) || comp_sym(c)) {
            const size_t halves = comp_sym(c) ? 2 : 1;  // compensated: hi and lo blocks
            if ((st = nb::sym_plan(p->n, p->block ? p->block / 32 : 0, p->bpt, c->device, &c->splan,
                                   comp_sym(c) ? 1 : 0, comp_sym(c) ? NB_SOURCE_AUTO : p->source_side,
                                   p->bands)) ||
                (st = dev_alloc((void **)&c->sym_t,
                                halves * c->splan.slots * c->splan.rb * sizeof(float4),
                                "symmetric scratch allocation")) ||
                (c->splan.nbands > 1 &&
                 (st = dev_alloc(&c->sym_acc, halves * n * sizeof(float4),
                                 "per-body sums of the banded source side"))) ||
                (st = dev_alloc((void **)&c->sym_s, halves * c->splan.spart_size * sizeof(float4),
                                c->splan.fixed ? "symmetric source-side accumulators (48 B per body)"
                                               : "symmetric source-side array (about N^2/(2 rb) entries; "
                                                 "NB_SOURCE_FIXED or NB_ALGO_FAST need O(N) scratch)"))) {
                free_ctx(c);
                return st;
            }
        }
        if ((st = dev_alloc((void **)&c->partial, pb, "partial-sum scratch allocation")) ||
            (st = dev_alloc(&c->acc_tmp, n * sizeof(double4), "energy scratch allocation")) ||
            (st = dev_alloc((void **)&c->e_blocks,
                            (size_t)(nb::energy_blocks(p->n) + 1) * 5 * sizeof(double),
                            "energy scratch allocation")) ||
            (st = dev_alloc((void **)&c->e_out, 8 * sizeof(double), "energy scratch allocation"))) {
            free_ctx(c);
            return st;
        }
    }
    c->shard_lo = 0;
    c->shard_hi = p->n;
    *out = c;
    return NB_OK;
}

int nb_create_shard(const nb_params *p, int rank, int nranks, nb_ctx **out)
{
    if (!out) return set_error(NB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!p) return set_error(NB_ERR_INVALID, "params is NULL");
    if (nranks < 1 || rank < 0 || rank >= nranks)
        return set_error(NB_ERR_INVALID, "nb_create_shard: rank must be in [0, nranks), nranks >= 1");
    const bool fast = p->precision == NB_F32 && p->algo == NB_ALGO_FAST;
    const bool exact = (p->precision == NB_F32 || p->precision == NB_F64) && p->algo == NB_ALGO_EXACT;
    if (!fast && !exact)
        return set_error(NB_ERR_UNSUPPORTED, "nb_create_shard: shards run the directed kernel (NB_F32, "
                                             "NB_ALGO_FAST) or the reference-exact one (NB_ALGO_EXACT)");
    int st = nb_create(p, out);
    if (st) return st;
    nb_ctx *c = *out;
    c->shard_rank = rank;
    c->shard_count = nranks;
    if (fast) {
        // whole target blocks per shard, so that the shard's CTAs write the
        // partial slots the single-GPU launch writes for those targets
        if ((st = nb::fast_shard(&c->plan, rank, nranks))) {
            free_ctx(c);
            *out = nullptr;
            return st;
        }
        c->shard_lo = c->plan.i_lo;
        c->shard_hi = c->plan.i_hi;
    } else {
        // the reference's split (body_task_mgpu.cu:41-49): n / nranks bodies
        // each, one more for the first n % nranks ranks
        const int q = p->n / nranks, r = p->n % nranks;
        c->shard_lo = rank < r ? rank * (q + 1) : rank * q + r;
        c->shard_hi = c->shard_lo + q + (rank < r ? 1 : 0);
    }
    return NB_OK;
}

int nb_shard_info(nb_ctx *c, int *info4)
{
    if (!c || !info4) return set_error(NB_ERR_INVALID, "ctx/info is NULL");
    info4[0] = c->shard_lo;
    info4[1] = c->shard_hi - c->shard_lo;
    info4[2] = c->shard_rank;
    info4[3] = c->shard_count;
    return NB_OK;
}

// Calls that need every body's fresh state, refused on a shard of a
// multi-rank partition (its other ranks' bodies are stale between steps).
static int refuse_shard(const nb_ctx *c, const char *what)
{
    if (c && c->shard_count > 1)
        return set_error(NB_ERR_UNSUPPORTED, std::string(what) +
                                                 ": not available on a shard of a multi-rank partition");
    return NB_OK;
}

// A fixed-point source side whose eps2 changed gets its scale rewritten on
// the stream of the next stepping call, before that call's force launches
// (and before any graph capture, which then does not contain it).
static int fx_refresh(nb_ctx *c, cudaStream_t s)
{
    if (!c->fx_dirty || !c->has_state) return NB_OK;
    int st = nb::sym_fx_rescale(c->splan, c->sym_s, (float)c->p.eps2, s);
    if (!st) c->fx_dirty = false;
    return st;
}

int nb_destroy(nb_ctx *c)
{
    if (!c) return NB_OK;
    // work queued on the caller's streams may still use the buffers.  A
    // device that cannot be synchronised because a thread outside the
    // library is capturing a graph keeps the context: freeing it could pull
    // memory from under that work
    const cudaError_t e = nb::device_sync();
    if (nb::is_capture_error(e)) {
        (void)cudaGetLastError();
        return nb::cuda_error(e, "nb_destroy: the device cannot be synchronised while another thread captures "
                                 "a graph; the context is kept, call again after the capture");
    }
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
    if (sb && is_comp(c)) {
        NB_CUDA(cudaMemcpyAsync(c->tmpA, pos, sb, cudaMemcpyDefault, s));
        NB_CUDA(cudaMemcpyAsync(c->tmpB, vel, sb, cudaMemcpyDefault, s));
        int st = nb::comp_split(c->tmpA, c->tmpB, (double4 *)c->pos[0], c->pos32, (float4 *)c->vel,
                                c->vel_lo, c->p.n, s);
        if (st) return st;
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    } else if (sb) {
        NB_CUDA(cudaMemcpyAsync(c->pos[0], pos, sb, cudaMemcpyDefault, s));
        NB_CUDA(cudaMemcpyAsync(c->vel, vel, sb, cudaMemcpyDefault, s));
        // symmetric contexts: zeroed source-side accumulators and the sum of
        // |m| their scale comes from
        if (uses_sym(c)) {
            int st = nb::sym_fx_prepare(c->splan, (const float4 *)c->pos[0], c->sym_s, (float)c->p.eps2, s);
            if (!st) c->fx_dirty = false;
            if (st) return st;
        }
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
    if (sb && is_comp(c)) {
        int st = nb::comp_join((const double4 *)c->pos[0], (const float4 *)c->vel, c->vel_lo,
                               c->tmpA, c->tmpB, c->p.n, s);
        if (st) return st;
        if (pos) NB_CUDA(cudaMemcpyAsync(pos, c->tmpA, sb, cudaMemcpyDefault, s));
        if (vel) NB_CUDA(cudaMemcpyAsync(vel, c->tmpB, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    } else if (sb) {
        if (pos) NB_CUDA(cudaMemcpyAsync(pos, c->pos[c->cur], sb, cudaMemcpyDefault, s));
        if (vel) NB_CUDA(cudaMemcpyAsync(vel, c->vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    return NB_OK;
}

int nb_state_ptrs(nb_ctx *c, void **pos_dev, void **vel_dev)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (pos_dev) *pos_dev = is_comp(c) ? c->pos[0] : c->pos[c->cur];
    if (vel_dev) *vel_dev = c->vel;
    return NB_OK;
}

// One step; when ev != nullptr, records ev[0] before the first kernel,
// ev[1] between the force and the integrate kernel and ev[2] at the end.
// acc_keep (symmetric FP32 contexts only): also the step's bare
// accelerations, read from the same force launch before the step consumes it.
static int step_once(nb_ctx *c, cudaStream_t s, void *acc_out, cudaEvent_t *ev = nullptr,
                     float4 *acc_keep = nullptr)
{
    const nb_params &p = c->p;
    void *po = c->pos[c->cur], *pn = c->pos[c->cur ^ 1];
    int st;
    if (ev) NB_CUDA(cudaEventRecord(ev[0], s));
    if (comp_sym(c)) {
        st = nb::sym_force(c->splan, c->pos32, (float)p.eps2, c->sym_t, c->sym_s, (float4 *)c->sym_acc, s);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[1], s));
        if (!st)
            st = nb::sym_comp_integrate(c->splan, c->sym_t, c->sym_s, (double4 *)c->pos[0], c->pos32,
                                        (float4 *)c->vel, c->vel_lo, (float)p.damping, (float)p.dt,
                                        p.dt, p.kick, (float)p.G, (double4 *)acc_out, s, (const float4 *)c->sym_acc);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[2], s));
        return st;  // positions are updated in place: no ping-pong
    }
    if (is_comp(c)) {
        st = nb::fast_force(c->plan, c->pos32, (float)p.eps2, c->partial, s, nb::SK_COMP);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[1], s));
        if (!st && acc_out)
            st = nb::fast_reduce(c->plan, c->partial, 1, c->pos32, (float)p.eps2, nullptr,
                                 (double4 *)acc_out, s);
        else if (!st)
            st = nb::comp_integrate(c->plan, c->partial, (double4 *)c->pos[0], c->pos32,
                                    (float4 *)c->vel, c->vel_lo, (float)p.damping, (float)p.dt,
                                    p.dt, p.kick, (float)p.G, s);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[2], s));
        return st;  // positions are updated in place: no ping-pong
    }
    if (f64_sym(c)) {
        st = ff_sym(c) ? nb::symff_force(c->splan, (const double4 *)po, p.eps2, c->ff_split, c->ff_range,
                                         (double4 *)c->sym_t, (double4 *)c->sym_s, (double4 *)c->sym_acc, s)
                       : nb::sym64_force(c->splan, (const double4 *)po, p.eps2, (double4 *)c->sym_t,
                                         (double4 *)c->sym_s, s);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[1], s));
        if (!st)
            st = nb::sym64_integrate(c->splan, (const double4 *)po, (double4 *)pn, (double4 *)c->vel,
                                     (const double4 *)c->sym_t, (const double4 *)c->sym_s, p.damping, p.dt,
                                     p.kick, p.G, (double4 *)acc_out, s, ff_sym(c) ? c->ff_range : nullptr,
                                     (const double4 *)c->sym_acc);
    } else if (p.precision == NB_F64) {
        st = nb::exact_step_f64(p.n, c->shard_lo, c->shard_hi, (const double4 *)po, (double4 *)pn,
                                (double4 *)c->vel, p.eps2,
                                p.damping, p.dt, p.kick, p.G, (double4 *)acc_out, p.block, s);
    } else if (p.algo == NB_ALGO_EXACT) {
        st = nb::exact_step_f32(p.n, c->shard_lo, c->shard_hi, (const float4 *)po, (float4 *)pn,
                                (float4 *)c->vel,
                                (float)p.eps2, (float)p.damping, (float)p.dt, p.kick, (float)p.G,
                                (float4 *)acc_out, p.block, s);
    } else if (p.algo == NB_ALGO_SYM) {
        st = nb::sym_force(c->splan, (const float4 *)po, (float)p.eps2, c->sym_t, c->sym_s,
                           (float4 *)c->sym_acc, s);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[1], s));
        if (!st && acc_keep)
            st = nb::sym_integrate(c->splan, (const float4 *)po, nullptr, nullptr, c->sym_t, c->sym_s,
                                   (const float4 *)c->sym_acc,
                                   (float)p.damping, (float)p.dt, p.kick, (float)p.G, acc_keep,
                                   s, 0);
        if (!st)
            st = nb::sym_integrate(c->splan, (const float4 *)po, (float4 *)pn, (float4 *)c->vel,
                                   c->sym_t, c->sym_s, (const float4 *)c->sym_acc, (float)p.damping,
                                   (float)p.dt, p.kick, (float)p.G, (float4 *)acc_out, s);
    } else {
        st = nb::fast_force(c->plan, (const float4 *)po, (float)p.eps2, c->partial, s);
        if (!st && ev) NB_CUDA(cudaEventRecord(ev[1], s));
        if (!st)
            st = nb::fast_integrate(c->plan, (const float4 *)po, (float4 *)pn, (float4 *)c->vel,
                                    c->partial, (float)p.damping, (float)p.dt, p.kick, (float)p.G,
                                    (float4 *)acc_out, s);
    }
    if (!st && ev) {
        if (!uses_fast(c) && !f64_sym(c)) NB_CUDA(cudaEventRecord(ev[1], s));  // exact: one fused kernel
        NB_CUDA(cudaEventRecord(ev[2], s));
    }
    if (!st && !acc_out) c->cur ^= 1;
    return st;
}

}  // extern "C"

// Steps per replayed graph: even, so that the ping-pong buffers are back in
// place after a replay and the graph can be replayed again.
constexpr int kGraphSteps = 16;

// Capture kGraphSteps steps from the current buffer into a graph.  The
// kernels' arguments (buffers, plans, parameters) stay fixed until
// nb_set_params, which destroys the captured graphs.  *out stays null when
// the capture does not take: a device-wide call made by code outside the
// library in another thread invalidates a capture without any fault of the
// steps.  Nothing captured has run and c->cur is as before, so the caller
// launches the steps one by one instead, where an error of the steps
// themselves then shows.
static void capture_step_graph(nb_ctx *c, cudaStream_t s, cudaGraphExec_t *out)
{
    *out = nullptr;
    const int cur0 = c->cur;
    cudaGraph_t g = nullptr;
    {
        std::shared_lock<std::shared_mutex> gate(nb::capture_gate());
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            int st = NB_OK;
            for (int i = 0; i < kGraphSteps && !st; ++i) st = step_once(c, s, nullptr);
            if (cudaStreamEndCapture(s, &g) != cudaSuccess || st) {
                if (g) cudaGraphDestroy(g);
                g = nullptr;
            }
        }
    }
    c->cur = cur0;
    if (g) {
        if (nb::graph_instantiate(out, g) != cudaSuccess) *out = nullptr;
        cudaGraphDestroy(g);
    }
    (void)cudaGetLastError();  // a capture that did not take leaves its error behind
}

// The side stream of nb_step and its two events, made on first use; all or
// nothing, so that a failed call leaves nothing half set up.
static int make_side_stream(nb_ctx *c)
{
    cudaStream_t ss = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaStreamCreateWithFlags(&ss, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (ss) cudaStreamDestroy(ss);
        return nb::cuda_error(e, "nb_step: side stream setup");
    }
    c->side_ev[0] = ev[0];
    c->side_ev[1] = ev[1];
    c->side_stream = ss;
    return NB_OK;
}

extern "C" {

int nb_step(nb_ctx *c, int steps, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (c->shard_count > 1 && steps > 1)
        return set_error(NB_ERR_INVALID, "nb_step: a shard steps once per call (the other shards' "
                                         "positions are exchanged between steps)");
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if ((st = fx_refresh(c, s))) return st;
    const bool legacy = s == nullptr || s == cudaStreamLegacy;
    if (legacy && c->p.n > 0 && steps >= 2 * kGraphSteps) {
        // the legacy default stream cannot be captured: enough steps for a
        // graph run on the side stream, ordered after the caller's earlier
        // work, and the caller's later work waits for them
        if (!c->side_stream && (st = make_side_stream(c))) return st;
        NB_CUDA(cudaEventRecord(c->side_ev[0], s));
        NB_CUDA(cudaStreamWaitEvent(c->side_stream, c->side_ev[0], 0));
        st = nb_step(c, steps, (void *)c->side_stream);
        // joined also after a failure, for whatever the steps launched
        cudaError_t e = cudaEventRecord(c->side_ev[1], c->side_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->side_ev[1], 0);
        if (st) return st;
        if (e != cudaSuccess) return nb::cuda_error(e, "nb_step: ordering the caller's stream after the steps");
        return NB_OK;
    }
    // launch step by step on the legacy default stream (a few steps), and
    // also on a stream the caller is capturing into a graph of its own (the
    // launches then go into the caller's graph)
    bool graphs = !legacy && c->p.n > 0;
    if (graphs) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        NB_CUDA(cudaStreamIsCapturing(s, &cs));
        graphs = cs == cudaStreamCaptureStatusNone;
    }
    if (graphs && steps >= 2 * kGraphSteps) {
        for (; steps >= kGraphSteps; steps -= kGraphSteps) {
            cudaGraphExec_t &g = c->step_graph[c->cur];
            if (!g) capture_step_graph(c, s, &g);
            if (!g) break;  // the capture did not take: the steps left go one by one
            NB_CUDA(cudaGraphLaunch(g, s));
        }
    }
    for (; steps > 0; --steps)
        if ((st = step_once(c, s, nullptr))) return st;
    return NB_OK;
}

int nb_set_params(nb_ctx *c, double eps2, double damping, double dt, double G)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!std::isfinite(eps2) || !std::isfinite(damping) || !std::isfinite(dt) || !std::isfinite(G))
        return set_error(NB_ERR_INVALID, "eps2, damping, dt and G must be finite");
    // captured graphs hold the old values as kernel arguments
    for (auto &g : c->step_graph)
        if (g) {
            nb::graph_exec_destroy(g);
            g = nullptr;
        }
    if (c->splan.fixed && eps2 != c->p.eps2) c->fx_dirty = true;  // rescaled before the next force launch
    c->p.eps2 = eps2;
    c->p.damping = damping;
    c->p.dt = dt;
    c->p.G = G;
    c->adj.ready = false;  // a recorded forward pass used the old values
    c->adj.live_last = false;
    return NB_OK;
}

int nb_step_timed(nb_ctx *c, int steps, float *ms_force, float *ms_integrate, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (c->shard_count > 1 && steps > 1)
        return set_error(NB_ERR_INVALID, "nb_step_timed: a shard steps once per call");
    if (!ms_force || !ms_integrate) return set_error(NB_ERR_INVALID, "ms outputs are NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    cudaStream_t s = (cudaStream_t)stream;
    if (int st = fx_refresh(c, s)) return st;
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
    if (int rs = refuse_shard(c, "nb_accel")) return rs;
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (c->p.n == 0) return NB_OK;
    if (!acc_dev) return set_error(NB_ERR_INVALID, "acc_dev is NULL");
    if (int st = fx_refresh(c, (cudaStream_t)stream)) return st;
    return step_once(c, (cudaStream_t)stream, acc_dev);
}

int nb_energy(nb_ctx *c, double *out5, void *accphi_dev, void *stream)
{
    if (int rs = refuse_shard(c, "nb_energy")) return rs;
    if (!c || !out5) return set_error(NB_ERR_INVALID, "ctx/out is NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (!(c->p.eps2 > 0.0)) return set_error(NB_ERR_INVALID, "nb_energy needs eps2 > 0");
    cudaStream_t s = (cudaStream_t)stream;
    const nb_params &p = c->p;
    int st;
    const bool exact32 = p.precision == NB_F32 && p.algo == NB_ALGO_EXACT;
    if (exact32 && p.n == 0) {
        for (int k = 0; k < 5; ++k) out5[k] = 0.0;
        return NB_OK;
    }
    if (exact32 && !c->e_pos64) {
        // first energy call of a reference-exact float context: its scratch,
        // all or nothing
        void *m[4] = {};
        const size_t bytes[4] = {(size_t)p.n * sizeof(double4), (size_t)p.n * sizeof(double4),
                                 (size_t)(nb::energy_blocks(p.n) + 1) * 5 * sizeof(double), 8 * sizeof(double)};
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = nb::dmalloc(&m[k], bytes[k]);
        if (e != cudaSuccess) {
            for (void *q : m) nb::dfree(q);
            return nb::cuda_error(e, "energy scratch allocation");
        }
        c->acc_tmp = m[1];
        c->e_blocks = (double *)m[2];
        c->e_out = (double *)m[3];
        c->e_pos64 = (double4 *)m[0];
    }
    if (exact32) {
        // FP64 potential pass on the float positions widened to double
        st = nb::widen_f32(p.n, (const float4 *)c->pos[c->cur], c->e_pos64, s);
        if (!st) st = nb::energy_phi_f64(p.n, c->e_pos64, p.eps2, (double4 *)c->acc_tmp, s);
        if (!st)
            st = nb::energy_reduce(p.n, nullptr, c->e_pos64, (const float4 *)c->vel, nullptr, nullptr,
                                   (const double4 *)c->acc_tmp, p.G, c->e_blocks, c->e_out, s);
        if (!st && accphi_dev) st = nb::narrow_f64(p.n, (const double4 *)c->acc_tmp, (float4 *)accphi_dev, s);
        if (st) return st;
        NB_CUDA(cudaMemcpyAsync(out5, c->e_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
        NB_CUDA(cudaStreamSynchronize(s));
        return NB_OK;
    }
    if (ff_sym(c)) {
        // the float-float symmetric pass with the potential, summed and
        // unscaled by the FP64 integrator into (acc, phi) per body
        const double4 *pos = (const double4 *)c->pos[c->cur];
        st = nb::symff_force(c->splan, pos, p.eps2, c->ff_split, c->ff_range, (double4 *)c->sym_t,
                             (double4 *)c->sym_s, (double4 *)c->sym_acc, s, 1);
        if (!st)
            st = nb::sym64_integrate(c->splan, pos, nullptr, nullptr, (const double4 *)c->sym_t,
                                     (const double4 *)c->sym_s, p.damping, p.dt, p.kick, p.G,
                                     (double4 *)c->acc_tmp, s, c->ff_range, (const double4 *)c->sym_acc);
        if (!st)
            st = nb::energy_reduce(p.n, nullptr, pos, nullptr, nullptr, nullptr,
                                   (const double4 *)c->acc_tmp, p.G, c->e_blocks, c->e_out, s,
                                   (const double4 *)c->vel);
    } else if (p.precision == NB_F64) {
        const double4 *pos = (const double4 *)c->pos[c->cur];
        st = nb::energy_phi_f64(p.n, pos, p.eps2, (double4 *)c->acc_tmp, s);
        if (!st)
            st = nb::energy_reduce(p.n, nullptr, pos, nullptr, nullptr, nullptr,
                                   (const double4 *)c->acc_tmp, p.G, c->e_blocks, c->e_out, s,
                                   (const double4 *)c->vel);
    } else if (is_comp(c)) {
        st = nb::fast_force(c->eplan, c->pos32, (float)p.eps2, c->partial, s, nb::SK_COMP | nb::SK_PHI);
        if (!st)
            st = nb::fast_reduce(c->eplan, c->partial, 1, c->pos32, (float)p.eps2, nullptr,
                                 (double4 *)c->acc_tmp, s);
        if (!st)
            st = nb::energy_reduce(p.n, c->pos32, (const double4 *)c->pos[0], (const float4 *)c->vel,
                                   c->vel_lo, nullptr, (const double4 *)c->acc_tmp, p.G,
                                   c->e_blocks, c->e_out, s);
    } else {
        const float4 *pos = (const float4 *)c->pos[c->cur];
        st = nb::fast_force(c->eplan, pos, (float)p.eps2, c->partial, s, nb::SK_PHI);
        if (!st)
            st = nb::fast_reduce(c->eplan, c->partial, 0, pos, (float)p.eps2, (float4 *)c->acc_tmp,
                                 nullptr, s);
        if (!st)
            st = nb::energy_reduce(p.n, pos, nullptr, (const float4 *)c->vel, nullptr,
                                   (const float4 *)c->acc_tmp, nullptr, p.G, c->e_blocks,
                                   c->e_out, s);
    }
    if (st) return st;
    if (accphi_dev && p.n)
        NB_CUDA(cudaMemcpyAsync(accphi_dev, c->acc_tmp,
                                (size_t)p.n * (c->elem == 8 ? sizeof(double4) : sizeof(float4)),
                                cudaMemcpyDeviceToDevice, s));
    NB_CUDA(cudaMemcpyAsync(out5, c->e_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
    NB_CUDA(cudaStreamSynchronize(s));
    return NB_OK;
}

// ---------------------------------------------------------------------------
// adjoint: forward with checkpoints, reverse pass with per-segment recompute
// ---------------------------------------------------------------------------
static int adj_reserve(nb_ctx *c, int nckpt, int every)
{
    const size_t n = (size_t)c->p.n;
    auto &A = c->adj;
    int st;
    if (!A.gm) {
        // gm is allocated last: without it, a retry after a failed
        // allocation starts from nothing
        nb::dfree(A.sym_t);
        nb::dfree(A.sym_s);
        nb::dfree(A.partial);
        nb::dfree(A.vel_tmp);
        nb::dfree(A.vel_tmp2);
        nb::dfree(A.lx);
        nb::dfree(A.lv);
        nb::dfree(A.gbuf);
        A.sym_t = A.sym_s = A.partial = A.vel_tmp = A.vel_tmp2 = A.lx = A.lv = A.gbuf = nullptr;
        A.sym = uses_sym(c);
        if (A.sym) {
            if ((st = nb::sym_vjp_plan(c->p.n, 0, 0, c->device, &A.splan)) ||
                (st = dev_alloc((void **)&A.sym_t, (size_t)A.splan.slots * A.splan.rb * sizeof(float4),
                                "adjoint allocation")) ||
                (st = dev_alloc((void **)&A.sym_s, (size_t)A.splan.spart_size * sizeof(float4),
                                "adjoint allocation")))
                return st;
        } else {
            if ((st = nb::adj_plan(c->p.n, 0, 0, c->device, &A.plan)) ||
                (st = dev_alloc((void **)&A.partial,
                                (size_t)A.plan.slots * A.plan.tbsize * sizeof(float4),
                                "adjoint allocation")))
                return st;
        }
        if ((st = dev_alloc((void **)&A.vel_tmp, n * sizeof(float4), "adjoint allocation")) ||
            (st = dev_alloc((void **)&A.vel_tmp2, n * sizeof(float4), "adjoint allocation")) ||
            (st = dev_alloc((void **)&A.lx, n * sizeof(float4), "adjoint allocation")) ||
            (st = dev_alloc((void **)&A.lv, n * sizeof(float4), "adjoint allocation")) ||
            (st = dev_alloc((void **)&A.gbuf, n * sizeof(float4), "adjoint allocation")) ||
            (st = dev_alloc((void **)&A.gm, n * sizeof(float), "adjoint allocation")))
            return st;
    }
    if (nckpt > A.cap_ckpt) {
        nb::dfree(A.ckpt_pos);
        nb::dfree(A.ckpt_vel);
        A.ckpt_pos = A.ckpt_vel = nullptr;
        A.cap_ckpt = 0;
        if ((st = dev_alloc((void **)&A.ckpt_pos, n * nckpt * sizeof(float4), "checkpoint allocation")) ||
            (st = dev_alloc((void **)&A.ckpt_vel, n * nckpt * sizeof(float4), "checkpoint allocation")))
            return st;
        A.cap_ckpt = nckpt;
    }
    if (every > A.cap_seg) {
        nb::dfree(A.seg_pos);
        nb::dfree(A.seg_acc);
        nb::dfree(A.seg_pos2);
        nb::dfree(A.seg_acc2);
        A.seg_pos = A.seg_acc = A.seg_pos2 = A.seg_acc2 = nullptr;
        A.cap_seg = 0;
        if ((st = dev_alloc((void **)&A.seg_pos, n * (every + 1) * sizeof(float4), "segment allocation")) ||
            (st = dev_alloc((void **)&A.seg_acc, n * every * sizeof(float4), "segment allocation")) ||
            (st = dev_alloc((void **)&A.seg_pos2, n * (every + 1) * sizeof(float4), "segment allocation")) ||
            (st = dev_alloc((void **)&A.seg_acc2, n * every * sizeof(float4), "segment allocation")))
            return st;
        A.cap_seg = every;
    }
    return NB_OK;
}

int nb_adj_forward(nb_ctx *c, int steps, int ckpt_every, void *stream, unsigned long long *generation)
{
    if (generation) *generation = 0;
    if (int rs = refuse_shard(c, "nb_adj_forward")) return rs;
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!uses_fast(c)) return set_error(NB_ERR_UNSUPPORTED, "the adjoint needs an NB_F32 fast context");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (steps < 1 || ckpt_every < 1) return set_error(NB_ERR_INVALID, "steps and ckpt_every must be >= 1");
    if (ckpt_every > steps) ckpt_every = steps;
    const int nckpt = (steps + ckpt_every - 1) / ckpt_every;
    int st = adj_reserve(c, nckpt, ckpt_every);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if ((st = fx_refresh(c, s))) return st;
    const size_t n = (size_t)c->p.n;
    auto &A = c->adj;
    const nb_params &p = c->p;
    // The last segment is the first one the reverse pass needs: its states
    // (and, for the reference kick, its accelerations) are kept in the
    // segment buffers as they are computed, so that segment is not
    // recomputed.  Same kernels, same bits as a recompute.
    const int t_last = (nckpt - 1) * ckpt_every;
    A.ready = false;
    A.live_last = false;
    for (int t = 0; t < steps; ++t) {
        if (t % ckpt_every == 0 && n) {
            const size_t k = (size_t)(t / ckpt_every) * n;
            NB_CUDA(cudaMemcpyAsync(A.ckpt_pos + k, c->pos[c->cur], n * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, s));
            NB_CUDA(cudaMemcpyAsync(A.ckpt_vel + k, c->vel, n * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, s));
        }
        const bool keep = n && t >= t_last;
        const size_t k = (size_t)(t - t_last);
        if (keep && t == t_last)
            NB_CUDA(cudaMemcpyAsync(A.seg_pos, c->pos[c->cur], n * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, s));
        const float4 *xk = (const float4 *)c->pos[c->cur];
        // reference kick: the bare acceleration at x_k from the step's own
        // force launch (the symmetric step reads it before consuming the
        // source-side sums; the directed partials stay in the scratch)
        float4 *ak = (keep && p.kick == NB_KICK_REFERENCE) ? A.seg_acc + k * n : nullptr;
        if ((st = step_once(c, s, nullptr, nullptr, uses_sym(c) ? ak : nullptr))) return st;
        if (!keep) continue;
        if (ak && !uses_sym(c) &&
            (st = nb::fast_reduce(c->plan, c->partial, 0, xk, (float)p.eps2, ak, nullptr, s)))
            return st;
        NB_CUDA(cudaMemcpyAsync(A.seg_pos + (k + 1) * n, c->pos[c->cur], n * sizeof(float4),
                                cudaMemcpyDeviceToDevice, s));
    }
    A.steps = steps;
    A.every = ckpt_every;
    A.nckpt = nckpt;
    A.ready = true;
    A.live_last = n > 0;
    A.generation += 1;
    if (generation) *generation = A.generation;
    return NB_OK;
}

int nb_adj_backward(nb_ctx *c, unsigned long long generation, const void *gx_T, const void *gv_T,
                    void *gx0, void *gv0, void *gm, void *stream)
{
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!c->adj.ready) return set_error(NB_ERR_STATE, "nb_adj_backward needs a preceding nb_adj_forward");
    if (generation != c->adj.generation)
        return set_error(NB_ERR_STATE, "nb_adj_backward: the context no longer holds that forward pass "
                                       "(a later nb_adj_forward replaced it)");
    if (c->p.n == 0) return NB_OK;
    if (!gx_T || !gx0 || !gv0 || !gm) return set_error(NB_ERR_INVALID, "NULL gradient buffer");
    auto &A = c->adj;
    const nb_params &p = c->p;
    const size_t n = (size_t)p.n;
    const float eps2 = (float)p.eps2, D = (float)p.damping, dt = (float)p.dt, G = (float)p.G;
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    NB_CUDA(cudaMemcpyAsync(A.lx, gx_T, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    if (gv_T)
        NB_CUDA(cudaMemcpyAsync(A.lv, gv_T, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    else
        NB_CUDA(cudaMemsetAsync(A.lv, 0, n * sizeof(float4), s));
    NB_CUDA(cudaMemsetAsync(A.gm, 0, n * sizeof(float), s));
    // Recompute segment `seg` from its checkpoint into segment buffer b on
    // stream rs, with the algorithm of the forward pass (same bits).
    auto recompute = [&](int seg, int b, cudaStream_t rs) -> int {
        float4 *sp = b ? A.seg_pos2 : A.seg_pos, *sa = b ? A.seg_acc2 : A.seg_acc;
        float4 *vt = b ? A.vel_tmp2 : A.vel_tmp;
        const int t0 = seg * A.every;
        const int len = (A.steps - t0) < A.every ? (A.steps - t0) : A.every;
        NB_CUDA(cudaMemcpyAsync(sp, A.ckpt_pos + (size_t)seg * n, n * sizeof(float4), cudaMemcpyDeviceToDevice, rs));
        NB_CUDA(cudaMemcpyAsync(vt, A.ckpt_vel + (size_t)seg * n, n * sizeof(float4), cudaMemcpyDeviceToDevice, rs));
        int st2;
        for (int k = 0; k < len; ++k) {
            const float4 *xk = sp + (size_t)k * n;
            float4 *xn = sp + (size_t)(k + 1) * n;
            if (uses_sym(c)) {
                if ((st2 = nb::sym_force(c->splan, xk, eps2, c->sym_t, c->sym_s, (float4 *)c->sym_acc, rs)))
                    return st2;
                if (p.kick == NB_KICK_REFERENCE &&
                    (st2 = nb::sym_integrate(c->splan, xk, nullptr, nullptr, c->sym_t, c->sym_s,
                                             (const float4 *)c->sym_acc, D, dt,
                                             p.kick, G, sa + (size_t)k * n, rs, 0)))
                    return st2;
                if ((st2 = nb::sym_integrate(c->splan, xk, xn, vt, c->sym_t, c->sym_s,
                                             (const float4 *)c->sym_acc, D, dt, p.kick, G, nullptr, rs)))
                    return st2;
                continue;
            }
            if ((st2 = nb::fast_force(c->plan, xk, eps2, c->partial, rs))) return st2;
            if (p.kick == NB_KICK_REFERENCE &&
                (st2 = nb::fast_reduce(c->plan, c->partial, 0, xk, eps2, sa + (size_t)k * n, nullptr, rs)))
                return st2;
            if ((st2 = nb::fast_integrate(c->plan, xk, xn, vt, c->partial, D, dt, p.kick, G, nullptr, rs)))
                return st2;
        }
        return NB_OK;
    };
    // Segments alternate between the two buffers, the last one in buffer 0
    // (where the forward pass leaves it).  While the reverse pass runs through
    // segment seg on `s`, segment seg-1 is recomputed on rstream into the
    // other buffer; each side waits on an event for the other.
    const int last = A.nckpt - 1;
    auto buf_of = [&](int seg) { return (last - seg) & 1; };
    const bool live = A.live_last;
    A.live_last = false;  // the buffers are reused from here on
    if (last > 0 && !A.rstream &&
        (st = nb::create_recompute_stream(&A.rstream, A.ev_rec, &A.ev_go)))
        return st;
    if (!live && (st = recompute(last, buf_of(last), s))) return st;
    bool have_g = false;
    for (int seg = last; seg >= 0; --seg) {
        const int b = buf_of(seg);
        if (seg < last) NB_CUDA(cudaStreamWaitEvent(s, A.ev_rec[b], 0));
        if (seg > 0) {
            // everything enqueued on s so far (the reverse of seg+1, which
            // used the other buffer, and any recompute on s) precedes it
            NB_CUDA(cudaEventRecord(A.ev_go, s));
            NB_CUDA(cudaStreamWaitEvent(A.rstream, A.ev_go, 0));
            if ((st = recompute(seg - 1, buf_of(seg - 1), A.rstream))) return st;
            NB_CUDA(cudaEventRecord(A.ev_rec[buf_of(seg - 1)], A.rstream));
        }
        const float4 *sp = b ? A.seg_pos2 : A.seg_pos, *sa = b ? A.seg_acc2 : A.seg_acc;
        const int t0 = seg * A.every;
        const int len = (A.steps - t0) < A.every ? (A.steps - t0) : A.every;
        // reverse through the segment
        for (int k = len - 1; k >= 0; --k) {
            const float4 *xk = sp + (size_t)k * n;
            const float4 *ak = sa + (size_t)k * n;
            if (!have_g) {
                if ((st = nb::adj_g(p.n, xk, A.lx, A.lv, A.gbuf, D, dt, p.kick, G, s))) return st;
                have_g = true;
            }
            const bool more = !(seg == 0 && k == 0);
            if (A.sym) {
                if ((st = nb::sym_vjp(A.splan, xk, A.gbuf, eps2, A.sym_t, A.sym_s, s)) ||
                    (st = nb::adj_update_sym(A.splan, A.sym_t, A.sym_s, xk, ak, A.lx, A.lv, A.gm, A.gbuf, D,
                                             dt, p.kick, G, more ? 1 : 0, s)))
                    return st;
                continue;
            }
            if ((st = nb::adj_vjp(A.plan, xk, A.gbuf, eps2, A.partial, s))) return st;
            if ((st = nb::adj_update(A.plan, A.partial, xk, ak, A.lx, A.lv, A.gm, A.gbuf, D, dt, p.kick, G,
                                     more ? 1 : 0, s)))
                return st;
        }
    }
    NB_CUDA(cudaMemcpyAsync(gx0, A.lx, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    NB_CUDA(cudaMemcpyAsync(gv0, A.lv, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    NB_CUDA(cudaMemcpyAsync(gm, A.gm, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return NB_OK;
}

int nb_launches_per_step(nb_ctx *c)
{
    if (!c) return -1;
    if (c->p.n == 0) return 0;
    // a banded symmetric plan: a force and a fold launch per band
    const int bands = (uses_sym(c) || comp_sym(c) || f64_sym(c)) && c->splan.nbands > 1 ? c->splan.nbands : 0;
    if (ff_sym(c)) return 4 + (bands ? 2 * bands - 1 : 0);  // scale reduction, split, force, integrate
    if (bands) return 2 * bands + 1;
    return (uses_fast(c) || is_comp(c) || f64_sym(c)) ? 2 : 1;
}

// Single-system autotuner: every compiled shape of the context's force
// kernel is timed on the current state (saved and restored), the fastest
// is kept.  Symmetric candidates whose triangular array would pass the
// budget are planned in bands (skipped when the shape has no banded form);
// the scratch is sized for the largest candidate tried and kept, so no step
// reallocates afterwards.
int nb_autotune(nb_ctx *c, int reps, const char *cache_path, void *stream, int *chosen2)
{
    if (int rs = refuse_shard(c, "nb_autotune")) return rs;
    if (!c) return set_error(NB_ERR_INVALID, "ctx is NULL");
    if (!c->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (reps < 1) reps = 3;
    cudaStream_t s = (cudaStream_t)stream;
    if (int fst = fx_refresh(c, s)) return fst;
    const nb_params &p = c->p;
    const bool symm = uses_sym(c) || comp_sym(c) || f64_sym(c);
    const bool fast = !symm && (uses_fast(c) || is_comp(c));
    auto report = [&](int a, int b) {
        if (chosen2) {
            chosen2[0] = a;
            chosen2[1] = b;
        }
    };
    if ((!symm && !fast) || p.n == 0) {  // the exact kernel: nothing to tune
        report(p.block, 0);
        return NB_OK;
    }
    // candidates: (warps per CTA, targets per lane) or (block, bodies per thread)
    std::vector<std::array<int, 2>> cands;
    if (ff_sym(c))
        cands = {{1, 2}, {1, 4}, {4, 4}, {8, 4}, {8, 8}};
    else if (f64_sym(c))
        cands = {{1, 8}, {1, 4}, {4, 8}, {8, 8}};
    else if (comp_sym(c))
        cands = {{1, 12}, {4, 12}, {8, 12}, {1, 8}, {8, 8}};
    else if (uses_sym(c))
        cands = {{1, 16}, {1, 8}, {1, 4}, {1, 20}, {2, 16}, {4, 20}, {8, 24}, {4, 8}, {8, 4}, {8, 8}};
    else if (is_comp(c))
        cands = {{256, 4}, {256, 8}};
    else
        cands = {{128, 2}, {128, 4}, {128, 8}, {256, 2}, {256, 4}, {256, 8}};
    const size_t ent = (p.precision == NB_F64) ? sizeof(double4) : sizeof(float4);  // symmetric entries
    const size_t halves = comp_sym(c) ? 2 : 1;
    const size_t mult = is_comp(c) ? 2 : 1;  // directed compensated partials: hi and lo
    const int cur_a = symm ? c->splan.warps : c->plan.block, cur_b = symm ? c->splan.bpt : c->plan.bpt;
    auto make = [&](int a, int b, nb::SymPlan *sp, nb::SkPlan *fp) -> int {
        if (symm) {
            if (ff_sym(c)) return nb::symff_plan(p.n, a, b, c->device, sp, p.bands);
            if (f64_sym(c)) return nb::sym64_plan(p.n, a, b, c->device, sp);
            return nb::sym_plan(p.n, a, b, c->device, sp, comp_sym(c) ? 1 : 0,
                                comp_sym(c) ? NB_SOURCE_AUTO : (c->splan.fixed ? NB_SOURCE_FIXED : NB_SOURCE_TRIANGULAR),
                                p.bands);
        }
        return nb::fast_plan(p.n, a, b, p.ctas_per_sm, c->device, fp, is_comp(c) ? nb::SK_COMP : 0);
    };
    auto t_bytes = [&](const nb::SymPlan &sp, const nb::SkPlan &fp) -> size_t {
        return symm ? halves * (size_t)sp.slots * sp.rb * ent : mult * (size_t)fp.slots * fp.tbsize * sizeof(float4);
    };
    auto s_bytes = [&](const nb::SymPlan &sp) -> size_t { return symm ? halves * (size_t)sp.spart_size * ent : 0; };

    // cache: device | mode | n -> shape
    cudaDeviceProp prop;
    NB_CUDA(cudaGetDeviceProperties(&prop, c->device));
    std::ostringstream key;
    key << "single|" << prop.name << "|sms" << prop.multiProcessorCount << "|prec" << p.precision << "|algo"
        << p.algo << "|n" << p.n;
    if (c->splan.fixed) key << "|fixedsource";  // its own compiled shapes
    std::string k = key.str();
    for (char &ch : k)
        if (ch == ' ') ch = '_';
    int best_a = cur_a, best_b = cur_b;
    bool cached = false;
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            std::string kk;
            int a = 0, b = 0;
            if ((ls >> kk >> a >> b) && kk == k) {
                best_a = a;
                best_b = b;
                cached = true;
            }
        }
    }
    // viable candidates and the scratch they need
    struct Cand {
        int a, b;
        nb::SymPlan sp;
        nb::SkPlan fp;
    };
    std::vector<Cand> viable;
    size_t need_t = 0, need_s = 0;
    for (auto &cd : cands) {
        if (cached && !(cd[0] == best_a && cd[1] == best_b)) continue;
        Cand v{cd[0], cd[1], {}, {}};
        if (make(v.a, v.b, &v.sp, &v.fp)) continue;  // not plannable (e.g. no occupancy)
        const bool current = v.a == cur_a && v.b == cur_b;
        if (symm && !current && (long long)s_bytes(v.sp) > nb::kSymSpartBudget) continue;
        need_t = std::max(need_t, t_bytes(v.sp, v.fp));
        need_s = std::max(need_s, s_bytes(v.sp));
        viable.push_back(v);
    }
    if (viable.empty()) {
        report(symm ? cur_a * 32 : cur_a, cur_b);
        return NB_OK;
    }
    // banded candidates fold into per-body sums: the context keeps a buffer
    // for them once one is timed
    bool banded = false;
    for (const Cand &v : viable) banded = banded || (symm && v.sp.nbands > 1);
    if (banded && !c->sym_acc) {
        cudaError_t ea = nb::dmalloc(&c->sym_acc, halves * (size_t)p.n * ent);
        if (ea != cudaSuccess) return nb::cuda_error(ea, "autotune scratch allocation");
    }
    if (!symm) {  // the directed scratch also serves the energy pass
        need_t = std::max(need_t, mult * (size_t)c->eplan.slots * c->eplan.tbsize * sizeof(float4));
    }
    // the plan from before stays usable on the new scratch (the fallback)
    need_t = std::max(need_t, t_bytes(c->splan, c->plan));
    need_s = std::max(need_s, s_bytes(c->splan));
    // scratch for every candidate and a copy of the state, all or nothing
    const size_t sb = state_bytes(c);
    const size_t n = (size_t)p.n;
    void *m[6] = {};
    const size_t bytes[6] = {need_t, need_s, sb, sb, is_comp(c) ? n * sizeof(float4) : 0,
                             is_comp(c) ? n * sizeof(float4) : 0};
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < 6 && e == cudaSuccess; ++q)
        if (bytes[q]) e = nb::dmalloc(&m[q], bytes[q]);
    if (e != cudaSuccess) {
        for (void *q : m) nb::dfree(q);
        return nb::cuda_error(e, "autotune scratch allocation");
    }
    void *pos_now = is_comp(c) ? c->pos[0] : c->pos[c->cur];
    const int cur0 = c->cur;
    e = cudaMemcpyAsync(m[2], pos_now, sb, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m[3], c->vel, is_comp(c) ? n * sizeof(float4) : sb,
                                              cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && is_comp(c)) e = cudaMemcpyAsync(m[4], c->pos32, n * sizeof(float4), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && is_comp(c)) e = cudaMemcpyAsync(m[5], c->vel_lo, n * sizeof(float4), cudaMemcpyDeviceToDevice, s);
    auto restore = [&]() -> cudaError_t {
        c->cur = cur0;
        void *dst = is_comp(c) ? c->pos[0] : c->pos[cur0];
        cudaError_t r = cudaMemcpyAsync(dst, m[2], sb, cudaMemcpyDeviceToDevice, s);
        if (r == cudaSuccess) r = cudaMemcpyAsync(c->vel, m[3], is_comp(c) ? n * sizeof(float4) : sb,
                                                  cudaMemcpyDeviceToDevice, s);
        if (r == cudaSuccess && is_comp(c)) r = cudaMemcpyAsync(c->pos32, m[4], n * sizeof(float4), cudaMemcpyDeviceToDevice, s);
        if (r == cudaSuccess && is_comp(c)) r = cudaMemcpyAsync(c->vel_lo, m[5], n * sizeof(float4), cudaMemcpyDeviceToDevice, s);
        return r;
    };
    // the context runs on the new scratch from here on; the captured graphs
    // and a recorded adjoint forward pass belong to the old plan
    for (auto &g : c->step_graph)
        if (g) {
            nb::graph_exec_destroy(g);
            g = nullptr;
        }
    c->adj.ready = false;
    c->adj.live_last = false;
    cudaStreamSynchronize(s);  // the old scratch may still be in use
    if (symm) {
        nb::dfree(c->sym_t);
        nb::dfree(c->sym_s);
        c->sym_t = (float4 *)m[0];
        c->sym_s = (float4 *)m[1];
        // a fixed-point source side starts zeroed, with its mass record
        if (e == cudaSuccess && uses_sym(c)) {
            int sp_st = nb::sym_fx_prepare(c->splan, (const float4 *)pos_now, c->sym_s, (float)p.eps2, s);
            if (sp_st) e = cudaErrorUnknown;
        }
    } else {
        nb::dfree(c->partial);
        c->partial = (float4 *)m[0];
    }
    int st = e == cudaSuccess ? NB_OK : nb::cuda_error(e, "autotune state copy");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!st && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        st = set_error(NB_ERR_CUDA, "autotune events");
    float best = 1e30f;
    const nb::SymPlan sp0 = c->splan;
    const nb::SkPlan fp0 = c->plan;
    const Cand *pick = nullptr;
    for (const Cand &v : viable) {
        if (st) break;
        if (symm) c->splan = v.sp;
        else c->plan = v.fp;
        if (viable.size() == 1) {  // a cached choice: nothing to time
            pick = &v;
            break;
        }
        st = step_once(c, s, nullptr);  // warm-up
        cudaError_t r = cudaEventRecord(e0, s);
        for (int q = 0; q < reps && !st && r == cudaSuccess; ++q) st = step_once(c, s, nullptr);
        if (r == cudaSuccess) r = cudaEventRecord(e1, s);
        if (r == cudaSuccess) r = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, e0, e1);
        if (r == cudaSuccess) r = restore();
        if (!st && r != cudaSuccess) st = nb::cuda_error(r, "autotune timing");
        if (!st && ms < best) {
            best = ms;
            pick = &v;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (!pick) {  // keep the plan from before (its scratch fits: the current shape was a candidate or smaller)
        c->splan = sp0;
        c->plan = fp0;
    } else if (symm) {
        c->splan = pick->sp;
    } else {
        c->plan = pick->fp;
    }
    restore();
    cudaStreamSynchronize(s);
    for (int q = 2; q < 6; ++q) nb::dfree(m[q]);
    if (st) return st;
    const int ra = symm ? c->splan.warps * 32 : c->plan.block, rb = symm ? c->splan.bpt : c->plan.bpt;
    if (cache_path && !cached && pick) {
        std::ofstream outf(cache_path, std::ios::app);
        if (outf) outf << k << " " << (symm ? c->splan.warps : c->plan.block) << " " << rb << "\n";
    }
    report(ra, rb);
    return NB_OK;
}

int nb_plan_info(nb_ctx *c, int *info5)
{
    if (!c || !info5) return set_error(NB_ERR_INVALID, "ctx/info is NULL");
    if (uses_sym(c) || comp_sym(c) || f64_sym(c)) {
        info5[0] = c->splan.warps * 32;
        info5[1] = c->splan.bpt;
        info5[2] = c->splan.grid;
        info5[3] = c->splan.rb;
        info5[4] = c->splan.slots;
        return NB_OK;
    }
    info5[0] = c->plan.block;
    info5[1] = c->plan.bpt;
    info5[2] = c->plan.grid;
    info5[3] = c->plan.tbsize;
    info5[4] = c->plan.slots;
    return NB_OK;
}

int nb_source_info(nb_ctx *c, int *info4)
{
    if (!c || !info4) return set_error(NB_ERR_INVALID, "ctx/info is NULL");
    info4[0] = 0;
    info4[1] = 1;
    info4[2] = 0;
    info4[3] = 0;
    if (uses_sym(c) || comp_sym(c) || f64_sym(c)) {
        const size_t ent = c->p.precision == NB_F64 ? sizeof(double4) : sizeof(float4);
        const size_t halves = comp_sym(c) ? 2 : 1;
        info4[0] = c->splan.fixed ? NB_SOURCE_FIXED : NB_SOURCE_TRIANGULAR;
        info4[1] = c->splan.nbands;
        info4[2] = (int)((halves * (size_t)c->splan.spart_size * ent) >> 20);
    }
    return NB_OK;
}

int nb_run_host(nb_ctx *c, const void *pos, const void *vel, int loops, int out_interval,
                void *outbuffer, double *timings, void *stream)
{
    if (int rs = refuse_shard(c, "nb_run_host")) return rs;
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
        // all three or none: a failed call leaves nothing half set up
        void *b3[3] = {nullptr, nullptr, nullptr};
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = nb::hmalloc(&b3[k], sb);
        if (e != cudaSuccess) {
            for (void *q : b3) nb::hfree(q);
            return nb::cuda_error(e, "pinned staging allocation");
        }
        c->stage_pos = b3[0];
        c->stage_vel = b3[1];
        c->stage_out = b3[2];
    }
    cudaEvent_t ev[2];
    for (int k = 0; k < 2; ++k) NB_CUDA(cudaEventCreate(&ev[k]));
    struct Guard {
        cudaEvent_t *e;
        ~Guard()
        {
            for (int k = 0; k < 2; ++k) cudaEventDestroy(e[k]);
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

    // frames: snapshot on the compute stream, D2H on the copy stream
    const int frames = loops / out_interval;
    if (frames > 0 && sb && !c->copy_stream) {
        // the copy stream is set last: a failed call leaves nothing half set up
        cudaStream_t cs = nullptr;
        void *snap[2] = {nullptr, nullptr}, *stage[2] = {nullptr, nullptr};
        cudaEvent_t es[2] = {nullptr, nullptr}, e0[2] = {nullptr, nullptr}, e1[2] = {nullptr, nullptr};
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = nb::dmalloc(&snap[k], sb);
            if (e == cudaSuccess) e = nb::hmalloc(&stage[k], sb);
            if (e == cudaSuccess) e = cudaEventCreate(&es[k]);
            if (e == cudaSuccess) e = cudaEventCreate(&e0[k]);
            if (e == cudaSuccess) e = cudaEventCreate(&e1[k]);
        }
        if (e != cudaSuccess) {
            for (int k = 0; k < 2; ++k) {
                nb::dfree(snap[k]);
                nb::hfree(stage[k]);
                if (es[k]) cudaEventDestroy(es[k]);
                if (e0[k]) cudaEventDestroy(e0[k]);
                if (e1[k]) cudaEventDestroy(e1[k]);
            }
            if (cs) cudaStreamDestroy(cs);
            return nb::cuda_error(e, "frame copy-out setup");
        }
        for (int k = 0; k < 2; ++k) {
            c->snap[k] = snap[k];
            c->stage[k] = stage[k];
            c->ev_snap[k] = es[k];
            c->ev_c0[k] = e0[k];
            c->ev_c1[k] = e1[k];
        }
        c->copy_stream = cs;
    }
    const int nstretch = (loops + out_interval - 1) / out_interval;
    while (c->events.size() < 2 * (size_t)nstretch) {
        cudaEvent_t e;
        NB_CUDA(cudaEventCreate(&e));
        c->events.push_back(e);
    }
    int pending[2] = {-1, -1};
    auto drain = [&](int slot) -> int {
        if (pending[slot] < 0) return NB_OK;
        NB_CUDA(cudaEventSynchronize(c->ev_c1[slot]));
        float cms = 0;
        NB_CUDA(cudaEventElapsedTime(&cms, c->ev_c0[slot], c->ev_c1[slot]));
        copyout += cms * 1e-3;
        std::memcpy((char *)outbuffer + (size_t)pending[slot] * sb, c->stage[slot], sb);
        pending[slot] = -1;
        return NB_OK;
    };

    // step loop; frame f (after step (f+1) * out_interval) goes to
    // outbuffer + f * 4n (body_task_sgpu.cu:116-125)
    int done = 0, k = 0;
    while (done < loops) {
        const int next_frame = (done / out_interval + 1) * out_interval;
        const int upto = next_frame < loops ? next_frame : loops;
        NB_CUDA(cudaEventRecord(c->events[2 * k], s));
        if ((st = nb_step(c, upto - done, stream))) return st;
        NB_CUDA(cudaEventRecord(c->events[2 * k + 1], s));
        ++k;
        done = upto;
        if (done % out_interval == 0 && sb) {
            const int f = done / out_interval - 1;
            const int slot = f & 1;
            if ((st = drain(slot))) return st;
            const void *cur = is_comp(c) ? c->pos[0] : c->pos[c->cur];
            NB_CUDA(cudaMemcpyAsync(c->snap[slot], cur, sb, cudaMemcpyDeviceToDevice, s));
            NB_CUDA(cudaEventRecord(c->ev_snap[slot], s));
            NB_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_snap[slot], 0));
            NB_CUDA(cudaEventRecord(c->ev_c0[slot], c->copy_stream));
            NB_CUDA(cudaMemcpyAsync(c->stage[slot], c->snap[slot], sb, cudaMemcpyDeviceToHost,
                                    c->copy_stream));
            NB_CUDA(cudaEventRecord(c->ev_c1[slot], c->copy_stream));
            pending[slot] = f;
        }
    }
    for (int slot = 0; slot < 2; ++slot)
        if ((st = drain(slot))) return st;
    NB_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < k; ++i) {
        NB_CUDA(cudaEventElapsedTime(&ms, c->events[2 * i], c->events[2 * i + 1]));
        kernel += ms * 1e-3;
    }
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
