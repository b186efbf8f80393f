// nb_batch.cu -- many independent systems of uneven size in one launch.
//
// The reference runs several nbody systems as separate UTC tasks, one kernel
// launch per system per step (benchapps/nbody/utc/nbody_mtask.cc:199-231).
// Here all systems share one persistent launch per step:
//  * bodies of all systems are concatenated (AoS float4, system s at
//    [off[s], off[s+1]));
//  * the iteration space is the concatenation over systems of
//    (warp target block of 32*BPT targets, 32-source group), and each warp of
//    the persistent grid takes an equal contiguous range of it (warp-level
//    stream-K), so small and large systems are balanced without per-size
//    launches;
//  * each warp stages its 32-source groups in its own shared-memory slice
//    (no CTA barriers: warps of a CTA may work on different systems);
//  * one partial per (warp, warp target block) goes to slot
//    warp + global block index; the integrate kernel sums them in warp order.
// The step loop is captured in a CUDA graph (nb_batch_run), and an autotuner
// picks the warps per CTA and bodies per lane.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "nb_internal.cuh"

namespace nb {

struct BatchDev {
    const int *sys_off;       // [nsys + 1] body offsets
    const long long *it_off;  // [nsys + 1] iteration offsets
    const int *tb_off;        // [nsys + 1] global warp-target-block offsets
    const int *body_sys;      // [nbody] system of each body
    int nsys;
};

__device__ __forceinline__ int find_sys(const long long *it_off, int nsys, long long it)
{
    int lo = 0, hi = nsys;  // it_off[lo] <= it < it_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (it_off[mid] <= it) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int WPB, int BPT>
__global__ void __launch_bounds__(32 * WPB) bk_force_kernel(const float4 *__restrict__ pos, BatchDev bd,
                                                            float eps2, float4 *__restrict__ partial,
                                                            long long total, int workers)
{
    constexpr int WTB = 32 * BPT;
    __shared__ __align__(16) float4 sP[WPB][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wid;
    if (w >= workers) return;
    long long it = sk_start(w, total, workers);
    const long long end = sk_start(w + 1, total, workers);
    if (it >= end) return;
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    int s = find_sys(bd.it_off, bd.nsys, it);
    while (it < end) {
        while (it >= bd.it_off[s + 1]) ++s;
        const int o = bd.sys_off[s];
        const int ns = bd.sys_off[s + 1] - o;
        const int ngroups = (ns + kGroup - 1) / kGroup;
        const long long base = bd.it_off[s];
        const int tbl = (int)((it - base) / ngroups);
        const long long blk_first = base + (long long)tbl * ngroups;
        const long long seg_end = end < blk_first + ngroups ? end : blk_first + ngroups;
        const int j0 = (int)(it - blk_first) * kGroup;
        const int j1 = min((int)(seg_end - blk_first) * kGroup, ns);

        float px[BPT], py[BPT], pz[BPT], ax[BPT], ay[BPT], az[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int li = tbl * WTB + lane + 32 * k;
            const float4 q = li < ns ? pos[o + li] : make_float4(0.f, 0.f, 0.f, 0.f);
            px[k] = q.x;
            py[k] = q.y;
            pz[k] = q.z;
            ax[k] = ay[k] = az[k] = 0.f;
        }
        float4 nxt = (j0 + lane < j1) ? pos[o + j0 + lane] : pad;
        for (int jt = j0; jt < j1; jt += kGroup) {
            __syncwarp();
            sP[wid][lane] = nxt;
            __syncwarp();
            if (jt + kGroup < j1) nxt = (jt + kGroup + lane < j1) ? pos[o + jt + kGroup + lane] : pad;
            const int cnt = min(kGroup, j1 - jt);
            const int cnt2 = (cnt + 1) & ~1;  // entries past cnt are zero-mass pads
            for (int j = 0; j < cnt2; j += 2) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float4 q = sP[wid][j + u];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float sc = (q.w * inv) * (inv * inv);
                        ax[k] = fmaf(rx, sc, ax[k]);
                        ay[k] = fmaf(ry, sc, ay[k]);
                        az[k] = fmaf(rz, sc, az[k]);
                    }
                }
            }
        }
        const long long slot = (long long)w + bd.tb_off[s] + tbl;
        float4 *dst = partial + slot * WTB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) dst[lane + 32 * k] = make_float4(ax[k], ay[k], az[k], 0.f);
        it = seg_end;
    }
}

__global__ void bk_integrate_kernel(const float4 *__restrict__ pos_old, float4 *__restrict__ pos_new,
                                    float4 *__restrict__ vel, const float4 *__restrict__ partial,
                                    BatchDev bd, int nbody, int wtb, long long total, int workers,
                                    float damping, float dt, int kick, float G,
                                    float4 *__restrict__ acc_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbody) return;
    const int s = bd.body_sys[i];
    const int o = bd.sys_off[s];
    const int ns = bd.sys_off[s + 1] - o;
    const int ngroups = (ns + kGroup - 1) / kGroup;
    const int li = i - o;
    const int tbl = li / wtb;
    const long long first = bd.it_off[s] + (long long)tbl * ngroups;
    const int c0 = sk_owner(first, total, workers);
    const int c1 = sk_owner(first + ngroups - 1, total, workers);
    const long long gtb = (long long)bd.tb_off[s] + tbl;
    const int lj = li - tbl * wtb;
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 q = partial[(c + gtb) * wtb + lj];
        ax = __fadd_rn(ax, q.x);
        ay = __fadd_rn(ay, q.y);
        az = __fadd_rn(az, q.z);
    }
    if (acc_out) {
        acc_out[i] = make_float4(ax, ay, az, 0.f);
        return;
    }
    float4 p = pos_old[i];
    float4 v = vel[i];
    const float k = kick == NB_KICK_REFERENCE ? p.w : G;
    v.x = __fadd_rn(v.x, __fmul_rn(__fmul_rn(ax, k), dt));
    v.y = __fadd_rn(v.y, __fmul_rn(__fmul_rn(ay, k), dt));
    v.z = __fadd_rn(v.z, __fmul_rn(__fmul_rn(az, k), dt));
    v.x = __fmul_rn(v.x, damping);
    v.y = __fmul_rn(v.y, damping);
    v.z = __fmul_rn(v.z, damping);
    p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
    p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
    p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
    pos_new[i] = p;
    vel[i] = v;
}

typedef void (*bk_kernel_t)(const float4 *, BatchDev, float, float4 *, long long, int);

static bk_kernel_t bk_kernel_for(int wpb, int bpt)
{
#define NB_BK(W, B) \
    if (wpb == W && bpt == B) return bk_force_kernel<W, B>;
    NB_BK(2, 4) NB_BK(2, 8) NB_BK(4, 2) NB_BK(4, 4) NB_BK(4, 8) NB_BK(8, 2) NB_BK(8, 4) NB_BK(8, 8)
#undef NB_BK
    return nullptr;
}

}  // namespace nb

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchPlan {
    int wpb = 0, bpt = 0, grid = 0, workers = 0;
    long long total = 0, total_wtb = 0, slots = 0;
};

struct nb_batch {
    nb_params p;
    int device = 0, sms = 0;
    int nsys = 0, nbody = 0;
    std::vector<int> sizes;
    int *d_sys_off = nullptr, *d_tb_off = nullptr, *d_body_sys = nullptr;
    long long *d_it_off = nullptr;
    float4 *pos[2] = {nullptr, nullptr};
    float4 *vel = nullptr;
    int cur = 0;
    bool has_state = false;
    float4 *partial = nullptr;
    size_t partial_cap = 0;  // float4 entries
    BatchPlan plan;
    // graph of `graph_steps` steps starting from pos[graph_cur]
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0, graph_cur = -1;
    // per-system plain plans for the baseline
    std::vector<nb::SkPlan> sys_plans;
    float4 *sys_partial = nullptr;
};

using nb::set_error;

static int batch_plan_for(nb_batch *b, int wpb, int bpt, BatchPlan *out, std::vector<long long> *it_off,
                          std::vector<int> *tb_off)
{
    nb::bk_kernel_t k = nb::bk_kernel_for(wpb, bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "batched kernel shape not compiled");
    const int wtb = 32 * bpt;
    it_off->assign(b->nsys + 1, 0);
    tb_off->assign(b->nsys + 1, 0);
    for (int s = 0; s < b->nsys; ++s) {
        const long long n = b->sizes[s];
        const long long ntb = (n + wtb - 1) / wtb, ng = (n + nb::kGroup - 1) / nb::kGroup;
        (*it_off)[s + 1] = (*it_off)[s] + ntb * ng;
        (*tb_off)[s + 1] = (*tb_off)[s] + (int)ntb;
    }
    int occ = 0;
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * wpb, 0));
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "batched kernel does not fit on an SM");
    BatchPlan p;
    p.wpb = wpb;
    p.bpt = bpt;
    p.total = (*it_off)[b->nsys];
    p.total_wtb = (*tb_off)[b->nsys];
    long long workers = (long long)b->sms * occ * wpb;
    if (p.total > 0 && workers > p.total) workers = p.total;
    p.workers = p.total > 0 ? (int)workers : 0;
    p.grid = (p.workers + wpb - 1) / wpb;
    p.slots = p.total > 0 ? p.workers + p.total_wtb - 1 : 0;
    *out = p;
    return NB_OK;
}

static int batch_apply_plan(nb_batch *b, int wpb, int bpt, cudaStream_t s)
{
    BatchPlan p;
    std::vector<long long> it_off;
    std::vector<int> tb_off;
    int st = batch_plan_for(b, wpb, bpt, &p, &it_off, &tb_off);
    if (st) return st;
    const size_t need = (size_t)p.slots * 32 * bpt;
    if (need > b->partial_cap) {
        cudaFree(b->partial);
        b->partial = nullptr;
        b->partial_cap = 0;
        cudaError_t e = cudaMalloc((void **)&b->partial, need * sizeof(float4));
        if (e != cudaSuccess) return nb::cuda_error(e, "batched scratch allocation");
        b->partial_cap = need;
    }
    NB_CUDA(cudaMemcpyAsync(b->d_it_off, it_off.data(), it_off.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, s));
    NB_CUDA(cudaMemcpyAsync(b->d_tb_off, tb_off.data(), tb_off.size() * sizeof(int),
                            cudaMemcpyHostToDevice, s));
    NB_CUDA(cudaStreamSynchronize(s));
    b->plan = p;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_cur = -1;
    }
    return NB_OK;
}

static nb::BatchDev batch_dev(const nb_batch *b)
{
    nb::BatchDev d;
    d.sys_off = b->d_sys_off;
    d.it_off = b->d_it_off;
    d.tb_off = b->d_tb_off;
    d.body_sys = b->d_body_sys;
    d.nsys = b->nsys;
    return d;
}

static int batch_step_once(nb_batch *b, cudaStream_t s)
{
    const BatchPlan &p = b->plan;
    if (b->nbody == 0) return NB_OK;
    const float4 *po = b->pos[b->cur];
    float4 *pn = b->pos[b->cur ^ 1];
    nb::bk_kernel_t k = nb::bk_kernel_for(p.wpb, p.bpt);
    k<<<p.grid, 32 * p.wpb, 0, s>>>(po, batch_dev(b), (float)b->p.eps2, b->partial, p.total, p.workers);
    NB_LAUNCH_CHECK("bk_force_kernel launch");
    nb::bk_integrate_kernel<<<(b->nbody + 255) / 256, 256, 0, s>>>(
        po, pn, b->vel, b->partial, batch_dev(b), b->nbody, 32 * p.bpt, p.total, p.workers,
        (float)b->p.damping, (float)b->p.dt, b->p.kick, (float)b->p.G, nullptr);
    NB_LAUNCH_CHECK("bk_integrate_kernel launch");
    b->cur ^= 1;
    return NB_OK;
}

static void free_batch(nb_batch *b)
{
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->d_sys_off);
    cudaFree(b->d_tb_off);
    cudaFree(b->d_body_sys);
    cudaFree(b->d_it_off);
    cudaFree(b->pos[0]);
    cudaFree(b->pos[1]);
    cudaFree(b->vel);
    cudaFree(b->partial);
    cudaFree(b->sys_partial);
    delete b;
}

extern "C" {

int nb_batch_create(const nb_params *p, int nsys, const int *sizes, nb_batch **out)
{
    if (!out) return set_error(NB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!p || nsys < 0 || (nsys > 0 && !sizes)) return set_error(NB_ERR_INVALID, "bad batch arguments");
    if (p->precision != NB_F32 || p->algo != NB_ALGO_FAST)
        return set_error(NB_ERR_UNSUPPORTED, "batches run the NB_F32 fast algorithm");
    if (p->kick != NB_KICK_REFERENCE && p->kick != NB_KICK_PHYSICAL)
        return set_error(NB_ERR_INVALID, "unknown kick mode");
    long long nbody = 0;
    for (int s = 0; s < nsys; ++s) {
        if (sizes[s] < 1) return set_error(NB_ERR_INVALID, "every system needs at least one body");
        nbody += sizes[s];
    }
    if (nbody > (1LL << 30)) return set_error(NB_ERR_INVALID, "batch too large");
    nb_batch *b = new nb_batch();
    b->p = *p;
    b->nsys = nsys;
    b->nbody = (int)nbody;
    b->sizes.assign(sizes, sizes + nsys);
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e != cudaSuccess) {
        delete b;
        return nb::cuda_error(e, "device query");
    }
    std::vector<int> sys_off(nsys + 1, 0), body_sys((size_t)nbody);
    for (int s = 0; s < nsys; ++s) {
        sys_off[s + 1] = sys_off[s] + sizes[s];
        for (int i = sys_off[s]; i < sys_off[s + 1]; ++i) body_sys[i] = s;
    }
    const size_t sb = (size_t)nbody * sizeof(float4);
#define NB_BALLOC(ptr, bytes)                                                  \
    do {                                                                       \
        cudaError_t _e = cudaMalloc((void **)&(ptr), (bytes) ? (bytes) : 16);  \
        if (_e != cudaSuccess) {                                               \
            free_batch(b);                                                     \
            return nb::cuda_error(_e, "batch allocation");                     \
        }                                                                      \
    } while (0)
    NB_BALLOC(b->d_sys_off, sizeof(int) * (nsys + 1));
    NB_BALLOC(b->d_tb_off, sizeof(int) * (nsys + 1));
    NB_BALLOC(b->d_it_off, sizeof(long long) * (nsys + 1));
    NB_BALLOC(b->d_body_sys, sizeof(int) * (size_t)nbody);
    NB_BALLOC(b->pos[0], sb);
    NB_BALLOC(b->pos[1], sb);
    NB_BALLOC(b->vel, sb);
#undef NB_BALLOC
    e = cudaMemcpy(b->d_sys_off, sys_off.data(), sizeof(int) * (nsys + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nbody)
        e = cudaMemcpy(b->d_body_sys, body_sys.data(), sizeof(int) * (size_t)nbody, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_batch(b);
        return nb::cuda_error(e, "batch tables");
    }
    const int wpb = p->block ? p->block / 32 : 4;
    const int bpt = p->bpt ? p->bpt : 4;
    int st = batch_apply_plan(b, wpb, bpt, nullptr);
    if (st) {
        free_batch(b);
        return st;
    }
    *out = b;
    return NB_OK;
}

int nb_batch_destroy(nb_batch *b)
{
    if (!b) return NB_OK;
    cudaDeviceSynchronize();
    free_batch(b);
    return NB_OK;
}

int nb_batch_set_state(nb_batch *b, const void *pos, const void *vel, int where, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    const size_t sb = (size_t)b->nbody * sizeof(float4);
    if (sb && (!pos || !vel)) return set_error(NB_ERR_INVALID, "pos/vel is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    b->cur = 0;
    if (sb) {
        NB_CUDA(cudaMemcpyAsync(b->pos[0], pos, sb, cudaMemcpyDefault, s));
        NB_CUDA(cudaMemcpyAsync(b->vel, vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    b->has_state = true;
    return NB_OK;
}

int nb_batch_get_state(nb_batch *b, void *pos, void *vel, int where, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    const size_t sb = (size_t)b->nbody * sizeof(float4);
    cudaStream_t s = (cudaStream_t)stream;
    if (sb) {
        if (pos) NB_CUDA(cudaMemcpyAsync(pos, b->pos[b->cur], sb, cudaMemcpyDefault, s));
        if (vel) NB_CUDA(cudaMemcpyAsync(vel, b->vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    return NB_OK;
}

int nb_batch_step(nb_batch *b, int steps, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    for (int i = 0; i < steps; ++i) {
        int st = batch_step_once(b, (cudaStream_t)stream);
        if (st) return st;
    }
    return NB_OK;
}

int nb_batch_run(nb_batch *b, int steps, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (steps == 0 || b->nbody == 0) return NB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (s == nullptr) return set_error(NB_ERR_INVALID, "nb_batch_run needs a non-default stream");
    if (!b->graph || b->graph_steps != steps || b->graph_cur != b->cur) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        const int cur0 = b->cur;
        cudaGraph_t g = nullptr;
        NB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int st = NB_OK;
        for (int i = 0; i < steps && !st; ++i) st = batch_step_once(b, s);
        cudaError_t e = cudaStreamEndCapture(s, &g);
        b->cur = cur0;
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return nb::cuda_error(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return nb::cuda_error(e, "cudaGraphInstantiate");
        b->graph_steps = steps;
        b->graph_cur = cur0;
    }
    NB_CUDA(cudaGraphLaunch(b->graph, s));
    if (steps % 2) b->cur ^= 1;
    return NB_OK;
}

int nb_batch_plan_info(nb_batch *b, long long *info6)
{
    if (!b || !info6) return set_error(NB_ERR_INVALID, "batch/info is NULL");
    info6[0] = b->plan.wpb;
    info6[1] = b->plan.bpt;
    info6[2] = b->plan.grid;
    info6[3] = b->plan.workers;
    info6[4] = b->plan.total;
    info6[5] = b->plan.slots;
    return NB_OK;
}

int nb_batch_set_shape(nb_batch *b, int warps_per_cta, int bodies_per_lane)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    return batch_apply_plan(b, warps_per_cta, bodies_per_lane, nullptr);
}

// Autotuner: times every compiled (warps per CTA, bodies per lane) shape on
// this batch (one warm-up step, then `reps` steps with CUDA events) and keeps
// the fastest.  The state is restored afterwards.  With cache_path, the
// choice is looked up / stored under a key of the device name and the batch's
// size histogram (log2 buckets).
int nb_batch_autotune(nb_batch *b, int reps, const char *cache_path, void *stream, int *chosen2)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (reps < 1) reps = 2;
    cudaStream_t s = (cudaStream_t)stream;
    cudaDeviceProp prop;
    NB_CUDA(cudaGetDeviceProperties(&prop, b->device));
    std::ostringstream key;
    key << prop.name << "|sms" << prop.multiProcessorCount << "|kick" << b->p.kick << "|";
    {
        std::map<int, int> hist;
        for (int n : b->sizes) {
            int lg = 0;
            while ((1 << (lg + 1)) <= n) ++lg;
            hist[lg]++;
        }
        for (auto &h : hist) key << h.first << ":" << h.second << ",";
    }
    std::string k = key.str();
    for (char &ch : k)
        if (ch == ' ') ch = '_';
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            std::string kk;
            int w = 0, bp = 0;
            if ((ls >> kk >> w >> bp) && kk == k) {
                int st = batch_apply_plan(b, w, bp, s);
                if (st) break;  // stale entry: tune again
                if (chosen2) {
                    chosen2[0] = w;
                    chosen2[1] = bp;
                }
                return NB_OK;
            }
        }
    }
    const size_t sb = (size_t)b->nbody * sizeof(float4);
    float4 *save_p = nullptr, *save_v = nullptr;
    if (sb) {
        NB_CUDA(cudaMalloc((void **)&save_p, sb));
        NB_CUDA(cudaMalloc((void **)&save_v, sb));
        NB_CUDA(cudaMemcpyAsync(save_p, b->pos[b->cur], sb, cudaMemcpyDeviceToDevice, s));
        NB_CUDA(cudaMemcpyAsync(save_v, b->vel, sb, cudaMemcpyDeviceToDevice, s));
    }
    const int cand[][2] = {{2, 4}, {2, 8}, {4, 2}, {4, 4}, {4, 8}, {8, 2}, {8, 4}, {8, 8}};
    float best = 1e30f;
    int bw = b->plan.wpb, bb = b->plan.bpt;
    cudaEvent_t e0, e1;
    NB_CUDA(cudaEventCreate(&e0));
    NB_CUDA(cudaEventCreate(&e1));
    int st = NB_OK;
    for (auto &c : cand) {
        if ((st = batch_apply_plan(b, c[0], c[1], s))) break;
        if ((st = batch_step_once(b, s))) break;
        NB_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps && !st; ++r) st = batch_step_once(b, s);
        NB_CUDA(cudaEventRecord(e1, s));
        NB_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        NB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            bw = c[0];
            bb = c[1];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!st) st = batch_apply_plan(b, bw, bb, s);
    if (sb) {
        b->cur = 0;
        cudaMemcpyAsync(b->pos[0], save_p, sb, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b->vel, save_v, sb, cudaMemcpyDeviceToDevice, s);
        cudaStreamSynchronize(s);
        cudaFree(save_p);
        cudaFree(save_v);
    }
    if (st) return st;
    if (cache_path) {
        std::ofstream outf(cache_path, std::ios::app);
        if (outf) outf << k << " " << bw << " " << bb << "\n";
    }
    if (chosen2) {
        chosen2[0] = bw;
        chosen2[1] = bb;
    }
    return NB_OK;
}

// The per-system baseline: every system stepped by its own plain stream-K
// launches (force + integrate per system per step), as separate tasks would.
int nb_batch_step_per_system(nb_batch *b, int steps, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    cudaStream_t s = (cudaStream_t)stream;
    if (b->sys_plans.empty() && b->nsys) {
        b->sys_plans.resize(b->nsys);
        size_t need = 0;
        for (int i = 0; i < b->nsys; ++i) {
            int st = nb::fast_plan(b->sizes[i], 0, 0, 0, b->device, &b->sys_plans[i], 0);
            if (st) return st;
            need = std::max(need, (size_t)b->sys_plans[i].slots * b->sys_plans[i].tbsize);
        }
        NB_CUDA(cudaMalloc((void **)&b->sys_partial, std::max<size_t>(need, 1) * sizeof(float4)));
    }
    std::vector<int> off(b->nsys + 1, 0);
    for (int i = 0; i < b->nsys; ++i) off[i + 1] = off[i] + b->sizes[i];
    for (int t = 0; t < steps; ++t) {
        for (int i = 0; i < b->nsys; ++i) {
            const float4 *po = b->pos[b->cur] + off[i];
            float4 *pn = b->pos[b->cur ^ 1] + off[i];
            int st = nb::fast_force(b->sys_plans[i], po, (float)b->p.eps2, b->sys_partial, s, 0);
            if (!st)
                st = nb::fast_integrate(b->sys_plans[i], po, pn, b->vel + off[i], b->sys_partial,
                                        (float)b->p.damping, (float)b->p.dt, b->p.kick, (float)b->p.G,
                                        nullptr, s);
            if (st) return st;
        }
        b->cur ^= 1;
    }
    return NB_OK;
}

int nb_batch_launches_per_step(nb_batch *b) { return b ? (b->nbody ? 2 : 0) : -1; }

}  // extern "C"
