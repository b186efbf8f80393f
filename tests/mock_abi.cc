// mock_abi.cc -- host-only stand-in for the C ABI (include/nbody_gb300.h)
// and the four CUDA runtime calls of the UTC task stand-in, so that the
// drop-in task (utc_gb300/task/body_task_gb300.cc) runs without a GPU.
// Test infrastructure: nb_run_host steps with the oracle's C restatement
// (oracle/nbody_oracle.c) and records what the task handed over.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>
#include <vector>

#include "nbody_gb300.h"
#include "nbody_oracle.h"

namespace {

std::string g_err;
int g_fake_stream_object;  // its address is the worker's "stream"
cudaStream_t g_fake_stream = reinterpret_cast<cudaStream_t>(&g_fake_stream_object);

struct Record {
    void *stream = nullptr;
    int calls = 0, n = 0, loops = 0, out_interval = 0, precision = -1, algo = -1, memtype = -1, kick = -1;
    double eps2 = 0, damping = 0, dt = 0;
} g_rec;
// every task worker makes and frees a stream: counted from many threads
std::atomic<int> g_streams_created{0}, g_streams_destroyed{0};

struct BatchRecord {
    int creates = 0, runs = 0, nsys = 0, destroys = 0, precision = -1, algo = -1;
    void *stream = nullptr;
} g_batch;

}  // namespace

struct nb_ctx {
    nb_params p;
    // shard contexts (nb_create_shard): every body's state in host memory,
    // two position buffers, the shard's range and its steps so far
    int rank = 0, nranks = 1, lo = 0, hi = 0, cur = 0, steps = 0;
    std::vector<double> x[2], v;
    std::vector<float> xf[2], vf;
};

struct nb_batch {
    nb_params p;
    std::vector<int> sizes;
    std::vector<double> x, v;
};

extern "C" {

// ---- CUDA runtime calls of utc_standin.h ----
cudaError_t cudaGetDevice(int *dev)
{
    *dev = 0;
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDeviceCount(int *count)
{
    *count = 1;
    return cudaSuccess;
}
cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned int)
{
    *s = g_fake_stream;
    ++g_streams_created;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t) { ++g_streams_destroyed; return cudaSuccess; }

// ---- the C ABI calls of the task ----
void nb_params_default(nb_params *p)
{
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

const char *nb_last_error(void) { return g_err.c_str(); }

int nb_create(const nb_params *p, nb_ctx **out)
{
    *out = nullptr;
    if (p->n == 3) {  // planted failure: the task must report it
        g_err = "mock: n == 3 is refused";
        return NB_ERR_INVALID;
    }
    *out = new nb_ctx{*p};
    return NB_OK;
}

int nb_destroy(nb_ctx *c)
{
    delete c;
    return NB_OK;
}

int nb_run_host(nb_ctx *c, const void *pos, const void *vel, int loops, int out_interval, void *outbuffer,
                double *timings, void *stream)
{
    const nb_params &p = c->p;
    g_rec.calls++;
    g_rec.stream = stream;
    g_rec.n = p.n;
    g_rec.loops = loops;
    g_rec.out_interval = out_interval;
    g_rec.precision = p.precision;
    g_rec.algo = p.algo;
    g_rec.memtype = p.memtype;
    g_rec.kick = p.kick;
    g_rec.eps2 = p.eps2;
    g_rec.damping = p.damping;
    g_rec.dt = p.dt;
    const size_t m = 4 * (size_t)p.n;
    if (p.precision == NB_F64) {
        std::vector<double> x((const double *)pos, (const double *)pos + m), v((const double *)vel,
                                                                               (const double *)vel + m);
        for (int f = 0; f < loops / out_interval; ++f) {
            orc_step_f64(p.n, x.data(), v.data(), p.eps2, p.damping, p.dt, out_interval, p.kick, p.G, 1);
            std::memcpy((double *)outbuffer + f * m, x.data(), m * sizeof(double));
        }
    } else {
        std::vector<float> x((const float *)pos, (const float *)pos + m), v((const float *)vel,
                                                                             (const float *)vel + m);
        for (int f = 0; f < loops / out_interval; ++f) {
            orc_step_f32(p.n, x.data(), v.data(), (float)p.eps2, (float)p.damping, (float)p.dt, out_interval,
                         p.kick, (float)p.G, 1);
            std::memcpy((float *)outbuffer + f * m, x.data(), m * sizeof(float));
        }
    }
    if (timings)
        for (int k = 0; k < 4; ++k) timings[k] = 1.0 + k;  // total, kernel, copy-in, copy-out
    return NB_OK;
}

// ---- shard contexts of the multi-GPU task (host memory stands for each
// "device"; planted failures: n == 5 refuses rank 1 at creation, n == 7 fails
// rank 1's fifth step) ----
int nb_create_shard(const nb_params *p, int rank, int nranks, nb_ctx **out)
{
    *out = nullptr;
    if (p->n == 5 && rank == 1) {
        g_err = "mock: shard 1 of a 5-body system is refused";
        return NB_ERR_INVALID;
    }
    nb_ctx *c = new nb_ctx{*p};
    c->rank = rank;
    c->nranks = nranks;
    const int q = p->n / nranks, r = p->n % nranks;
    c->lo = rank < r ? rank * (q + 1) : rank * q + r;
    c->hi = c->lo + q + (rank < r ? 1 : 0);
    *out = c;
    return NB_OK;
}

int nb_shard_info(nb_ctx *c, int *info4)
{
    info4[0] = c->lo;
    info4[1] = c->hi - c->lo;
    info4[2] = c->rank;
    info4[3] = c->nranks;
    return NB_OK;
}

int nb_set_state(nb_ctx *c, const void *pos, const void *vel, int, void *)
{
    const size_t m = 4 * (size_t)c->p.n;
    if (c->p.precision == NB_F64) {
        c->x[0].assign((const double *)pos, (const double *)pos + m);
        c->x[1] = c->x[0];
        c->v.assign((const double *)vel, (const double *)vel + m);
    } else {
        c->xf[0].assign((const float *)pos, (const float *)pos + m);
        c->xf[1] = c->xf[0];
        c->vf.assign((const float *)vel, (const float *)vel + m);
    }
    c->cur = 0;
    return NB_OK;
}

// One step of the shard's range: the oracle's step of every body, of which
// the range is kept (a target's result does not depend on the others'
// velocities or on the partition)
int nb_step(nb_ctx *c, int steps, void *)
{
    if (steps != 1) {
        g_err = "mock: a shard steps once per call";
        return NB_ERR_INVALID;
    }
    if (c->p.n == 7 && c->rank == 1 && ++c->steps == 5) {
        g_err = "mock: planted failure of shard 1's fifth step";
        return NB_ERR_CUDA;
    }
    const nb_params &p = c->p;
    const size_t a = 4 * (size_t)c->lo, b = 4 * (size_t)c->hi;
    if (p.precision == NB_F64) {
        std::vector<double> x = c->x[c->cur], v = c->v;
        orc_step_f64(p.n, x.data(), v.data(), p.eps2, p.damping, p.dt, 1, p.kick, p.G, 1);
        std::copy(x.begin() + a, x.begin() + b, c->x[c->cur ^ 1].begin() + a);
        std::copy(v.begin() + a, v.begin() + b, c->v.begin() + a);
    } else {
        std::vector<float> x = c->xf[c->cur], v = c->vf;
        orc_step_f32(p.n, x.data(), v.data(), (float)p.eps2, (float)p.damping, (float)p.dt, 1, p.kick,
                     (float)p.G, 1);
        std::copy(x.begin() + a, x.begin() + b, c->xf[c->cur ^ 1].begin() + a);
        std::copy(v.begin() + a, v.begin() + b, c->vf.begin() + a);
    }
    c->cur ^= 1;
    return NB_OK;
}

int nb_state_ptrs(nb_ctx *c, void **pos_dev, void **vel_dev)
{
    const bool f64 = c->p.precision == NB_F64;
    if (pos_dev) *pos_dev = f64 ? (void *)c->x[c->cur].data() : (void *)c->xf[c->cur].data();
    if (vel_dev) *vel_dev = f64 ? (void *)c->v.data() : (void *)c->vf.data();
    return NB_OK;
}

cudaError_t cudaMemcpyPeerAsync(void *dst, int, const void *src, int, size_t bytes, cudaStream_t)
{
    std::memcpy(dst, src, bytes);
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void *dst, const void *src, size_t bytes, cudaMemcpyKind, cudaStream_t)
{
    std::memcpy(dst, src, bytes);
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t) { return "mock CUDA error"; }

// ---- the timing events and the batch calls of a task group ----
cudaError_t cudaEventCreate(cudaEvent_t *e)
{
    *e = reinterpret_cast<cudaEvent_t>(&g_fake_stream_object);
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t)
{
    *ms = 1.0f;
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }

int nb_batch_create(const nb_params *p, int nsys, const int *sizes, nb_batch **out)
{
    *out = nullptr;
    for (int i = 0; i < nsys; ++i)
        if (sizes[i] == 3) {  // planted failure: every member must report it
            g_err = "mock: a system of 3 bodies is refused";
            return NB_ERR_INVALID;
        }
    nb_batch *b = new nb_batch();
    b->p = *p;
    b->sizes.assign(sizes, sizes + nsys);
    size_t total = 0;
    for (int n : b->sizes) total += 4 * (size_t)n;
    b->x.resize(total);
    b->v.resize(total);
    g_batch.creates++;
    g_batch.nsys = nsys;
    g_batch.precision = p->precision;
    g_batch.algo = p->algo;
    *out = b;
    return NB_OK;
}

int nb_batch_destroy(nb_batch *b)
{
    if (b) g_batch.destroys++;
    delete b;
    return NB_OK;
}

int nb_batch_set_state(nb_batch *b, const void *pos, const void *vel, int, void *)
{
    const size_t m = b->x.size(), w = b->p.precision == NB_F64 ? 8 : 4;
    for (size_t k = 0; k < m; ++k) {  // kept as double: exact for either state type
        b->x[k] = w == 8 ? ((const double *)pos)[k] : (double)((const float *)pos)[k];
        b->v[k] = w == 8 ? ((const double *)vel)[k] : (double)((const float *)vel)[k];
    }
    return NB_OK;
}

int nb_batch_get_state(nb_batch *b, void *pos, void *vel, int, void *)
{
    const size_t m = b->x.size();
    for (size_t k = 0; k < m; ++k) {
        if (b->p.precision == NB_F64) {
            if (pos) ((double *)pos)[k] = b->x[k];
            if (vel) ((double *)vel)[k] = b->v[k];
        } else {
            if (pos) ((float *)pos)[k] = (float)b->x[k];
            if (vel) ((float *)vel)[k] = (float)b->v[k];
        }
    }
    return NB_OK;
}

// each system stepped alone by the oracle, in the state's precision
int nb_batch_run(nb_batch *b, int steps, void *stream)
{
    const nb_params &p = b->p;
    g_batch.runs++;
    g_batch.stream = stream;
    size_t o = 0;
    for (int n : b->sizes) {
        const size_t m = 4 * (size_t)n;
        if (p.precision == NB_F64) {
            orc_step_f64(n, &b->x[o], &b->v[o], p.eps2, p.damping, p.dt, steps, p.kick, p.G, 1);
        } else {
            std::vector<float> x(b->x.begin() + o, b->x.begin() + o + m), v(b->v.begin() + o, b->v.begin() + o + m);
            orc_step_f32(n, x.data(), v.data(), (float)p.eps2, (float)p.damping, (float)p.dt, steps, p.kick,
                         (float)p.G, 1);
            std::copy(x.begin(), x.end(), b->x.begin() + o);
            std::copy(v.begin(), v.end(), b->v.begin() + o);
        }
        o += m;
    }
    return NB_OK;
}

// ---- what the test reads back ----
void mock_batch_record(int *ints6, void **stream)
{
    const int v[6] = {g_batch.creates, g_batch.runs, g_batch.nsys, g_batch.destroys, g_batch.precision,
                      g_batch.algo};
    std::memcpy(ints6, v, sizeof(v));
    *stream = g_batch.stream;
}
void mock_batch_reset(void) { g_batch = BatchRecord(); }
void *mock_fake_stream(void) { return g_fake_stream; }
void mock_record(void **stream, int *ints9, double *dbl3)
{
    *stream = g_rec.stream;
    const int v[9] = {g_rec.calls, g_rec.n, g_rec.loops, g_rec.out_interval, g_rec.precision, g_rec.algo,
                      g_rec.memtype, g_streams_created.load(), g_streams_destroyed.load()};
    std::memcpy(ints9, v, sizeof(v));
    dbl3[0] = g_rec.eps2;
    dbl3[1] = g_rec.damping;
    dbl3[2] = g_rec.dt;
}

}  // extern "C"
