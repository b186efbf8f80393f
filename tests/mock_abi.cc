// mock_abi.cc -- host-only stand-in for the C ABI (include/nbody_gb300.h)
// and the four CUDA runtime calls of the UTC task stand-in, so that the
// drop-in task (utc_gb300/task/body_task_gb300.cc) runs without a GPU.
// Test infrastructure: nb_run_host steps with the oracle's C restatement
// (oracle/nbody_oracle.c) and records what the task handed over.
#include <cuda_runtime.h>

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
    int streams_created = 0, streams_destroyed = 0;
} g_rec;

}  // namespace

struct nb_ctx {
    nb_params p;
};

extern "C" {

// ---- CUDA runtime calls of utc_standin.h ----
cudaError_t cudaGetDevice(int *dev)
{
    *dev = 0;
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned int)
{
    *s = g_fake_stream;
    ++g_rec.streams_created;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t) { ++g_rec.streams_destroyed; return cudaSuccess; }

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

// ---- what the test reads back ----
void *mock_fake_stream(void) { return g_fake_stream; }
void mock_record(void **stream, int *ints9, double *dbl3)
{
    *stream = g_rec.stream;
    const int v[9] = {g_rec.calls, g_rec.n, g_rec.loops, g_rec.out_interval, g_rec.precision, g_rec.algo,
                      g_rec.memtype, g_rec.streams_created, g_rec.streams_destroyed};
    std::memcpy(ints9, v, sizeof(v));
    dbl3[0] = g_rec.eps2;
    dbl3[1] = g_rec.damping;
    dbl3[2] = g_rec.dt;
}

}  // extern "C"
