// body_task_mgpu_gb300.cc -- BodySystemMGPU_GB300<T>, the drop-in for the
// UTC nbody multi-GPU task (one thread per GPU, a shard of the targets each).
#include "body_task_mgpu_gb300.h"

#include <chrono>
#include <cstdio>
#include <type_traits>

#include <cuda_runtime.h>

template <typename T>
void BodySystemMGPU_GB300<T>::initImpl(unsigned int numBodies, T softeningSquared, T damping, T *pos,
                                       T *vel)
{
    // body_task_mgpu.cu:18-57: thread 0 keeps the parameters and pointers;
    // every thread's range follows from its rank when it runs
    if (__localThreadId == 0) {
        m_numBodies = numBodies;
        m_softeningSquared = softeningSquared;
        m_damping = damping;
        m_pos = pos;
        m_vel = vel;
        m_cur.assign(__numLocalThreads, nullptr);
        m_dev.assign(__numLocalThreads, 0);
        m_first.assign(__numLocalThreads, 0);
        m_count.assign(__numLocalThreads, 0);
    }
    intra_Barrier();
}

namespace {

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

template <typename T>
void BodySystemMGPU_GB300<T>::runImpl(double runtime[][4], int loops, int outInterval, int blocksize,
                                      T deltaTime, T *outbuffer, iUtc::MemType memtype)
{
    (void)memtype;  // the shards copy straight from and to the caller's arrays
    const int rank = __localThreadId, nranks = __numLocalThreads;
    const cudaStream_t s = __streamId;
    const size_t row = 4 * sizeof(T);
    const auto t_all = std::chrono::steady_clock::now();
    double kernel = 0, copyin = 0, copyout = 0;
    int st = NB_OK;
    std::string what;
    auto fail = [&](int code, const char *where) {
        if (st == NB_OK) {
            st = code;
            what = std::string(where) + ": " + nb_last_error();
        }
    };
    auto cuda_fail = [&](cudaError_t e, const char *where) {
        if (e != cudaSuccess && st == NB_OK) {
            st = NB_ERR_CUDA;
            what = std::string(where) + ": " + cudaGetErrorString(e);
        }
    };

    // set-up: this thread's shard context on its device, every body's state
    nb_params p;
    nb_params_default(&p);
    p.n = (int)m_numBodies;
    p.precision = std::is_same<T, double>::value ? NB_F64 : NB_F32;
    p.algo = m_algo >= 0 ? m_algo : (std::is_same<T, double>::value ? NB_ALGO_EXACT : NB_ALGO_FAST);
    p.kick = m_kick;
    p.eps2 = (double)m_softeningSquared;
    p.damping = (double)m_damping;
    p.dt = (double)deltaTime;
    if (p.algo == NB_ALGO_EXACT) p.block = blocksize;
    if (rank == 0) m_status.store(NB_OK);  // before the set-up barrier: nobody sets it until the end
    nb_ctx *ctx = nullptr;
    auto t = std::chrono::steady_clock::now();
    int rc = nb_create_shard(&p, rank, nranks, &ctx);
    if (rc) fail(rc, "nb_create_shard");
    int info[4] = {0, 0, rank, nranks};
    if (!st && (rc = nb_shard_info(ctx, info))) fail(rc, "nb_shard_info");
    if (!st && (rc = nb_set_state(ctx, m_pos, m_vel, NB_HOST, (void *)s))) fail(rc, "nb_set_state");
    copyin += seconds_since(t);
    m_first[rank] = info[0];
    m_count[rank] = info[1];
    m_dev[rank] = __deviceId;
    if (st) m_setup_failed.store(1);
    intra_Barrier();
    bool stop = m_setup_failed.load() != 0;
    if (outInterval <= 0) outInterval = loops > 0 ? loops : 1;

    for (int i = 0; i < loops && !stop;) {
        // phase A: this thread's step; publish its current buffer
        t = std::chrono::steady_clock::now();
        if (!st && (rc = nb_step(ctx, 1, (void *)s))) fail(rc, "nb_step");
        if (!st) cuda_fail(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        kernel += seconds_since(t);
        void *cur = nullptr;
        if (!st && (rc = nb_state_ptrs(ctx, &cur, nullptr))) fail(rc, "nb_state_ptrs");
        m_cur[rank] = cur;
        ++i;
        if (!st && i % outInterval == 0 && info[1] > 0) {
            // this thread's range of the frame (body_task_mgpu.cu:156-160)
            t = std::chrono::steady_clock::now();
            const size_t frame = (size_t)(i / outInterval - 1) * 4 * (size_t)m_numBodies;
            cuda_fail(cudaMemcpyAsync(outbuffer + frame + 4 * (size_t)info[0],
                                      (const char *)cur + row * info[0], row * info[1],
                                      cudaMemcpyDeviceToHost, s),
                      "frame copy");
            if (!st) cuda_fail(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            copyout += seconds_since(t);
        }
        if (st) m_failed.store(1);
        intra_Barrier();
        if (m_failed.load()) break;
        // phase B: this thread's new range into every other thread's buffer
        if (nranks > 1 && i < loops && info[1] > 0) {
            t = std::chrono::steady_clock::now();
            for (int j = 0; j < nranks && !st; ++j) {
                if (j == rank) continue;
                cuda_fail(cudaMemcpyPeerAsync((char *)m_cur[j] + row * info[0], m_dev[j],
                                              (const char *)cur + row * info[0], __deviceId, row * info[1], s),
                          "cudaMemcpyPeerAsync");
            }
            if (!st) cuda_fail(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            copyin += seconds_since(t);
        }
        if (st) m_exchange_failed.store(1);
        intra_Barrier();
        stop = m_exchange_failed.load() != 0;
    }
    if (ctx) nb_destroy(ctx);
    if (st) {
        std::fprintf(stderr, "BodySystemMGPU_GB300::runImpl (thread %d): status %d: %s\n", rank, st,
                     what.c_str());
        int expected = NB_OK;
        m_status.compare_exchange_strong(expected, st);
    }
    if (runtime) {
        runtime[rank][0] = seconds_since(t_all);
        runtime[rank][1] = kernel;
        runtime[rank][2] = copyin;
        runtime[rank][3] = copyout;
    }
    intra_Barrier();
    if (rank == 0) {  // the next run starts clean
        m_setup_failed.store(0);
        m_failed.store(0);
        m_exchange_failed.store(0);
    }
    intra_Barrier();
}

template class BodySystemMGPU_GB300<float>;
template class BodySystemMGPU_GB300<double>;

// ---------------------------------------------------------------------------
// flat entry points, so that non-C++ callers (the test harness) can drive the
// multi-GPU task as the app does: `nthreads` threads, runtime[nthreads][4]
// ---------------------------------------------------------------------------
template <typename T>
static int mgpu_run(unsigned n, T eps2, T damping, T *pos, T *vel, double *runtime, int loops, int outInterval,
                    int blocksize, T dt, T *outbuffer, int nthreads, int algo)
{
    iUtc::Task<BodySystemMGPU_GB300<T>> nbody(iUtc::ProcList(nthreads, 0), iUtc::TaskType::gpu_task);
    if (algo >= 0) nbody.userObject()->setAlgo(algo);
    nbody.init(n, eps2, damping, pos, vel);
    nbody.run(reinterpret_cast<double(*)[4]>(runtime), loops, outInterval, blocksize, dt, outbuffer,
              iUtc::MemType::pageable);
    nbody.wait();
    return nbody.userObject()->lastStatus();
}

extern "C" {

int nbt_mgpu_run_f32(unsigned n, float eps2, float damping, float *pos, float *vel, double *runtime, int loops,
                     int outInterval, int blocksize, float dt, float *outbuffer, int nthreads, int algo)
{
    return mgpu_run<float>(n, eps2, damping, pos, vel, runtime, loops, outInterval, blocksize, dt, outbuffer,
                           nthreads, algo);
}

int nbt_mgpu_run_f64(unsigned n, double eps2, double damping, double *pos, double *vel, double *runtime,
                     int loops, int outInterval, int blocksize, double dt, double *outbuffer, int nthreads,
                     int algo)
{
    return mgpu_run<double>(n, eps2, damping, pos, vel, runtime, loops, outInterval, blocksize, dt, outbuffer,
                            nthreads, algo);
}

}  // extern "C"
