// body_task_gb300.cc -- BodySystemGB300<T>, the UTC nbody task drop-in.
#include "body_task_gb300.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <type_traits>

#include <cuda_runtime.h>

#include "nbody_init.h"

template <typename T>
void BodySystemGB300<T>::initImpl(unsigned int numBodies, T softeningSquared, T damping, T *pos,
                                  T *vel)
{
    // body_task_sgpu.cu:14-38: thread 0 keeps the parameters and the host
    // pointers; the arrays are read at run time, not copied here
    if (__localThreadId == 0) {
        m_numBodies = numBodies;
        m_softeningSquared = softeningSquared;
        m_damping = damping;
        m_pos = pos;
        m_vel = vel;
    }
    intra_Barrier();
}

// nb_destroy / nb_batch_destroy keep what they were given while another
// thread of the process is capturing a graph (the device cannot be
// synchronised then): try again for up to ten seconds for that capture to end
template <typename F>
static void destroy_when_possible(F destroy)
{
    for (int k = 0; k < 1000 && destroy() != NB_OK; ++k) std::this_thread::sleep_for(std::chrono::milliseconds(10));
}

template <typename T>
void BodySystemGB300<T>::runImpl(double *runtime, int loops, int outInterval, int blocksize,
                                 T deltaTime, T *outbuffer, iUtc::MemType memtype)
{
    nb_params p;
    nb_params_default(&p);
    p.n = (int)m_numBodies;
    p.precision = std::is_same<T, double>::value ? NB_F64 : NB_F32;
    p.algo = m_algo >= 0 ? m_algo : NB_ALGO_SYM;
    p.kick = m_kick;
    p.eps2 = (double)m_softeningSquared;
    p.damping = (double)m_damping;
    p.dt = (double)deltaTime;
    if (p.algo == NB_ALGO_EXACT) p.block = blocksize;
    p.memtype = memtype == iUtc::MemType::pinned    ? NB_MEM_PINNED
                : memtype == iUtc::MemType::unified ? NB_MEM_UNIFIED
                                                    : NB_MEM_PAGEABLE;
    if (m_group) {
        BodyTaskGroupMember<T> m{m_numBodies, m_softeningSquared, m_damping, deltaTime, m_pos, m_vel, loops,
                                 outInterval, m_algo, m_kick, outbuffer, runtime};
        m_status = m_group->join(&m);
        if (m_status != NB_OK)
            std::fprintf(stderr, "BodySystemGB300::runImpl: status %d: %s\n", m_status, m.error.c_str());
        return;
    }
    double t[4] = {0, 0, 0, 0};
    nb_ctx *ctx = nullptr;
    int st = nb_create(&p, &ctx);
    if (st == NB_OK)
        st = nb_run_host(ctx, m_pos, m_vel, loops, outInterval, outbuffer, t,
                         (void *)__streamId);
    if (st != NB_OK)
        std::fprintf(stderr, "BodySystemGB300::runImpl: status %d: %s\n", st, nb_last_error());
    if (ctx) destroy_when_possible([ctx] { return nb_destroy(ctx); });
    m_status = st;
    if (runtime)
        for (int k = 0; k < 4; ++k) runtime[k] = t[k];
}

template <typename T>
int BodyTaskGroup<T>::join(BodyTaskGroupMember<T> *m)
{
    std::unique_lock<std::mutex> lk(m_mu);
    m->taken = m->done = false;
    m_arrived.push_back(m);
    if ((int)m_arrived.size() == m_members) {  // the last to arrive runs the round
        std::vector<BodyTaskGroupMember<T> *> ms;
        ms.swap(m_arrived);
        for (auto *x : ms) x->taken = true;
        lk.unlock();
        runBatch(ms);
        lk.lock();
        for (auto *x : ms) x->done = true;
        m_cv.notify_all();
        return m->status;
    }
    if (!m_cv.wait_for(lk, std::chrono::duration<double>(m_timeout), [m] { return m->taken; })) {
        // the round did not fill in time: it ends for every member that came
        for (auto *x : m_arrived) {
            x->status = NB_ERR_STATE;
            x->error = "task group: " + std::to_string(m_arrived.size()) + " of " + std::to_string(m_members) +
                       " members arrived within the timeout";
            x->done = true;
        }
        m_arrived.clear();
        m_cv.notify_all();
        return m->status;
    }
    m_cv.wait(lk, [m] { return m->done; });  // the round's batch is running
    return m->status;
}

// The members' systems concatenated into one nb_batch on a stream of its
// own; frames and timers as runImpl writes them for one system.
template <typename T>
int BodyTaskGroup<T>::runBatch(const std::vector<BodyTaskGroupMember<T> *> &ms)
{
    const auto t0 = std::chrono::steady_clock::now();
    const BodyTaskGroupMember<T> &a = *ms[0];
    std::string msg;
    int st = NB_OK;
    for (auto *x : ms)
        if (x->eps2 != a.eps2 || x->damping != a.damping || x->dt != a.dt || x->loops != a.loops ||
            x->outInterval != a.outInterval || x->algo != a.algo || x->kick != a.kick) {
            st = NB_ERR_INVALID;
            msg = "task group: members differ in eps2, damping, dt, loops, outInterval, algorithm or kick mode";
        }
    if (!st && (a.loops < 0 || a.outInterval <= 0)) {
        st = NB_ERR_INVALID;
        msg = "task group: loops must be >= 0 and outInterval > 0";
    }
    for (auto *x : ms)
        if (!st && x->n > 0 && (!x->pos || !x->vel || (a.loops >= a.outInterval && !x->outbuffer))) {
            st = NB_ERR_INVALID;
            msg = "task group: a member's pos, vel or outbuffer is NULL";
        }
    const int nsys = (int)ms.size();
    std::vector<int> sizes(nsys);
    std::vector<size_t> off(nsys + 1, 0);
    for (int i = 0; i < nsys; ++i) {
        sizes[i] = (int)ms[i]->n;
        off[i + 1] = off[i] + 4 * (size_t)ms[i]->n;
    }
    nb_params p;
    nb_params_default(&p);
    p.precision = std::is_same<T, double>::value ? NB_F64 : NB_F32;
    p.algo = a.algo >= 0 ? a.algo : NB_ALGO_SYM;
    p.kick = a.kick;
    p.eps2 = (double)a.eps2;
    p.damping = (double)a.damping;
    p.dt = (double)a.dt;
    std::vector<T> P(off[nsys]), V(off[nsys]);
    for (int i = 0; i < nsys && !st; ++i) {
        std::memcpy(&P[off[i]], ms[i]->pos, 4 * (size_t)ms[i]->n * sizeof(T));
        std::memcpy(&V[off[i]], ms[i]->vel, 4 * (size_t)ms[i]->n * sizeof(T));
    }
    const bool batchable = p.algo == NB_ALGO_SYM || (p.precision == NB_F32 && p.algo == NB_ALGO_FAST);
    if (!st && !batchable) {
        // the reference-exact and FP64-pipe kernels have no batched form:
        // the members' systems run one after another, each as runImpl runs
        // it alone, each member with its own timers
        cudaStream_t s1 = nullptr;
        if (cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking) != cudaSuccess) {
            st = NB_ERR_CUDA;
            msg = "task group: cannot create the run's stream";
        }
        for (auto *x : ms) {
            double t[4] = {0, 0, 0, 0};
            nb_params q = p;
            q.n = (int)x->n;
            nb_ctx *ctx = nullptr;
            int sx = st ? st : nb_create(&q, &ctx);
            if (!sx) sx = nb_run_host(ctx, x->pos, x->vel, a.loops, a.outInterval, x->outbuffer, t, (void *)s1);
            x->status = sx;
            x->error = sx && !st ? nb_last_error() : msg;
            if (ctx) destroy_when_possible([ctx] { return nb_destroy(ctx); });
            if (x->runtime && !sx)
                for (int k = 0; k < 4; ++k) x->runtime[k] = t[k];
        }
        if (s1) cudaStreamDestroy(s1);
        return st;
    }
    nb_batch *b = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e[4] = {};
    float copyin = 0.f, kernel = 0.f, copyout = 0.f, ms_ = 0.f;
    if (!st && (st = nb_batch_create(&p, nsys, sizes.data(), &b))) msg = nb_last_error();
    if (!st && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        st = NB_ERR_CUDA;
        msg = "task group: cannot create the batch's stream";
    }
    for (int k = 0; k < 4 && !st; ++k)
        if (cudaEventCreate(&e[k]) != cudaSuccess) {
            st = NB_ERR_CUDA;
            msg = "task group: cannot create timing events";
        }
    if (!st) {
        cudaEventRecord(e[0], s);
        if ((st = nb_batch_set_state(b, P.data(), V.data(), NB_HOST, s))) msg = nb_last_error();
        cudaEventRecord(e[1], s);
        cudaEventSynchronize(e[1]);
        cudaEventElapsedTime(&copyin, e[0], e[1]);
    }
    // frame f after (f + 1) * outInterval steps, to outbuffer + f * 4N
    for (int done = 0; !st && done < a.loops;) {
        const int upto = std::min(a.loops, (done / a.outInterval + 1) * a.outInterval);
        cudaEventRecord(e[0], s);
        if ((st = nb_batch_run(b, upto - done, s))) msg = nb_last_error();
        cudaEventRecord(e[1], s);
        done = upto;
        if (!st && done % a.outInterval == 0) {
            cudaEventRecord(e[2], s);
            if ((st = nb_batch_get_state(b, P.data(), nullptr, NB_HOST, s))) msg = nb_last_error();
            cudaEventRecord(e[3], s);
            cudaEventSynchronize(e[3]);
            cudaEventElapsedTime(&ms_, e[2], e[3]);
            copyout += ms_;
            const size_t f = (size_t)(done / a.outInterval - 1);
            for (int i = 0; i < nsys && !st; ++i)
                std::memcpy(ms[i]->outbuffer + f * 4 * (size_t)ms[i]->n, &P[off[i]],
                            4 * (size_t)ms[i]->n * sizeof(T));
        }
        cudaEventSynchronize(e[1]);
        cudaEventElapsedTime(&ms_, e[0], e[1]);
        kernel += ms_;
    }
    for (auto &x : e)
        if (x) cudaEventDestroy(x);
    if (s) cudaStreamDestroy(s);
    if (b) destroy_when_possible([b] { return nb_batch_destroy(b); });
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (auto *x : ms) {
        x->status = st;
        x->error = msg;
        if (x->runtime && !st) {
            x->runtime[0] = total;
            x->runtime[1] = kernel * 1e-3;
            x->runtime[2] = copyin * 1e-3;
            x->runtime[3] = copyout * 1e-3;
        }
    }
    return st;
}

template class BodySystemGB300<float>;
template class BodySystemGB300<double>;
template class BodyTaskGroup<float>;
template class BodyTaskGroup<double>;

// ---------------------------------------------------------------------------
// flat entry points of the task library, so that non-C++ callers (the test
// harness) can drive the task exactly as the app does
// ---------------------------------------------------------------------------
template <typename T>
static int task_run(unsigned n, T eps2, T damping, T *pos, T *vel, double *runtime, int loops,
                    int outInterval, int blocksize, T dt, T *outbuffer, int memtype, int algo,
                    int device)
{
    iUtc::Task<BodySystemGB300<T>> nbody(iUtc::ProcList(0), iUtc::TaskType::gpu_task, device);
    nbody.userObject()->setAlgo(algo);
    nbody.init(n, eps2, damping, pos, vel);
    nbody.run(runtime, loops, outInterval, blocksize, dt, outbuffer,
              memtype == 1 ? iUtc::MemType::pinned
                           : (memtype == 2 ? iUtc::MemType::unified : iUtc::MemType::pageable));
    nbody.wait();
    return nbody.userObject()->lastStatus();
}

// nsys tasks in one group of `members` (members > nsys leaves the group
// short, so that its timeout ends the round), each run as the app runs it;
// eps2[i] is system i's softening squared (members must agree on it)
template <typename T>
static int task_group_run(int nsys, const int *sizes, T **pos, T **vel, T **out, const T *eps2, T damping, T dt,
                          int loops, int outInterval, int members, double timeout_s, int *status,
                          double *runtime)
{
    BodyTaskGroup<T> group(members, timeout_s);
    std::vector<std::unique_ptr<iUtc::Task<BodySystemGB300<T>>>> tasks;
    for (int i = 0; i < nsys; ++i) {
        tasks.emplace_back(new iUtc::Task<BodySystemGB300<T>>(iUtc::ProcList(0), iUtc::TaskType::gpu_task));
        tasks[i]->userObject()->setGroup(&group);
        tasks[i]->init((unsigned)sizes[i], eps2[i], damping, pos[i], vel[i]);
    }
    for (int i = 0; i < nsys; ++i)
        tasks[i]->run(runtime ? runtime + 4 * i : (double *)nullptr, loops, outInterval, 256, dt, out[i],
                      iUtc::MemType::pageable);
    int worst = NB_OK;
    for (int i = 0; i < nsys; ++i) {
        tasks[i]->wait();
        status[i] = tasks[i]->userObject()->lastStatus();
        if (status[i] != NB_OK) worst = status[i];
    }
    return worst;
}

extern "C" {

int nbt_group_run_f32(int nsys, const int *sizes, float **pos, float **vel, float **out, const float *eps2,
                      float damping, float dt, int loops, int outInterval, int members, double timeout_s,
                      int *status, double *runtime)
{
    return task_group_run<float>(nsys, sizes, pos, vel, out, eps2, damping, dt, loops, outInterval, members,
                                 timeout_s, status, runtime);
}

int nbt_group_run_f64(int nsys, const int *sizes, double **pos, double **vel, double **out, const double *eps2,
                      double damping, double dt, int loops, int outInterval, int members, double timeout_s,
                      int *status, double *runtime)
{
    return task_group_run<double>(nsys, sizes, pos, vel, out, eps2, damping, dt, loops, outInterval, members,
                                  timeout_s, status, runtime);
}

int nbt_run_f32(unsigned n, float eps2, float damping, float *pos, float *vel, double *runtime,
                int loops, int outInterval, int blocksize, float dt, float *outbuffer,
                int memtype, int algo, int device)
{
    return task_run<float>(n, eps2, damping, pos, vel, runtime, loops, outInterval, blocksize, dt,
                           outbuffer, memtype, algo, device);
}

int nbt_run_f64(unsigned n, double eps2, double damping, double *pos, double *vel,
                double *runtime, int loops, int outInterval, int blocksize, double dt,
                double *outbuffer, int memtype, int algo, int device)
{
    return task_run<double>(n, eps2, damping, pos, vel, runtime, loops, outInterval, blocksize,
                            dt, outbuffer, memtype, algo, device);
}

/* The app's initialiser task (NbodyInit<T>, nbody_init.h) from a fresh
 * rand() state: srand(seed), then randomizeBodies(config). */
int nbt_randomize_f32(int config, float *pos, float *vel, float clusterScale,
                      float velocityScale, int n, unsigned seed)
{
    std::srand(seed);
    iUtc::Task<NbodyInit<float>> init(iUtc::ProcList(0));
    init.run((NBodyConfig)config, pos, vel, (float *)nullptr, clusterScale, velocityScale, n, true);
    init.wait();
    return 0;
}

int nbt_randomize_f64(int config, double *pos, double *vel, float clusterScale,
                      float velocityScale, int n, unsigned seed)
{
    std::srand(seed);
    iUtc::Task<NbodyInit<double>> init(iUtc::ProcList(0));
    init.run((NBodyConfig)config, pos, vel, (float *)nullptr, clusterScale, velocityScale, n, true);
    init.wait();
    return 0;
}

}  // extern "C"
