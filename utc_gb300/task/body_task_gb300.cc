// body_task_gb300.cc -- BodySystemGB300<T>, the UTC nbody task drop-in.
#include "body_task_gb300.h"

#include <cstdio>
#include <cstdlib>
#include <type_traits>

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
    double t[4] = {0, 0, 0, 0};
    nb_ctx *ctx = nullptr;
    int st = nb_create(&p, &ctx);
    if (st == NB_OK)
        st = nb_run_host(ctx, m_pos, m_vel, loops, outInterval, outbuffer, t,
                         (void *)__streamId);
    if (st != NB_OK)
        std::fprintf(stderr, "BodySystemGB300::runImpl: status %d: %s\n", st, nb_last_error());
    nb_destroy(ctx);
    m_status = st;
    if (runtime)
        for (int k = 0; k < 4; ++k) runtime[k] = t[k];
}

template class BodySystemGB300<float>;
template class BodySystemGB300<double>;

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

extern "C" {

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
