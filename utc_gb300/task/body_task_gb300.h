/*
 * body_task_gb300.h -- drop-in replacement for the UTC nbody GPU task.
 *
 * Same class shape and signatures as the reference's BodySystemSGPU<T>
 * (benchapps/nbody/utc/sgpu/body_task_sgpu.h:16-41):
 *   initImpl(numBodies, softeningSquared, damping, pos, vel) stores the
 *     parameters and the caller's host pointers without copying
 *     (body_task_sgpu.cu:14-38);
 *   runImpl(runtime[4], loops, outInterval, blocksize, deltaTime, outbuffer,
 *     memtype) copies the state to the GPU, runs `loops` steps on the task's
 *     stream and writes the positions after every outInterval-th step to
 *     outbuffer + (step/outInterval - 1)*4N; runtime[] gets {total, kernel,
 *     copyin, copyout} seconds (body_task_sgpu.cu:40-137).
 * The work goes through the C ABI (include/nbody_gb300.h) on
 * UserTaskBase::__streamId.  Both state types run the symmetric kernel
 * (NB_ALGO_SYM) by default: in FP32 for T = float; for T = double with
 * FP64-accurate float-float pair terms on the FP32 pipe (not bit-identical
 * to the sequential reference; setAlgo(NB_ALGO_SYM_FP64) keeps FP64
 * arithmetic throughout, setAlgo(NB_ALGO_EXACT) gives the reference-exact
 * kernel).  `blocksize` is
 * the CTA size of the exact kernel; the other kernels choose their own
 * launch shape.
 * Errors do not stop the process: the message goes to stderr (as the
 * reference's checkCudaErr does) and lastStatus() keeps the code.
 */
#ifndef UTC_GB300_BODY_TASK_GB300_H_
#define UTC_GB300_BODY_TASK_GB300_H_

#include <condition_variable>
#include <mutex>
#include <string>
#include <vector>

#include "nbody_gb300.h"
#include "utc_standin.h"

template <typename T>
class BodyTaskGroup;

template <typename T>
class BodySystemGB300 : public UserTaskBase {
private:
    unsigned int m_numBodies = 0;
    T *m_pos = nullptr;
    T *m_vel = nullptr;
    T m_softeningSquared = T(0);
    T m_damping = T(1);
    int m_algo = -1;  // -1: default for T
    int m_kick = NB_KICK_REFERENCE;
    int m_status = NB_OK;
    BodyTaskGroup<T> *m_group = nullptr;

public:
    void initImpl(unsigned int numBodies, T softeningSquared, T damping, T *pos, T *vel);

    void runImpl(double *runtime, int loops, int outInterval, int blocksize, T deltaTime,
                 T *outbuffer, iUtc::MemType memtype);

    /* extensions (not in the reference): force algorithm and kick mode */
    void setAlgo(int algo) { m_algo = algo; }
    void setKick(int kick) { m_kick = kick; }
    /* run as a member of a group (below); nullptr: run alone */
    void setGroup(BodyTaskGroup<T> *group) { m_group = group; }
    int lastStatus() const { return m_status; }
};

/* What a task hands to its group: its system, its run's arguments and
 * where its results go. */
template <typename T>
struct BodyTaskGroupMember {
    unsigned int n;
    T eps2, damping, dt;
    const T *pos, *vel;
    int loops, outInterval, algo, kick;
    T *outbuffer;
    double *runtime;
    int status = NB_OK;
    std::string error;   // the message behind a failing status
    bool taken = false;  // a member's round has started running
    bool done = false;   // ... and has finished
};

/* Extension (not in the reference): tasks whose runs go as one batch.  The
 * reference's multi-task app (benchapps/nbody/utc/nbody_mtask.cc:199-231)
 * runs one Task<BodySystemSGPU> per system, each on its own stream.  Tasks
 * given the same group meet in runImpl; the last to arrive runs every
 * member's system as one nb_batch (one launch pair per step for all
 * systems, each frame's steps one CUDA graph) on its own stream, then
 * writes every member's frames and timers, and the others return with it.
 * Algorithms without a batched kernel (NB_ALGO_EXACT, NB_ALGO_SYM_FP64) run
 * the members' systems one after another instead, each as it runs alone.
 * Members may differ in N; they must share eps2, damping, dt, loops,
 * outInterval, algorithm and kick mode, else every member of that round
 * gets NB_ERR_INVALID.  A member waits at most timeout_s for the group to
 * fill; a round that does not fill in time ends with NB_ERR_STATE for the
 * members that came, whose outbuffers stay untouched.  memtype and
 * blocksize do not apply (the batch copies from the caller's arrays and
 * chooses its own launch shape).  A group serves any number of rounds of
 * `members` runs each. */
template <typename T>
class BodyTaskGroup {
public:
    explicit BodyTaskGroup(int members, double timeout_s = 600.0)
        : m_members(members > 0 ? members : 1), m_timeout(timeout_s)
    {
    }
    int members() const { return m_members; }
    /* called by runImpl on the member's task thread; returns its status */
    int join(BodyTaskGroupMember<T> *m);

private:
    int runBatch(const std::vector<BodyTaskGroupMember<T> *> &ms);

    const int m_members;
    const double m_timeout;
    std::mutex m_mu;
    std::condition_variable m_cv;
    std::vector<BodyTaskGroupMember<T> *> m_arrived;
    long long m_round = 0;  // rounds finished or abandoned
    bool m_running = false;
};

extern template class BodySystemGB300<float>;
extern template class BodySystemGB300<double>;
extern template class BodyTaskGroup<float>;
extern template class BodyTaskGroup<double>;

#endif
