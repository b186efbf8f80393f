/*
 * body_task_mgpu_gb300.h -- drop-in replacement for the UTC nbody
 * multi-GPU task.
 *
 * Same class shape and signatures as the reference's BodySystemMGPU<T>
 * (benchapps/nbody/utc-snode-mgpu/mgpu/body_task_mgpu.h:16-44), a task of
 * several threads of one process, one GPU each:
 *   initImpl(numBodies, softeningSquared, damping, pos, vel) keeps the
 *     parameters and the caller's host pointers (body_task_mgpu.cu:18-57);
 *   runImpl(runtime[][4], loops, outInterval, blocksize, deltaTime,
 *     outbuffer, memtype): every thread advances its own range of target
 *     bodies for `loops` steps and writes that range of the positions after
 *     every outInterval-th step to outbuffer + (step/outInterval - 1)*4N;
 *     runtime[thread] gets {total, kernel, copyin, copyout} seconds
 *     (body_task_mgpu.cu:59-163).
 *
 * Design on GB300: each thread holds a shard context (nb_create_shard) on
 * its own device with every body's state resident in its HBM.  Per step a
 * thread launches its shard's step on its own stream, then copies its new
 * range straight into the other threads' position buffers (device-to-
 * device peer copies: NVLink between GPUs, a plain device copy when threads
 * share a GPU), where the reference copies every body's positions in from a
 * host buffer and its range back out (body_task_mgpu.cu:102-151).  Two
 * barriers a step keep the threads in lockstep: after every step (each
 * thread then knows the others' current buffers and that nobody still reads
 * them) and after every exchange.  No kernel waits for another thread's
 * work; the waits are host-side.
 *
 * T = float runs the directed fast kernel: whole target blocks per thread,
 * and the threads' results together equal a single-GPU NB_ALGO_FAST run bit
 * for bit.  T = double runs the reference-exact kernel with the reference's
 * split (n / threads bodies each, one more for the first n % threads),
 * equal to the sequential reference bit for bit.  setAlgo(NB_ALGO_EXACT)
 * takes the exact kernel for float too.  Errors do not stop the process:
 * the message goes to stderr and lastStatus() keeps the first failing
 * thread's code of the last run.
 */
#ifndef UTC_GB300_BODY_TASK_MGPU_GB300_H_
#define UTC_GB300_BODY_TASK_MGPU_GB300_H_

#include <atomic>
#include <string>
#include <vector>

#include "nbody_gb300.h"
#include "utc_standin.h"

template <typename T>
class BodySystemMGPU_GB300 : public UserTaskBase {
private:
    unsigned int m_numBodies = 0;
    T m_softeningSquared = T(0);
    T m_damping = T(1);
    T *m_pos = nullptr;
    T *m_vel = nullptr;
    int m_algo = -1;  // -1: default for T
    int m_kick = NB_KICK_REFERENCE;
    std::atomic<int> m_status{NB_OK};
    // a thread failed in one phase of the run: set only within that phase and
    // read by every thread after the barrier that ends it, so that all
    // threads leave the step loop at the same barrier
    std::atomic<int> m_setup_failed{0}, m_failed{0}, m_exchange_failed{0};
    std::vector<void *> m_cur;       // per thread: its context's current position buffer
    std::vector<int> m_dev;          // per thread: its device
    std::vector<int> m_first, m_count;

public:
    void initImpl(unsigned int numBodies, T softeningSquared, T damping, T *pos, T *vel);

    void runImpl(double runtime[][4], int loops, int outInterval, int blocksize, T deltaTime,
                 T *outbuffer, iUtc::MemType memtype);

    /* extensions (not in the reference): force algorithm and kick mode */
    void setAlgo(int algo) { m_algo = algo; }
    void setKick(int kick) { m_kick = kick; }
    int lastStatus() const { return m_status.load(); }
};

extern template class BodySystemMGPU_GB300<float>;
extern template class BodySystemMGPU_GB300<double>;

#endif
