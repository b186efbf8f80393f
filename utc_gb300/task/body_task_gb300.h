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

#include "nbody_gb300.h"
#include "utc_standin.h"

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

public:
    void initImpl(unsigned int numBodies, T softeningSquared, T damping, T *pos, T *vel);

    void runImpl(double *runtime, int loops, int outInterval, int blocksize, T deltaTime,
                 T *outbuffer, iUtc::MemType memtype);

    /* extensions (not in the reference): force algorithm and kick mode */
    void setAlgo(int algo) { m_algo = algo; }
    void setKick(int kick) { m_kick = kick; }
    int lastStatus() const { return m_status; }
};

extern template class BodySystemGB300<float>;
extern template class BodySystemGB300<double>;

#endif
