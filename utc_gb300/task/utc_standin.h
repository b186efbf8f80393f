/*
 * utc_standin.h -- the part of UTC's task API that the nbody GPU task uses,
 * as a single-process stand-in (UTC itself needs MPI and Boost).
 *
 * Mirrors the reference's interface and threading contract:
 *  - Task<T>(ProcList, TaskType) creates the user object and one worker
 *    thread (UTC/include/Task.inc:624-855, UTC/src/gpu/TaskGPU.cc:195-343);
 *  - init(args...) / run(args...) bind T::initImpl / T::runImpl and enqueue
 *    them on the worker, returning at once (Task.inc:264-281, 432-445,
 *    TaskGPU.cc:345-363); wait() blocks until they have run (Task.inc:523-542,
 *    TaskGPU.cc:375-390);
 *  - a gpu_task worker selects its device and creates its own non-blocking
 *    stream before the first job and exposes them through the thread-locals
 *    UserTaskBase::__streamId / __deviceId (UTC/src/gpu/UtcGpuContext.cc:
 *    28-93, UTC/src/UserTaskBase.cc:64-119).
 * MemType mirrors UTC/include/gpu/GpuData.h:17-22.
 */
#ifndef UTC_GB300_UTC_STANDIN_H_
#define UTC_GB300_UTC_STANDIN_H_

#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>

namespace iUtc {

enum class MemType { unknown = -1, pageable, pinned, unified };
enum class TaskType { unknown = -1, cpu_task, gpu_task };

/* Placement of task threads.  Only single-process, single-thread placements
 * exist here: ProcList(rank) and ProcList(nthreads, rank) with nthreads 1. */
class ProcList {
public:
    explicit ProcList(int rank = 0) : m_threads(1), m_rank(rank) {}
    ProcList(int nthreads, int rank) : m_threads(nthreads), m_rank(rank) {}
    int threads() const { return m_threads; }
    int rank() const { return m_rank; }

private:
    int m_threads, m_rank;
};

/* UtcContext::getContext (UTC/src/UtcContext.cc:35-40) for one process. */
class UtcContext {
public:
    static UtcContext &getContext(int = 0, char ** = nullptr)
    {
        static UtcContext ctx;
        return ctx;
    }
    int numProcs() const { return 1; }
    int getProcRank() const { return 0; }
};

/* iUtc::Timer (UTC/include/Timer.h:25-71): wall seconds. */
class Timer {
public:
    void start() { m_t0 = std::chrono::steady_clock::now(); }
    double stop() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - m_t0).count();
    }

private:
    std::chrono::steady_clock::time_point m_t0 = std::chrono::steady_clock::now();
};

}  // namespace iUtc

/* Base of user tasks (UTC/include/UserTaskBase.h:28-104): the thread-locals a
 * task body reads. */
class UserTaskBase {
public:
    virtual ~UserTaskBase() {}
    static inline thread_local int __localThreadId = 0;
    static inline thread_local int __globalThreadId = 0;
    static inline thread_local int __processIdInWorld = 0;
    static inline thread_local cudaStream_t __streamId = nullptr;
    static inline thread_local int __deviceId = 0;
    int __numLocalThreads = 1;
    int __numGlobalThreads = 1;
    /* one thread per task here, so the intra-task barrier is a no-op */
    void intra_Barrier() {}
};

namespace iUtc {

template <class T>
class Task {
public:
    explicit Task(ProcList rl = ProcList(0), TaskType tt = TaskType::cpu_task, int device = -1)
        : m_type(tt), m_device(device), m_obj(new T())
    {
        (void)rl;
        m_thread = std::thread([this] { worker(); });
    }
    ~Task()
    {
        finish();
        delete m_obj;
    }
    Task(const Task &) = delete;
    Task &operator=(const Task &) = delete;

    template <typename... Args>
    void init(Args... args)
    {
        enqueue(std::bind(&T::initImpl, m_obj, args...));
    }
    template <typename... Args>
    void run(Args... args)
    {
        enqueue(std::bind(&T::runImpl, m_obj, args...));
    }
    template <typename... Args>
    void exec(void (T::*fn)(Args...), Args... args)
    {
        enqueue(std::bind(fn, m_obj, args...));
    }
    void wait()
    {
        std::unique_lock<std::mutex> lk(m_mu);
        m_cv.wait(lk, [this] { return m_jobs.empty() && !m_busy; });
    }
    void finish()
    {
        {
            std::lock_guard<std::mutex> lk(m_mu);
            if (m_stop) return;
            m_stop = true;
        }
        m_cv.notify_all();
        if (m_thread.joinable()) m_thread.join();
    }
    T *userObject() { return m_obj; }

private:
    void enqueue(std::function<void()> job)
    {
        {
            std::lock_guard<std::mutex> lk(m_mu);
            m_jobs.push_back(std::move(job));
        }
        m_cv.notify_all();
    }
    void worker()
    {
        cudaStream_t stream = nullptr;
        if (m_type == TaskType::gpu_task) {
            int dev = m_device;
            if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) dev = 0;
            if (cudaSetDevice(dev) != cudaSuccess ||
                cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) {
                std::fprintf(stderr, "Task: cannot set up device %d and its stream\n", dev);
                stream = nullptr;
            }
            UserTaskBase::__deviceId = dev;
            UserTaskBase::__streamId = stream;
        }
        UserTaskBase::__localThreadId = 0;
        UserTaskBase::__globalThreadId = 0;
        for (;;) {
            std::function<void()> job;
            {
                std::unique_lock<std::mutex> lk(m_mu);
                m_cv.wait(lk, [this] { return !m_jobs.empty() || m_stop; });
                if (m_jobs.empty()) break;  // stop requested and queue drained
                job = std::move(m_jobs.front());
                m_jobs.pop_front();
                m_busy = true;
            }
            job();
            {
                std::lock_guard<std::mutex> lk(m_mu);
                m_busy = false;
            }
            m_cv.notify_all();
        }
        if (stream) cudaStreamDestroy(stream);
    }

    TaskType m_type;
    int m_device;
    T *m_obj;
    std::thread m_thread;
    std::mutex m_mu;
    std::condition_variable m_cv;
    std::deque<std::function<void()>> m_jobs;
    bool m_busy = false;
    bool m_stop = false;
};

}  // namespace iUtc

#endif
