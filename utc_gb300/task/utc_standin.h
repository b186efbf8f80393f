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
 *    28-93, UTC/src/UserTaskBase.cc:64-119);
 *  - a task placed on ProcList(nthreads, rank) has nthreads worker threads:
 *    every job runs on all of them (UTC runs a task's initImpl/runImpl on
 *    each of its threads, UTC/src/gpu/TaskGPU.cc:170-178), with
 *    __localThreadId = 0..nthreads-1, __numLocalThreads = nthreads and
 *    intra_Barrier() a barrier of the task's threads (UTC/src/Barrier.cc:
 *    173); thread k of a gpu_task uses device k % (device count), as UTC's
 *    CudaDeviceManager::getAvailableGpu does (CudaDeviceManager.cc:141-143),
 *    unless the task was given a device.
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
#include <memory>
#include <thread>
#include <vector>

namespace iUtc {

enum class MemType { unknown = -1, pageable, pinned, unified };
enum class TaskType { unknown = -1, cpu_task, gpu_task };

/* Placement of task threads: one process; ProcList(rank) is one thread,
 * ProcList(nthreads, rank) nthreads threads of that process. */
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

namespace iUtc {

/* A reusable barrier of a fixed number of threads. */
class ThreadBarrier {
public:
    explicit ThreadBarrier(int n) : m_n(n) {}
    void wait()
    {
        std::unique_lock<std::mutex> lk(m_mu);
        const unsigned long long gen = m_gen;
        if (++m_count == m_n) {
            m_count = 0;
            ++m_gen;
            m_cv.notify_all();
        } else {
            m_cv.wait(lk, [&] { return m_gen != gen; });
        }
    }

private:
    std::mutex m_mu;
    std::condition_variable m_cv;
    int m_n, m_count = 0;
    unsigned long long m_gen = 0;
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
    /* barrier of the task's threads (a no-op for a one-thread task) */
    void intra_Barrier()
    {
        if (__barrier) __barrier->wait();
    }
    std::shared_ptr<iUtc::ThreadBarrier> __barrier;
};

namespace iUtc {

template <class T>
class Task {
public:
    explicit Task(ProcList rl = ProcList(0), TaskType tt = TaskType::cpu_task, int device = -1)
        : m_type(tt), m_device(device), m_obj(new T())
    {
        m_nthreads = rl.threads() > 0 ? rl.threads() : 1;
        m_obj->__numLocalThreads = m_nthreads;
        m_obj->__numGlobalThreads = m_nthreads;
        if (m_nthreads > 1) m_obj->__barrier = std::make_shared<ThreadBarrier>(m_nthreads);
        m_next.assign(m_nthreads, 0);
        for (int k = 0; k < m_nthreads; ++k) m_threads.emplace_back([this, k] { worker(k); });
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
    /* until every thread has run every job enqueued so far */
    void wait()
    {
        std::unique_lock<std::mutex> lk(m_mu);
        m_cv.wait(lk, [this] {
            for (size_t x : m_next)
                if (x < m_jobs.size()) return false;
            return m_busy == 0;
        });
    }
    void finish()
    {
        {
            std::lock_guard<std::mutex> lk(m_mu);
            if (m_stop) return;
            m_stop = true;
        }
        m_cv.notify_all();
        for (auto &t : m_threads)
            if (t.joinable()) t.join();
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
    void worker(int k)
    {
        cudaStream_t stream = nullptr;
        if (m_type == TaskType::gpu_task) {
            int dev = m_device;
            if (dev < 0 && m_nthreads > 1) {
                int count = 0;
                if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) count = 1;
                dev = k % count;
            }
            if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) dev = 0;
            if (cudaSetDevice(dev) != cudaSuccess ||
                cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) {
                std::fprintf(stderr, "Task: cannot set up device %d and its stream\n", dev);
                stream = nullptr;
            }
            UserTaskBase::__deviceId = dev;
            UserTaskBase::__streamId = stream;
        }
        UserTaskBase::__localThreadId = k;
        UserTaskBase::__globalThreadId = k;
        for (;;) {
            std::function<void()> job;
            {
                std::unique_lock<std::mutex> lk(m_mu);
                m_cv.wait(lk, [this, k] { return m_next[k] < m_jobs.size() || m_stop; });
                if (m_next[k] >= m_jobs.size()) break;  // stop requested and every job run
                job = m_jobs[m_next[k]];
                ++m_busy;
            }
            job();
            {
                std::lock_guard<std::mutex> lk(m_mu);
                ++m_next[k];
                --m_busy;
            }
            m_cv.notify_all();
        }
        if (stream) cudaStreamDestroy(stream);
    }

    TaskType m_type;
    int m_device;
    int m_nthreads = 1;
    T *m_obj;
    std::vector<std::thread> m_threads;
    std::mutex m_mu;
    std::condition_variable m_cv;
    std::vector<std::function<void()>> m_jobs;  // every job, in order; run by every thread
    std::vector<size_t> m_next;                 // per thread: the next job to run
    int m_busy = 0;
    bool m_stop = false;
};

}  // namespace iUtc

#endif
