/*
 * nbody_mtask_main.cc -- the multi-task nbody app on GB300, with the
 * reference's flags and flow (benchapps/nbody/utc/nbody_mtask.cc:55-272):
 * T systems of N bodies each, initialised one after another from the same
 * rand() stream (NbodyInit, SHELL), advanced `-l` steps with a frame every
 * `-o` steps, timers printed as the reference prints them.
 *
 *   -v print timers      -t threads (must be 1)   -p processes (must be 1)
 *   -m 0|1|2 memtype     -i preset 0..6           -l iterations
 *   -o output interval   -n bodies per system     -b block size
 *   -T number of systems (tasks)
 * additions:
 *   -B 1|0|2  1 (default): all systems in one batched launch per step
 *           (nb_batch_*, one CUDA graph); 0: the reference's pattern, one
 *           Task<BodySystemGB300<T>> per system, all running at once; 2:
 *           one task per system as in 0, the tasks joined in one
 *           BodyTaskGroup, so that their runs go as one batch
 *   -F      float state (the reference fixes FTYPE=double)
 *   -a 0|2  batched force algorithm for float state: 0 directed, 2 symmetric
 *           (default); double-state batches run the float-float symmetric
 *           kernel.  With -B 0 and -B 2 the value goes to every task
 *           (setAlgo; -a 1 and -a 3 also serve single tasks there)
 *   -O file write every system's frames (system 0's frames, then system
 *           1's, ...) in the app's text format; the reference parses -O
 *           and writes nothing
 * The reference's time_record.txt bookkeeping (print_time) is the benchmark
 * scripts', not the app's, and is not kept.
 */
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <vector>
#include <unistd.h>

#include <cuda_runtime.h>

#include "body_task_gb300.h"
#include "nbody_init.h"

using namespace iUtc;

template <typename FTYPE>
static int run_batched(int ntasks, int numBodies, int iteration, int outInterval, const NBodyParams &prm,
                       std::vector<FTYPE *> &pos, std::vector<FTYPE *> &vel, std::vector<FTYPE *> &out,
                       int algo, double runtime[4])
{
    const bool f64 = sizeof(FTYPE) == 8;
    const size_t per = (size_t)numBodies * 4;
    std::vector<FTYPE> P(per * ntasks), V(per * ntasks);
    for (int i = 0; i < ntasks; ++i) {
        std::memcpy(&P[per * i], pos[i], per * sizeof(FTYPE));
        std::memcpy(&V[per * i], vel[i], per * sizeof(FTYPE));
    }
    nb_params p;
    nb_params_default(&p);
    p.precision = f64 ? NB_F64 : NB_F32;
    p.algo = f64 ? NB_ALGO_SYM : (algo >= 0 ? algo : NB_ALGO_SYM);
    p.kick = NB_KICK_REFERENCE;
    p.eps2 = (double)((FTYPE)prm.m_softening * (FTYPE)prm.m_softening);
    p.damping = (double)(FTYPE)prm.m_damping;
    p.dt = (double)(FTYPE)prm.m_timestep;
    std::vector<int> sizes(ntasks, numBodies);
    nb_batch *b = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    int st = nb_batch_create(&p, ntasks, sizes.data(), &b);
    cudaStream_t s = nullptr;
    cudaEvent_t e[4] = {};
    if (!st && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) st = NB_ERR_CUDA;
    for (int k = 0; k < 4 && !st; ++k)
        if (cudaEventCreate(&e[k]) != cudaSuccess) st = NB_ERR_CUDA;
    float copyin = 0.f, kernel = 0.f, copyout = 0.f, ms = 0.f;
    if (!st) {
        cudaEventRecord(e[0], s);
        st = nb_batch_set_state(b, P.data(), V.data(), NB_HOST, s);
        cudaEventRecord(e[1], s);
        cudaEventSynchronize(e[1]);
        cudaEventElapsedTime(&copyin, e[0], e[1]);
    }
    // frame f after (f + 1) * outInterval steps, to out[i] + f * 4N
    for (int done = 0; !st && done < iteration;) {
        const int upto = std::min(iteration, (done / outInterval + 1) * outInterval);
        cudaEventRecord(e[0], s);
        st = nb_batch_run(b, upto - done, s);
        cudaEventRecord(e[1], s);
        done = upto;
        if (!st && done % outInterval == 0) {
            cudaEventRecord(e[2], s);
            st = nb_batch_get_state(b, P.data(), nullptr, NB_HOST, s);
            cudaEventRecord(e[3], s);
            cudaEventSynchronize(e[3]);
            cudaEventElapsedTime(&ms, e[2], e[3]);
            copyout += ms;
            const int f = done / outInterval - 1;
            for (int i = 0; i < ntasks && !st; ++i)
                std::memcpy(out[i] + (size_t)f * per, &P[per * i], per * sizeof(FTYPE));
        }
        cudaEventSynchronize(e[1]);
        cudaEventElapsedTime(&ms, e[0], e[1]);
        kernel += ms;
    }
    if (st) std::cerr << "nbody_mtask: status " << st << ": " << nb_last_error() << std::endl;
    for (auto &x : e)
        if (x) cudaEventDestroy(x);
    if (s) cudaStreamDestroy(s);
    nb_batch_destroy(b);
    runtime[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    runtime[1] = kernel * 1e-3;
    runtime[2] = copyin * 1e-3;
    runtime[3] = copyout * 1e-3;
    return st;
}

template <typename FTYPE>
static int run_app(bool printTime, int paraSelect, int iteration, int outInterval, int numBodies, int ntasks,
                   const char *outfilename, int blocksize, MemType memtype, int mode, int algo)
{
    NBodyParams activeParams = nbody_demo_params(paraSelect, numBodies);
    const int frames = iteration / outInterval + 1;
    const size_t per = (size_t)numBodies * 4;
    std::vector<FTYPE *> pos, vel, out;
    {
        Task<NbodyInit<FTYPE>> bodyInit(ProcList(0));
        for (int i = 0; i < ntasks; ++i) {
            pos.push_back(new FTYPE[per]);
            vel.push_back(new FTYPE[per]);
            out.push_back(new FTYPE[per * frames]);
            bodyInit.run(NBODY_CONFIG_SHELL, pos[i], vel[i], (float *)nullptr, activeParams.m_clusterScale,
                         activeParams.m_velocityScale, numBodies, true);
            bodyInit.wait();
            std::memcpy(out[i], pos[i], per * sizeof(FTYPE));
        }
    }
    double runtime[5] = {0, 0, 0, 0, 0};
    int status = NB_OK;
    const auto t0 = std::chrono::steady_clock::now();
    if (mode == 1) {
        std::vector<FTYPE *> frames1(ntasks);
        for (int i = 0; i < ntasks; ++i) frames1[i] = out[i] + per;
        status = run_batched<FTYPE>(ntasks, numBodies, iteration, outInterval, activeParams, pos, vel, frames1,
                                    algo, runtime);
    } else {
        std::vector<Task<BodySystemGB300<FTYPE>> *> tasks;
        std::vector<std::vector<double>> rts(ntasks, std::vector<double>(4, 0.0));
        BodyTaskGroup<FTYPE> group(ntasks);
        for (int i = 0; i < ntasks; ++i) {
            auto *t = new Task<BodySystemGB300<FTYPE>>(ProcList(0), TaskType::gpu_task);
            if (mode == 2) t->userObject()->setGroup(&group);
            if (algo >= 0) t->userObject()->setAlgo(algo);
            t->init((unsigned)numBodies, (FTYPE)activeParams.m_softening * (FTYPE)activeParams.m_softening,
                    (FTYPE)activeParams.m_damping, pos[i], vel[i]);
            tasks.push_back(t);
        }
        for (int i = 0; i < ntasks; ++i)
            tasks[i]->run(rts[i].data(), iteration, outInterval, blocksize, (FTYPE)activeParams.m_timestep,
                          out[i] + per, memtype);
        for (int i = 0; i < ntasks; ++i) {
            tasks[i]->wait();
            if (tasks[i]->userObject()->lastStatus() != NB_OK) status = tasks[i]->userObject()->lastStatus();
            // the reference sums its tasks' timers; a group's members all
            // carry the one batch's timers
            for (int j = 0; j < 4; ++j) runtime[j] = mode == 2 ? std::max(runtime[j], rts[i][j]) : runtime[j] + rts[i][j];
            delete tasks[i];
        }
    }
    const double totaltime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    if (outfilename && status == NB_OK) {
        FILE *fp = std::fopen(outfilename, "w");
        if (!fp) {
            std::cout << "Cann't open the output file !!!" << std::endl;
            return 1;
        }
        Task<Output<FTYPE>> outtask(ProcList(0));
        for (int i = 0; i < ntasks; ++i)
            for (int f = 0; f < frames; ++f) {
                float timestamp = f * activeParams.m_timestep;
                outtask.run(&fp, out[i] + (size_t)f * per, timestamp, numBodies);
                outtask.wait();
            }
        std::fclose(fp);
    }
    for (int i = 0; i < ntasks; ++i) {
        delete[] pos[i];
        delete[] vel[i];
        delete[] out[i];
    }

    std::cout << "Test complete !!!" << std::endl;
    if (printTime) {
        std::cout << "\tbody system info:" << std::endl;
        std::cout << "\t\tTotal bodies : " << numBodies << std::endl;
        std::cout << "\t\tIterations: " << iteration << std::endl;
        std::cout << "\t\tOutput frames: " << frames << std::endl;
        std::cout << "\t\tNumber of tasks: " << ntasks << std::endl;
        std::cout << "\ttime info: " << std::endl;
        std::cout << "\t\treal total runtime: " << std::fixed << std::setprecision(4) << 1000 * totaltime
                  << std::endl;
        std::cout << "\t\ttotal runtime: " << std::fixed << std::setprecision(4) << 1000 * runtime[0] << "(ms)"
                  << std::endl;
        std::cout << "\t\tkernel time: " << std::fixed << std::setprecision(4) << 1000 * runtime[1] << "(ms)"
                  << std::endl;
        std::cout << "\t\tcopyin time: " << std::fixed << std::setprecision(4) << 1000 * runtime[2] << "(ms)"
                  << std::endl;
        std::cout << "\t\tcopyout time: " << std::fixed << std::setprecision(4) << 1000 * runtime[3] << "(ms)"
                  << std::endl;
    }
    return status == NB_OK ? 0 : 2;
}

int main(int argc, char **argv)
{
    bool printTime = false, useFloat = false;
    int mode = 1;
    int paraSelect = 0, iteration = 1, outInterval = 0, numBodies = 1024, ntasks = 1;
    int blocksize = 256, nthreads = 1, nprocess = 1, mtype = 0, algo = -1;
    char *outfilename = nullptr;
    UtcContext &ctx = UtcContext::getContext(argc, argv);
    int opt;
    while ((opt = getopt(argc, argv, "vt:p:m:i:l:o:O:n:b:T:B:Fa:")) != EOF) {
        switch (opt) {
        case 'v': printTime = true; break;
        case 't': nthreads = std::atoi(optarg); break;
        case 'p': nprocess = std::atoi(optarg); break;
        case 'm': mtype = std::atoi(optarg); break;
        case 'i': paraSelect = std::atoi(optarg); break;
        case 'o': outInterval = std::atoi(optarg); break;
        case 'O': outfilename = optarg; break;
        case 'l': iteration = std::atoi(optarg); break;
        case 'n': numBodies = std::atoi(optarg); break;
        case 'b': blocksize = std::atoi(optarg); break;
        case 'T': ntasks = std::atoi(optarg); break;
        case 'B': mode = std::atoi(optarg); break;
        case 'F': useFloat = true; break;
        case 'a': algo = std::atoi(optarg); break;
        default: break;
        }
    }
    if (nprocess != ctx.numProcs()) {
        std::cerr << "process number not match with arguments '-p' !!!\n";
        return 1;
    }
    if (nthreads != 1) {
        std::cerr << "require one thread !!!\n";
        return 1;
    }
    MemType memtype = MemType::pageable;
    if (mtype == 1) memtype = MemType::pinned;
    else if (mtype == 2) memtype = MemType::unified;
    else if (mtype != 0) std::cerr << "wrong memory type for -m !!!" << std::endl;
    if (outInterval <= 0) outInterval = iteration;
    if (paraSelect > 6) paraSelect = 0;
    if (blocksize <= 0) blocksize = 256;
    if (ntasks < 1) ntasks = 1;
    if (numBodies % blocksize != 0) {
        std::cout << "number of bodies is scaled to multiple of " << blocksize << std::endl;
        numBodies = (numBodies / blocksize + 1) * blocksize;
    }
    if (useFloat)
        return run_app<float>(printTime, paraSelect, iteration, outInterval, numBodies, ntasks, outfilename,
                              blocksize, memtype, mode, algo);
    return run_app<double>(printTime, paraSelect, iteration, outInterval, numBodies, ntasks, outfilename,
                           blocksize, memtype, mode, algo);
}
