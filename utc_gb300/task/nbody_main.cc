/*
 * nbody_main.cc -- the nbody app driver on the GB300 task, with the
 * reference's flags and flow (benchapps/nbody/utc/nbody_main.cc:68-271):
 *
 *   -v print timers      -t threads               -p processes (must be 1)
 *   -m 0|1|2 memtype     -i preset 0..6           -l iterations
 *   -o output interval   -O output file           -n bodies
 *   -b block size (exact kernel CTA size; N is rounded up to a multiple)
 * additions:
 *   -F  use float state (the reference fixes FTYPE=double at compile time)
 *   -a 0|1|2|3  force algorithm: 0 directed fast (float only), 1 reference-exact,
 *             2 symmetric (the default; float-float pair terms for double),
 *             3 symmetric in FP64 arithmetic throughout (double only)
 *
 * Bodies come from NbodyInit (SHELL), run through Task<BodySystemGB300<T>>,
 * frames go through Task<Output<T>>; timers are printed as the reference
 * prints them.  With -t N > 1 the bodies run through the multi-GPU task
 * Task<BodySystemMGPU_GB300<T>>(ProcList(N, 0)), as the reference's
 * multi-GPU app does (benchapps/nbody/utc-snode-mgpu/nbody_main.cc:209-236:
 * one thread per GPU, timers averaged over the threads).
 */
#include <array>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <iomanip>
#include <iostream>
#include <unistd.h>

#include "body_task_gb300.h"
#include "body_task_mgpu_gb300.h"
#include "nbody_init.h"

using namespace iUtc;

template <typename FTYPE>
static int run_app(bool printTime, int paraSelect, int iteration, int outInterval, int numBodies,
                   const char *outfilename, int blocksize, MemType memtype, int algo, int nthreads)
{
    NBodyParams activeParams = nbody_demo_params(paraSelect, numBodies);
    FTYPE *body_pos = new FTYPE[(size_t)numBodies * 4];
    FTYPE *body_vel = new FTYPE[(size_t)numBodies * 4];
    float *body_color = new float[(size_t)numBodies * 4];
    {
        Task<NbodyInit<FTYPE>> bodyInit(ProcList(0));
        bodyInit.run(NBODY_CONFIG_SHELL, body_pos, body_vel, body_color,
                     activeParams.m_clusterScale, activeParams.m_velocityScale, numBodies, true);
        bodyInit.wait();
    }
    const int frames = iteration / outInterval + 1;
    FTYPE *body_outBuffer = new FTYPE[(size_t)numBodies * 4 * frames];
    std::memcpy(body_outBuffer, body_pos, sizeof(FTYPE) * 4 * (size_t)numBodies);

    double runtime[4] = {0, 0, 0, 0};
    int status;
    if (nthreads > 1) {
        std::vector<std::array<double, 4>> runtime_m(nthreads);
        Task<BodySystemMGPU_GB300<FTYPE>> nbody(ProcList(nthreads, 0), TaskType::gpu_task);
        if (algo >= 0) nbody.userObject()->setAlgo(algo);
        nbody.init((unsigned)numBodies,
                   (FTYPE)activeParams.m_softening * (FTYPE)activeParams.m_softening,
                   (FTYPE)activeParams.m_damping, body_pos, body_vel);
        nbody.run(reinterpret_cast<double(*)[4]>(runtime_m.data()), iteration, outInterval, blocksize,
                  (FTYPE)activeParams.m_timestep, body_outBuffer + (size_t)numBodies * 4, memtype);
        nbody.wait();
        status = nbody.userObject()->lastStatus();
        for (int i = 0; i < nthreads; i++)
            for (int j = 0; j < 4; j++) runtime[j] += runtime_m[i][j] / nthreads;
    } else {
        Task<BodySystemGB300<FTYPE>> nbody(ProcList(0), TaskType::gpu_task);
        if (algo >= 0) nbody.userObject()->setAlgo(algo);
        nbody.init((unsigned)numBodies,
                   (FTYPE)activeParams.m_softening * (FTYPE)activeParams.m_softening,
                   (FTYPE)activeParams.m_damping, body_pos, body_vel);
        nbody.run(runtime, iteration, outInterval, blocksize, (FTYPE)activeParams.m_timestep,
                  body_outBuffer + (size_t)numBodies * 4, memtype);
        nbody.wait();
        status = nbody.userObject()->lastStatus();
    }

    if (outfilename) {
        FILE *fp = std::fopen(outfilename, "w");
        if (!fp) {
            std::cout << "Cann't open the output file !!!" << std::endl;
            return 1;
        }
        Task<Output<FTYPE>> outtask(ProcList(0));
        for (int i = 0; i < frames; i++) {
            float timestamp = i * activeParams.m_timestep;
            outtask.run(&fp, &body_outBuffer[(size_t)i * numBodies * 4], timestamp, numBodies);
            outtask.wait();
        }
        std::fclose(fp);
    }
    delete[] body_pos;
    delete[] body_vel;
    delete[] body_color;
    delete[] body_outBuffer;

    std::cout << "Test complete !!!" << std::endl;
    if (printTime) {
        std::cout << "\tbody system info:" << std::endl;
        std::cout << "\t\tTotal bodies : " << numBodies << std::endl;
        std::cout << "\t\tIterations: " << iteration << std::endl;
        std::cout << "\t\tOutput frames: " << frames << std::endl;
        std::cout << "\ttime info: " << std::endl;
        std::cout << "\t\ttotal runtime: " << std::fixed << std::setprecision(4)
                  << 1000 * runtime[0] << "(ms)" << std::endl;
        std::cout << "\t\tkernel time: " << std::fixed << std::setprecision(4)
                  << 1000 * runtime[1] << "(ms)" << std::endl;
        std::cout << "\t\tcopyin time: " << std::fixed << std::setprecision(4)
                  << 1000 * runtime[2] << "(ms)" << std::endl;
        std::cout << "\t\tcopyout time: " << std::fixed << std::setprecision(4)
                  << 1000 * runtime[3] << "(ms)" << std::endl;
    }
    return status == NB_OK ? 0 : 2;
}

int main(int argc, char **argv)
{
    bool printTime = false, useFloat = false;
    int paraSelect = 0, iteration = 1, outInterval = 0, numBodies = 1024;
    int blocksize = 256, nthreads = 1, nprocess = 1, mtype = 0, algo = -1;
    char *outfilename = nullptr;
    UtcContext &ctx = UtcContext::getContext(argc, argv);
    int opt;
    while ((opt = getopt(argc, argv, "vt:p:m:i:l:o:O:n:b:Fa:")) != EOF) {
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
        case 'F': useFloat = true; break;
        case 'a': algo = std::atoi(optarg); break;
        default: break;
        }
    }
    if (nprocess != ctx.numProcs()) {
        std::cerr << "process number not match with arguments '-p' !!!\n";
        return 1;
    }
    if (nthreads < 1) {
        std::cerr << "require at least one thread !!!\n";
        return 1;
    }
    MemType memtype = MemType::pageable;
    if (mtype == 1) memtype = MemType::pinned;
    else if (mtype == 2) memtype = MemType::unified;
    else if (mtype != 0) std::cerr << "wrong memory type for -m !!!" << std::endl;
    if (outInterval == 0) outInterval = iteration;
    if (paraSelect > 6) paraSelect = 0;
    if (blocksize <= 0) blocksize = 256;
    if (numBodies % blocksize != 0) {
        std::cout << "number of bodies is scaled to multiple of " << blocksize << std::endl;
        numBodies = (numBodies / blocksize + 1) * blocksize;
    }
    if (useFloat)
        return run_app<float>(printTime, paraSelect, iteration, outInterval, numBodies, outfilename,
                              blocksize, memtype, algo, nthreads);
    return run_app<double>(printTime, paraSelect, iteration, outInterval, numBodies, outfilename,
                           blocksize, memtype, algo, nthreads);
}
