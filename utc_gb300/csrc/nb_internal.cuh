// nb_internal.cuh -- shared declarations of the GB300 nbody library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "nbody_gb300.h"

namespace nb {

// ---------------------------------------------------------------------------
// error reporting (thread-local last error, status codes)
// ---------------------------------------------------------------------------
int set_error(int status, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);

#define NB_CUDA(call)                                              \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::nb::cuda_error(_e, #call); \
    } while (0)

#define NB_LAUNCH_CHECK(what)                                     \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::nb::cuda_error(_e, what); \
    } while (0)

// ---------------------------------------------------------------------------
// packed f32x2 arithmetic (sm_100+ FFMA2 / FADD2 / FMUL2)
// ---------------------------------------------------------------------------
typedef unsigned long long f2;  // two floats in one 64-bit register pair

__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Position used for the padding sources of a partial tile: zero mass makes
// its term exactly zero (m * finite = 0), the distance keeps d2 finite > 0.
constexpr float kPadCoord = 1.0e15f;

// ---------------------------------------------------------------------------
// stream-K plan of the fast force kernel
// ---------------------------------------------------------------------------
// The iteration space is (target block tb, source group g) with groups of
// kGroup sources; it = tb * ngroups + g.  CTA c of `grid` owns iterations
// [start(c), start(c+1)), start(c) = floor(c * total / grid), so every CTA
// gets the same number of pair evaluations up to one group.  A CTA writes
// one partial acceleration per target block it touches, into slot c + tb
// (distinct for distinct (c, tb) because CTA ranges are ordered).
constexpr int kGroup = 32;

struct SkPlan {
    int n = 0;
    int block = 0;     // threads per CTA
    int npair = 0;     // packed target pairs per thread (bodies per thread / 2)
    int tbsize = 0;    // targets per block = block * 2 * npair
    int ntb = 0;       // target blocks
    int ngroups = 0;   // source groups per target block
    long long total = 0;
    int grid = 0;      // persistent CTAs
    int slots = 0;     // grid + ntb - 1
};

__host__ __device__ __forceinline__ long long sk_start(long long c, long long total, int grid)
{
    return (c * total) / grid;
}
// CTA that owns iteration `it`: the largest c with start(c) <= it.
__host__ __device__ __forceinline__ int sk_owner(long long it, long long total, int grid)
{
    return (int)(((it + 1) * (long long)grid - 1) / total);
}

// Fast-path entry points (nb_fast.cu)
int fast_plan(int n, int block, int bpt, int ctas_per_sm, int device, SkPlan *plan);
int fast_force(const SkPlan &plan, const float4 *pos, float eps2, float4 *partial,
               cudaStream_t s);
// Reduce the partial slots and integrate (acc_out != nullptr: write the bare
// acceleration instead of integrating).
int fast_integrate(const SkPlan &plan, const float4 *pos_old, float4 *pos_new, float4 *vel,
                   const float4 *partial, float damping, float dt, int kick, float G,
                   float4 *acc_out, cudaStream_t s);

// Exact-path entry points (nb_exact.cu)
int exact_step_f32(int n, const float4 *pos_old, float4 *pos_new, float4 *vel, float eps2,
                   float damping, float dt, int kick, float G, float4 *acc_out, int block,
                   cudaStream_t s);
int exact_step_f64(int n, const double4 *pos_old, double4 *pos_new, double4 *vel, double eps2,
                   double damping, double dt, int kick, double G, double4 *acc_out, int block,
                   cudaStream_t s);

// FMA peak probe (nb_fast.cu)
int probe_fma(int iters, int packed, double *flops, float *ms, cudaStream_t s);

}  // namespace nb
