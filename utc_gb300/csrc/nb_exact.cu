// nb_exact.cu -- reference-exact all-pairs step (float and double).
//
// Reproduces the reference's sequential BodySystem<T>::update bit for bit
// (benchapps/nbody/seq/bodysystem.h:71-96, bodysystem.cc:103-182):
//  * every operation is an unfused IEEE round-to-nearest intrinsic in the
//    reference's order (no FMA contraction);
//  * each target sums its sources in index order j = 0..n-1;
//  * 1/sqrt(d2): the reference computes 1.0/sqrtf(d2) with a double
//    division rounded back to float.  Double rounding of a quotient of
//    floats through double (53 >= 2*24+2 bits) is innocuous, so that value
//    equals the correctly rounded float reciprocal __frcp_rn(__fsqrt_rn(d2)).
// This is the drop-in path for the app's default FTYPE double and the
// parity anchor for float; it is not the throughput path.
#include "nb_internal.cuh"

namespace nb {

template <typename T> struct vec4_of;
template <> struct vec4_of<float> { typedef float4 type; };
template <> struct vec4_of<double> { typedef double4 type; };

__device__ __forceinline__ float e_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double e_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float e_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double e_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float e_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double e_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float e_rinvsqrt(float x) { return __frcp_rn(__fsqrt_rn(x)); }
__device__ __forceinline__ double e_rinvsqrt(double x) { return __drcp_rn(__dsqrt_rn(x)); }

// Targets i_begin <= i < i_end against all n sources: a target's result does
// not depend on which other targets a launch covers (a shard of the targets
// gives the full launch's bits).
template <typename T>
__global__ void exact_step_kernel(const typename vec4_of<T>::type *__restrict__ pos_old,
                                  typename vec4_of<T>::type *__restrict__ pos_new,
                                  typename vec4_of<T>::type *__restrict__ vel, int n, int i_begin,
                                  int i_end, T eps2, T damping, T dt, int kick, T G,
                                  typename vec4_of<T>::type *__restrict__ acc_out)
{
    typedef typename vec4_of<T>::type V4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V4 *sp = reinterpret_cast<V4 *>(smem_raw);
    const int nt = blockDim.x;
    const int i = i_begin + blockIdx.x * nt + threadIdx.x;
    V4 pi;
    if (i < i_end) {
        pi = pos_old[i];
    } else {
        pi.x = pi.y = pi.z = pi.w = T(0);
    }
    T ax = T(0), ay = T(0), az = T(0);
    for (int jt = 0; jt < n; jt += nt) {
        __syncthreads();
        if (jt + (int)threadIdx.x < n) sp[threadIdx.x] = pos_old[jt + threadIdx.x];
        __syncthreads();
        const int cnt = min(nt, n - jt);
        for (int j = 0; j < cnt; ++j) {
            const V4 pj = sp[j];
            const T r0 = e_sub(pj.x, pi.x);
            const T r1 = e_sub(pj.y, pi.y);
            const T r2 = e_sub(pj.z, pi.z);
            T d = e_add(e_add(e_mul(r0, r0), e_mul(r1, r1)), e_mul(r2, r2));
            d = e_add(d, eps2);
            const T inv = e_rinvsqrt(d);
            const T inv3 = e_mul(e_mul(inv, inv), inv);
            const T s = e_mul(pj.w, inv3);
            ax = e_add(ax, e_mul(r0, s));
            ay = e_add(ay, e_mul(r1, s));
            az = e_add(az, e_mul(r2, s));
        }
    }
    if (i >= i_end) return;
    if (acc_out) {
        V4 a;
        a.x = ax;
        a.y = ay;
        a.z = az;
        a.w = T(0);
        acc_out[i] = a;
        return;
    }
    V4 v = vel[i];
    const T k = kick == NB_KICK_REFERENCE ? pi.w : G;
    v.x = e_add(v.x, e_mul(e_mul(ax, k), dt));
    v.y = e_add(v.y, e_mul(e_mul(ay, k), dt));
    v.z = e_add(v.z, e_mul(e_mul(az, k), dt));
    v.x = e_mul(v.x, damping);
    v.y = e_mul(v.y, damping);
    v.z = e_mul(v.z, damping);
    pi.x = e_add(pi.x, e_mul(v.x, dt));
    pi.y = e_add(pi.y, e_mul(v.y, dt));
    pi.z = e_add(pi.z, e_mul(v.z, dt));
    pos_new[i] = pi;
    vel[i] = v;
}

template <typename T>
static int exact_launch(int n, int i_begin, int i_end, const typename vec4_of<T>::type *pos_old,
                        typename vec4_of<T>::type *pos_new, typename vec4_of<T>::type *vel,
                        T eps2, T damping, T dt, int kick, T G,
                        typename vec4_of<T>::type *acc_out, int block, cudaStream_t s)
{
    const int nt = i_end - i_begin;  // targets of this launch
    if (n == 0 || nt <= 0) return NB_OK;
    if (block <= 0) block = 256;
    if (block % 32 != 0 || block > 1024)
        return set_error(NB_ERR_INVALID, "exact kernel block size must be a multiple of 32, <= 1024");
    // The results do not depend on the CTA size (every thread sums its
    // sources in index order), so the requested size is only an upper bound:
    // halve it while that lowers the most warps one SM has to run (a small N
    // in large CTAs leaves SMs idle: N=16384 in CTAs of 256 covers 64 of
    // 152 SMs).  Ties keep the larger CTA.
    int dev = 0, sms = 0;
    NB_CUDA(cudaGetDevice(&dev));
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto load = [&](int b) {
        const long long grid = ((long long)nt + b - 1) / b;
        return ((grid + sms - 1) / sms) * (b / 32);
    };
    for (int b = block / 2; b >= 32 && b % 32 == 0; b /= 2)
        if (load(b) < load(block)) block = b;
    const size_t smem = sizeof(typename vec4_of<T>::type) * block;
    exact_step_kernel<T><<<(nt + block - 1) / block, block, smem, s>>>(pos_old, pos_new, vel, n, i_begin,
                                                                      i_end, eps2, damping, dt, kick, G,
                                                                      acc_out);
    NB_LAUNCH_CHECK("exact_step_kernel launch");
    return NB_OK;
}

int exact_step_f32(int n, int i_begin, int i_end, const float4 *pos_old, float4 *pos_new, float4 *vel,
                   float eps2, float damping, float dt, int kick, float G, float4 *acc_out, int block,
                   cudaStream_t s)
{
    return exact_launch<float>(n, i_begin, i_end, pos_old, pos_new, vel, eps2, damping, dt, kick, G,
                               acc_out, block, s);
}

int exact_step_f64(int n, int i_begin, int i_end, const double4 *pos_old, double4 *pos_new,
                   double4 *vel, double eps2, double damping, double dt, int kick, double G,
                   double4 *acc_out, int block, cudaStream_t s)
{
    return exact_launch<double>(n, i_begin, i_end, pos_old, pos_new, vel, eps2, damping, dt, kick, G,
                                acc_out, block, s);
}

}  // namespace nb
