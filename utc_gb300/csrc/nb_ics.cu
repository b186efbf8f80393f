// nb_ics.cu -- seeded initial conditions generated on the GPU.
//
// The reference draws its bodies on the host with the C library's rand()
// (randomizeBodies, benchapps/nbody/seq/nbody.h:89-250; kept bit-exact in
// utc_gb300/task/nbody_init.h for the app).  For large synthetic workloads
// the bodies are drawn here instead, one thread per body, from a
// counter-based generator: stream k of body i of seed s is
//   splitmix64(s ^ splitmix64(i * 256 + k)),  k < 256
// (the SplitMix64 finaliser, Steele, Lea & Flood 2014), so a body's draw does
// not depend on the launch shape or on the other bodies.
//  * uniform cube: positions U[-1,1]^3, velocities U[-vmax,vmax]^3, masses
//    U[0.5,1.5]/n (total mass ~ 1);
//  * Plummer sphere (Aarseth, Henon & Wielen 1974): r = a / sqrt(X^-2/3 - 1)
//    with X uniform in (0, 0.999], speeds q * v_esc(r) with q drawn by
//    rejection from q^2 (1 - q^2)^(7/2), isotropic directions, masses M/n;
//    then the centre of mass and its velocity are moved to the origin
//    (FP64 block sums reduced in order by one block: deterministic);
//  * the reference app's own three configurations (randomizeBodies,
//    benchapps/nbody/seq/nbody.h:89-250) with this generator in place of
//    rand(), a = clusterScale, vmax = velocityScale, masses 1, vel.w = 1:
//    random (positions uniform in the ball of radius s = a max(1, n/1024),
//    velocities uniform in the ball of radius s vmax), shell (a unit
//    direction drawn by rejection from the cube, each coordinate scaled by
//    its own draw from [2.5a, 4a], velocity (pos x axis) a vmax with axis z,
//    or (y, x, 1) normalised when the direction is within 1e-6 of z) and
//    expand (positions uniform in the ball of radius s = a n/1024, or a when
//    s < 1; velocity the same point times s vmax).
#include <cmath>

#include "nb_internal.cuh"

namespace nb {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// uniform double in [0, 1) from 53 random bits
__device__ __forceinline__ double u01(unsigned long long seed, unsigned long long i, unsigned k)
{
    const unsigned long long h = splitmix64(seed ^ splitmix64(i * 256ull + k));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

template <typename V4>
__device__ __forceinline__ V4 mk4(double x, double y, double z, double w)
{
    V4 r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.w = w;
    return r;
}

// A point uniform in the unit ball by rejection from the cube: tries use
// streams k0, k0 + 1, ... (3 per try, 40 tries).  All 40 fail with
// probability 0.476^40 ~ 1e-13; then the last candidate is pulled inside.
__device__ __forceinline__ void ball_point(unsigned long long seed, unsigned long long id, unsigned k0,
                                           double &x, double &y, double &z, double &len)
{
    for (unsigned t = 0; t < 40; ++t) {
        x = 2.0 * u01(seed, id, k0 + 3 * t) - 1.0;
        y = 2.0 * u01(seed, id, k0 + 3 * t + 1) - 1.0;
        z = 2.0 * u01(seed, id, k0 + 3 * t + 2) - 1.0;
        len = sqrt(x * x + y * y + z * z);
        if (len <= 1.0) return;
    }
    x *= 0.5 / len;
    y *= 0.5 / len;
    z *= 0.5 / len;
    len = 0.5;
}

template <typename V4>
__global__ void ics_kernel(int kind, int n, unsigned long long seed, double a, double G, double M,
                           double vmax, V4 *__restrict__ pos, V4 *__restrict__ vel)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long id = (unsigned long long)i;
    if (kind == 2 || kind == 4) {  // reference random / expand
        double x, y, z, len;
        ball_point(seed, id, 8, x, y, z, len);
        double s = a * fmax(1.0, n / 1024.0);
        if (kind == 4) {
            s = a * (n / 1024.0);
            if (s < 1.0) s = a;
            pos[i] = mk4<V4>(x * s, y * s, z * s, 1.0);
            vel[i] = mk4<V4>(x * s * vmax, y * s * vmax, z * s * vmax, 1.0);
            return;
        }
        double vx, vy, vz, vlen;
        ball_point(seed, id, 128, vx, vy, vz, vlen);
        pos[i] = mk4<V4>(x * s, y * s, z * s, 1.0);
        vel[i] = mk4<V4>(vx * s * vmax, vy * s * vmax, vz * s * vmax, 1.0);
        return;
    }
    if (kind == 3) {  // reference shell
        double x, y, z, len;
        ball_point(seed, id, 8, x, y, z, len);
        if (len > 1e-6) {  // one FP64 division instead of three
            const double il = 1.0 / len;
            x *= il;
            y *= il;
            z *= il;
        }
        const double inner = 2.5 * a, outer = 4.0 * a;
        const double px = x * (inner + (outer - inner) * u01(seed, id, 128));
        const double py = y * (inner + (outer - inner) * u01(seed, id, 129));
        const double pz = z * (inner + (outer - inner) * u01(seed, id, 130));
        double ax = 0.0, ay = 0.0, az = 1.0;
        if (1.0 - z < 1e-6) {
            const double il = rsqrt(y * y + x * x + 1.0);
            ax = y * il;
            ay = x * il;
            az = il;
        }
        const double vs = a * vmax;
        pos[i] = mk4<V4>(px, py, pz, 1.0);
        vel[i] = mk4<V4>((py * az - pz * ay) * vs, (pz * ax - px * az) * vs, (px * ay - py * ax) * vs, 1.0);
        return;
    }
    if (kind == 0) {  // uniform cube
        pos[i] = mk4<V4>(2.0 * u01(seed, id, 0) - 1.0, 2.0 * u01(seed, id, 1) - 1.0,
                         2.0 * u01(seed, id, 2) - 1.0, (0.5 + u01(seed, id, 3)) / n);
        vel[i] = mk4<V4>(vmax * (2.0 * u01(seed, id, 4) - 1.0), vmax * (2.0 * u01(seed, id, 5) - 1.0),
                         vmax * (2.0 * u01(seed, id, 6) - 1.0), 1.0);
        return;
    }
    // Plummer sphere
    // x1^(-2/3) as rcbrt(x1)^2, (1 - q^2)^3.5 as t^3 sqrt(t) and
    // (r^2 + a^2)^(-1/4) as rsqrt(sqrt(.)): the same quantities without pow,
    // whose FP64 log/exp dominated the sampler on a part with a slow FP64 pipe
    const double x1 = fmax(0.999 * u01(seed, id, 0), 1e-300);
    const double c1 = rcbrt(x1);
    const double r = a / sqrt(c1 * c1 - 1.0);
    double ct = 2.0 * u01(seed, id, 1) - 1.0;
    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double sp, cp;
    sincospi(2.0 * u01(seed, id, 2), &sp, &cp);
    pos[i] = mk4<V4>(r * st * cp, r * st * sp, r * ct, M / n);
    // speed fraction q by rejection from g(q) = q^2 (1 - q^2)^3.5 (max < 0.1);
    // each try is accepted with probability 7 pi / 512 / 0.1 = 0.43, so all 64
    // tries miss with probability ~2e-16; then q falls back to the mode of g,
    // sqrt(2/9)
    double q = 0.4714045207910317;
    for (unsigned t = 0; t < 64; ++t) {
        const double qq = u01(seed, id, 8 + 2 * t);
        const double yy = 0.1 * u01(seed, id, 9 + 2 * t);
        const double t1 = 1.0 - qq * qq;
        if (yy < qq * qq * (t1 * t1 * t1 * sqrt(t1))) {
            q = qq;
            break;
        }
    }
    const double vesc = sqrt(2.0 * G * M) * rsqrt(sqrt(r * r + a * a));
    ct = 2.0 * u01(seed, id, 3) - 1.0;
    st = sqrt(fmax(0.0, 1.0 - ct * ct));
    sincospi(2.0 * u01(seed, id, 4), &sp, &cp);
    const double v = q * vesc;
    vel[i] = mk4<V4>(v * st * cp, v * st * sp, v * ct, 1.0);
}

// centre of mass / velocity (mass-weighted) in FP64: block partials, then
// one block of 7 x 128 threads sums them in a fixed order (thread (q, j)
// takes partials j, j + 128, ...; then a tree over j)
constexpr int kIcsBlock = 256;
constexpr int kIcsFinal = 128;

template <typename V4>
__global__ void ics_moments_kernel(int n, const V4 *__restrict__ pos, const V4 *__restrict__ vel,
                                   double *__restrict__ part)
{
    __shared__ double red[7][kIcsBlock];
    const int i = blockIdx.x * kIcsBlock + threadIdx.x;
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    if (i < n) {
        const double m = pos[i].w;
        v[0] = m * pos[i].x;
        v[1] = m * pos[i].y;
        v[2] = m * pos[i].z;
        v[3] = m * vel[i].x;
        v[4] = m * vel[i].y;
        v[5] = m * vel[i].z;
        v[6] = m;
    }
    for (int q = 0; q < 7; ++q) red[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int w = kIcsBlock / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int q = 0; q < 7; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 7) part[(size_t)blockIdx.x * 7 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(7 * kIcsFinal)
    ics_moments_final(const double *__restrict__ part, int nblocks, double *__restrict__ out)
{
    __shared__ double red[7][kIcsFinal];
    const int q = threadIdx.x / kIcsFinal, j = threadIdx.x % kIcsFinal;
    double s = 0;
#pragma unroll 8
    for (int b = j; b < nblocks; b += kIcsFinal) s += part[(size_t)b * 7 + q];
    red[q][j] = s;
    __syncthreads();
    for (int w = kIcsFinal / 2; w > 0; w >>= 1) {
        if (j < w) red[q][j] += red[q][j + w];
        __syncthreads();
    }
    if (j == 0) out[q] = red[q][0];
}

template <typename V4>
__global__ void ics_recenter_kernel(int n, V4 *__restrict__ pos, V4 *__restrict__ vel,
                                    const double *__restrict__ mom)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double M = mom[6] > 0 ? mom[6] : 1.0;
    pos[i].x -= mom[0] / M;
    pos[i].y -= mom[1] / M;
    pos[i].z -= mom[2] / M;
    vel[i].x -= mom[3] / M;
    vel[i].y -= mom[4] / M;
    vel[i].z -= mom[5] / M;
}

template <typename V4>
static int ics_launch(int kind, int n, unsigned long long seed, double a, double G, double M,
                      double vmax, V4 *pos, V4 *vel, double *scratch, cudaStream_t s)
{
    const int blocks = (n + kIcsBlock - 1) / kIcsBlock;
    ics_kernel<V4><<<blocks, kIcsBlock, 0, s>>>(kind, n, seed, a, G, M, vmax, pos, vel);
    NB_LAUNCH_CHECK("ics_kernel launch");
    if (kind == 1) {
        ics_moments_kernel<V4><<<blocks, kIcsBlock, 0, s>>>(n, pos, vel, scratch + 8);
        NB_LAUNCH_CHECK("ics_moments_kernel launch");
        ics_moments_final<<<1, 7 * kIcsFinal, 0, s>>>(scratch + 8, blocks, scratch);
        NB_LAUNCH_CHECK("ics_moments_final launch");
        ics_recenter_kernel<V4><<<blocks, kIcsBlock, 0, s>>>(n, pos, vel, scratch);
        NB_LAUNCH_CHECK("ics_recenter_kernel launch");
    }
    return NB_OK;
}

size_t ics_scratch_doubles(int n) { return 8 + 7 * (size_t)((n + kIcsBlock - 1) / kIcsBlock); }

}  // namespace nb

extern "C" int nb_ics_generate(int kind, int n, unsigned long long seed, double a, double G,
                               double M, double vmax, int precision, void *pos_dev, void *vel_dev,
                               void *scratch_dev, void *stream)
{
    if (kind < 0 || kind > 4)
        return nb::set_error(NB_ERR_INVALID,
                             "nb_ics_generate: kind is 0 (cube), 1 (Plummer), 2 (random), 3 (shell) or 4 (expand)");
    if (n < 0 || n > NB_MAX_BODIES) return nb::set_error(NB_ERR_INVALID, "nb_ics_generate: n must be in [0, 2^30]");
    if (precision != NB_F32 && precision != NB_F64)
        return nb::set_error(NB_ERR_INVALID, "nb_ics_generate: precision is NB_F32 or NB_F64");
    if (n == 0) return NB_OK;
    if (!pos_dev || !vel_dev || (kind == 1 && !scratch_dev))
        return nb::set_error(NB_ERR_INVALID, "nb_ics_generate: NULL buffer");
    if (!(a > 0) || !std::isfinite(G) || !std::isfinite(M) || !std::isfinite(vmax))
        return nb::set_error(NB_ERR_INVALID, "nb_ics_generate: bad parameters");
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == NB_F32)
        return nb::ics_launch<float4>(kind, n, seed, a, G, M, vmax, (float4 *)pos_dev, (float4 *)vel_dev,
                                      (double *)scratch_dev, s);
    return nb::ics_launch<double4>(kind, n, seed, a, G, M, vmax, (double4 *)pos_dev, (double4 *)vel_dev,
                                   (double *)scratch_dev, s);
}

extern "C" size_t nb_ics_scratch_bytes(int n) { return nb::ics_scratch_doubles(n) * sizeof(double); }
