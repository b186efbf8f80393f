// nb_sym64.cu -- symmetric all-pairs step in FP64 (NB_F64 with NB_ALGO_SYM).
//
// The app's default state type is double (benchapps/nbody/utc/nbody_main.cc
// FTYPE).  The reference's GPU kernel evaluates every ordered pair in double
// with a correctly rounded sqrt and a division
// (benchapps/nbody/cuda/bodysystem_kernel.cu:21-56), which on a part with a
// narrow FP64 pipe costs some 40 FP64 operations per interaction.  This
// kernel keeps FP64 everywhere but
//  * evaluates each unordered pair once on the layout of the FP32 symmetric
//    kernel (nb_sym.cu: row blocks of 32*BPT targets x 32-body chunks, the
//    chunk rotating through the warp with its reaction);
//  * takes 1/sqrt(d2) from the FP64 approximate reciprocal square root
//    refined by two Newton-Raphson steps, y <- y + (y/2)(1 - d2 y^2), each
//    squaring the relative error (the approximation's ~1e-7 becomes ~1e-14,
//    then rounding level);
// 24 FP64 operations and one approximation per pair: 12 per interaction.
// Results agree with the FP64 oracle to rounding (the tests hold them to
// 1e-13 relative); they are not bit-identical to it (NB_ALGO_EXACT is).
// Range: d2 must be a normal FP64 number (eps2 > 0 keeps it there).
#include "nb_internal.cuh"

namespace nb {

template <int W, int BPT, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) sym64_force_kernel(const double4 *__restrict__ pos, int n,
                                                                   double eps2, double4 *__restrict__ tpart,
                                                                   double4 *__restrict__ spart,
                                                                   long long total, int nc, int nrb)
{
    constexpr int WB = 32 * BPT;
    constexpr int RB = W * WB;
    constexpr int RC = RB / 32;
    __shared__ __align__(16) double4 sC[32];
    __shared__ double sF[3][W][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int c = blockIdx.x;
    long long it = sk_start(c, total, gridDim.x);
    const long long end = sk_start(c + 1, total, gridDim.x);
    const double4 pad = make_double4(1.0e150, 1.0e150, 1.0e150, 0.0);
    const double4 zero = make_double4(0.0, 0.0, 0.0, 0.0);

    while (it < end) {
        const int I = sym_row_of(it, nc, RC, nrb);
        const long long rfirst = sym_prefix(I, nc, RC);
        const long long rend = sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB + wid * WB;

        // nm = -m: the reaction on the chunk body points along -r; missing
        // targets get zero mass
        double px[BPT], py[BPT], pz[BPT], nm[BPT], ax[BPT], ay[BPT], az[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tbase + lane + 32 * k;
            const double4 q = i < n ? pos[i] : zero;
            px[k] = q.x;
            py[k] = q.y;
            pz[k] = q.z;
            nm[k] = -q.w;
            ax[k] = ay[k] = az[k] = 0.0;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            __syncthreads();  // previous chunk: sC reads and sF reads are done
            if (wid == 0) sC[lane] = (jb + lane < n) ? pos[jb + lane] : pad;
            __syncthreads();
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 2
                for (int j = 0; j < 32; ++j) {
                    const double4 q = sC[j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const double rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        double d2 = fma(rx, rx, eps2);
                        d2 = fma(ry, ry, d2);
                        d2 = fma(rz, rz, d2);
                        const double inv = rsqrt64(d2);
                        const double s = (q.w * inv) * (inv * inv);
                        ax[k] = fma(rx, s, ax[k]);
                        ay[k] = fma(ry, s, ay[k]);
                        az[k] = fma(rz, s, az[k]);
                    }
                }
            } else {
                double fx = 0.0, fy = 0.0, fz = 0.0;
#pragma unroll 1
                for (int r = 0; r < 32; ++r) {
                    const double4 q = sC[(lane + r) & 31];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const double rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        double d2 = fma(rx, rx, eps2);
                        d2 = fma(ry, ry, d2);
                        d2 = fma(rz, rz, d2);
                        const double inv = rsqrt64(d2);
                        const double inv3 = inv * (inv * inv);
                        const double st = q.w * inv3;
                        const double ss = nm[k] * inv3;
                        ax[k] = fma(rx, st, ax[k]);
                        ay[k] = fma(ry, st, ay[k]);
                        az[k] = fma(rz, st, az[k]);
                        fx = fma(rx, ss, fx);
                        fy = fma(ry, ss, fy);
                        fz = fma(rz, ss, fz);
                    }
                    const int from = (lane + 1) & 31;
                    fx = __shfl_sync(0xffffffffu, fx, from);
                    fy = __shfl_sync(0xffffffffu, fy, from);
                    fz = __shfl_sync(0xffffffffu, fz, from);
                }
                // lane l now holds the reaction on chunk body l from this warp
                sF[0][wid][lane] = fx;
                sF[1][wid][lane] = fy;
                sF[2][wid][lane] = fz;
                __syncthreads();
                if (wid == 0 && jb + lane < n) {
                    double sx = 0.0, sy = 0.0, sz = 0.0;
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        sx += sF[0][w][lane];
                        sy += sF[1][w][lane];
                        sz += sF[2][w][lane];
                    }
                    spart[sym_soff(I, n, RB) + (jb + lane - (I + 1) * RB)] = make_double4(sx, sy, sz, 0.0);
                }
            }
        }
        double4 *dst = tpart + (size_t)(c + I) * RB + wid * WB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) dst[lane + 32 * k] = make_double4(ax[k], ay[k], az[k], 0.0);
        it = seg_end;
    }
}

// Per body: target-side slots (CTA order) + source-side rows 0..I-1 (row
// order), then the reference's kick / damping / drift in its order with
// unfused IEEE operations (bodysystem.cc:135-182), or the bare acceleration.
__global__ void sym64_integrate_kernel(const double4 *__restrict__ pos_old, double4 *__restrict__ pos_new,
                                       double4 *__restrict__ vel, const double4 *__restrict__ tpart,
                                       const double4 *__restrict__ spart, int n, int rb, int nc, int nrb,
                                       long long total, int grid, double damping, double dt, int kick,
                                       double G, double4 *__restrict__ acc_out,
                                       const unsigned long long *__restrict__ ffrange,
                                       const double4 *__restrict__ accsum)
{
    // bodies from the last one down: the longest row walks start first
    const int i = n - 1 - (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < 0) return;
    // w: the potential sum_j m_j / sqrt(d2), j != i, when the force pass
    // recorded it (the float-float energy pass), else 0
    double ax = 0.0, ay = 0.0, az = 0.0, aw = 0.0;
    if (accsum) {  // banded plan: the fold kernel's sums
        const double4 q = accsum[i];
        ax = q.x;
        ay = q.y;
        az = q.z;
        aw = q.w;
    } else {
        const int rc = rb / 32;
        const int I = i / rb;
        const int c0 = sk_owner(sym_prefix(I, nc, rc), total, grid);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1, total, grid);
        const int li = i - I * rb;
        for (int c = c0; c <= c1; ++c) {
            const double4 q = tpart[(size_t)(c + I) * rb + li];
            ax = __dadd_rn(ax, q.x);
            ay = __dadd_rn(ay, q.y);
            az = __dadd_rn(az, q.z);
            aw = __dadd_rn(aw, q.w);
        }
        long long off = (long long)i - rb;  // row r at soff(r) + i - (r + 1) rb
        for (int r = 0; r < I; ++r) {
            const double4 q = spart[off];
            off += (long long)n - (long long)(r + 2) * rb;
            ax = __dadd_rn(ax, q.x);
            ay = __dadd_rn(ay, q.y);
            az = __dadd_rn(az, q.z);
            aw = __dadd_rn(aw, q.w);
        }
    }
    if (ffrange) {
        // float-float path: its sums are in units scaled by 2^kx (positions)
        // and 2^km (masses), kx = -e(max |x|), km = -e(max m) with
        // 2^(e-1) <= v < 2^e; a = a_scaled * 2^(2 kx - km) and
        // phi = phi_scaled * 2^(kx - km), exact
        auto ex = [](unsigned long long b) {
            const int f = (int)((b >> 52) & 0x7ff);
            return (f == 0 || f == 0x7ff) ? 0 : f - 1022;
        };
        const int em = ex(ffrange[1]), ex0 = ex(ffrange[0]);
        const int k = em - 2 * ex0;
        ax = ldexp(ax, k);
        ay = ldexp(ay, k);
        az = ldexp(az, k);
        aw = ldexp(aw, em - ex0);
    }
    if (acc_out) {
        acc_out[i] = make_double4(ax, ay, az, aw);
        return;
    }
    double4 p = pos_old[i];
    double4 v = vel[i];
    const double k = kick == NB_KICK_REFERENCE ? p.w : G;
    v.x = __dadd_rn(v.x, __dmul_rn(__dmul_rn(ax, k), dt));
    v.y = __dadd_rn(v.y, __dmul_rn(__dmul_rn(ay, k), dt));
    v.z = __dadd_rn(v.z, __dmul_rn(__dmul_rn(az, k), dt));
    v.x = __dmul_rn(v.x, damping);
    v.y = __dmul_rn(v.y, damping);
    v.z = __dmul_rn(v.z, damping);
    p.x = __dadd_rn(p.x, __dmul_rn(v.x, dt));
    p.y = __dadd_rn(p.y, __dmul_rn(v.y, dt));
    p.z = __dadd_rn(p.z, __dmul_rn(v.z, dt));
    pos_new[i] = p;
    vel[i] = v;
}

typedef void (*sym64_kernel_t)(const double4 *, int, double, double4 *, double4 *, long long, int, int);

static sym64_kernel_t sym64_kernel_for(int w, int bpt)
{
    if (w == 1 && bpt == 8) return sym64_force_kernel<1, 8, 8>;
    if (w == 1 && bpt == 4) return sym64_force_kernel<1, 4, 8>;
    if (w == 4 && bpt == 8) return sym64_force_kernel<4, 8, 2>;
    if (w == 8 && bpt == 8) return sym64_force_kernel<8, 8, 1>;
    return nullptr;
}

int sym64_plan(int n, int warps, int bpt, int device, SymPlan *pl)
{
    if (warps == 0 && bpt == 0) {
        // one-warp CTAs x 8 targets (row block 256), then 4 x 8 (1024),
        // 8 x 8 (2048) while the source-side array (32 B entries) is over
        // budget
        static const int shapes[3][2] = {{1, 8}, {4, 8}, {8, 8}};
        int s = 0;
        while (s < 2 && sym_spart_entries(n, shapes[s][0] * 32 * shapes[s][1]) * (long long)sizeof(double4) >
                            kSymSpartBudget)
            ++s;
        warps = shapes[s][0];
        bpt = shapes[s][1];
        // small systems: 4 targets per lane when 8 give fewer than four
        // (row, chunk) items per SM
        if (warps == 1 && n > 0) {
            int sms = 0;
            NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
            const int rb = 32 * bpt, nrb = (n + rb - 1) / rb, nc = (n + 31) / 32;
            if (sym_prefix(nrb, nc, bpt) < 4ll * sms) bpt = 4;
        }
    }
    sym64_kernel_t k = sym64_kernel_for(warps, bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "FP64 symmetric kernel shape not compiled");
    SymPlan p;
    p.n = n;
    p.warps = warps;
    p.bpt = bpt;
    p.rb = warps * 32 * bpt;
    p.nc = (n + 31) / 32;
    p.nrb = (n + p.rb - 1) / p.rb;
    p.total = n > 0 ? sym_prefix(p.nrb, p.nc, p.rb / 32) : 0;
    int sms = 0, occ = 0;
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * warps, 0));
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "FP64 symmetric kernel does not fit on an SM");
    long long grid = (long long)sms * occ;
    if (p.total > 0 && grid > p.total) grid = p.total;
    p.grid = p.total > 0 ? (int)grid : 0;
    p.slots = p.total > 0 ? p.grid + p.nrb - 1 : 0;
    p.spart_size = sym_spart_entries(n, p.rb);
    *pl = p;
    return NB_OK;
}

int sym64_force(const SymPlan &p, const double4 *pos, double eps2, double4 *tpart, double4 *spart,
                cudaStream_t s)
{
    if (p.total == 0) return NB_OK;
    sym64_kernel_t k = sym64_kernel_for(p.warps, p.bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "FP64 symmetric kernel shape not compiled");
    k<<<p.grid, 32 * p.warps, 0, s>>>(pos, p.n, eps2, tpart, spart, p.total, p.nc, p.nrb);
    NB_LAUNCH_CHECK("sym64_force_kernel launch");
    return NB_OK;
}

int sym64_integrate(const SymPlan &p, const double4 *pos_old, double4 *pos_new, double4 *vel,
                    const double4 *tpart, const double4 *spart, double damping, double dt, int kick,
                    double G, double4 *acc_out, cudaStream_t s, const unsigned long long *ffrange,
                    const double4 *accsum)
{
    if (p.n == 0) return NB_OK;
    if (p.nbands > 1 && !accsum) return set_error(NB_ERR_INVALID, "sym64_integrate: a banded plan needs its per-body sums");
    sym64_integrate_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(pos_old, pos_new, vel, tpart, spart, p.n, p.rb,
                                                             p.nc, p.nrb, p.total, p.grid, damping, dt, kick,
                                                             G, acc_out, ffrange, p.nbands > 1 ? accsum : nullptr);
    NB_LAUNCH_CHECK("sym64_integrate_kernel launch");
    return NB_OK;
}

}  // namespace nb
