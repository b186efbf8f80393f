// nb_batch.cu -- many independent systems of uneven size in one launch.
//
// The reference runs several nbody systems as separate UTC tasks, one kernel
// launch per system per step (benchapps/nbody/utc/nbody_mtask.cc:199-231).
// Here all systems share one persistent launch per step:
//  * bodies of all systems are concatenated (AoS float4, system s at
//    [off[s], off[s+1]));
//  * the iteration space is the concatenation over systems of
//    (warp target block of 32*BPT targets, 32-source group), and each warp of
//    the persistent grid takes an equal contiguous range of it (warp-level
//    stream-K), so small and large systems are balanced without per-size
//    launches;
//  * each warp stages its 32-source groups in its own shared-memory slice
//    (no CTA barriers: warps of a CTA may work on different systems);
//  * one partial per (warp, warp target block) goes to slot
//    warp + global block index; the integrate kernel sums them in warp order.
// The step loop is captured in a CUDA graph (nb_batch_run), and an autotuner
// picks the warps per CTA and bodies per lane.
//
// NB_ALGO_SYM batches use the single-system symmetric layout per system (a
// warp's row block of 32*BPT targets paired with every 32-body chunk at or
// after its start, each unordered pair once; the chunk rotates through the
// warp carrying its reaction), all systems' (row, chunk) items concatenated
// and split over warps the same way.  Each item belongs to one warp, which
// writes the reactions on its chunk bodies to the system's triangular
// source-side array; target-side partials go to slot warp + global row.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "nb_ff.cuh"
#include "nb_internal.cuh"

namespace nb {

struct BatchDev {
    const int *sys_off;       // [nsys + 1] body offsets
    const long long *it_off;  // [nsys + 1] iteration offsets
    const int *tb_off;        // [nsys + 1] global warp-target-block offsets
    const int *body_sys;      // [nbody] system of each body
    int nsys;
};

__device__ __forceinline__ int find_sys(const long long *it_off, int nsys, long long it)
{
    int lo = 0, hi = nsys;  // it_off[lo] <= it < it_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (it_off[mid] <= it) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int WPB, int BPT>
__global__ void __launch_bounds__(32 * WPB) bk_force_kernel(const float4 *__restrict__ pos, BatchDev bd,
                                                            float eps2, float4 *__restrict__ partial,
                                                            long long total, int workers)
{
    constexpr int WTB = 32 * BPT;
    __shared__ __align__(16) float4 sP[WPB][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wid;
    if (w >= workers) return;
    long long it = sk_start(w, total, workers);
    const long long end = sk_start(w + 1, total, workers);
    if (it >= end) return;
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    int s = find_sys(bd.it_off, bd.nsys, it);
    while (it < end) {
        while (it >= bd.it_off[s + 1]) ++s;
        const int o = bd.sys_off[s];
        const int ns = bd.sys_off[s + 1] - o;
        const int ngroups = (ns + kGroup - 1) / kGroup;
        const long long base = bd.it_off[s];
        const int tbl = (int)((it - base) / ngroups);
        const long long blk_first = base + (long long)tbl * ngroups;
        const long long seg_end = end < blk_first + ngroups ? end : blk_first + ngroups;
        const int j0 = (int)(it - blk_first) * kGroup;
        const int j1 = min((int)(seg_end - blk_first) * kGroup, ns);

        float px[BPT], py[BPT], pz[BPT], ax[BPT], ay[BPT], az[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int li = tbl * WTB + lane + 32 * k;
            const float4 q = li < ns ? pos[o + li] : make_float4(0.f, 0.f, 0.f, 0.f);
            px[k] = q.x;
            py[k] = q.y;
            pz[k] = q.z;
            ax[k] = ay[k] = az[k] = 0.f;
        }
        float4 nxt = (j0 + lane < j1) ? pos[o + j0 + lane] : pad;
        for (int jt = j0; jt < j1; jt += kGroup) {
            __syncwarp();
            sP[wid][lane] = nxt;
            __syncwarp();
            if (jt + kGroup < j1) nxt = (jt + kGroup + lane < j1) ? pos[o + jt + kGroup + lane] : pad;
            const int cnt = min(kGroup, j1 - jt);
            const int cnt2 = (cnt + 1) & ~1;  // entries past cnt are zero-mass pads
            for (int j = 0; j < cnt2; j += 2) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float4 q = sP[wid][j + u];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float sc = (q.w * inv) * (inv * inv);
                        ax[k] = fmaf(rx, sc, ax[k]);
                        ay[k] = fmaf(ry, sc, ay[k]);
                        az[k] = fmaf(rz, sc, az[k]);
                    }
                }
            }
        }
        const long long slot = (long long)w + bd.tb_off[s] + tbl;
        float4 *dst = partial + slot * WTB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) dst[lane + 32 * k] = make_float4(ax[k], ay[k], az[k], 0.f);
        it = seg_end;
    }
}

// The reference's kick / damping / drift (unfused, its order), or the bare
// acceleration when acc_out != nullptr.
__device__ __forceinline__ void batch_kick_drift(int i, float ax, float ay, float az,
                                                 const float4 *__restrict__ pos_old,
                                                 float4 *__restrict__ pos_new, float4 *__restrict__ vel,
                                                 float damping, float dt, int kick, float G,
                                                 float4 *__restrict__ acc_out)
{
    if (acc_out) {
        acc_out[i] = make_float4(ax, ay, az, 0.f);
        return;
    }
    float4 p = pos_old[i];
    float4 v = vel[i];
    const float k = kick == NB_KICK_REFERENCE ? p.w : G;
    v.x = __fadd_rn(v.x, __fmul_rn(__fmul_rn(ax, k), dt));
    v.y = __fadd_rn(v.y, __fmul_rn(__fmul_rn(ay, k), dt));
    v.z = __fadd_rn(v.z, __fmul_rn(__fmul_rn(az, k), dt));
    v.x = __fmul_rn(v.x, damping);
    v.y = __fmul_rn(v.y, damping);
    v.z = __fmul_rn(v.z, damping);
    p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
    p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
    p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
    pos_new[i] = p;
    vel[i] = v;
}

__global__ void bk_integrate_kernel(const float4 *__restrict__ pos_old, float4 *__restrict__ pos_new,
                                    float4 *__restrict__ vel, const float4 *__restrict__ partial,
                                    BatchDev bd, int nbody, int wtb, long long total, int workers,
                                    float damping, float dt, int kick, float G,
                                    float4 *__restrict__ acc_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbody) return;
    const int s = bd.body_sys[i];
    const int o = bd.sys_off[s];
    const int ns = bd.sys_off[s + 1] - o;
    const int ngroups = (ns + kGroup - 1) / kGroup;
    const int li = i - o;
    const int tbl = li / wtb;
    const long long first = bd.it_off[s] + (long long)tbl * ngroups;
    const int c0 = sk_owner(first, total, workers);
    const int c1 = sk_owner(first + ngroups - 1, total, workers);
    const long long gtb = (long long)bd.tb_off[s] + tbl;
    const int lj = li - tbl * wtb;
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 q = partial[(c + gtb) * wtb + lj];
        ax = __fadd_rn(ax, q.x);
        ay = __fadd_rn(ay, q.y);
        az = __fadd_rn(az, q.z);
    }
    batch_kick_drift(i, ax, ay, az, pos_old, pos_new, vel, damping, dt, kick, G, acc_out);
}


struct BatchSymDev {
    const int *sys_off;       // [nsys + 1] body offsets
    const long long *it_off;  // [nsys + 1] (row, chunk) item offsets
    const int *row_off;       // [nsys + 1] global row offsets
    const long long *sp_off;  // [nsys + 1] source-side array offsets (float4)
    const int *body_sys;      // [nbody] system of each body
    int nsys;
};

template <int WPB, int BPT>
__global__ void __launch_bounds__(32 * WPB) bks_force_kernel(const float4 *__restrict__ pos, BatchSymDev bd,
                                                             float eps2, float4 *__restrict__ tpart,
                                                             float4 *__restrict__ spart, long long total,
                                                             int workers)
{
    constexpr int RB = 32 * BPT;
    constexpr int RC = BPT;
    __shared__ __align__(16) float4 sC[WPB][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wid;
    if (w >= workers) return;
    long long it = sk_start(w, total, workers);
    const long long end = sk_start(w + 1, total, workers);
    if (it >= end) return;
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    int s = find_sys(bd.it_off, bd.nsys, it);
    while (it < end) {
        while (it >= bd.it_off[s + 1]) ++s;
        const int o = bd.sys_off[s];
        const int ns = bd.sys_off[s + 1] - o;
        const int nc = (ns + 31) / 32, nrb = (ns + RB - 1) / RB;
        const long long base = bd.it_off[s];
        const int I = sym_row_of(it - base, nc, RC, nrb);
        const long long rfirst = base + sym_prefix(I, nc, RC);
        const long long rend = base + sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB;

        float px[BPT], py[BPT], pz[BPT], nm[BPT], ax[BPT], ay[BPT], az[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int li = tbase + lane + 32 * k;
            // missing targets get zero mass: their reactions on the chunk are 0
            const float4 q = li < ns ? pos[o + li] : make_float4(0.f, 0.f, 0.f, 0.f);
            px[k] = q.x;
            py[k] = q.y;
            pz[k] = q.z;
            nm[k] = -q.w;
            ax[k] = ay[k] = az[k] = 0.f;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            __syncwarp();  // previous chunk's reads are done
            sC[wid][lane] = (jb + lane < ns) ? pos[o + jb + lane] : pad;
            __syncwarp();
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 4
                for (int j = 0; j < 32; ++j) {
                    const float4 q = sC[wid][j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float sc = (q.w * inv) * (inv * inv);
                        ax[k] = fmaf(rx, sc, ax[k]);
                        ay[k] = fmaf(ry, sc, ay[k]);
                        az[k] = fmaf(rz, sc, az[k]);
                    }
                }
            } else {
                float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll 2
                for (int r = 0; r < 32; ++r) {
                    const float4 q = sC[wid][(lane + r) & 31];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float inv3 = inv * (inv * inv);
                        const float st = q.w * inv3;
                        const float ss = nm[k] * inv3;
                        ax[k] = fmaf(rx, st, ax[k]);
                        ay[k] = fmaf(ry, st, ay[k]);
                        az[k] = fmaf(rz, st, az[k]);
                        fx = fmaf(rx, ss, fx);
                        fy = fmaf(ry, ss, fy);
                        fz = fmaf(rz, ss, fz);
                    }
                    const int from = (lane + 1) & 31;
                    fx = __shfl_sync(0xffffffffu, fx, from);
                    fy = __shfl_sync(0xffffffffu, fy, from);
                    fz = __shfl_sync(0xffffffffu, fz, from);
                }
                // lane l holds the reaction on chunk body l
                if (jb + lane < ns)
                    spart[bd.sp_off[s] + sym_soff(I, ns, RB) + (jb + lane - (I + 1) * RB)] =
                        make_float4(fx, fy, fz, 0.f);
            }
        }
        float4 *dst = tpart + ((long long)w + bd.row_off[s] + I) * RB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) dst[lane + 32 * k] = make_float4(ax[k], ay[k], az[k], 0.f);
        it = seg_end;
    }
}

// Per body: target-side slots of its row (warp order), then the source-side
// entries of rows 0..I-1 of its system (row order), then kick / drift.
__global__ void bks_integrate_kernel(const float4 *__restrict__ pos_old, float4 *__restrict__ pos_new,
                                     float4 *__restrict__ vel, const float4 *__restrict__ tpart,
                                     const float4 *__restrict__ spart, BatchSymDev bd, int nbody, int rb,
                                     long long total, int workers, float damping, float dt, int kick,
                                     float G, float4 *__restrict__ acc_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbody) return;
    const int s = bd.body_sys[i];
    const int o = bd.sys_off[s];
    const int ns = bd.sys_off[s + 1] - o;
    const int li = i - o;
    const int rc = rb / 32;
    const int nc = (ns + 31) / 32;
    const int I = li / rb;
    const long long base = bd.it_off[s];
    const int c0 = sk_owner(base + sym_prefix(I, nc, rc), total, workers);
    const int c1 = sk_owner(base + sym_prefix(I + 1, nc, rc) - 1, total, workers);
    const long long grow = (long long)bd.row_off[s] + I;
    const int lj = li - I * rb;
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 q = tpart[(c + grow) * rb + lj];
        ax = __fadd_rn(ax, q.x);
        ay = __fadd_rn(ay, q.y);
        az = __fadd_rn(az, q.z);
    }
    long long off = bd.sp_off[s] + li - rb;  // row r at soff(r) + li - (r + 1) rb
    for (int r = 0; r < I; ++r) {
        const float4 q = spart[off];
        off += (long long)ns - (long long)(r + 2) * rb;
        ax = __fadd_rn(ax, q.x);
        ay = __fadd_rn(ay, q.y);
        az = __fadd_rn(az, q.z);
    }
    batch_kick_drift(i, ax, ay, az, pos_old, pos_new, vel, damping, dt, kick, G, acc_out);
}

// Float-float batched symmetric kernel for FP64 state: the layout and work
// split of bks_force_kernel, the pair arithmetic of symff_force_kernel
// (nb_ff.cuh; grid-split positions scaled by the batch's powers of two),
// each chunk's target sums folded into FP64, reactions written as FP64.
template <int WPB, int BPT>
__global__ void __launch_bounds__(32 * WPB)
    bksff_force_kernel(const float4 *__restrict__ H, const float4 *__restrict__ Mi, const float4 *__restrict__ Lo,
                       BatchSymDev bd, double eps2, const unsigned long long *__restrict__ range,
                       double4 *__restrict__ tpart, double4 *__restrict__ spart, long long total, int workers)
{
    constexpr int RB = 32 * BPT;
    constexpr int RC = BPT;
    __shared__ __align__(16) float4 sH[WPB][32], sM[WPB][32], sL[WPB][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wid;
    if (w >= workers) return;
    long long it = sk_start(w, total, workers);
    const long long end = sk_start(w + 1, total, workers);
    if (it >= end) return;
    // eps2 in the scaled units (x 2^(2 kx)), as a float-float
    const double e2s = ldexp(eps2, -2 * ff_exponent(range[0]));
    const float eh = __double2float_rn(e2s), el = __double2float_rn(e2s - (double)eh);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    int s = find_sys(bd.it_off, bd.nsys, it);
    while (it < end) {
        while (it >= bd.it_off[s + 1]) ++s;
        const int o = bd.sys_off[s];
        const int ns = bd.sys_off[s + 1] - o;
        const int nc = (ns + 31) / 32, nrb = (ns + RB - 1) / RB;
        const long long base = bd.it_off[s];
        const int I = sym_row_of(it - base, nc, RC, nrb);
        const long long rfirst = base + sym_prefix(I, nc, RC);
        const long long rend = base + sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB;
        // missing targets: zero mass, so their reactions are 0; masses
        // negated: reactions point along -r
        float pxh[BPT], pxm[BPT], pxl[BPT], pyh[BPT], pym[BPT], pyl[BPT], pzh[BPT], pzm[BPT], pzl[BPT];
        float nmh[BPT], nml[BPT];
        double ax[BPT], ay[BPT], az[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int li = tbase + lane + 32 * k;
            const float4 a = li < ns ? H[o + li] : zero;
            const float4 m = li < ns ? Mi[o + li] : zero;
            const float4 q = li < ns ? Lo[o + li] : zero;
            pxh[k] = a.x; pxm[k] = m.x; pxl[k] = q.x;
            pyh[k] = a.y; pym[k] = m.y; pyl[k] = q.y;
            pzh[k] = a.z; pzm[k] = m.z; pzl[k] = q.z;
            nmh[k] = -a.w; nml[k] = -m.w;
            ax[k] = ay[k] = az[k] = 0.0;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            const bool in = jb + lane < ns;
            __syncwarp();  // previous chunk's reads are done
            // padding: far away (scaled coordinates are below 1), no mass
            sH[wid][lane] = in ? H[o + jb + lane] : make_float4(1.0e6f, 1.0e6f, 1.0e6f, 0.f);
            sM[wid][lane] = in ? Mi[o + jb + lane] : zero;
            sL[wid][lane] = in ? Lo[o + jb + lane] : zero;
            __syncwarp();
            float Axh[BPT], Axl[BPT], Ayh[BPT], Ayl[BPT], Azh[BPT], Azl[BPT];
#pragma unroll
            for (int k = 0; k < BPT; ++k) Axh[k] = Axl[k] = Ayh[k] = Ayl[k] = Azh[k] = Azl[k] = 0.f;
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 1
                for (int j = 0; j < 32; ++j) {
                    const float4 a = sH[wid][j], am = sM[wid][j], q = sL[wid][j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        FFPair f;
                        ff_pair<false>(a, am, q, pxh[k], pxm[k], pxl[k], pyh[k], pym[k], pyl[k], pzh[k], pzm[k],
                                       pzl[k], 0.f, 0.f, eh, el, f);
                        ff_acc(Axh[k], Axl[k], f.rxh, f.rxl, f.wjh, f.wjl);
                        ff_acc(Ayh[k], Ayl[k], f.ryh, f.ryl, f.wjh, f.wjl);
                        ff_acc(Azh[k], Azl[k], f.rzh, f.rzl, f.wjh, f.wjl);
                    }
                }
            } else {
                float Fxh = 0.f, Fxl = 0.f, Fyh = 0.f, Fyl = 0.f, Fzh = 0.f, Fzl = 0.f;
#pragma unroll 1
                for (int r = 0; r < 32; ++r) {
                    const int idx = (lane + r) & 31;
                    const float4 a = sH[wid][idx], am = sM[wid][idx], q = sL[wid][idx];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        FFPair f;
                        ff_pair<true>(a, am, q, pxh[k], pxm[k], pxl[k], pyh[k], pym[k], pyl[k], pzh[k], pzm[k],
                                      pzl[k], nmh[k], nml[k], eh, el, f);
                        ff_acc(Axh[k], Axl[k], f.rxh, f.rxl, f.wjh, f.wjl);
                        ff_acc(Ayh[k], Ayl[k], f.ryh, f.ryl, f.wjh, f.wjl);
                        ff_acc(Azh[k], Azl[k], f.rzh, f.rzl, f.wjh, f.wjl);
                        ff_acc(Fxh, Fxl, f.rxh, f.rxl, f.wih, f.wil);
                        ff_acc(Fyh, Fyl, f.ryh, f.ryl, f.wih, f.wil);
                        ff_acc(Fzh, Fzl, f.rzh, f.rzl, f.wih, f.wil);
                    }
                    const int from = (lane + 1) & 31;
                    Fxh = __shfl_sync(0xffffffffu, Fxh, from);
                    Fxl = __shfl_sync(0xffffffffu, Fxl, from);
                    Fyh = __shfl_sync(0xffffffffu, Fyh, from);
                    Fyl = __shfl_sync(0xffffffffu, Fyl, from);
                    Fzh = __shfl_sync(0xffffffffu, Fzh, from);
                    Fzl = __shfl_sync(0xffffffffu, Fzl, from);
                }
                // lane l holds the reaction on chunk body l
                if (in)
                    spart[bd.sp_off[s] + sym_soff(I, ns, RB) + (jb + lane - (I + 1) * RB)] =
                        make_double4((double)Fxh + (double)Fxl, (double)Fyh + (double)Fyl,
                                     (double)Fzh + (double)Fzl, 0.0);
            }
#pragma unroll
            for (int k = 0; k < BPT; ++k) {
                ax[k] += (double)Axh[k] + (double)Axl[k];
                ay[k] += (double)Ayh[k] + (double)Ayl[k];
                az[k] += (double)Azh[k] + (double)Azl[k];
            }
        }
        double4 *dst = tpart + ((long long)w + bd.row_off[s] + I) * RB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) dst[lane + 32 * k] = make_double4(ax[k], ay[k], az[k], 0.0);
        it = seg_end;
    }
}

// Per body: FP64 sums of the target-side slots of its row (warp order) and
// the source-side entries of rows 0..I-1 of its system (row order), the
// batch's scaling undone (a = a_scaled * 2^(2 kx - km), exact), then the
// reference's kick / damping / drift in its order with unfused IEEE
// operations (bodysystem.cc:135-182), or the bare acceleration.
__global__ void bksff_integrate_kernel(const double4 *__restrict__ pos_old, double4 *__restrict__ pos_new,
                                       double4 *__restrict__ vel, const double4 *__restrict__ tpart,
                                       const double4 *__restrict__ spart, BatchSymDev bd, int nbody, int rb,
                                       long long total, int workers, double damping, double dt, int kick,
                                       double G, const unsigned long long *__restrict__ range,
                                       double4 *__restrict__ acc_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbody) return;
    const int s = bd.body_sys[i];
    const int o = bd.sys_off[s];
    const int ns = bd.sys_off[s + 1] - o;
    const int li = i - o;
    const int rc = rb / 32;
    const int nc = (ns + 31) / 32;
    const int I = li / rb;
    const long long base = bd.it_off[s];
    const int c0 = sk_owner(base + sym_prefix(I, nc, rc), total, workers);
    const int c1 = sk_owner(base + sym_prefix(I + 1, nc, rc) - 1, total, workers);
    const long long grow = (long long)bd.row_off[s] + I;
    const int lj = li - I * rb;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int c = c0; c <= c1; ++c) {
        const double4 q = tpart[(c + grow) * rb + lj];
        ax = __dadd_rn(ax, q.x);
        ay = __dadd_rn(ay, q.y);
        az = __dadd_rn(az, q.z);
    }
    long long off = bd.sp_off[s] + li - rb;  // row r at soff(r) + li - (r + 1) rb
    for (int r = 0; r < I; ++r) {
        const double4 q = spart[off];
        off += (long long)ns - (long long)(r + 2) * rb;
        ax = __dadd_rn(ax, q.x);
        ay = __dadd_rn(ay, q.y);
        az = __dadd_rn(az, q.z);
    }
    const int k2 = ff_exponent(range[1]) - 2 * ff_exponent(range[0]);
    ax = ldexp(ax, k2);
    ay = ldexp(ay, k2);
    az = ldexp(az, k2);
    if (acc_out) {
        acc_out[i] = make_double4(ax, ay, az, 0.0);
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

typedef void (*bksff_kernel_t)(const float4 *, const float4 *, const float4 *, BatchSymDev, double,
                               const unsigned long long *, double4 *, double4 *, long long, int);

static bksff_kernel_t bksff_kernel_for(int wpb, int bpt)
{
#define NB_BKSFF(W, B) \
    if (wpb == W && bpt == B) return bksff_force_kernel<W, B>;
    NB_BKSFF(1, 2) NB_BKSFF(1, 4) NB_BKSFF(2, 2) NB_BKSFF(2, 4) NB_BKSFF(4, 2) NB_BKSFF(4, 4)
#undef NB_BKSFF
    return nullptr;
}

typedef void (*bks_kernel_t)(const float4 *, BatchSymDev, float, float4 *, float4 *, long long, int);

static bks_kernel_t bks_kernel_for(int wpb, int bpt)
{
#define NB_BKS(W, B) \
    if (wpb == W && bpt == B) return bks_force_kernel<W, B>;
    NB_BKS(1, 8) NB_BKS(1, 12) NB_BKS(1, 16) NB_BKS(2, 8) NB_BKS(2, 16) NB_BKS(4, 8) NB_BKS(4, 16)
#undef NB_BKS
    return nullptr;
}

// Batched adjoint: the vector-Jacobian product of one step for every system
// (same algebra as vjp_pair_kernel in nb_adjoint.cu: out_k = m_k P - q g_k -
// 3 Q and dm_k = -sum inv^3 r.g_j), warp-level stream-K over the batch.
template <int WPB, int BPT>
__global__ void __launch_bounds__(32 * WPB) bk_vjp_kernel(const float4 *__restrict__ pos,
                                                          const float4 *__restrict__ gbuf, BatchDev bd,
                                                          float eps2, float4 *__restrict__ partial,
                                                          long long total, int workers)
{
    constexpr int WTB = 32 * BPT;
    __shared__ __align__(16) float4 sP[WPB][32];
    __shared__ __align__(16) float4 sG[WPB][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wid;
    if (w >= workers) return;
    long long it = sk_start(w, total, workers);
    const long long end = sk_start(w + 1, total, workers);
    if (it >= end) return;
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    int s = find_sys(bd.it_off, bd.nsys, it);
    while (it < end) {
        while (it >= bd.it_off[s + 1]) ++s;
        const int o = bd.sys_off[s];
        const int ns = bd.sys_off[s + 1] - o;
        const int ngroups = (ns + kGroup - 1) / kGroup;
        const long long base = bd.it_off[s];
        const int tbl = (int)((it - base) / ngroups);
        const long long blk_first = base + (long long)tbl * ngroups;
        const long long seg_end = end < blk_first + ngroups ? end : blk_first + ngroups;
        const int j0 = (int)(it - blk_first) * kGroup;
        const int j1 = min((int)(seg_end - blk_first) * kGroup, ns);

        float px[BPT], py[BPT], pz[BPT], pm[BPT], gx[BPT], gy[BPT], gz[BPT];
        float Px[BPT], Py[BPT], Pz[BPT], Q0[BPT], Q1[BPT], Q2[BPT], q[BPT], dm[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int li = tbl * WTB + lane + 32 * k;
            const float4 a = li < ns ? pos[o + li] : zero;
            const float4 g = li < ns ? gbuf[o + li] : zero;
            px[k] = a.x; py[k] = a.y; pz[k] = a.z; pm[k] = a.w;
            gx[k] = g.x; gy[k] = g.y; gz[k] = g.z;
            Px[k] = Py[k] = Pz[k] = Q0[k] = Q1[k] = Q2[k] = q[k] = dm[k] = 0.f;
        }
        float4 nxp = (j0 + lane < j1) ? pos[o + j0 + lane] : pad;
        float4 nxg = (j0 + lane < j1) ? gbuf[o + j0 + lane] : zero;
        for (int jt = j0; jt < j1; jt += kGroup) {
            __syncwarp();
            sP[wid][lane] = nxp;
            sG[wid][lane] = nxg;
            __syncwarp();
            if (jt + kGroup < j1) {
                const int jn = jt + kGroup + lane;
                nxp = jn < j1 ? pos[o + jn] : pad;
                nxg = jn < j1 ? gbuf[o + jn] : zero;
            }
            const int cnt = min(kGroup, j1 - jt);
            for (int j = 0; j < cnt; ++j) {
                const float4 sv = sP[wid][j];
                const float4 g = sG[wid][j];
#pragma unroll
                for (int k = 0; k < BPT; ++k) {
                    const float rx = sv.x - px[k], ry = sv.y - py[k], rz = sv.z - pz[k];
                    float d2 = fmaf(rx, rx, eps2);
                    d2 = fmaf(ry, ry, d2);
                    d2 = fmaf(rz, rz, d2);
                    const float inv = rsqrt_approx(d2);
                    const float inv2 = inv * inv;
                    const float inv3 = inv2 * inv;
                    const float inv5 = inv3 * inv2;
                    Px[k] = fmaf(inv3, g.x, Px[k]);
                    Py[k] = fmaf(inv3, g.y, Py[k]);
                    Pz[k] = fmaf(inv3, g.z, Pz[k]);
                    q[k] = fmaf(inv3, sv.w, q[k]);
                    const float rgj = fmaf(rz, g.z, fmaf(ry, g.y, rx * g.x));
                    const float rgk = fmaf(rz, gz[k], fmaf(ry, gy[k], rx * gx[k]));
                    const float cc = inv5 * fmaf(pm[k], rgj, -(sv.w * rgk));
                    Q0[k] = fmaf(cc, rx, Q0[k]);
                    Q1[k] = fmaf(cc, ry, Q1[k]);
                    Q2[k] = fmaf(cc, rz, Q2[k]);
                    dm[k] = fmaf(inv3, rgj, dm[k]);
                }
            }
        }
        const long long slot = (long long)w + bd.tb_off[s] + tbl;
        float4 *dst = partial + slot * WTB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const float ox = fmaf(pm[k], Px[k], fmaf(-q[k], gx[k], -3.f * Q0[k]));
            const float oy = fmaf(pm[k], Py[k], fmaf(-q[k], gy[k], -3.f * Q1[k]));
            const float oz = fmaf(pm[k], Pz[k], fmaf(-q[k], gz[k], -3.f * Q2[k]));
            dst[lane + 32 * k] = make_float4(ox, oy, oz, -dm[k]);
        }
        it = seg_end;
    }
}

__global__ void bk_adj_update_kernel(const float4 *__restrict__ partial, BatchDev bd, int nbody,
                                     int wtb, long long total, int workers,
                                     const float4 *__restrict__ pos, const float4 *__restrict__ acc,
                                     float4 *__restrict__ lx, float4 *__restrict__ lv,
                                     float *__restrict__ gm, float4 *__restrict__ gbuf,
                                     float damping, float dt, int kick, float G, int want_next_g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbody) return;
    const int s = bd.body_sys[i];
    const int o = bd.sys_off[s];
    const int ns = bd.sys_off[s + 1] - o;
    const int ngroups = (ns + kGroup - 1) / kGroup;
    const int li = i - o;
    const int tbl = li / wtb;
    const long long first = bd.it_off[s] + (long long)tbl * ngroups;
    const int c0 = sk_owner(first, total, workers);
    const int c1 = sk_owner(first + ngroups - 1, total, workers);
    const long long gtb = (long long)bd.tb_off[s] + tbl;
    const int lj = li - tbl * wtb;
    float ox = 0.f, oy = 0.f, oz = 0.f, odm = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 qv = partial[(c + gtb) * wtb + lj];
        ox += qv.x;
        oy += qv.y;
        oz += qv.z;
        odm += qv.w;
    }
    adj_body_update(i, ox, oy, oz, odm, pos, acc, lx, lv, gm, gbuf, damping, dt, kick, G, want_next_g);
}

// Symmetric batched VJP: sym_vjp_kernel's pair algebra (nb_adjoint.cu: each
// unordered pair once, the chunk body's eight reaction sums rotating through
// the warp) on the symmetric batched layout of bks_force_kernel.
template <int WPB, int BPT>
__global__ void __launch_bounds__(32 * WPB) bks_vjp_kernel(const float4 *__restrict__ pos,
                                                           const float4 *__restrict__ gbuf, BatchSymDev bd,
                                                           float eps2, float4 *__restrict__ tpart,
                                                           float4 *__restrict__ spart, long long total,
                                                           int workers)
{
    constexpr int RB = 32 * BPT;
    constexpr int RC = BPT;
    __shared__ __align__(16) float4 sC[WPB][32];
    __shared__ __align__(16) float4 sG[WPB][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wid;
    if (w >= workers) return;
    long long it = sk_start(w, total, workers);
    const long long end = sk_start(w + 1, total, workers);
    if (it >= end) return;
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    int s = find_sys(bd.it_off, bd.nsys, it);
    while (it < end) {
        while (it >= bd.it_off[s + 1]) ++s;
        const int o = bd.sys_off[s];
        const int ns = bd.sys_off[s + 1] - o;
        const int nc = (ns + 31) / 32, nrb = (ns + RB - 1) / RB;
        const long long base = bd.it_off[s];
        const int I = sym_row_of(it - base, nc, RC, nrb);
        const long long rfirst = base + sym_prefix(I, nc, RC);
        const long long rend = base + sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB;

        // missing targets: zero mass and zero g, so every term they give is 0
        float px[BPT], py[BPT], pz[BPT], pm[BPT], gx[BPT], gy[BPT], gz[BPT];
        float Px[BPT], Py[BPT], Pz[BPT], Q0[BPT], Q1[BPT], Q2[BPT], q[BPT], dm[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int li = tbase + lane + 32 * k;
            const float4 a = li < ns ? pos[o + li] : zero;
            const float4 g = li < ns ? gbuf[o + li] : zero;
            px[k] = a.x; py[k] = a.y; pz[k] = a.z; pm[k] = a.w;
            gx[k] = g.x; gy[k] = g.y; gz[k] = g.z;
            Px[k] = Py[k] = Pz[k] = Q0[k] = Q1[k] = Q2[k] = q[k] = dm[k] = 0.f;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            __syncwarp();  // previous chunk's reads are done
            sC[wid][lane] = (jb + lane < ns) ? pos[o + jb + lane] : pad;
            sG[wid][lane] = (jb + lane < ns) ? gbuf[o + jb + lane] : zero;
            __syncwarp();
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 2
                for (int j = 0; j < 32; ++j) {
                    const float4 sb = sC[wid][j];
                    const float4 g = sG[wid][j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = sb.x - px[k], ry = sb.y - py[k], rz = sb.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float inv2 = inv * inv;
                        const float inv3 = inv2 * inv;
                        const float inv5 = inv3 * inv2;
                        Px[k] = fmaf(inv3, g.x, Px[k]);
                        Py[k] = fmaf(inv3, g.y, Py[k]);
                        Pz[k] = fmaf(inv3, g.z, Pz[k]);
                        q[k] = fmaf(inv3, sb.w, q[k]);
                        const float rgj = fmaf(rz, g.z, fmaf(ry, g.y, rx * g.x));
                        const float rgk = fmaf(rz, gz[k], fmaf(ry, gy[k], rx * gx[k]));
                        const float cc = inv5 * fmaf(pm[k], rgj, -(sb.w * rgk));
                        Q0[k] = fmaf(cc, rx, Q0[k]);
                        Q1[k] = fmaf(cc, ry, Q1[k]);
                        Q2[k] = fmaf(cc, rz, Q2[k]);
                        dm[k] = fmaf(inv3, rgj, dm[k]);
                    }
                }
            } else {
                float rPx = 0.f, rPy = 0.f, rPz = 0.f, rq = 0.f, rQ0 = 0.f, rQ1 = 0.f, rQ2 = 0.f, rw = 0.f;
#pragma unroll 2
                for (int r = 0; r < 32; ++r) {
                    const int idx = (lane + r) & 31;
                    const float4 sb = sC[wid][idx];
                    const float4 g = sG[wid][idx];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = sb.x - px[k], ry = sb.y - py[k], rz = sb.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float inv2 = inv * inv;
                        const float inv3 = inv2 * inv;
                        const float inv5 = inv3 * inv2;
                        const float rgj = fmaf(rz, g.z, fmaf(ry, g.y, rx * g.x));
                        const float rgk = fmaf(rz, gz[k], fmaf(ry, gy[k], rx * gx[k]));
                        const float cc = inv5 * fmaf(pm[k], rgj, -(sb.w * rgk));
                        Px[k] = fmaf(inv3, g.x, Px[k]);
                        Py[k] = fmaf(inv3, g.y, Py[k]);
                        Pz[k] = fmaf(inv3, g.z, Pz[k]);
                        q[k] = fmaf(inv3, sb.w, q[k]);
                        Q0[k] = fmaf(cc, rx, Q0[k]);
                        Q1[k] = fmaf(cc, ry, Q1[k]);
                        Q2[k] = fmaf(cc, rz, Q2[k]);
                        dm[k] = fmaf(inv3, rgj, dm[k]);
                        rPx = fmaf(inv3, gx[k], rPx);
                        rPy = fmaf(inv3, gy[k], rPy);
                        rPz = fmaf(inv3, gz[k], rPz);
                        rq = fmaf(inv3, pm[k], rq);
                        rQ0 = fmaf(-cc, rx, rQ0);
                        rQ1 = fmaf(-cc, ry, rQ1);
                        rQ2 = fmaf(-cc, rz, rQ2);
                        rw = fmaf(inv3, rgk, rw);
                    }
                    const int from = (lane + 1) & 31;
                    rPx = __shfl_sync(0xffffffffu, rPx, from);
                    rPy = __shfl_sync(0xffffffffu, rPy, from);
                    rPz = __shfl_sync(0xffffffffu, rPz, from);
                    rq = __shfl_sync(0xffffffffu, rq, from);
                    rQ0 = __shfl_sync(0xffffffffu, rQ0, from);
                    rQ1 = __shfl_sync(0xffffffffu, rQ1, from);
                    rQ2 = __shfl_sync(0xffffffffu, rQ2, from);
                    rw = __shfl_sync(0xffffffffu, rw, from);
                }
                // lane l holds chunk body l's reaction
                if (jb + lane < ns) {
                    const float4 sb = sC[wid][lane], gb = sG[wid][lane];
                    const float ox = fmaf(sb.w, rPx, fmaf(-rq, gb.x, -3.f * rQ0));
                    const float oy = fmaf(sb.w, rPy, fmaf(-rq, gb.y, -3.f * rQ1));
                    const float oz = fmaf(sb.w, rPz, fmaf(-rq, gb.z, -3.f * rQ2));
                    spart[bd.sp_off[s] + sym_soff(I, ns, RB) + (jb + lane - (I + 1) * RB)] =
                        make_float4(ox, oy, oz, rw);
                }
            }
        }
        float4 *dst = tpart + ((long long)w + bd.row_off[s] + I) * RB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const float ox = fmaf(pm[k], Px[k], fmaf(-q[k], gx[k], -3.f * Q0[k]));
            const float oy = fmaf(pm[k], Py[k], fmaf(-q[k], gy[k], -3.f * Q1[k]));
            const float oz = fmaf(pm[k], Pz[k], fmaf(-q[k], gz[k], -3.f * Q2[k]));
            dst[lane + 32 * k] = make_float4(ox, oy, oz, -dm[k]);
        }
        it = seg_end;
    }
}

// Symmetric batched reverse-step update: target-side slots (warp order) and
// source-side rows (row order) of the body's system, then the per-body update.
__global__ void bks_adj_update_kernel(const float4 *__restrict__ tpart, const float4 *__restrict__ spart,
                                      BatchSymDev bd, int nbody, int rb, long long total, int workers,
                                      const float4 *__restrict__ pos, const float4 *__restrict__ acc,
                                      float4 *__restrict__ lx, float4 *__restrict__ lv,
                                      float *__restrict__ gm, float4 *__restrict__ gbuf, float damping,
                                      float dt, int kick, float G, int want_next_g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbody) return;
    const int s = bd.body_sys[i];
    const int o = bd.sys_off[s];
    const int ns = bd.sys_off[s + 1] - o;
    const int li = i - o;
    const int rc = rb / 32;
    const int nc = (ns + 31) / 32;
    const int I = li / rb;
    const long long base = bd.it_off[s];
    const int c0 = sk_owner(base + sym_prefix(I, nc, rc), total, workers);
    const int c1 = sk_owner(base + sym_prefix(I + 1, nc, rc) - 1, total, workers);
    const long long grow = (long long)bd.row_off[s] + I;
    const int lj = li - I * rb;
    float ox = 0.f, oy = 0.f, oz = 0.f, odm = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 qv = tpart[(c + grow) * rb + lj];
        ox += qv.x;
        oy += qv.y;
        oz += qv.z;
        odm += qv.w;
    }
    long long off = bd.sp_off[s] + li - rb;  // row r at soff(r) + li - (r + 1) rb
    for (int r = 0; r < I; ++r) {
        const float4 qv = spart[off];
        off += (long long)ns - (long long)(r + 2) * rb;
        ox += qv.x;
        oy += qv.y;
        oz += qv.z;
        odm += qv.w;
    }
    adj_body_update(i, ox, oy, oz, odm, pos, acc, lx, lv, gm, gbuf, damping, dt, kick, G, want_next_g);
}

typedef void (*bks_vjp_t)(const float4 *, const float4 *, BatchSymDev, float, float4 *, float4 *, long long,
                          int);

static bks_vjp_t bks_vjp_for(int wpb, int bpt)
{
    if (wpb == 1 && bpt == 10) return bks_vjp_kernel<1, 10>;
    if (wpb == 1 && bpt == 8) return bks_vjp_kernel<1, 8>;
    return nullptr;
}

typedef void (*bk_vjp_t)(const float4 *, const float4 *, BatchDev, float, float4 *, long long, int);

static bk_vjp_t bk_vjp_for(int wpb, int bpt)
{
    if (wpb == 4 && bpt == 2) return bk_vjp_kernel<4, 2>;
    if (wpb == 4 && bpt == 4) return bk_vjp_kernel<4, 4>;
    if (wpb == 8 && bpt == 4) return bk_vjp_kernel<8, 4>;
    return nullptr;
}

typedef void (*bk_kernel_t)(const float4 *, BatchDev, float, float4 *, long long, int);

static bk_kernel_t bk_kernel_for(int wpb, int bpt)
{
#define NB_BK(W, B) \
    if (wpb == W && bpt == B) return bk_force_kernel<W, B>;
    NB_BK(2, 4) NB_BK(2, 8) NB_BK(4, 2) NB_BK(4, 4) NB_BK(4, 8) NB_BK(8, 2) NB_BK(8, 4) NB_BK(8, 8)
#undef NB_BK
    return nullptr;
}

}  // namespace nb

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchPlan {
    int wpb = 0, bpt = 0, grid = 0, workers = 0;
    long long total = 0, total_wtb = 0, slots = 0;
    long long spart = 0;  // symmetric: float4 entries of all source-side arrays
};

struct nb_batch {
    nb_params p;
    int device = 0, sms = 0;
    int nsys = 0, nbody = 0;
    std::vector<int> sizes;
    int *d_sys_off = nullptr, *d_tb_off = nullptr, *d_body_sys = nullptr;
    long long *d_it_off = nullptr;
    float4 *pos[2] = {nullptr, nullptr};
    float4 *vel = nullptr;
    int cur = 0;
    bool has_state = false;
    float4 *partial = nullptr;
    size_t partial_cap = 0;  // float4 entries
    // NB_ALGO_SYM: source-side arrays of all systems and their offsets
    bool sym = false;
    long long *d_sp_off = nullptr;
    float4 *spart = nullptr;
    size_t spart_cap = 0;
    BatchPlan plan;
    // graph of `graph_steps` steps starting from pos[graph_cur]
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0, graph_cur = -1;
    // scratch of the per-system baseline (target-side and source-side)
    float4 *sys_partial = nullptr, *sys_spart = nullptr;
    // NB_F64 state (NB_ALGO_SYM): pos / vel / partial / spart hold double4
    // (twice the float4 entries), stepped by the float-float batched kernel
    // from the scaled grid split (3 nbody float4) and the batch's
    // scale record
    bool f64 = false;
    float4 *ff_split = nullptr;
    unsigned long long *ff_range = nullptr;
    // plan, scratch and device tables agree; false after a failed plan change
    // (launches then refuse to run rather than use a stale or NULL scratch)
    bool plan_ok = false;
    // adjoint: VJP plan (own iteration tables), checkpoints, reverse buffers
    BatchPlan vplan;
    long long *d_it_off_v = nullptr;
    int *d_tb_off_v = nullptr;
    float4 *vpartial = nullptr;
    long long *d_sp_off_v = nullptr;  // symmetric VJP: source-side offsets
    float4 *vspart = nullptr;         // and arrays
    bool adj_live_last = false;       // last segment's states left by the forward
    int adj_steps = 0, adj_every = 0, adj_nckpt = 0, cap_ckpt = 0, cap_seg = 0;
    bool adj_ready = false;
    unsigned long long adj_generation = 0;  // number of the recorded forward pass
    float4 *ckpt_pos = nullptr, *ckpt_vel = nullptr, *seg_pos = nullptr, *seg_acc = nullptr;
    // second segment buffer and stream: segment s-1 is recomputed on rstream
    // while the reverse pass runs through segment s
    float4 *seg_pos2 = nullptr, *seg_acc2 = nullptr, *vel_tmp2 = nullptr;
    cudaStream_t rstream = nullptr;
    cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_go = nullptr;
    float4 *vel_tmp = nullptr, *lx = nullptr, *lv = nullptr, *gbuf = nullptr;
    float *gm = nullptr;
};

using nb::set_error;

static int batch_plan_for(nb_batch *b, int wpb, int bpt, BatchPlan *out, std::vector<long long> *it_off,
                          std::vector<int> *tb_off, std::vector<long long> *sp_off)
{
    const void *k = b->f64 ? (const void *)nb::bksff_kernel_for(wpb, bpt)
                    : b->sym ? (const void *)nb::bks_kernel_for(wpb, bpt)
                             : (const void *)nb::bk_kernel_for(wpb, bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "batched kernel shape not compiled");
    const int wtb = 32 * bpt;
    it_off->assign(b->nsys + 1, 0);
    tb_off->assign(b->nsys + 1, 0);
    sp_off->assign(b->nsys + 1, 0);
    for (int s = 0; s < b->nsys; ++s) {
        const long long n = b->sizes[s];
        const long long ntb = (n + wtb - 1) / wtb, ng = (n + nb::kGroup - 1) / nb::kGroup;
        // directed: (target block, source group) items; symmetric: (row,
        // chunk) items of the triangular layout, rows of 32 * bpt bodies
        const long long items = b->sym ? nb::sym_prefix(ntb, (int)ng, bpt) : ntb * ng;
        (*it_off)[s + 1] = (*it_off)[s] + items;
        (*tb_off)[s + 1] = (*tb_off)[s] + (int)ntb;
        (*sp_off)[s + 1] = (*sp_off)[s] + (b->sym ? nb::sym_spart_entries((int)n, wtb) : 0);
    }
    int occ = 0;
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * wpb, 0));
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "batched kernel does not fit on an SM");
    BatchPlan p;
    p.wpb = wpb;
    p.bpt = bpt;
    p.total = (*it_off)[b->nsys];
    p.total_wtb = (*tb_off)[b->nsys];
    p.spart = (*sp_off)[b->nsys];
    long long workers = (long long)b->sms * occ * wpb;
    if (p.total > 0 && workers > p.total) workers = p.total;
    p.workers = p.total > 0 ? (int)workers : 0;
    p.grid = (p.workers + wpb - 1) / wpb;
    p.slots = p.total > 0 ? p.workers + p.total_wtb - 1 : 0;
    *out = p;
    return NB_OK;
}

static int batch_apply_plan(nb_batch *b, int wpb, int bpt, cudaStream_t s)
{
    BatchPlan p;
    std::vector<long long> it_off, sp_off;
    std::vector<int> tb_off;
    int st = batch_plan_for(b, wpb, bpt, &p, &it_off, &tb_off, &sp_off);
    if (st) return st;
    // from here on the scratch, the tables or both change: the captured graph
    // (its arguments) and the old plan are void until this call succeeds
    b->plan_ok = false;
    if (b->graph) {
        nb::graph_exec_destroy(b->graph);
        b->graph = nullptr;
        b->graph_cur = -1;
    }
    const size_t wide = b->f64 ? 2 : 1;  // float4 entries per partial entry
    const size_t need = (size_t)p.slots * 32 * bpt * wide;
    if (need > b->partial_cap) {
        nb::dfree(b->partial);
        b->partial = nullptr;
        b->partial_cap = 0;
        cudaError_t e = nb::dmalloc((void **)&b->partial, need * sizeof(float4));
        if (e != cudaSuccess) return nb::cuda_error(e, "batched scratch allocation");
        b->partial_cap = need;
    }
    if ((size_t)p.spart * wide > b->spart_cap) {
        nb::dfree(b->spart);
        b->spart = nullptr;
        b->spart_cap = 0;
        cudaError_t e = nb::dmalloc((void **)&b->spart, (size_t)p.spart * wide * sizeof(float4));
        if (e != cudaSuccess) return nb::cuda_error(e, "batched source-side allocation");
        b->spart_cap = (size_t)p.spart * wide;
    }
    if (b->sym)
        NB_CUDA(cudaMemcpyAsync(b->d_sp_off, sp_off.data(), sp_off.size() * sizeof(long long),
                                cudaMemcpyHostToDevice, s));
    NB_CUDA(cudaMemcpyAsync(b->d_it_off, it_off.data(), it_off.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, s));
    NB_CUDA(cudaMemcpyAsync(b->d_tb_off, tb_off.data(), tb_off.size() * sizeof(int),
                            cudaMemcpyHostToDevice, s));
    NB_CUDA(cudaStreamSynchronize(s));
    b->plan = p;
    b->plan_ok = true;
    return NB_OK;
}

static nb::BatchDev batch_dev(const nb_batch *b)
{
    nb::BatchDev d;
    d.sys_off = b->d_sys_off;
    d.it_off = b->d_it_off;
    d.tb_off = b->d_tb_off;
    d.body_sys = b->d_body_sys;
    d.nsys = b->nsys;
    return d;
}

static nb::BatchSymDev batch_sym_dev(const nb_batch *b)
{
    nb::BatchSymDev d;
    d.sys_off = b->d_sys_off;
    d.it_off = b->d_it_off;
    d.row_off = b->d_tb_off;
    d.sp_off = b->d_sp_off;
    d.body_sys = b->d_body_sys;
    d.nsys = b->nsys;
    return d;
}

// The batched force pass at positions po (partials into the batch scratch).
static int batch_force(nb_batch *b, const float4 *po, cudaStream_t s)
{
    const BatchPlan &p = b->plan;
    if (b->nbody == 0) return NB_OK;
    if (!b->plan_ok)
        return set_error(NB_ERR_STATE, "batch has no valid launch plan (a plan change or autotune failed)");
    if (b->f64) {
        float4 *H = b->ff_split, *M = H + b->nbody, *L = M + b->nbody;
        int st = nb::ff_scale_split((const double4 *)po, b->nbody, b->sms, H, M, L, b->ff_range, s);
        if (st) return st;
        nb::bksff_kernel_t k = nb::bksff_kernel_for(p.wpb, p.bpt);
        k<<<p.grid, 32 * p.wpb, 0, s>>>(H, M, L, batch_sym_dev(b), b->p.eps2, b->ff_range, (double4 *)b->partial,
                                        (double4 *)b->spart, p.total, p.workers);
        NB_LAUNCH_CHECK("bksff_force_kernel launch");
        return NB_OK;
    }
    if (b->sym) {
        nb::bks_kernel_t k = nb::bks_kernel_for(p.wpb, p.bpt);
        k<<<p.grid, 32 * p.wpb, 0, s>>>(po, batch_sym_dev(b), (float)b->p.eps2, b->partial, b->spart,
                                        p.total, p.workers);
        NB_LAUNCH_CHECK("bks_force_kernel launch");
        return NB_OK;
    }
    nb::bk_kernel_t k = nb::bk_kernel_for(p.wpb, p.bpt);
    k<<<p.grid, 32 * p.wpb, 0, s>>>(po, batch_dev(b), (float)b->p.eps2, b->partial, p.total, p.workers);
    NB_LAUNCH_CHECK("bk_force_kernel launch");
    return NB_OK;
}

// Sum the partials of the last force pass and integrate from po into pn (vel
// in place), or with acc_out write the bare accelerations instead.
static int batch_integrate(nb_batch *b, const float4 *po, float4 *pn, float4 *vel, float4 *acc_out,
                           cudaStream_t s)
{
    const BatchPlan &p = b->plan;
    if (b->nbody == 0) return NB_OK;
    if (!b->plan_ok)
        return set_error(NB_ERR_STATE, "batch has no valid launch plan (a plan change or autotune failed)");
    if (b->f64) {
        nb::bksff_integrate_kernel<<<(b->nbody + 255) / 256, 256, 0, s>>>(
            (const double4 *)po, (double4 *)pn, (double4 *)vel, (const double4 *)b->partial,
            (const double4 *)b->spart, batch_sym_dev(b), b->nbody, 32 * p.bpt, p.total, p.workers, b->p.damping,
            b->p.dt, b->p.kick, b->p.G, b->ff_range, (double4 *)acc_out);
        NB_LAUNCH_CHECK("bksff_integrate_kernel launch");
        return NB_OK;
    }
    if (b->sym) {
        nb::bks_integrate_kernel<<<(b->nbody + 255) / 256, 256, 0, s>>>(
            po, pn, vel, b->partial, b->spart, batch_sym_dev(b), b->nbody, 32 * p.bpt, p.total,
            p.workers, (float)b->p.damping, (float)b->p.dt, b->p.kick, (float)b->p.G, acc_out);
        NB_LAUNCH_CHECK("bks_integrate_kernel launch");
        return NB_OK;
    }
    nb::bk_integrate_kernel<<<(b->nbody + 255) / 256, 256, 0, s>>>(
        po, pn, vel, b->partial, batch_dev(b), b->nbody, 32 * p.bpt, p.total, p.workers,
        (float)b->p.damping, (float)b->p.dt, b->p.kick, (float)b->p.G, acc_out);
    NB_LAUNCH_CHECK("bk_integrate_kernel launch");
    return NB_OK;
}

// One batched step from po into pn (vel in place); with acc_out the second
// kernel writes the bare accelerations instead of integrating.
static int batch_force_step(nb_batch *b, const float4 *po, float4 *pn, float4 *vel,
                            float4 *acc_out, cudaStream_t s)
{
    int st = batch_force(b, po, s);
    return st ? st : batch_integrate(b, po, pn, vel, acc_out, s);
}

static int batch_step_once(nb_batch *b, cudaStream_t s)
{
    if (b->nbody == 0) return NB_OK;
    int st = batch_force_step(b, b->pos[b->cur], b->pos[b->cur ^ 1], b->vel, nullptr, s);
    if (st) return st;
    b->cur ^= 1;
    return NB_OK;
}

// VJP plan: its own tables for 32 * bpt targets per warp block (directed:
// (system, target block, source group) items; symmetric: (system, row,
// chunk) items with the source-side offsets)
static int batch_vplan_setup(nb_batch *b)
{
    if (b->d_it_off_v) return NB_OK;
    const int wpb = b->sym ? 1 : 4, bpt = b->sym ? 10 : 4, wtb = 32 * bpt;
    const void *k = b->sym ? (const void *)nb::bks_vjp_for(wpb, bpt) : (const void *)nb::bk_vjp_for(wpb, bpt);
    std::vector<long long> it_off(b->nsys + 1, 0), sp_off(b->nsys + 1, 0);
    std::vector<int> tb_off(b->nsys + 1, 0);
    for (int q = 0; q < b->nsys; ++q) {
        const long long n = b->sizes[q];
        const long long ntb = (n + wtb - 1) / wtb, ng = (n + nb::kGroup - 1) / nb::kGroup;
        it_off[q + 1] = it_off[q] + (b->sym ? nb::sym_prefix(ntb, (int)ng, bpt) : ntb * ng);
        tb_off[q + 1] = tb_off[q] + (int)ntb;
        sp_off[q + 1] = sp_off[q] + (b->sym ? nb::sym_spart_entries((int)n, wtb) : 0);
    }
    int occ = 0;
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * wpb, 0));
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "batched adjoint kernel does not fit on an SM");
    BatchPlan p;
    p.wpb = wpb;
    p.bpt = bpt;
    p.total = it_off[b->nsys];
    p.total_wtb = tb_off[b->nsys];
    p.spart = sp_off[b->nsys];
    long long workers = (long long)b->sms * occ * wpb;
    if (p.total > 0 && workers > p.total) workers = p.total;
    p.workers = p.total > 0 ? (int)workers : 0;
    p.grid = (p.workers + wpb - 1) / wpb;
    p.slots = p.total > 0 ? p.workers + p.total_wtb - 1 : 0;
    // d_it_off_v, which marks the setup as done, is set last: a failed call
    // frees what it made and leaves nothing half set up
    const size_t nb4 = std::max<size_t>((size_t)b->nbody, 1) * sizeof(float4);
    const size_t ns = (size_t)b->nsys + 1;
    void *m[11] = {};
    const size_t bytes[11] = {sizeof(long long) * ns, sizeof(int) * ns, sizeof(long long) * ns,
                              std::max<size_t>((size_t)p.slots * wtb, 1) * sizeof(float4),
                              std::max<size_t>((size_t)p.spart, 1) * sizeof(float4),
                              nb4, nb4, nb4, nb4, nb4,
                              std::max<size_t>((size_t)b->nbody, 1) * sizeof(float)};
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < 11 && e == cudaSuccess; ++q) e = nb::dmalloc(&m[q], bytes[q]);
    if (e == cudaSuccess) e = nb::dmemcpy(m[0], it_off.data(), bytes[0], cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = nb::dmemcpy(m[1], tb_off.data(), bytes[1], cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = nb::dmemcpy(m[2], sp_off.data(), bytes[2], cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        for (void *q : m) nb::dfree(q);
        return nb::cuda_error(e, "batched adjoint allocation");
    }
    b->d_tb_off_v = (int *)m[1];
    b->d_sp_off_v = (long long *)m[2];
    b->vpartial = (float4 *)m[3];
    b->vspart = (float4 *)m[4];
    b->vel_tmp = (float4 *)m[5];
    b->vel_tmp2 = (float4 *)m[6];
    b->lx = (float4 *)m[7];
    b->lv = (float4 *)m[8];
    b->gbuf = (float4 *)m[9];
    b->gm = (float *)m[10];
    b->vplan = p;
    b->d_it_off_v = (long long *)m[0];
    return NB_OK;
}

static void free_batch(nb_batch *b)
{
    if (!b) return;
    if (b->graph) nb::graph_exec_destroy(b->graph);
    nb::dfree(b->d_sys_off);
    nb::dfree(b->d_tb_off);
    nb::dfree(b->d_body_sys);
    nb::dfree(b->d_it_off);
    nb::dfree(b->pos[0]);
    nb::dfree(b->pos[1]);
    nb::dfree(b->vel);
    nb::dfree(b->partial);
    nb::dfree(b->spart);
    nb::dfree(b->d_sp_off);
    nb::dfree(b->sys_partial);
    nb::dfree(b->sys_spart);
    nb::dfree(b->ff_split);
    nb::dfree(b->ff_range);
    nb::dfree(b->d_it_off_v);
    nb::dfree(b->d_tb_off_v);
    nb::dfree(b->vpartial);
    nb::dfree(b->d_sp_off_v);
    nb::dfree(b->vspart);
    nb::dfree(b->ckpt_pos);
    nb::dfree(b->ckpt_vel);
    nb::dfree(b->seg_pos);
    nb::dfree(b->seg_acc);
    nb::dfree(b->vel_tmp);
    nb::dfree(b->seg_pos2);
    nb::dfree(b->seg_acc2);
    nb::dfree(b->vel_tmp2);
    if (b->rstream) cudaStreamDestroy(b->rstream);
    for (auto &e : b->ev_rec)
        if (e) cudaEventDestroy(e);
    if (b->ev_go) cudaEventDestroy(b->ev_go);
    nb::dfree(b->lx);
    nb::dfree(b->lv);
    nb::dfree(b->gbuf);
    nb::dfree(b->gm);
    delete b;
}

extern "C" {

int nb_batch_create(const nb_params *p, int nsys, const int *sizes, nb_batch **out)
{
    if (!out) return set_error(NB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!p || nsys < 0 || (nsys > 0 && !sizes)) return set_error(NB_ERR_INVALID, "bad batch arguments");
    if (!((p->precision == NB_F32 && (p->algo == NB_ALGO_FAST || p->algo == NB_ALGO_SYM)) ||
          (p->precision == NB_F64 && p->algo == NB_ALGO_SYM)))
        return set_error(NB_ERR_UNSUPPORTED,
                         "batches run NB_F32 with the fast or symmetric algorithm, or NB_F64 with the symmetric one");
    if (p->kick != NB_KICK_REFERENCE && p->kick != NB_KICK_PHYSICAL)
        return set_error(NB_ERR_INVALID, "unknown kick mode");
    // batches always keep the triangular source side; the field is checked
    // only for a valid value
    if (p->source_side < NB_SOURCE_AUTO || p->source_side > NB_SOURCE_FIXED)
        return set_error(NB_ERR_INVALID, "unknown source_side");
    if (!std::isfinite(p->eps2) || !std::isfinite(p->damping) || !std::isfinite(p->dt) || !std::isfinite(p->G))
        return set_error(NB_ERR_INVALID, "eps2, damping, dt and G must be finite");
    long long nbody = 0;
    for (int s = 0; s < nsys; ++s) {
        if (sizes[s] < 1) return set_error(NB_ERR_INVALID, "every system needs at least one body");
        nbody += sizes[s];
    }
    if (nbody > NB_MAX_BODIES) return set_error(NB_ERR_INVALID, "batch too large (more than 2^30 bodies)");
    nb_batch *b = new nb_batch();
    b->p = *p;
    b->nsys = nsys;
    b->nbody = (int)nbody;
    b->sizes.assign(sizes, sizes + nsys);
    b->sym = p->algo == NB_ALGO_SYM;
    b->f64 = p->precision == NB_F64;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e != cudaSuccess) {
        delete b;
        return nb::cuda_error(e, "device query");
    }
    std::vector<int> sys_off(nsys + 1, 0), body_sys((size_t)nbody);
    for (int s = 0; s < nsys; ++s) {
        sys_off[s + 1] = sys_off[s] + sizes[s];
        for (int i = sys_off[s]; i < sys_off[s + 1]; ++i) body_sys[i] = s;
    }
    const size_t sb = (size_t)nbody * (b->f64 ? sizeof(double4) : sizeof(float4));
#define NB_BALLOC(ptr, bytes)                                                  \
    do {                                                                       \
        cudaError_t _e = nb::dmalloc((void **)&(ptr), (bytes) ? (bytes) : 16);  \
        if (_e != cudaSuccess) {                                               \
            free_batch(b);                                                     \
            return nb::cuda_error(_e, "batch allocation");                     \
        }                                                                      \
    } while (0)
    NB_BALLOC(b->d_sys_off, sizeof(int) * (nsys + 1));
    NB_BALLOC(b->d_tb_off, sizeof(int) * (nsys + 1));
    NB_BALLOC(b->d_it_off, sizeof(long long) * (nsys + 1));
    NB_BALLOC(b->d_sp_off, sizeof(long long) * (nsys + 1));
    NB_BALLOC(b->d_body_sys, sizeof(int) * (size_t)nbody);
    NB_BALLOC(b->pos[0], sb);
    NB_BALLOC(b->pos[1], sb);
    NB_BALLOC(b->vel, sb);
    if (b->f64) {
        NB_BALLOC(b->ff_split, 3 * (size_t)nbody * sizeof(float4));
        NB_BALLOC(b->ff_range, 2 * sizeof(unsigned long long));
    }
#undef NB_BALLOC
    e = nb::dmemcpy(b->d_sys_off, sys_off.data(), sizeof(int) * (nsys + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nbody)
        e = nb::dmemcpy(b->d_body_sys, body_sys.data(), sizeof(int) * (size_t)nbody, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_batch(b);
        return nb::cuda_error(e, "batch tables");
    }
    // defaults: float symmetric one-warp workers x 16 targets, directed
    // 4 x 4, float-float (FP64 state) one-warp workers x 2
    const int wpb = p->block ? p->block / 32 : (b->sym ? 1 : 4);
    const int bpt = p->bpt ? p->bpt : (b->f64 ? 2 : (b->sym ? 16 : 4));
    int st = batch_apply_plan(b, wpb, bpt, nullptr);
    if (st) {
        free_batch(b);
        return st;
    }
    *out = b;
    return NB_OK;
}

int nb_batch_destroy(nb_batch *b)
{
    if (!b) return NB_OK;
    const cudaError_t e = nb::device_sync();
    if (nb::is_capture_error(e)) {  // as nb_destroy: keep what may still be in use
        (void)cudaGetLastError();
        return nb::cuda_error(e, "nb_batch_destroy: the device cannot be synchronised while another thread "
                                 "captures a graph; the batch is kept, call again after the capture");
    }
    free_batch(b);
    return NB_OK;
}

int nb_batch_set_state(nb_batch *b, const void *pos, const void *vel, int where, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    const size_t sb = (size_t)b->nbody * (b->f64 ? sizeof(double4) : sizeof(float4));
    if (sb && (!pos || !vel)) return set_error(NB_ERR_INVALID, "pos/vel is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    b->cur = 0;
    if (sb) {
        NB_CUDA(cudaMemcpyAsync(b->pos[0], pos, sb, cudaMemcpyDefault, s));
        NB_CUDA(cudaMemcpyAsync(b->vel, vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    b->has_state = true;
    return NB_OK;
}

int nb_batch_get_state(nb_batch *b, void *pos, void *vel, int where, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    const size_t sb = (size_t)b->nbody * (b->f64 ? sizeof(double4) : sizeof(float4));
    cudaStream_t s = (cudaStream_t)stream;
    if (sb) {
        if (pos) NB_CUDA(cudaMemcpyAsync(pos, b->pos[b->cur], sb, cudaMemcpyDefault, s));
        if (vel) NB_CUDA(cudaMemcpyAsync(vel, b->vel, sb, cudaMemcpyDefault, s));
        if (where == NB_HOST) NB_CUDA(cudaStreamSynchronize(s));
    }
    return NB_OK;
}

int nb_batch_step(nb_batch *b, int steps, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    for (int i = 0; i < steps; ++i) {
        int st = batch_step_once(b, (cudaStream_t)stream);
        if (st) return st;
    }
    return NB_OK;
}

int nb_batch_run(nb_batch *b, int steps, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (steps < 0) return set_error(NB_ERR_INVALID, "steps must be >= 0");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (steps == 0 || b->nbody == 0) return NB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (s == nullptr) return set_error(NB_ERR_INVALID, "nb_batch_run needs a non-default stream");
    {
        // inside the caller's own capture of this stream: launch the steps
        // into that capture instead of nesting one
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        NB_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs != cudaStreamCaptureStatusNone) {
            for (int i = 0; i < steps; ++i) {
                int st = batch_step_once(b, s);
                if (st) return st;
            }
            return NB_OK;
        }
    }
    if (!b->graph || b->graph_steps != steps || b->graph_cur != b->cur) {
        if (b->graph) {
            nb::graph_exec_destroy(b->graph);
            b->graph = nullptr;
        }
        // a capture that does not take (a device-wide call made by code
        // outside the library in another thread invalidates it) ran nothing
        // and leaves b->cur as it was: the steps then go one by one, where an
        // error of the steps themselves shows
        const int cur0 = b->cur;
        cudaGraph_t g = nullptr;
        {
            std::shared_lock<std::shared_mutex> gate(nb::capture_gate());
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                int st = NB_OK;
                for (int i = 0; i < steps && !st; ++i) st = batch_step_once(b, s);
                if (cudaStreamEndCapture(s, &g) != cudaSuccess || st) {
                    if (g) cudaGraphDestroy(g);
                    g = nullptr;
                }
            }
        }
        b->cur = cur0;
        if (g) {
            if (nb::graph_instantiate(&b->graph, g) != cudaSuccess) b->graph = nullptr;
            cudaGraphDestroy(g);
        }
        (void)cudaGetLastError();
        if (!b->graph) {
            for (int i = 0; i < steps; ++i) {
                int st = batch_step_once(b, s);
                if (st) return st;
            }
            return NB_OK;
        }
        b->graph_steps = steps;
        b->graph_cur = cur0;
    }
    NB_CUDA(cudaGraphLaunch(b->graph, s));
    if (steps % 2) b->cur ^= 1;
    return NB_OK;
}

int nb_batch_set_params(nb_batch *b, double eps2, double damping, double dt, double G)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!std::isfinite(eps2) || !std::isfinite(damping) || !std::isfinite(dt) || !std::isfinite(G))
        return set_error(NB_ERR_INVALID, "eps2, damping, dt and G must be finite");
    if (b->graph) {  // it holds the old values as kernel arguments
        nb::graph_exec_destroy(b->graph);
        b->graph = nullptr;
        b->graph_cur = -1;
    }
    b->p.eps2 = eps2;
    b->p.damping = damping;
    b->p.dt = dt;
    b->p.G = G;
    b->adj_ready = false;
    b->adj_live_last = false;
    return NB_OK;
}

int nb_batch_plan_info(nb_batch *b, long long *info6)
{
    if (!b || !info6) return set_error(NB_ERR_INVALID, "batch/info is NULL");
    info6[0] = b->plan.wpb;
    info6[1] = b->plan.bpt;
    info6[2] = b->plan.grid;
    info6[3] = b->plan.workers;
    info6[4] = b->plan.total;
    info6[5] = b->plan.slots;
    return NB_OK;
}

int nb_batch_set_shape(nb_batch *b, int warps_per_cta, int bodies_per_lane)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    return batch_apply_plan(b, warps_per_cta, bodies_per_lane, nullptr);
}

// Autotuner: times every compiled (warps per CTA, bodies per lane) shape on
// this batch (one warm-up step, then `reps` steps with CUDA events) and keeps
// the fastest.  The state is restored afterwards.  With cache_path, the
// choice is looked up / stored under a key of the device name and the batch's
// size histogram (log2 buckets).
int nb_batch_autotune(nb_batch *b, int reps, const char *cache_path, void *stream, int *chosen2)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (reps < 1) reps = 2;
    cudaStream_t s = (cudaStream_t)stream;
    cudaDeviceProp prop;
    NB_CUDA(cudaGetDeviceProperties(&prop, b->device));
    std::ostringstream key;
    key << prop.name << "|sms" << prop.multiProcessorCount << "|kick" << b->p.kick
        << (b->f64 ? "|symff" : (b->sym ? "|sym" : "|dir")) << "|";
    {
        std::map<int, int> hist;
        for (int n : b->sizes) {
            int lg = 0;
            while ((2LL << lg) <= n) ++lg;
            hist[lg]++;
        }
        for (auto &h : hist) key << h.first << ":" << h.second << ",";
    }
    std::string k = key.str();
    for (char &ch : k)
        if (ch == ' ') ch = '_';
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            std::string kk;
            int w = 0, bp = 0;
            if ((ls >> kk >> w >> bp) && kk == k) {
                int st = batch_apply_plan(b, w, bp, s);
                if (st) break;  // stale entry: tune again
                if (chosen2) {
                    chosen2[0] = w;
                    chosen2[1] = bp;
                }
                return NB_OK;
            }
        }
    }
    const size_t sb = (size_t)b->nbody * (b->f64 ? sizeof(double4) : sizeof(float4));
    float4 *save_p = nullptr, *save_v = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto release = [&] {
        nb::dfree(save_p);
        nb::dfree(save_v);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t ce = cudaSuccess;
    if (sb) {
        ce = nb::dmalloc((void **)&save_p, sb);
        if (ce == cudaSuccess) ce = nb::dmalloc((void **)&save_v, sb);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(save_p, b->pos[b->cur], sb, cudaMemcpyDeviceToDevice, s);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(save_v, b->vel, sb, cudaMemcpyDeviceToDevice, s);
    }
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaStreamSynchronize(s);  // a copy may be in flight
        release();
        return nb::cuda_error(ce, "autotune setup");
    }
    static const int cand_dir[][2] = {{2, 4}, {2, 8}, {4, 2}, {4, 4}, {4, 8}, {8, 2}, {8, 4}, {8, 8}};
    static const int cand_sym[][2] = {{1, 8}, {1, 12}, {1, 16}, {2, 8}, {2, 16}, {4, 8}, {4, 16}};
    static const int cand_ff[][2] = {{1, 2}, {1, 4}, {2, 2}, {2, 4}, {4, 2}, {4, 4}};
    std::vector<std::array<int, 2>> cands;
    if (b->f64)
        for (auto &c : cand_ff) cands.push_back({c[0], c[1]});
    else if (b->sym)
        for (auto &c : cand_sym) cands.push_back({c[0], c[1]});
    else
        for (auto &c : cand_dir) cands.push_back({c[0], c[1]});
    float best = 1e30f;
    const int w0 = b->plan.wpb, b0 = b->plan.bpt;
    int bw = w0, bb = b0;
    int st = NB_OK;
    for (auto &c : cands) {
        if ((st = batch_apply_plan(b, c[0], c[1], s))) break;
        if ((st = batch_step_once(b, s))) break;
        cudaError_t te = cudaEventRecord(e0, s);
        for (int r = 0; r < reps && !st && te == cudaSuccess; ++r) st = batch_step_once(b, s);
        if (st) break;
        if (te == cudaSuccess) te = cudaEventRecord(e1, s);
        if (te == cudaSuccess) te = cudaEventSynchronize(e1);
        float ms = 0;
        if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
        if (te != cudaSuccess) {
            st = nb::cuda_error(te, "autotune timing");
            break;
        }
        if (ms < best) {
            best = ms;
            bw = c[0];
            bb = c[1];
        }
    }
    if (!st) st = batch_apply_plan(b, bw, bb, s);
    if (st) batch_apply_plan(b, w0, b0, s);  // back to the plan from before, if it still fits
    if (sb) {  // the candidates' steps are undone
        b->cur = 0;
        cudaMemcpyAsync(b->pos[0], save_p, sb, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b->vel, save_v, sb, cudaMemcpyDeviceToDevice, s);
    }
    cudaStreamSynchronize(s);
    release();
    if (st) return st;
    if (cache_path) {
        std::ofstream outf(cache_path, std::ios::app);
        if (outf) outf << k << " " << bw << " " << bb << "\n";
    }
    if (chosen2) {
        chosen2[0] = bw;
        chosen2[1] = bb;
    }
    return NB_OK;
}

}  // extern "C"

// Plans of every system on its own (the per-system baselines): directed
// stream-K plans, or symmetric plans for NB_ALGO_SYM batches, and the largest
// scratch each kind needs.
struct SysPlans {
    std::vector<nb::SkPlan> dir;
    std::vector<nb::SymPlan> sym;  // float symmetric or float-float (FP64 state)
    std::vector<int> off;          // body offsets of the systems
    size_t tpart = 1, spart = 1;   // float4 entries (double4 state: twice the partial entries)
};

static int sys_plans_for(nb_batch *b, SysPlans *out)
{
    SysPlans sp;
    const size_t wide = b->f64 ? 2 : 1;
    sp.off.assign(b->nsys + 1, 0);
    for (int i = 0; i < b->nsys; ++i) {
        sp.off[i + 1] = sp.off[i] + b->sizes[i];
        int st;
        if (b->sym) {
            nb::SymPlan q;
            if ((st = b->f64 ? nb::symff_plan(b->sizes[i], 0, 0, b->device, &q, -1)
                             : nb::sym_plan(b->sizes[i], 0, 0, b->device, &q, 0, NB_SOURCE_TRIANGULAR, -1)))
                return st;
            sp.tpart = std::max(sp.tpart, (size_t)q.slots * q.rb * wide);
            sp.spart = std::max(sp.spart, (size_t)q.spart_size * wide);
            sp.sym.push_back(q);
        } else {
            nb::SkPlan q;
            if ((st = nb::fast_plan(b->sizes[i], 0, 0, 0, b->device, &q, 0))) return st;
            sp.tpart = std::max(sp.tpart, (size_t)q.slots * q.tbsize);
            sp.dir.push_back(q);
        }
    }
    *out = std::move(sp);
    return NB_OK;
}

// System i stepped on its own from pos[c] into pos[c ^ 1]: force + integrate
// launches (float-float for FP64 state: its own scale record `range` and
// its slice of the split buffer).
static int sys_step(const nb_batch *b, const SysPlans &sp, int i, int c, float4 *tpart, float4 *spart,
                    unsigned long long *range, cudaStream_t s)
{
    const nb_params &p = b->p;
    const int o = sp.off[i];
    int st;
    if (b->f64) {
        const double4 *po = (const double4 *)b->pos[c] + o;
        double4 *pn = (double4 *)b->pos[c ^ 1] + o, *vel = (double4 *)b->vel + o;
        if ((st = nb::symff_force(sp.sym[i], po, p.eps2, b->ff_split + 3 * (size_t)o, range, (double4 *)tpart,
                                  (double4 *)spart, nullptr, s)))
            return st;
        return nb::sym64_integrate(sp.sym[i], po, pn, vel, (const double4 *)tpart, (const double4 *)spart,
                                   p.damping, p.dt, p.kick, p.G, nullptr, s, range);
    }
    const float4 *po = b->pos[c] + o;
    float4 *pn = b->pos[c ^ 1] + o, *vel = b->vel + o;
    if (b->sym) {
        if ((st = nb::sym_force(sp.sym[i], po, (float)p.eps2, tpart, spart, nullptr, s))) return st;
        return nb::sym_integrate(sp.sym[i], po, pn, vel, tpart, spart, nullptr, (float)p.damping, (float)p.dt,
                                 p.kick, (float)p.G, nullptr, s);
    }
    if ((st = nb::fast_force(sp.dir[i], po, (float)p.eps2, tpart, s, 0))) return st;
    return nb::fast_integrate(sp.dir[i], po, pn, vel, tpart, (float)p.damping, (float)p.dt, p.kick,
                              (float)p.G, nullptr, s);
}

extern "C" {

// The per-system baseline: every system stepped by its own launches (force +
// integrate per system per step, the batch's algorithm), as separate tasks
// would, on one stream.
int nb_batch_step_per_system(nb_batch *b, int steps, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    cudaStream_t s = (cudaStream_t)stream;
    SysPlans sp;
    int st = sys_plans_for(b, &sp);
    if (st) return st;
    if (!b->sys_partial) {
        // both or neither: a failure leaves no half-allocated pair behind
        float4 *t = nullptr, *u = nullptr;
        cudaError_t e = nb::dmalloc((void **)&t, sp.tpart * sizeof(float4));
        if (e == cudaSuccess) e = nb::dmalloc((void **)&u, sp.spart * sizeof(float4));
        if (e != cudaSuccess) {
            nb::dfree(t);
            return nb::cuda_error(e, "per-system baseline scratch allocation");
        }
        b->sys_partial = t;
        b->sys_spart = u;
    }
    for (int t = 0; t < steps; ++t) {
        for (int i = 0; i < b->nsys; ++i) {
            if ((st = sys_step(b, sp, i, b->cur, b->sys_partial, b->sys_spart, b->ff_range, s))) return st;
        }
        b->cur ^= 1;
    }
    return NB_OK;
}

// Baseline in the reference's multi-task pattern (benchapps/nbody/utc/
// nbody_mtask.cc:199-231 with BodySystemSGPU::runImpl, body_task_sgpu.cu:
// 85-127): `ntasks` host threads, each with its own stream, run their share
// of the systems one after another; every system step is a force and an
// integrate launch followed by a stream synchronise.  Blocks until done.
int nb_batch_step_tasks(nb_batch *b, int steps, int ntasks)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (ntasks < 1 || steps < 0) return set_error(NB_ERR_INVALID, "ntasks >= 1 and steps >= 0");
    NB_CUDA(nb::device_sync());
    if (ntasks > b->nsys) ntasks = b->nsys > 0 ? b->nsys : 1;
    SysPlans sp;
    int st0 = sys_plans_for(b, &sp);
    if (st0) return st0;
    std::vector<float4 *> tscratch(ntasks, nullptr), sscratch(ntasks, nullptr);
    std::vector<unsigned long long *> ranges(ntasks, nullptr);  // float-float scale records
    std::vector<cudaStream_t> streams(ntasks, nullptr);
    auto release = [&] {
        for (int t = 0; t < ntasks; ++t) {
            nb::dfree(tscratch[t]);
            nb::dfree(sscratch[t]);
            nb::dfree(ranges[t]);
            if (streams[t]) cudaStreamDestroy(streams[t]);
        }
    };
    for (int t = 0; t < ntasks; ++t) {
        cudaError_t e = nb::dmalloc((void **)&tscratch[t], sp.tpart * sizeof(float4));
        if (e == cudaSuccess) e = nb::dmalloc((void **)&sscratch[t], sp.spart * sizeof(float4));
        if (e == cudaSuccess) e = nb::dmalloc((void **)&ranges[t], 2 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&streams[t], cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            release();
            return nb::cuda_error(e, "per-system task baseline setup");
        }
    }
    const int cur = b->cur, dev = b->device;
    std::vector<int> status(ntasks, NB_OK);
    std::vector<std::thread> workers;
    for (int t = 0; t < ntasks; ++t) {
        workers.emplace_back([&, t] {
            cudaSetDevice(dev);
            for (int i = t; i < b->nsys && status[t] == NB_OK; i += ntasks) {
                int c = cur;
                for (int k = 0; k < steps && status[t] == NB_OK; ++k) {
                    int st = sys_step(b, sp, i, c, tscratch[t], sscratch[t], ranges[t], streams[t]);
                    if (!st && cudaStreamSynchronize(streams[t]) != cudaSuccess) st = NB_ERR_CUDA;
                    status[t] = st;
                    c ^= 1;
                }
            }
        });
    }
    for (auto &w : workers) w.join();
    release();
    for (int t = 0; t < ntasks; ++t)
        if (status[t]) return set_error(status[t], "per-system task baseline failed");
    if (steps % 2) b->cur ^= 1;
    return NB_OK;
}

int nb_batch_launches_per_step(nb_batch *b)
{
    if (!b) return -1;
    if (!b->nbody) return 0;
    return b->f64 ? 4 : 2;  // float-float: scale reduction, split, force, integrate
}

// Batched adjoint: every system's state advanced `steps` steps with a
// checkpoint every ckpt_every steps, then the reverse pass for all systems
// at once (same contract as nb_adj_forward / nb_adj_backward, over the
// concatenated bodies).
int nb_batch_adj_forward(nb_batch *b, int steps, int ckpt_every, void *stream,
                         unsigned long long *generation)
{
    if (generation) *generation = 0;
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (b->f64) return set_error(NB_ERR_UNSUPPORTED, "the batched adjoint runs NB_F32 batches");
    if (!b->has_state) return set_error(NB_ERR_STATE, "no state loaded");
    if (steps < 1 || ckpt_every < 1) return set_error(NB_ERR_INVALID, "steps and ckpt_every must be >= 1");
    if (ckpt_every > steps) ckpt_every = steps;
    int st = batch_vplan_setup(b);
    if (st) return st;
    const int nckpt = (steps + ckpt_every - 1) / ckpt_every;
    const size_t n = (size_t)b->nbody;
    if (nckpt > b->cap_ckpt) {
        nb::dfree(b->ckpt_pos);
        nb::dfree(b->ckpt_vel);
        b->ckpt_pos = b->ckpt_vel = nullptr;
        b->cap_ckpt = 0;
        NB_CUDA(nb::dmalloc((void **)&b->ckpt_pos, std::max<size_t>(n * nckpt, 1) * sizeof(float4)));
        NB_CUDA(nb::dmalloc((void **)&b->ckpt_vel, std::max<size_t>(n * nckpt, 1) * sizeof(float4)));
        b->cap_ckpt = nckpt;
    }
    if (ckpt_every > b->cap_seg) {
        nb::dfree(b->seg_pos);
        nb::dfree(b->seg_acc);
        nb::dfree(b->seg_pos2);
        nb::dfree(b->seg_acc2);
        b->seg_pos = b->seg_acc = b->seg_pos2 = b->seg_acc2 = nullptr;
        b->cap_seg = 0;
        NB_CUDA(nb::dmalloc((void **)&b->seg_pos, std::max<size_t>(n * (ckpt_every + 1), 1) * sizeof(float4)));
        NB_CUDA(nb::dmalloc((void **)&b->seg_acc, std::max<size_t>(n * ckpt_every, 1) * sizeof(float4)));
        NB_CUDA(nb::dmalloc((void **)&b->seg_pos2, std::max<size_t>(n * (ckpt_every + 1), 1) * sizeof(float4)));
        NB_CUDA(nb::dmalloc((void **)&b->seg_acc2, std::max<size_t>(n * ckpt_every, 1) * sizeof(float4)));
        b->cap_seg = ckpt_every;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // as nb_adj_forward: the last segment's states (and reference-kick
    // accelerations) stay in the segment buffers, so the reverse pass does
    // not recompute that segment
    const int t_last = (nckpt - 1) * ckpt_every;
    b->adj_ready = false;
    b->adj_live_last = false;
    for (int t = 0; t < steps; ++t) {
        if (t % ckpt_every == 0 && n) {
            const size_t k = (size_t)(t / ckpt_every) * n;
            NB_CUDA(cudaMemcpyAsync(b->ckpt_pos + k, b->pos[b->cur], n * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, s));
            NB_CUDA(cudaMemcpyAsync(b->ckpt_vel + k, b->vel, n * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, s));
        }
        const bool keep = n && t >= t_last;
        const size_t k = (size_t)(t - t_last);
        if (keep && t == t_last)
            NB_CUDA(cudaMemcpyAsync(b->seg_pos, b->pos[b->cur], n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
        const float4 *xk = b->pos[b->cur];
        if ((st = batch_step_once(b, s))) return st;
        if (!keep) continue;
        if (b->p.kick == NB_KICK_REFERENCE &&
            (st = batch_integrate(b, xk, nullptr, nullptr, b->seg_acc + k * n, s)))
            return st;
        NB_CUDA(cudaMemcpyAsync(b->seg_pos + (k + 1) * n, b->pos[b->cur], n * sizeof(float4),
                                cudaMemcpyDeviceToDevice, s));
    }
    b->adj_steps = steps;
    b->adj_every = ckpt_every;
    b->adj_nckpt = nckpt;
    b->adj_ready = true;
    b->adj_live_last = n > 0;
    b->adj_generation += 1;
    if (generation) *generation = b->adj_generation;
    return NB_OK;
}

int nb_batch_adj_backward(nb_batch *b, unsigned long long generation, const void *gx_T,
                          const void *gv_T, void *gx0, void *gv0, void *gm, void *stream)
{
    if (!b) return set_error(NB_ERR_INVALID, "batch is NULL");
    if (b->f64) return set_error(NB_ERR_UNSUPPORTED, "the batched adjoint runs NB_F32 batches");
    if (!b->adj_ready) return set_error(NB_ERR_STATE, "nb_batch_adj_backward needs a preceding nb_batch_adj_forward");
    if (generation != b->adj_generation)
        return set_error(NB_ERR_STATE, "nb_batch_adj_backward: the batch no longer holds that forward pass "
                                       "(a later nb_batch_adj_forward replaced it)");
    if (b->nbody == 0) return NB_OK;
    if (!gx_T || !gx0 || !gv0 || !gm) return set_error(NB_ERR_INVALID, "NULL gradient buffer");
    const size_t n = (size_t)b->nbody;
    const nb_params &p = b->p;
    const float eps2 = (float)p.eps2, D = (float)p.damping, dt = (float)p.dt, G = (float)p.G;
    cudaStream_t s = (cudaStream_t)stream;
    nb::BatchDev vd = batch_dev(b);
    vd.it_off = b->d_it_off_v;
    vd.tb_off = b->d_tb_off_v;
    nb::BatchSymDev vsd = batch_sym_dev(b);
    vsd.it_off = b->d_it_off_v;
    vsd.row_off = b->d_tb_off_v;
    vsd.sp_off = b->d_sp_off_v;
    const BatchPlan &vp = b->vplan;
    nb::bk_vjp_t vk = b->sym ? nullptr : nb::bk_vjp_for(vp.wpb, vp.bpt);
    nb::bks_vjp_t vks = b->sym ? nb::bks_vjp_for(vp.wpb, vp.bpt) : nullptr;
    int st;
    NB_CUDA(cudaMemcpyAsync(b->lx, gx_T, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    if (gv_T)
        NB_CUDA(cudaMemcpyAsync(b->lv, gv_T, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    else
        NB_CUDA(cudaMemsetAsync(b->lv, 0, n * sizeof(float4), s));
    NB_CUDA(cudaMemsetAsync(b->gm, 0, n * sizeof(float), s));
    // Recompute segment `seg` from its checkpoint into buffer k on stream rs
    // (one force pass per step; with the reference kick its partials also
    // give the accelerations).  Same kernels, same bits as the forward pass.
    auto recompute = [&](int seg, int kb, cudaStream_t rs) -> int {
        float4 *sp = kb ? b->seg_pos2 : b->seg_pos, *sa = kb ? b->seg_acc2 : b->seg_acc;
        float4 *vt = kb ? b->vel_tmp2 : b->vel_tmp;
        const int t0 = seg * b->adj_every;
        const int len = (b->adj_steps - t0) < b->adj_every ? (b->adj_steps - t0) : b->adj_every;
        NB_CUDA(cudaMemcpyAsync(sp, b->ckpt_pos + (size_t)seg * n, n * sizeof(float4), cudaMemcpyDeviceToDevice, rs));
        NB_CUDA(cudaMemcpyAsync(vt, b->ckpt_vel + (size_t)seg * n, n * sizeof(float4), cudaMemcpyDeviceToDevice, rs));
        int st2;
        for (int k = 0; k < len; ++k) {
            const float4 *xk = sp + (size_t)k * n;
            if ((st2 = batch_force(b, xk, rs))) return st2;
            if (p.kick == NB_KICK_REFERENCE &&
                (st2 = batch_integrate(b, xk, nullptr, nullptr, sa + (size_t)k * n, rs)))
                return st2;
            if ((st2 = batch_integrate(b, xk, sp + (size_t)(k + 1) * n, vt, nullptr, rs))) return st2;
        }
        return NB_OK;
    };
    // As in nb_adj_backward: segments alternate between the two buffers (the
    // last one in buffer 0, where the forward pass leaves it), and segment
    // seg-1 is recomputed on rstream while the reverse pass runs through seg.
    const int last = b->adj_nckpt - 1;
    auto buf_of = [&](int seg) { return (last - seg) & 1; };
    const bool live = b->adj_live_last;
    b->adj_live_last = false;  // the segment buffers are reused from here on
    if (last > 0 && !b->rstream &&
        (st = nb::create_recompute_stream(&b->rstream, b->ev_rec, &b->ev_go)))
        return st;
    if (!live && (st = recompute(last, buf_of(last), s))) return st;
    bool have_g = false;
    for (int seg = last; seg >= 0; --seg) {
        const int kb = buf_of(seg);
        if (seg < last) NB_CUDA(cudaStreamWaitEvent(s, b->ev_rec[kb], 0));
        if (seg > 0) {
            NB_CUDA(cudaEventRecord(b->ev_go, s));
            NB_CUDA(cudaStreamWaitEvent(b->rstream, b->ev_go, 0));
            if ((st = recompute(seg - 1, buf_of(seg - 1), b->rstream))) return st;
            NB_CUDA(cudaEventRecord(b->ev_rec[buf_of(seg - 1)], b->rstream));
        }
        const float4 *sp = kb ? b->seg_pos2 : b->seg_pos, *sa = kb ? b->seg_acc2 : b->seg_acc;
        const int t0 = seg * b->adj_every;
        const int len = (b->adj_steps - t0) < b->adj_every ? (b->adj_steps - t0) : b->adj_every;
        for (int k = len - 1; k >= 0; --k) {
            const float4 *xk = sp + (size_t)k * n;
            const float4 *ak = sa + (size_t)k * n;
            if (!have_g) {
                if ((st = nb::adj_g(b->nbody, xk, b->lx, b->lv, b->gbuf, D, dt, p.kick, G, s))) return st;
                have_g = true;
            }
            const bool more = !(seg == 0 && k == 0);
            if (b->sym) {
                if (vp.total > 0) {
                    vks<<<vp.grid, 32 * vp.wpb, 0, s>>>(xk, b->gbuf, vsd, eps2, b->vpartial, b->vspart,
                                                         vp.total, vp.workers);
                    NB_LAUNCH_CHECK("bks_vjp_kernel launch");
                }
                nb::bks_adj_update_kernel<<<(b->nbody + 255) / 256, 256, 0, s>>>(
                    b->vpartial, b->vspart, vsd, b->nbody, 32 * vp.bpt, vp.total, vp.workers, xk, ak, b->lx,
                    b->lv, b->gm, b->gbuf, D, dt, p.kick, G, more ? 1 : 0);
                NB_LAUNCH_CHECK("bks_adj_update_kernel launch");
                continue;
            }
            if (vp.total > 0) {
                vk<<<vp.grid, 32 * vp.wpb, 0, s>>>(xk, b->gbuf, vd, eps2, b->vpartial, vp.total, vp.workers);
                NB_LAUNCH_CHECK("bk_vjp_kernel launch");
            }
            nb::bk_adj_update_kernel<<<(b->nbody + 255) / 256, 256, 0, s>>>(
                b->vpartial, vd, b->nbody, 32 * vp.bpt, vp.total, vp.workers, xk, ak, b->lx, b->lv, b->gm,
                b->gbuf, D, dt, p.kick, G, more ? 1 : 0);
            NB_LAUNCH_CHECK("bk_adj_update_kernel launch");
        }
    }
    NB_CUDA(cudaMemcpyAsync(gx0, b->lx, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    NB_CUDA(cudaMemcpyAsync(gv0, b->lv, n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    NB_CUDA(cudaMemcpyAsync(gm, b->gm, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return NB_OK;
}

}  // extern "C"
