// nb_sym.cu -- symmetric all-pairs force kernel (each unordered pair once).
//
// The reference evaluates every ordered pair (i, j) separately
// (benchapps/nbody/cuda/bodysystem_kernel.cu:60-85).  The pair term is odd in
// r, so the contribution of j to i and of i to j share r, d2, 1/sqrt(d2) and
// inv^3: evaluating the pair once and applying it to both bodies costs 16
// FP32 operations and one rsqrt for two interactions instead of 24 and two.
// The individual terms are the same numbers as in the directed evaluation;
// only the order in which each body's terms are summed changes.
//
// Layout of the work:
//  * bodies are cut into row blocks of RB = W*32*BPT; a CTA of W warps owns a
//    row block's targets (each lane BPT of them, in registers);
//  * the columns are 32-body chunks; row I is paired with every chunk at or
//    after its own start.  Chunks inside row I are evaluated directed (target
//    side only: both orders of each pair occur there); chunks after row I are
//    evaluated symmetrically;
//  * in a symmetric chunk the 32 bodies sit in shared memory and rotate
//    through the warp: at step r lane l pairs its targets with chunk body
//    (l + r) mod 32 and carries that body's accumulated reaction, passing it
//    to lane l - 1 with one shuffle per component, so after 32 steps lane l
//    holds the reaction on chunk body l from the warp's targets; the W warps'
//    reactions are summed in warp order through shared memory and stored in
//    the source-side array spart (row I, body), a triangular layout;
//  * (row, chunk) items are split stream-K over persistent CTAs; target-side
//    partials go to slot cta + row as in the directed kernel.
// The integrate kernel adds, per body, its target-side slots (CTA order) and
// its source-side entries spart[0..I_b-1][b] (row order): deterministic.
//
// Bands (template flag BAND; plans with nbands > 1, where the triangular
// array, about N^2 / (2 rb) float4, would pass kSymSpartBudget, or on
// request through nb_params.bands).  The row blocks are cut into bands of
// consecutive rows whose entries fit the budget; the force kernel runs once
// per band over the band's (row, chunk) items (stream-K over the band), all
// bands reusing one source-side buffer and one set of target-side slots,
// and after each band sym_fold_kernel adds, per body, the band's target-side
// slots (if the body's row is in the band) and its source-side rows into a
// running per-body sum, which the integrator then takes.  Fixed order
// throughout, so still deterministic.  A band costs about 1.5 ms of tail
// and fold at N = 2^20, so only sizes whose force pass takes seconds use
// more than a few.
//
// Fixed-point source side (template flag FX; plans with fixed = 1, chosen
// by nb_params.source_side, or where even bands would not do: more than
// SymPlan::kMaxBands of them).  The CTA's reaction on a chunk body,
// summed over its warps as above, is added straight into per-body 64-bit
// integer accumulators with integer atomics.  Integer addition is
// associative, so the sums do not depend on the order the CTAs run in: the
// step stays deterministic, and the source side takes 48 B per body.  Each
// reaction v is split into two integers, hi = round(v / 2^(e-61)) and
// lo = round((v - hi 2^(e-61)) / 2^(e-83)), exact for |v| >= 2^(e-60) (the
// float's 24 significant bits fit) and within 2^(e-84) below.  The exponent
// comes from a bound on every partial and total reaction: a body at
// distance r adds at most m r / (r^2 + eps2)^(3/2) <= (2 / (3 sqrt 3)) m /
// eps2, so B = 0.385 sum|m| / eps2 bounds them all, and 2^e > 2 B keeps the
// hi sums below 2^62 (the lo words stay below 2^22 per reaction).  The
// source side is so summed essentially exactly, for any eps2 > 0.  The scale
// sits in a record after the accumulators, written at nb_set_state (and for
// a new eps2) by sym_fx_prepare / sym_fx_rescale; the integrator zeroes the
// accumulators after reading them.  On GB300 this variant ran 2-10 % slower
// than the triangular array of the same shape (the pair loop's schedule
// shifts with the code around it; 3513 against 3593 G interactions/s for
// the banded 4 x 20 triangular plan at N = 2^21).
//
// Compensated variant (COMP): each target's per-chunk partial sum (32
// sources) is folded into a two-sum (hi, lo) pair, the W warps' reactions on
// a chunk body are combined with two-sums, and both halves are written (lo
// block after the hi block of tpart and of spart); the compensated
// integrator sums them with two-sums.
//
// Shape.  The loop is issue-bound (16 FP32 instructions + 1 MUFU per pair,
// plus one LDS and three SHFL per lane and rotation step), and its issue
// rate improves with more independent targets per lane rather than with more
// warps: one-warp CTAs with 16 targets per lane (225 registers, 8 warps per
// SM) run 15 % faster than 8-warp CTAs with 8 targets per lane (80 registers,
// 24 warps per SM) on GB300.  Small row blocks make the triangular
// source-side array large (about N^2 / (2 rb) float4), so the default shape
// grows to 4 warps x 20 targets when that array would pass kSymSpartBudget,
// and is cut into bands beyond that.
#include "nb_internal.cuh"

namespace nb {

// Record after the fixed-point accumulators: x = sum |m|, y = 2^(61-e),
// z = 2^(e-61), w = 2^(83-e).
__device__ __forceinline__ const float4 *fx_record(const unsigned long long *acc, int n)
{
    return reinterpret_cast<const float4 *>(acc + 6ll * n);
}

// v added to the accumulators hi_p (units z = 2^(e-61)) and lo_p (units
// 1/w = 2^(e-83)).  The products with powers of two are exact; rem is exact
// (|v y| < 2^23 makes (float)h exact, otherwise v y is an integer and
// rem = 0).  The adds compile to fire-and-forget reductions.
__device__ __forceinline__ void fx_add(unsigned long long *hi_p, unsigned long long *lo_p, float v,
                                       const float4 &r)
{
    const long long h = __float2ll_rn(v * r.y);
    const float rem = fmaf(-(float)h, r.z, v);
    const long long l = __float2ll_rn(rem * r.w);
    atomicAdd(hi_p, (unsigned long long)h);
    atomicAdd(lo_p, (unsigned long long)l);
}

// A reaction (fx, fy, fz) on body j into the fixed-point accumulators.
__device__ __forceinline__ void fx_emit(unsigned long long *acc, int n, int j, float fx, float fy, float fz)
{
    const float4 r = __ldg(fx_record(acc, n));
    const long long nn = n;
    fx_add(acc + j, acc + 3 * nn + j, fx, r);
    fx_add(acc + nn + j, acc + 4 * nn + j, fy, r);
    fx_add(acc + 2 * nn + j, acc + 5 * nn + j, fz, r);
}

// FX: spart is the fixed-point accumulator buffer (with its record), not
// the triangular array.  BAND: one band of a banded plan, items
// [it0, it0 + total) covering row blocks from r0 on: target-side slot
// c + I - r0, source-side entries offset by soff0 (the band's first entry).
template <int W, int BPT, int MINB, bool COMP, bool FX = false, bool BAND = false>
__global__ void __launch_bounds__(32 * W, MINB) sym_force_kernel(const float4 *__restrict__ pos, int n,
                                                           float eps2, float4 *__restrict__ tpart,
                                                           float4 *__restrict__ spart,
                                                           long long total, int nc, int nrb,
                                                           long long tlo, long long slo, long long it0,
                                                           int r0, long long soff0)
{
    constexpr int WB = 32 * BPT;
    constexpr int RB = W * WB;
    constexpr int RC = RB / 32;
    __shared__ __align__(16) float4 sC[32];
    __shared__ float sF[3][W][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int c = blockIdx.x;
    long long it = sk_start(c, total, gridDim.x);
    long long end = sk_start(c + 1, total, gridDim.x);
    if constexpr (BAND) {
        it += it0;
        end += it0;
    }
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);

    while (it < end) {
        const int I = sym_row_of(it, nc, RC, nrb);
        const long long rfirst = sym_prefix(I, nc, RC);
        const long long rend = sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB + wid * WB;

        // nm = -m: the reaction on the chunk body points along -r
        float px[BPT], py[BPT], pz[BPT], nm[BPT], ax[BPT], ay[BPT], az[BPT];
        // COMP: compensated target sums (hi in h*, lo in l*)
        constexpr int CB = COMP ? BPT : 1;
        float hx[CB], hy[CB], hz[CB], lx[CB], ly[CB], lz[CB];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tbase + lane + 32 * k;
            // missing targets get zero mass: their reactions on the chunk are 0
            const float4 q = i < n ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            px[k] = q.x;
            py[k] = q.y;
            pz[k] = q.z;
            nm[k] = -q.w;
            ax[k] = ay[k] = az[k] = 0.f;
            if constexpr (COMP) hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            __syncthreads();  // previous chunk: sC reads and sF reads are done
            if (wid == 0) sC[lane] = (jb + lane < n) ? pos[jb + lane] : pad;
            __syncthreads();
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 4
                for (int j = 0; j < 32; ++j) {
                    const float4 q = sC[j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float s = (q.w * inv) * (inv * inv);
                        ax[k] = fmaf(rx, s, ax[k]);
                        ay[k] = fmaf(ry, s, ay[k]);
                        az[k] = fmaf(rz, s, az[k]);
                    }
                }
            } else {
                float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll 2
                for (int r = 0; r < 32; ++r) {
                    const float4 q = sC[(lane + r) & 31];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = q.x - px[k], ry = q.y - py[k], rz = q.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float inv3 = inv * (inv * inv);
                        const float st = q.w * inv3;    // on the target, from the chunk body
                        const float ss = nm[k] * inv3;  // on the chunk body, from the target
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
                // lane l now holds the reaction on chunk body l from this warp
                sF[0][wid][lane] = fx;
                sF[1][wid][lane] = fy;
                sF[2][wid][lane] = fz;
                __syncthreads();
                if (FX && wid == 0 && jb + lane < n) {
                    float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        sx += sF[0][w][lane];
                        sy += sF[1][w][lane];
                        sz += sF[2][w][lane];
                    }
                    fx_emit(reinterpret_cast<unsigned long long *>(spart), n, jb + lane, sx, sy, sz);
                } else if (wid == 0 && jb + lane < n) {
                    long long so = sym_soff(I, n, RB) + (jb + lane - (I + 1) * RB);
                    if constexpr (BAND) so -= soff0;
                    if constexpr (COMP) {
                        float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, e;
#pragma unroll
                        for (int w = 0; w < W; ++w) {
                            two_sum(sx, sF[0][w][lane], sx, e);
                            cx = __fadd_rn(cx, e);
                            two_sum(sy, sF[1][w][lane], sy, e);
                            cy = __fadd_rn(cy, e);
                            two_sum(sz, sF[2][w][lane], sz, e);
                            cz = __fadd_rn(cz, e);
                        }
                        spart[so] = make_float4(sx, sy, sz, 0.f);
                        spart[slo + so] = make_float4(cx, cy, cz, 0.f);
                    } else {
                        float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
                        for (int w = 0; w < W; ++w) {
                            sx += sF[0][w][lane];
                            sy += sF[1][w][lane];
                            sz += sF[2][w][lane];
                        }
                        spart[so] = make_float4(sx, sy, sz, 0.f);
                    }
                }
            }
            if constexpr (COMP) {
                // fold this chunk's 32-source partial sums into (hi, lo)
#pragma unroll
                for (int k = 0; k < BPT; ++k) {
                    float e;
                    two_sum(hx[k], ax[k], hx[k], e);
                    lx[k] = __fadd_rn(lx[k], e);
                    two_sum(hy[k], ay[k], hy[k], e);
                    ly[k] = __fadd_rn(ly[k], e);
                    two_sum(hz[k], az[k], hz[k], e);
                    lz[k] = __fadd_rn(lz[k], e);
                    ax[k] = ay[k] = az[k] = 0.f;
                }
            }
        }
        float4 *dst = tpart + (size_t)(c + I - (BAND ? r0 : 0)) * RB + wid * WB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            if constexpr (COMP) {
                dst[lane + 32 * k] = make_float4(hx[k], hy[k], hz[k], 0.f);
                dst[tlo + lane + 32 * k] = make_float4(lx[k], ly[k], lz[k], 0.f);
            } else {
                dst[lane + 32 * k] = make_float4(ax[k], ay[k], az[k], 0.f);
            }
        }
        it = seg_end;
    }
}

// Packed variant: each lane's targets as NP f32x2 pairs (targets k and
// k + NP of the lane), every pair-term operation one FADD2/FMUL2/FFMA2 for
// two targets; the chunk body is duplicated into register pairs; the
// reaction on the chunk body is accumulated as a pair (one half per target of
// the pair) and folded to a scalar before each shuffle.  Same work layout,
// partials and results' order of summation as sym_force_kernel.
template <int W, int NP>
__global__ void __launch_bounds__(32 * W) sym_force_kernel_f2(const float4 *__restrict__ pos, int n,
                                                              float eps2, float4 *__restrict__ tpart,
                                                              float4 *__restrict__ spart,
                                                              long long total, int nc, int nrb,
                                                              long long, long long, long long, int,
                                                              long long)
{
    constexpr int BPT = 2 * NP;
    constexpr int WB = 32 * BPT;
    constexpr int RB = W * WB;
    constexpr int RC = RB / 32;
    __shared__ __align__(16) float4 sC[32];
    __shared__ float sF[3][W][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int c = blockIdx.x;
    long long it = sk_start(c, total, gridDim.x);
    const long long end = sk_start(c + 1, total, gridDim.x);
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    const f2 EPS2 = f2_pack(eps2, eps2);
    const f2 ZERO = f2_pack(0.f, 0.f);

    while (it < end) {
        const int I = sym_row_of(it, nc, RC, nrb);
        const long long rfirst = sym_prefix(I, nc, RC);
        const long long rend = sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB + wid * WB;

        f2 PX[NP], PY[NP], PZ[NP], NM[NP], AX[NP], AY[NP], AZ[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const int i0 = tbase + lane + 32 * p;
            const int i1 = i0 + 32 * NP;
            const float4 q0 = i0 < n ? pos[i0] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 q1 = i1 < n ? pos[i1] : make_float4(0.f, 0.f, 0.f, 0.f);
            PX[p] = f2_pack(q0.x, q1.x);
            PY[p] = f2_pack(q0.y, q1.y);
            PZ[p] = f2_pack(q0.z, q1.z);
            NM[p] = f2_pack(-q0.w, -q1.w);  // negated: reactions point along -r
            AX[p] = AY[p] = AZ[p] = ZERO;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            __syncthreads();
            if (wid == 0) sC[lane] = (jb + lane < n) ? pos[jb + lane] : pad;
            __syncthreads();
            const bool diag = kc < (I + 1) * RC;
            float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll 2
            for (int r = 0; r < 32; ++r) {
                const float4 q = sC[diag ? r : ((lane + r) & 31)];
                const f2 XB = f2_pack(q.x, q.x), YB = f2_pack(q.y, q.y);
                const f2 ZB = f2_pack(q.z, q.z), MB = f2_pack(q.w, q.w);
                f2 FX = f2_pack(fx, 0.f), FY = f2_pack(fy, 0.f), FZ = f2_pack(fz, 0.f);
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    const f2 rx = f2_sub(XB, PX[p]);
                    const f2 ry = f2_sub(YB, PY[p]);
                    const f2 rz = f2_sub(ZB, PZ[p]);
                    f2 d2 = f2_fma(rx, rx, EPS2);
                    d2 = f2_fma(ry, ry, d2);
                    d2 = f2_fma(rz, rz, d2);
                    float dlo, dhi;
                    f2_unpack(d2, dlo, dhi);
                    const f2 inv = f2_pack(rsqrt_approx(dlo), rsqrt_approx(dhi));
                    const f2 inv3 = f2_mul(f2_mul(inv, inv), inv);
                    const f2 st = f2_mul(MB, inv3);
                    AX[p] = f2_fma(rx, st, AX[p]);
                    AY[p] = f2_fma(ry, st, AY[p]);
                    AZ[p] = f2_fma(rz, st, AZ[p]);
                    if (!diag) {
                        const f2 ss = f2_mul(NM[p], inv3);
                        FX = f2_fma(rx, ss, FX);
                        FY = f2_fma(ry, ss, FY);
                        FZ = f2_fma(rz, ss, FZ);
                    }
                }
                if (!diag) {
                    float lo, hi;
                    f2_unpack(FX, lo, hi);
                    fx = lo + hi;
                    f2_unpack(FY, lo, hi);
                    fy = lo + hi;
                    f2_unpack(FZ, lo, hi);
                    fz = lo + hi;
                    const int from = (lane + 1) & 31;
                    fx = __shfl_sync(0xffffffffu, fx, from);
                    fy = __shfl_sync(0xffffffffu, fy, from);
                    fz = __shfl_sync(0xffffffffu, fz, from);
                }
            }
            if (!diag) {
                sF[0][wid][lane] = fx;
                sF[1][wid][lane] = fy;
                sF[2][wid][lane] = fz;
                __syncthreads();
                if (wid == 0 && jb + lane < n) {
                    float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        sx += sF[0][w][lane];
                        sy += sF[1][w][lane];
                        sz += sF[2][w][lane];
                    }
                    spart[sym_soff(I, n, RB) + (jb + lane - (I + 1) * RB)] = make_float4(sx, sy, sz, 0.f);
                }
            }
        }
        float4 *dst = tpart + (size_t)(c + I) * RB + wid * WB;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            float x0, x1, y0, y1, z0, z1;
            f2_unpack(AX[p], x0, x1);
            f2_unpack(AY[p], y0, y1);
            f2_unpack(AZ[p], z0, z1);
            dst[lane + 32 * p] = make_float4(x0, y0, z0, 0.f);
            dst[lane + 32 * (p + NP)] = make_float4(x1, y1, z1, 0.f);
        }
        it = seg_end;
    }
}

// Per body: target-side slots + source-side rows 0..I_b-1, then the
// reference's kick / damping / drift (unfused, its order).  Four threads
// share a body: thread q of the quad sums slots c0+q, c0+q+4, ... and rows
// q, q+4, ... in order, and the quad combines its four sums as
// (s0 + s1) + (s2 + s3) (fixed order: deterministic).  The row walk, up to
// nrb - 1 entries for the last row block, is what bounds the kernel; split
// four ways it is a quarter as long.  Bodies are taken from the last one
// down, so the blocks with the longest walks start first instead of forming
// the tail (19.7 -> 18.1 us at N = 65536 on GB300; the sums are the same).
constexpr int kSymIntegBlock = 256;

// fxacc != nullptr: the fixed-point source side; thread 0 of the quad adds
// its total to the target-side sum in FP64 (one rounding) and, with
// consume, zeroes the body's six accumulators for the next force launch.
// accsum != nullptr (banded plans): the folded sums, taken as they are.
__global__ void __launch_bounds__(kSymIntegBlock) sym_integrate_kernel(
    const float4 *__restrict__ pos_old, float4 *__restrict__ pos_new, float4 *__restrict__ vel,
    const float4 *__restrict__ tpart, const float4 *__restrict__ spart, int n, int rb, int nc, int nrb,
    long long total, int grid, float damping, float dt, int kick, float G, float4 *__restrict__ acc_out,
    unsigned long long *__restrict__ fxacc, int consume, const float4 *__restrict__ accsum)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = n - 1 - (int)(t >> 2), q = (int)(t & 3);
    const bool live = i >= 0;  // dead threads still take part in the shuffles
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (live && accsum) {
        if (q == 0) {
            const float4 a4 = accsum[i];
            ax = a4.x;
            ay = a4.y;
            az = a4.z;
        }
    } else if (live) {
        const int rc = rb / 32;
        const int I = i / rb;
        const int c0 = sk_owner(sym_prefix(I, nc, rc), total, grid);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1, total, grid);
        const int li = i - I * rb;
        for (int c = c0 + q; c <= c1; c += 4) {
            const float4 v4 = tpart[(size_t)(c + I) * rb + li];
            ax = __fadd_rn(ax, v4.x);
            ay = __fadd_rn(ay, v4.y);
            az = __fadd_rn(az, v4.z);
        }
        if (!fxacc) {
#pragma unroll 4
            for (int r = q; r < I; r += 4) {
                const float4 v4 = spart[sym_soff(r, n, rb) + (i - (long long)(r + 1) * rb)];
                ax = __fadd_rn(ax, v4.x);
                ay = __fadd_rn(ay, v4.y);
                az = __fadd_rn(az, v4.z);
            }
        }
    }
    ax = __fadd_rn(ax, __shfl_xor_sync(0xffffffffu, ax, 1));
    ay = __fadd_rn(ay, __shfl_xor_sync(0xffffffffu, ay, 1));
    az = __fadd_rn(az, __shfl_xor_sync(0xffffffffu, az, 1));
    ax = __fadd_rn(ax, __shfl_xor_sync(0xffffffffu, ax, 2));
    ay = __fadd_rn(ay, __shfl_xor_sync(0xffffffffu, ay, 2));
    az = __fadd_rn(az, __shfl_xor_sync(0xffffffffu, az, 2));
    if (!live || q != 0) return;
    if (fxacc) {
        // units 2^(e-61) and 2^(e-83) as doubles, from the record's 2^(e-61)
        const float4 rec = *fx_record(fxacc, n);
        const double lhi = (double)rec.z, llo = (double)rec.z * 0x1p-22;
        const long long nn = n;
        unsigned long long *a = fxacc + i;
        const double sx = (double)(long long)a[0] * lhi + (double)(long long)a[3 * nn] * llo;
        const double sy = (double)(long long)a[nn] * lhi + (double)(long long)a[4 * nn] * llo;
        const double sz = (double)(long long)a[2 * nn] * lhi + (double)(long long)a[5 * nn] * llo;
        ax = (float)((double)ax + sx);
        ay = (float)((double)ay + sy);
        az = (float)((double)az + sz);
        if (consume) a[0] = a[nn] = a[2 * nn] = a[3 * nn] = a[4 * nn] = a[5 * nn] = 0ull;
    }
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

// After band [r0, r1) of a banded plan (items [it0, it0 + bt) over gb CTAs):
// per body, the running sum (zero before the first band) plus, if the body's
// row block is in the band, its target-side slots in CTA order, then the
// band's source-side rows before the body's row block in row order.  Fixed
// order throughout: deterministic.  Bodies from the last one down, as in
// sym_integrate_kernel (the longest row walks first).
__global__ void __launch_bounds__(256) sym_fold_kernel(const float4 *__restrict__ tpart,
                                                       const float4 *__restrict__ spart,
                                                       float4 *__restrict__ accsum, int n, int rb, int nc,
                                                       long long it0, long long bt, int gb, int r0, int r1,
                                                       long long soff0, int first)
{
    const int i = n - 1 - (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < 0) return;
    const int I = i / rb;
    if (I < r0) return;  // rows before the band get nothing from it (r0 = 0 for the first band)
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (!first) {
        const float4 a4 = accsum[i];
        ax = a4.x;
        ay = a4.y;
        az = a4.z;
    }
    if (I < r1) {
        const int rc = rb / 32;
        const int c0 = sk_owner(sym_prefix(I, nc, rc) - it0, bt, gb);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1 - it0, bt, gb);
        const int li = i - I * rb;
        for (int c = c0; c <= c1; ++c) {
            const float4 v4 = tpart[(size_t)(c + I - r0) * rb + li];
            ax = __fadd_rn(ax, v4.x);
            ay = __fadd_rn(ay, v4.y);
            az = __fadd_rn(az, v4.z);
        }
    }
    const int rend = I < r1 ? I : r1;
#pragma unroll 4
    for (int r = r0; r < rend; ++r) {
        const float4 v4 = spart[sym_soff(r, n, rb) - soff0 + (i - (long long)(r + 1) * rb)];
        ax = __fadd_rn(ax, v4.x);
        ay = __fadd_rn(ay, v4.y);
        az = __fadd_rn(az, v4.z);
    }
    accsum[i] = make_float4(ax, ay, az, 0.f);
}

// The compensated fold: running (S, C) per body in accsum[0..n) and
// accsum[n..2n), each partial (hi, lo) added as the compensated integrator
// adds it (two-sum into S, its error and lo into C).
__global__ void __launch_bounds__(256) sym_fold_comp_kernel(const float4 *__restrict__ tpart,
                                                            const float4 *__restrict__ spart, long long tlo,
                                                            long long slo, float4 *__restrict__ accsum, int n,
                                                            int rb, int nc, long long it0, long long bt, int gb,
                                                            int r0, int r1, long long soff0, int first)
{
    const int i = n - 1 - (int)(blockIdx.x * blockDim.x + threadIdx.x);  // longest walks first
    if (i < 0) return;
    const int I = i / rb;
    if (I < r0) return;
    float4 S = make_float4(0.f, 0.f, 0.f, 0.f), C = S;
    if (!first) {
        S = accsum[i];
        C = accsum[(size_t)n + i];
    }
    float e;
    auto add = [&](const float4 h, const float4 l) {
        two_sum(S.x, h.x, S.x, e);
        C.x = __fadd_rn(C.x, __fadd_rn(e, l.x));
        two_sum(S.y, h.y, S.y, e);
        C.y = __fadd_rn(C.y, __fadd_rn(e, l.y));
        two_sum(S.z, h.z, S.z, e);
        C.z = __fadd_rn(C.z, __fadd_rn(e, l.z));
    };
    if (I < r1) {
        const int rc = rb / 32;
        const int c0 = sk_owner(sym_prefix(I, nc, rc) - it0, bt, gb);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1 - it0, bt, gb);
        const int li = i - I * rb;
        for (int c = c0; c <= c1; ++c) {
            const size_t k = (size_t)(c + I - r0) * rb + li;
            add(tpart[k], tpart[tlo + k]);
        }
    }
    const int rend = I < r1 ? I : r1;
    for (int r = r0; r < rend; ++r) {
        const long long k = sym_soff(r, n, rb) - soff0 + (i - (long long)(r + 1) * rb);
        add(spart[k], spart[slo + k]);
    }
    accsum[i] = S;
    accsum[(size_t)n + i] = C;
}

typedef void (*sym_kernel_t)(const float4 *, int, float, float4 *, float4 *, long long, int, int,
                             long long, long long, long long, int, long long);

// bpt > 0: scalar kernel with bpt bodies per lane (the third template
// argument asks for that many resident CTAs per SM); bpt < 0: packed f32x2
// kernel with -bpt bodies per lane.  comp: the compensated kernel (scalar
// shapes with up to 12 targets per lane: 13 registers per target).
static sym_kernel_t sym_kernel_for(int w, int bpt, int comp, int fixed = 0, int band = 0)
{
    if (band) {  // banded triangular plans: the default shapes
        if (fixed) return nullptr;
        if (comp) {
            if (w == 1 && bpt == 12) return sym_force_kernel<1, 12, 8, true, false, true>;
            if (w == 4 && bpt == 12) return sym_force_kernel<4, 12, 2, true, false, true>;
            return nullptr;
        }
        if (w == 1 && bpt == 16) return sym_force_kernel<1, 16, 8, false, false, true>;
        if (w == 4 && bpt == 20) return sym_force_kernel<4, 20, 2, false, false, true>;
        if (w == 1 && bpt == 8) return sym_force_kernel<1, 8, 8, false, false, true>;
        if (w == 1 && bpt == 4) return sym_force_kernel<1, 4, 8, false, false, true>;
        return nullptr;
    }
    if (fixed) {  // fixed-point source side: one-warp shapes
        if (comp) return nullptr;
        if (w == 1 && bpt == 16) return sym_force_kernel<1, 16, 8, false, true>;
        if (w == 1 && bpt == 8) return sym_force_kernel<1, 8, 8, false, true>;
        if (w == 1 && bpt == 4) return sym_force_kernel<1, 4, 8, false, true>;
        return nullptr;
    }
    if (comp) {
        if (w == 1 && bpt == 12) return sym_force_kernel<1, 12, 8, true>;
        if (w == 4 && bpt == 12) return sym_force_kernel<4, 12, 2, true>;
        if (w == 8 && bpt == 12) return sym_force_kernel<8, 12, 1, true>;
        if (w == 1 && bpt == 8) return sym_force_kernel<1, 8, 8, true>;
        if (w == 8 && bpt == 8) return sym_force_kernel<8, 8, 1, true>;
        return nullptr;
    }
    if (w == 1 && bpt == 16) return sym_force_kernel<1, 16, 8, false>;
    if (w == 1 && bpt == 8) return sym_force_kernel<1, 8, 8, false>;
    if (w == 1 && bpt == 4) return sym_force_kernel<1, 4, 8, false>;
    if (w == 1 && bpt == 20) return sym_force_kernel<1, 20, 8, false>;
    if (w == 2 && bpt == 16) return sym_force_kernel<2, 16, 4, false>;
    if (w == 4 && bpt == 20) return sym_force_kernel<4, 20, 2, false>;
    if (w == 8 && bpt == 24) return sym_force_kernel<8, 24, 1, false>;
    if (w == 4 && bpt == 8) return sym_force_kernel<4, 8, 1, false>;
    if (w == 8 && bpt == 4) return sym_force_kernel<8, 4, 1, false>;
    if (w == 8 && bpt == 8) return sym_force_kernel<8, 8, 1, false>;
    if (w == 8 && bpt == -8) return sym_force_kernel_f2<8, 4>;
    if (w == 4 && bpt == -8) return sym_force_kernel_f2<4, 4>;
    if (w == 8 && bpt == -4) return sym_force_kernel_f2<8, 2>;
    return nullptr;
}

int sym_plan(int n, int warps, int bpt, int device, SymPlan *pl, int comp, int source_side, int bands)
{
    if (source_side < NB_SOURCE_AUTO || source_side > NB_SOURCE_FIXED)
        return set_error(NB_ERR_INVALID, "source_side is NB_SOURCE_AUTO, NB_SOURCE_TRIANGULAR or NB_SOURCE_FIXED");
    if (comp && source_side == NB_SOURCE_FIXED)
        return set_error(NB_ERR_UNSUPPORTED, "the compensated kernel keeps its triangular (hi, lo) source side");
    int fixed = source_side == NB_SOURCE_FIXED ? 1 : 0;
    const bool given = warps != 0 || bpt != 0;
    // triangular plans go to bands where the array would pass the budget;
    // bands = -1 grows the row block instead
    const bool may_band = !fixed && bands >= 0;
    SymPlan p;
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (!given && fixed) {
            warps = 1;
            bpt = 16;
            int sms = 0;  // fewer targets per lane for small systems, as below
            NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
            while (bpt > 4 && n > 0) {
                const int rb = 32 * bpt, nrb = (n + rb - 1) / rb, nc = (n + 31) / 32;
                if (sym_prefix(nrb, nc, bpt) >= 4ll * sms) break;
                bpt /= 2;
            }
        }
        if (warps == 0 && bpt == 0) {
            // plain: one-warp CTAs x 16 targets (row block 512), then 4 x 20
            // (2560) while the source-side array is over budget, and beyond
            // that 4 x 20 in bands (without bands: 8 x 24, 6144).
            // Compensated (hi and lo halves): 1 x 12 (384), 4 x 12 (1536),
            // then 4 x 12 in bands (without bands: 8 x 12, 3072).
            static const int plain[3][2] = {{1, 16}, {4, 20}, {8, 24}};
            static const int compd[3][2] = {{1, 12}, {4, 12}, {8, 12}};
            const int(*shapes)[2] = comp ? compd : plain;
            const long long halves = comp ? 2 : 1;
            const int last = may_band ? 1 : 2;
            int s = 0;
            while (s < last && halves * sym_spart_entries(n, shapes[s][0] * 32 * shapes[s][1]) *
                                   (long long)sizeof(float4) >
                               kSymSpartBudget)
                ++s;
            warps = shapes[s][0];
            bpt = shapes[s][1];
            // small systems: fewer targets per lane until there are at least
            // four (row, chunk) items per resident warp slot of an SM, so the
            // launch is not a few long items (at N=1024, 16 targets per lane
            // give 48 items)
            if (!comp && warps == 1) {
                int sms = 0;
                NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
                while (bpt > 4 && n > 0) {
                    const int rb = 32 * bpt, nrb = (n + rb - 1) / rb, nc = (n + 31) / 32;
                    if (sym_prefix(nrb, nc, bpt) >= 4ll * sms) break;
                    bpt /= 2;
                }
            }
        }
        if (warps == 0) warps = 8;
        if (bpt == 0) bpt = 8;
        p = SymPlan();
        p.n = n;
        p.warps = warps;
        p.bpt = bpt;
        p.comp = comp;
        p.fixed = fixed;
        p.rb = warps * 32 * (bpt < 0 ? -bpt : bpt);
        p.nc = (n + 31) / 32;
        p.nrb = (n + p.rb - 1) / p.rb;
        p.spart_size = fixed ? sym_fx_entries(n) : sym_spart_entries(n, p.rb);
        p.band_row[0] = 0;
        p.band_row[1] = p.nrb;
        const long long entry = (comp ? 2 : 1) * (long long)sizeof(float4);  // hi and lo halves
        if (may_band && !fixed && n > 0 && (bands > 1 || p.spart_size * entry > kSymSpartBudget)) {
            long long mx = 0;
            const int k = sym_make_bands(n, p.rb, kSymSpartBudget / entry, bands > 1 ? bands : 0, p.band_row, &mx);
            if (k == 0) {
                // more bands than a plan holds (N above about 3.6e7 with the
                // 4 x 20 shape): the automatic choice takes the fixed-point
                // source side instead
                if (given || source_side != NB_SOURCE_AUTO)
                    return set_error(NB_ERR_UNSUPPORTED, "the triangular source side would need more than 512 bands");
                fixed = 1;
                warps = bpt = 0;
                continue;
            }
            p.nbands = k;
            p.spart_size = mx;
        }
        break;
    }
    sym_kernel_t k = sym_kernel_for(p.warps, p.bpt, comp, p.fixed, p.nbands > 1);
    if (!k)
        return set_error(NB_ERR_UNSUPPORTED, p.fixed ? "symmetric kernel shape not compiled with the fixed-point "
                                                       "source side (one warp x 4, 8 or 16 targets)"
                                         : p.nbands > 1 ? "symmetric kernel shape not compiled for bands (one warp "
                                                          "x 4, 8 or 16 targets, 4 warps x 20; compensated: "
                                                          "1 or 4 warps x 12)"
                                                        : "symmetric kernel shape not compiled");
    p.total = n > 0 ? sym_prefix(p.nrb, p.nc, p.rb / 32) : 0;
    int sms = 0, occ = 0;
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * p.warps, 0));
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "symmetric kernel does not fit on an SM");
    long long grid = (long long)sms * occ;
    if (p.total > 0 && grid > p.total) grid = p.total;
    p.grid = p.total > 0 ? (int)grid : 0;
    p.slots = p.total > 0 ? p.grid + p.nrb - 1 : 0;
    p.sms = sms;
    *pl = p;
    return NB_OK;
}

// The record of a fixed plan: sum |m| of n bodies by one block in a fixed
// order (per-thread strided sums, then a tree), then the scale for eps2
// (with_sum 0: keep the recorded sum, a new eps2 only).
constexpr int kFxBlock = 1024;

__global__ void __launch_bounds__(kFxBlock) fx_record_kernel(const float4 *__restrict__ pos, int n, float eps2,
                                                             unsigned long long *__restrict__ acc, int with_sum)
{
    __shared__ float red[kFxBlock];
    float4 *rec = reinterpret_cast<float4 *>(acc + 6ll * n);
    float msum = 0.f;
    if (with_sum) {
        float sum = 0.f;
        for (int i = (int)threadIdx.x; i < n; i += kFxBlock) sum += fabsf(pos[i].w);
        red[threadIdx.x] = sum;
        __syncthreads();
        for (int w = kFxBlock / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        msum = red[0];
    } else {
        msum = rec->x;
    }
    if (threadIdx.x != 0) return;
    // B = 2 / (3 sqrt 3) sum|m| / eps2 bounds every reaction; 2^e > 2 B
    const float b = 0.38490018f * msum / eps2;
    int e = -40;
    if (b > 0.f && b <= 3.0e38f) {
        frexpf(b, &e);  // b < 2^e
        e += 1;
    } else if (b > 0.f) {
        e = 120;  // eps2 = 0: the self pair makes every result NaN anyway
    }
    e = max(-40, min(120, e));
    *rec = make_float4(msum, __int_as_float((127 + 61 - e) << 23), __int_as_float((127 + e - 61) << 23),
                       __int_as_float((127 + 83 - e) << 23));
}

int sym_fx_prepare(const SymPlan &p, const float4 *pos, float4 *spart, float eps2, cudaStream_t s)
{
    if (!p.fixed || p.n == 0) return NB_OK;
    NB_CUDA(cudaMemsetAsync(spart, 0, 6 * sizeof(unsigned long long) * (size_t)p.n, s));
    fx_record_kernel<<<1, kFxBlock, 0, s>>>(pos, p.n, eps2, reinterpret_cast<unsigned long long *>(spart), 1);
    NB_LAUNCH_CHECK("fx_record_kernel launch");
    return NB_OK;
}

int sym_fx_rescale(const SymPlan &p, float4 *spart, float eps2, cudaStream_t s)
{
    if (!p.fixed || p.n == 0) return NB_OK;
    fx_record_kernel<<<1, kFxBlock, 0, s>>>(nullptr, p.n, eps2, reinterpret_cast<unsigned long long *>(spart), 0);
    NB_LAUNCH_CHECK("fx_record_kernel launch");
    return NB_OK;
}

int sym_force(const SymPlan &p, const float4 *pos, float eps2, float4 *tpart, float4 *spart,
              float4 *accsum, cudaStream_t s)
{
    if (p.total == 0) return NB_OK;
    sym_kernel_t k = sym_kernel_for(p.warps, p.bpt, p.comp, p.fixed, p.nbands > 1);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "symmetric kernel shape not compiled");
    // lo blocks (compensated plans) follow the hi blocks
    const long long tlo = (long long)p.slots * p.rb, slo = p.spart_size;
    if (p.nbands <= 1) {
        k<<<p.grid, 32 * p.warps, 0, s>>>(pos, p.n, eps2, tpart, spart, p.total, p.nc, p.nrb, tlo, slo, 0, 0, 0);
        NB_LAUNCH_CHECK("sym_force_kernel launch");
        return NB_OK;
    }
    if (!accsum) return set_error(NB_ERR_INVALID, "sym_force: a banded plan needs its per-body sums");
    const int rc = p.rb / 32;
    for (int b = 0; b < p.nbands; ++b) {
        const int r0 = p.band_row[b], r1 = p.band_row[b + 1];
        const long long it0 = sym_prefix(r0, p.nc, rc), bt = sym_prefix(r1, p.nc, rc) - it0;
        const long long soff0 = sym_soff(r0, p.n, p.rb);
        const int gb = (int)(bt < p.grid ? bt : p.grid);
        k<<<gb, 32 * p.warps, 0, s>>>(pos, p.n, eps2, tpart, spart, bt, p.nc, p.nrb, tlo, slo, it0, r0, soff0);
        NB_LAUNCH_CHECK("sym_force_kernel launch");
        if (p.comp)
            sym_fold_comp_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(tpart, spart, tlo, slo, accsum, p.n, p.rb, p.nc,
                                                                   it0, bt, gb, r0, r1, soff0, b == 0);
        else
            sym_fold_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(tpart, spart, accsum, p.n, p.rb, p.nc, it0, bt, gb, r0,
                                                              r1, soff0, b == 0);
        NB_LAUNCH_CHECK("sym_fold_kernel launch");
    }
    return NB_OK;
}

int sym_integrate(const SymPlan &p, const float4 *pos_old, float4 *pos_new, float4 *vel,
                  const float4 *tpart, const float4 *spart, const float4 *accsum, float damping, float dt,
                  int kick, float G, float4 *acc_out, cudaStream_t s, int consume)
{
    if (p.n == 0) return NB_OK;
    if (p.nbands > 1 && !accsum) return set_error(NB_ERR_INVALID, "sym_integrate: a banded plan needs its per-body sums");
    const long long threads = 4ll * p.n;  // a quad of threads per body
    unsigned long long *fxacc =
        p.fixed ? reinterpret_cast<unsigned long long *>(const_cast<float4 *>(spart)) : nullptr;
    sym_integrate_kernel<<<(unsigned)((threads + kSymIntegBlock - 1) / kSymIntegBlock), kSymIntegBlock, 0, s>>>(
        pos_old, pos_new, vel, tpart, spart, p.n, p.rb, p.nc, p.nrb, p.total, p.grid, damping, dt, kick,
        G, acc_out, fxacc, consume, p.nbands > 1 ? accsum : nullptr);
    NB_LAUNCH_CHECK("sym_integrate_kernel launch");
    return NB_OK;
}

}  // namespace nb
