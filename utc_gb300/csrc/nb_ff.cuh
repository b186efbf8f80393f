// nb_ff.cuh -- float-float (double-single) device arithmetic shared by the
// float-float symmetric kernels for FP64 state (nb_symff.cu, single system;
// nb_batch.cu, batches).  Published techniques: Knuth's two-sum, Dekker's
// fast two-sum, the FMA two-product, Halley's iteration for 1/sqrt.  A
// float-float number is hi + lo with |lo| <= ulp(hi)/2 (about 48 bits).
#pragma once

#include "nb_internal.cuh"

namespace nb {

// Knuth's two-sum: s + e == a + b exactly.
__device__ __forceinline__ void ff_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Dekker's fast two-sum, exact when |a| >= |b| (or a == 0).
__device__ __forceinline__ void ff_fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// r = s - p from grid-split coordinates (x = h + m + l with h, m and l on
// the grids 2^-20, 2^-44 and 2^-68 of the scaled units, |x| < 1), as a
// normalized float-float.  The three differences are exact (each fits 24
// bits); A + B is split by Dekker's fast two-sum (|A| >= 2^-20 >= |B|, or
// A == 0) and the low part added once: r to 2^-47 relative, exactly when the
// high parts cancel (close pairs).
__device__ __forceinline__ void ff_diff(float sh, float sm, float sl, float ph, float pm, float pl, float &rh,
                                        float &rl)
{
    const float A = __fsub_rn(sh, ph), B = __fsub_rn(sm, pm), C = __fsub_rn(sl, pl);
    float s1, e1;
    ff_fast_two_sum(A, B, s1, e1);
    ff_fast_two_sum(s1, __fadd_rn(e1, C), rh, rl);
}

// A += r * w (float-float, renormalized)
__device__ __forceinline__ void ff_acc(float &Ah, float &Al, float rh, float rl, float wh, float wl)
{
    const float p = __fmul_rn(rh, wh);
    float e = __fmaf_rn(rh, wh, -p);
    e = __fmaf_rn(rh, wl, e);
    e = __fmaf_rn(rl, wh, e);
    float s, t;
    ff_two_sum(Ah, p, s, t);
    ff_fast_two_sum(s, __fadd_rn(Al, __fadd_rn(t, e)), Ah, Al);
}

struct FFPair {
    float rxh, rxl, ryh, ryl, rzh, rzl;  // r = x_j - x_i
    float wjh, wjl;                      // m_j inv^3 (weight on the target)
    float wih, wil;                      // m_i inv^3 with m_i as passed (reaction)
    float yh, yl;                        // inv = 1/sqrt(|r|^2 + eps2)
};

// A += v (float-float, renormalized)
__device__ __forceinline__ void ff_add(float &Ah, float &Al, float vh, float vl)
{
    float s, t;
    ff_two_sum(Ah, vh, s, t);
    ff_fast_two_sum(s, __fadd_rn(Al, __fadd_rn(t, vl)), Ah, Al);
}

// m * y for a float-float mass (mh, ml) and y (yh, yl), unnormalized
__device__ __forceinline__ void ff_mul(float mh, float ml, float yh, float yl, float &ph, float &pl)
{
    ph = __fmul_rn(mh, yh);
    float e = __fmaf_rn(mh, yh, -ph);
    e = __fmaf_rn(mh, yl, e);
    pl = __fmaf_rn(ml, yh, e);
}

// Pair pieces for source (sH, sM, sL) and target (p*), eps2 = eh + el.
template <bool REACT>
__device__ __forceinline__ void ff_pair(float4 sH, float4 sM, float4 sL, float pxh, float pxm, float pxl, float pyh,
                                        float pym, float pyl, float pzh, float pzm, float pzl, float mih, float mil,
                                        float eh, float el, FFPair &o)
{
    ff_diff(sH.x, sM.x, sL.x, pxh, pxm, pxl, o.rxh, o.rxl);
    ff_diff(sH.y, sM.y, sL.y, pyh, pym, pyl, o.ryh, o.ryl);
    ff_diff(sH.z, sM.z, sL.z, pzh, pzm, pzl, o.rzh, o.rzl);
    // squares as (p, e) with p + e = r^2 to float-float accuracy
    const float qx = __fmul_rn(o.rxh, o.rxh), qy = __fmul_rn(o.ryh, o.ryh), qz = __fmul_rn(o.rzh, o.rzh);
    float ex = __fmaf_rn(o.rxh, o.rxh, -qx), ey = __fmaf_rn(o.ryh, o.ryh, -qy), ez = __fmaf_rn(o.rzh, o.rzh, -qz);
    ex = __fmaf_rn(__fadd_rn(o.rxh, o.rxh), o.rxl, ex);
    ey = __fmaf_rn(__fadd_rn(o.ryh, o.ryh), o.ryl, ey);
    ez = __fmaf_rn(__fadd_rn(o.rzh, o.rzh), o.rzl, ez);
    float S, t1, t2, t3;
    ff_two_sum(eh, qx, S, t1);
    ff_two_sum(S, qy, S, t2);
    ff_two_sum(S, qz, S, t3);
    const float L = __fadd_rn(__fadd_rn(__fadd_rn(el, ex), __fadd_rn(ey, ez)), __fadd_rn(__fadd_rn(t1, t2), t3));
    float Dh, Dl;
    ff_fast_two_sum(S, L, Dh, Dl);  // all terms >= 0: |S| >= |L|
    // 1/sqrt(D): the FP32 approximation, one Newton step in FP32 (error
    // near 2^-24, so that u below is near 2^-23 and the roundings that scale
    // with it stay near 2^-47), then one Halley step in float-float
    const float ya = rsqrt_approx(Dh);
    const float y0 = __fmaf_rn(__fmul_rn(ya, 0.5f), __fmaf_rn(-Dh, __fmul_rn(ya, ya), 1.0f), ya);
    const float q = __fmul_rn(y0, y0);
    const float qe = __fmaf_rn(y0, y0, -q);
    const float t = __fmul_rn(Dh, q);
    float c = __fmaf_rn(Dh, q, -t);
    c = __fmaf_rn(Dh, qe, c);
    c = __fmaf_rn(Dl, q, c);
    const float u = __fsub_rn(__fsub_rn(1.0f, t), c);  // 1 - t is exact (t near 1)
    const float corr = __fmul_rn(y0, __fmul_rn(u, __fmaf_rn(0.375f, u, 0.5f)));
    float yh, yl;
    ff_fast_two_sum(y0, corr, yh, yl);
    o.yh = yh;
    o.yl = yl;
    // inv^3 = y^3
    const float p2 = __fmul_rn(yh, yh);
    float e2 = __fmaf_rn(yh, yh, -p2);
    e2 = __fmaf_rn(__fadd_rn(yh, yh), yl, e2);
    const float p3 = __fmul_rn(p2, yh);
    float e3 = __fmaf_rn(p2, yh, -p3);
    e3 = __fmaf_rn(p2, yl, e3);
    e3 = __fmaf_rn(e2, yh, e3);
    float y3h, y3l;
    ff_fast_two_sum(p3, e3, y3h, y3l);
    // weights (mass as the float-float h + m of its split)
    o.wjh = __fmul_rn(sH.w, y3h);
    float we = __fmaf_rn(sH.w, y3h, -o.wjh);
    we = __fmaf_rn(sH.w, y3l, we);
    o.wjl = __fmaf_rn(sM.w, y3h, we);
    if (REACT) {
        o.wih = __fmul_rn(mih, y3h);
        float wr = __fmaf_rn(mih, y3h, -o.wih);
        wr = __fmaf_rn(mih, y3l, wr);
        o.wil = __fmaf_rn(mil, y3h, wr);
    }
}

// binary exponent e of a non-negative double given by its bits, with
// 2^(e-1) <= v < 2^e; 0 for zero, subnormal, infinite or NaN values
__device__ __forceinline__ int ff_exponent(unsigned long long bits)
{
    const int field = (int)((bits >> 52) & 0x7ff);
    return (field == 0 || field == 0x7ff) ? 0 : field - 1022;
}


}  // namespace nb
