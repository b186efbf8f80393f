// nb_symff.cu -- FP64-accurate symmetric step in float-float arithmetic
// (NB_F64 with NB_ALGO_SYM).
//
// The app's default state type is double (benchapps/nbody/utc/nbody_main.cc
// FTYPE), and the reference evaluates every ordered pair in FP64
// (benchapps/nbody/cuda/bodysystem_kernel.cu:21-56).  On GB300 the FP64 pipe
// runs at about 1/76 of the FP32 rate (measured: 1.06 TFLOP/s DFMA against
// 78.5 TFLOP/s FFMA), so the FP64 symmetric kernel (nb_sym64.cu) is held to
// some 45 G interactions/s however it is arranged.  This kernel gets FP64
// accuracy from the FP32 pipe instead, with the standard float-float
// (double-single) techniques:
//  * error-free sums: Knuth's two-sum (s + e == a + b exactly) and Dekker's
//    fast two-sum for |a| >= |b|;
//  * error-free products from the FMA: p = a*b, e = fma(a, b, -p);
//  * float-float numbers hi + lo with |lo| <= ulp(hi)/2, about 48 bits.
// Per step, positions and masses are scaled by exact powers of two (the
// largest coordinate and the largest mass into [1/2, 1), found by a
// reduction on the device); each scaled coordinate is split on fixed grids
// into three floats, h (2^-20), m (2^-44) and l (2^-68), h + m + l == x
// exactly for |x| >= 2^-16 and to 2^-69 below that (the mass into a
// float-float).  Per unordered pair (the symmetric layout of nb_sym.cu: row
// blocks of 32*BPT targets per warp x 32-body chunks, the chunk rotating
// through the warp with its reaction):
//  * r = x_j - x_i: the three grid differences are exact; two fast
//    two-sums normalize them to a float-float, to 2^-47 relative and
//    exactly for close pairs -- also far from the origin, where a two-float
//    split of the positions would lose the bits below 2^-49 |x|;
//  * d2 = |r|^2 + eps2 in float-float;
//  * 1/sqrt(d2): the FP32 approximation refined by one FP32 Newton step
//    (to ~2^-24) and one Halley step in float-float, y = y0 (1 + t/2 +
//    3t^2/8) with t = 1 - d2 y0^2 formed from an error-free y0^2 (cubic
//    convergence; the small t keeps the correction's roundings near 2^-47);
//  * inv^3, the weights m_j inv^3 and m_i inv^3, and the six products with
//    r in float-float; target and reaction sums in float-float, renormalized
//    after every term.
// Each target's 32-source chunk sum is folded into FP64 accumulators; each
// reaction (one chunk body, the warp's 32*BPT targets) is written as FP64.
// The FP64 integrator of nb_sym64.cu then sums the partials in FP64, undoes
// the scaling and integrates.  The default shape, one warp x 2 targets
// (row blocks of 64 bodies: a triangular array of N^2 / 4 bytes), is kept at
// every size: past N = 185k the array is cut into bands of at most 8 GiB as
// in nb_sym.cu (symff_fold_kernel folds each band in FP64), which ran 9-22 %
// faster on GB300 than growing the row block (315 against 288 and 259 G
// interactions/s at N = 2^19 and 2^20).  196 FP32 operations and one approximation
// per pair (98 per interaction); results within a few 1e-15 of the FP64
// oracle (FP64 arithmetic: a few 1e-16), not bit-identical (NB_ALGO_EXACT is).
// Range: the scaled squared distances and eps2 must stay normal floats:
// eps2 >= 2^-100 max|x|^2 and body masses >= 2^-100 of the largest.
#include "nb_ff.cuh"

namespace nb {


// range[0] = bits of max |coordinate|, range[1] = bits of max |mass| (non-
// negative doubles order like their bit patterns); range zeroed beforehand.
__global__ void ff_range_kernel(const double4 *__restrict__ pos, int n, unsigned long long *__restrict__ range)
{
    unsigned long long mc = 0, mm = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double4 q = pos[i];
        const double c = fmax(fabs(q.x), fmax(fabs(q.y), fabs(q.z)));
        const unsigned long long bc = (unsigned long long)__double_as_longlong(c);
        const unsigned long long bm = (unsigned long long)__double_as_longlong(fabs(q.w));
        mc = bc > mc ? bc : mc;
        mm = bm > mm ? bm : mm;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, mc, o);
        const unsigned long long b = __shfl_xor_sync(0xffffffffu, mm, o);
        mc = a > mc ? a : mc;
        mm = b > mm ? b : mm;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&range[0], mc);
        atomicMax(&range[1], mm);
    }
}

// Scaled split: coordinates x * 2^kx (below 1 in magnitude) on the grids
// H: 2^-20, M: 2^-44, L: 2^-68 (H + M + L == x * 2^kx exactly when
// |x * 2^kx| >= 2^-16, otherwise to 2^-69); the mass m * 2^km as the
// float-float H + M (L unused).
__global__ void ff_split_kernel(const double4 *__restrict__ pos, int n, const unsigned long long *__restrict__ range,
                                float4 *__restrict__ H, float4 *__restrict__ M, float4 *__restrict__ L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int kx = -ff_exponent(range[0]), km = -ff_exponent(range[1]);
    const double4 q = pos[i];
    const double v[4] = {ldexp(q.x, kx), ldexp(q.y, kx), ldexp(q.z, kx), ldexp(q.w, km)};
    float h[4], m[4], l[4];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double gh = ldexp(rint(ldexp(v[k], 20)), -20);  // |gh| <= 1: 21 bits
        const double r1 = v[k] - gh;                              // exact, |r1| <= 2^-21
        const double gm = ldexp(rint(ldexp(r1, 44)), -44);       // 24 bits
        const double r2 = r1 - gm;                                // exact, |r2| <= 2^-45
        h[k] = (float)gh;
        m[k] = (float)gm;
        l[k] = (float)ldexp(rint(ldexp(r2, 68)), -68);            // 24 bits
    }
    h[3] = __double2float_rn(v[3]);
    m[3] = __double2float_rn(v[3] - (double)h[3]);
    l[3] = 0.f;
    H[i] = make_float4(h[0], h[1], h[2], h[3]);
    M[i] = make_float4(m[0], m[1], m[2], m[3]);
    L[i] = make_float4(l[0], l[1], l[2], l[3]);
}

// PHI: also the potential sum_j m_j inv (j != i) in the partials' w, the
// reaction's included (energy pass).
// BAND: one band of a banded plan, as in sym_force_kernel: items
// [it0, it0 + total) from row block r0 on, target-side slot c + I - r0,
// source-side entries offset by soff0.
template <int W, int BPT, int MINB, bool PHI, bool BAND = false>
__global__ void __launch_bounds__(32 * W, MINB)
    symff_force_kernel(const float4 *__restrict__ H, const float4 *__restrict__ Mi, const float4 *__restrict__ Lo,
                       int n, double eps2, const unsigned long long *__restrict__ range,
                       double4 *__restrict__ tpart, double4 *__restrict__ spart, long long total, int nc, int nrb,
                       long long it0, int r0, long long soff0)
{
    constexpr int WB = 32 * BPT;
    constexpr int RB = W * WB;
    constexpr int RC = RB / 32;
    __shared__ __align__(16) float4 sH[32], sM[32], sL[32];
    __shared__ double sF[4][W][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int c = blockIdx.x;
    // eps2 in the scaled units (x 2^(2 kx)), as a float-float
    const double e2s = ldexp(eps2, -2 * ff_exponent(range[0]));
    const float eh = __double2float_rn(e2s), el = __double2float_rn(e2s - (double)eh);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    long long it = sk_start(c, total, gridDim.x);
    long long end = sk_start(c + 1, total, gridDim.x);
    if constexpr (BAND) {
        it += it0;
        end += it0;
    }

    while (it < end) {
        const int I = sym_row_of(it, nc, RC, nrb);
        const long long rfirst = sym_prefix(I, nc, RC);
        const long long rend = sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB + wid * WB;

        // missing targets: zero mass, so their reactions are 0; masses
        // negated: reactions point along -r
        float pxh[BPT], pxm[BPT], pxl[BPT], pyh[BPT], pym[BPT], pyl[BPT], pzh[BPT], pzm[BPT], pzl[BPT];
        float nmh[BPT], nml[BPT];
        double ax[BPT], ay[BPT], az[BPT], aphi[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tbase + lane + 32 * k;
            const float4 a = i < n ? H[i] : zero;
            const float4 m = i < n ? Mi[i] : zero;
            const float4 b = i < n ? Lo[i] : zero;
            pxh[k] = a.x; pxm[k] = m.x; pxl[k] = b.x;
            pyh[k] = a.y; pym[k] = m.y; pyl[k] = b.y;
            pzh[k] = a.z; pzm[k] = m.z; pzl[k] = b.z;
            nmh[k] = -a.w; nml[k] = -m.w;
            ax[k] = ay[k] = az[k] = aphi[k] = 0.0;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            const bool in = jb + lane < n;
            __syncthreads();  // previous chunk: shared reads are done
            if (wid == 0) {
                // padding: far away (scaled coordinates are below 1), no mass
                sH[lane] = in ? H[jb + lane] : make_float4(1.0e6f, 1.0e6f, 1.0e6f, 0.f);
                sM[lane] = in ? Mi[jb + lane] : zero;
                sL[lane] = in ? Lo[jb + lane] : zero;
            }
            __syncthreads();
            float Axh[BPT], Axl[BPT], Ayh[BPT], Ayl[BPT], Azh[BPT], Azl[BPT], Aph[BPT], Apl[BPT];
#pragma unroll
            for (int k = 0; k < BPT; ++k)
                Axh[k] = Axl[k] = Ayh[k] = Ayl[k] = Azh[k] = Azl[k] = Aph[k] = Apl[k] = 0.f;
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 1
                for (int j = 0; j < 32; ++j) {
                    const float4 a = sH[j], am = sM[j], b = sL[j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        FFPair w;
                        ff_pair<false>(a, am, b, pxh[k], pxm[k], pxl[k], pyh[k], pym[k], pyl[k], pzh[k], pzm[k],
                                       pzl[k], 0.f, 0.f, eh, el, w);
                        ff_acc(Axh[k], Axl[k], w.rxh, w.rxl, w.wjh, w.wjl);
                        ff_acc(Ayh[k], Ayl[k], w.ryh, w.ryl, w.wjh, w.wjl);
                        ff_acc(Azh[k], Azl[k], w.rzh, w.rzl, w.wjh, w.wjl);
                        if (PHI && jb + j != tbase + lane + 32 * k) {  // no self term
                            float vh, vl;
                            ff_mul(a.w, am.w, w.yh, w.yl, vh, vl);
                            ff_add(Aph[k], Apl[k], vh, vl);
                        }
                    }
                }
            } else {
                float Fxh = 0.f, Fxl = 0.f, Fyh = 0.f, Fyl = 0.f, Fzh = 0.f, Fzl = 0.f, Fph = 0.f, Fpl = 0.f;
#pragma unroll 1
                for (int r = 0; r < 32; ++r) {
                    const int idx = (lane + r) & 31;
                    const float4 a = sH[idx], am = sM[idx], b = sL[idx];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        FFPair w;
                        ff_pair<true>(a, am, b, pxh[k], pxm[k], pxl[k], pyh[k], pym[k], pyl[k], pzh[k], pzm[k],
                                      pzl[k], nmh[k], nml[k], eh, el, w);
                        ff_acc(Axh[k], Axl[k], w.rxh, w.rxl, w.wjh, w.wjl);
                        ff_acc(Ayh[k], Ayl[k], w.ryh, w.ryl, w.wjh, w.wjl);
                        ff_acc(Azh[k], Azl[k], w.rzh, w.rzl, w.wjh, w.wjl);
                        ff_acc(Fxh, Fxl, w.rxh, w.rxl, w.wih, w.wil);
                        ff_acc(Fyh, Fyl, w.ryh, w.ryl, w.wih, w.wil);
                        ff_acc(Fzh, Fzl, w.rzh, w.rzl, w.wih, w.wil);
                        if (PHI) {
                            float vh, vl;
                            ff_mul(a.w, am.w, w.yh, w.yl, vh, vl);
                            ff_add(Aph[k], Apl[k], vh, vl);
                            ff_mul(-nmh[k], -nml[k], w.yh, w.yl, vh, vl);
                            ff_add(Fph, Fpl, vh, vl);
                        }
                    }
                    const int from = (lane + 1) & 31;
                    Fxh = __shfl_sync(0xffffffffu, Fxh, from);
                    Fxl = __shfl_sync(0xffffffffu, Fxl, from);
                    Fyh = __shfl_sync(0xffffffffu, Fyh, from);
                    Fyl = __shfl_sync(0xffffffffu, Fyl, from);
                    Fzh = __shfl_sync(0xffffffffu, Fzh, from);
                    Fzl = __shfl_sync(0xffffffffu, Fzl, from);
                    if (PHI) {
                        Fph = __shfl_sync(0xffffffffu, Fph, from);
                        Fpl = __shfl_sync(0xffffffffu, Fpl, from);
                    }
                }
                // lane l now holds the reaction on chunk body l from this warp
                const double fx = (double)Fxh + (double)Fxl, fy = (double)Fyh + (double)Fyl,
                             fz = (double)Fzh + (double)Fzl, fp = PHI ? (double)Fph + (double)Fpl : 0.0;
                long long so = sym_soff(I, n, RB) + (jb + lane - (I + 1) * RB);
                if constexpr (BAND) so -= soff0;
                if (W == 1) {
                    if (in) spart[so] = make_double4(fx, fy, fz, fp);
                } else {
                    sF[0][wid][lane] = fx;
                    sF[1][wid][lane] = fy;
                    sF[2][wid][lane] = fz;
                    sF[3][wid][lane] = fp;
                    __syncthreads();
                    if (wid == 0 && in) {
                        double sx = 0.0, sy = 0.0, sz = 0.0, sp = 0.0;
#pragma unroll
                        for (int w = 0; w < W; ++w) {
                            sx += sF[0][w][lane];
                            sy += sF[1][w][lane];
                            sz += sF[2][w][lane];
                            sp += sF[3][w][lane];
                        }
                        spart[so] = make_double4(sx, sy, sz, sp);
                    }
                }
            }
            // fold the chunk's sums into FP64
#pragma unroll
            for (int k = 0; k < BPT; ++k) {
                ax[k] += (double)Axh[k] + (double)Axl[k];
                ay[k] += (double)Ayh[k] + (double)Ayl[k];
                az[k] += (double)Azh[k] + (double)Azl[k];
                if (PHI) aphi[k] += (double)Aph[k] + (double)Apl[k];
            }
        }
        double4 *dst = tpart + (size_t)(c + I - (BAND ? r0 : 0)) * RB + wid * WB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) dst[lane + 32 * k] = make_double4(ax[k], ay[k], az[k], aphi[k]);
        it = seg_end;
    }
}

typedef void (*symff_kernel_t)(const float4 *, const float4 *, const float4 *, int, double,
                               const unsigned long long *, double4 *, double4 *, long long, int, int, long long,
                               int, long long);

static symff_kernel_t symff_kernel_for(int w, int bpt, bool phi = false, bool band = false)
{
    if (band) {  // banded plans: the one-warp shapes
        if (w == 1 && bpt == 2)
            return phi ? symff_force_kernel<1, 2, 16, true, true> : symff_force_kernel<1, 2, 16, false, true>;
        if (w == 1 && bpt == 4)
            return phi ? symff_force_kernel<1, 4, 8, true, true> : symff_force_kernel<1, 4, 8, false, true>;
        return nullptr;
    }
    if (w == 1 && bpt == 2) return phi ? symff_force_kernel<1, 2, 16, true> : symff_force_kernel<1, 2, 16, false>;
    if (w == 1 && bpt == 4) return phi ? symff_force_kernel<1, 4, 8, true> : symff_force_kernel<1, 4, 8, false>;
    if (w == 4 && bpt == 4) return phi ? symff_force_kernel<4, 4, 2, true> : symff_force_kernel<4, 4, 2, false>;
    if (w == 8 && bpt == 4) return phi ? symff_force_kernel<8, 4, 1, true> : symff_force_kernel<8, 4, 1, false>;
    if (w == 8 && bpt == 8) return phi ? symff_force_kernel<8, 8, 1, true> : symff_force_kernel<8, 8, 1, false>;
    return nullptr;
}

int symff_plan(int n, int warps, int bpt, int device, SymPlan *pl, int bands)
{
    const bool given = warps != 0 || bpt != 0;
    if (!given) {
        // one-warp CTAs x 2 targets (row block 64), its source-side array
        // (32 B entries) in bands where it would pass the budget; without
        // bands 1 x 4 (128), 4 x 4 (512), 8 x 4 (1024), 8 x 8 (2048) take
        // over instead
        static const int shapes[5][2] = {{1, 2}, {1, 4}, {4, 4}, {8, 4}, {8, 8}};
        int s = 0;
        if (bands < 0)
            while (s < 4 && sym_spart_entries(n, shapes[s][0] * 32 * shapes[s][1]) * (long long)sizeof(double4) >
                                kSymSpartBudget)
                ++s;
        warps = shapes[s][0];
        bpt = shapes[s][1];
    }
    SymPlan p;
    p.n = n;
    p.warps = warps;
    p.bpt = bpt;
    p.rb = warps * 32 * bpt;
    p.nc = (n + 31) / 32;
    p.nrb = (n + p.rb - 1) / p.rb;
    p.spart_size = sym_spart_entries(n, p.rb);
    p.band_row[0] = 0;
    p.band_row[1] = p.nrb;
    if (bands >= 0 && n > 0 &&
        (bands > 1 || p.spart_size * (long long)sizeof(double4) > kSymSpartBudget)) {
        long long mx = 0;
        const int k = sym_make_bands(n, p.rb, kSymSpartBudget / (long long)sizeof(double4), bands > 1 ? bands : 0,
                                     p.band_row, &mx);
        if (k == 0)
            return set_error(NB_ERR_UNSUPPORTED, "the float-float source side would need more than 512 bands");
        p.nbands = k;
        p.spart_size = mx;
    }
    const bool band = p.nbands > 1;
    symff_kernel_t k = symff_kernel_for(warps, bpt, false, band);
    if (!k)
        return set_error(NB_ERR_UNSUPPORTED, band ? "float-float symmetric kernel shape not compiled for bands "
                                                    "(one warp x 2 or 4 targets)"
                                                  : "float-float symmetric kernel shape not compiled");
    p.total = n > 0 ? sym_prefix(p.nrb, p.nc, p.rb / 32) : 0;
    int sms = 0, occ = 0;
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * warps, 0));
    int occ_phi = 0;  // the energy pass runs on the same plan
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_phi, symff_kernel_for(warps, bpt, true, band),
                                                          32 * warps, 0));
    if (occ_phi < occ) occ = occ_phi;
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "float-float symmetric kernel does not fit on an SM");
    long long grid = (long long)sms * occ;
    if (p.total > 0 && grid > p.total) grid = p.total;
    p.grid = p.total > 0 ? (int)grid : 0;
    p.slots = p.total > 0 ? p.grid + p.nrb - 1 : 0;
    p.sms = sms;
    *pl = p;
    return NB_OK;
}

// After band [r0, r1) of a banded plan: the running per-body sums (x, y, z
// and the potential in w), as sym_fold_kernel does for float partials.
__global__ void __launch_bounds__(256) symff_fold_kernel(const double4 *__restrict__ tpart,
                                                         const double4 *__restrict__ spart,
                                                         double4 *__restrict__ accsum, int n, int rb, int nc,
                                                         long long it0, long long bt, int gb, int r0, int r1,
                                                         long long soff0, int first)
{
    const int i = n - 1 - (int)(blockIdx.x * blockDim.x + threadIdx.x);  // longest walks first
    if (i < 0) return;
    const int I = i / rb;
    if (I < r0) return;  // rows before the band get nothing from it (r0 = 0 for the first band)
    double4 a = first ? make_double4(0.0, 0.0, 0.0, 0.0) : accsum[i];
    if (I < r1) {
        const int rc = rb / 32;
        const int c0 = sk_owner(sym_prefix(I, nc, rc) - it0, bt, gb);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1 - it0, bt, gb);
        const int li = i - I * rb;
        for (int c = c0; c <= c1; ++c) {
            const double4 q = tpart[(size_t)(c + I - r0) * rb + li];
            a.x = __dadd_rn(a.x, q.x);
            a.y = __dadd_rn(a.y, q.y);
            a.z = __dadd_rn(a.z, q.z);
            a.w = __dadd_rn(a.w, q.w);
        }
    }
    const int rend = I < r1 ? I : r1;
#pragma unroll 4
    for (int r = r0; r < rend; ++r) {
        const double4 q = spart[sym_soff(r, n, rb) - soff0 + (i - (long long)(r + 1) * rb)];
        a.x = __dadd_rn(a.x, q.x);
        a.y = __dadd_rn(a.y, q.y);
        a.z = __dadd_rn(a.z, q.z);
        a.w = __dadd_rn(a.w, q.w);
    }
    accsum[i] = a;
}

int ff_scale_split(const double4 *pos, int n, int sms, float4 *H, float4 *M, float4 *L, unsigned long long *range,
                   cudaStream_t s)
{
    if (n == 0) return NB_OK;
    NB_CUDA(cudaMemsetAsync(range, 0, 2 * sizeof(unsigned long long), s));
    const long long want = (n + 255) / 256, cap = 4ll * (sms > 0 ? sms : 1);
    const long long blocks = want < cap ? want : cap;
    ff_range_kernel<<<(unsigned)blocks, 256, 0, s>>>(pos, n, range);
    NB_LAUNCH_CHECK("ff_range_kernel launch");
    ff_split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pos, n, range, H, M, L);
    NB_LAUNCH_CHECK("ff_split_kernel launch");
    return NB_OK;
}

int symff_force(const SymPlan &p, const double4 *pos, double eps2, float4 *split, unsigned long long *range,
                double4 *tpart, double4 *spart, double4 *accsum, cudaStream_t s, int phi)
{
    if (p.n == 0) return NB_OK;
    symff_kernel_t k = symff_kernel_for(p.warps, p.bpt, phi != 0, p.nbands > 1);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "float-float symmetric kernel shape not compiled");
    if (p.nbands > 1 && !accsum) return set_error(NB_ERR_INVALID, "symff_force: a banded plan needs its per-body sums");
    float4 *H = split, *M = split + p.n, *L = split + 2 * (size_t)p.n;
    int st = ff_scale_split(pos, p.n, p.sms, H, M, L, range, s);
    if (st) return st;
    if (p.nbands <= 1) {
        k<<<p.grid, 32 * p.warps, 0, s>>>(H, M, L, p.n, eps2, range, tpart, spart, p.total, p.nc, p.nrb, 0, 0, 0);
        NB_LAUNCH_CHECK("symff_force_kernel launch");
        return NB_OK;
    }
    const int rc = p.rb / 32;
    for (int b = 0; b < p.nbands; ++b) {
        const int r0 = p.band_row[b], r1 = p.band_row[b + 1];
        const long long it0 = sym_prefix(r0, p.nc, rc), bt = sym_prefix(r1, p.nc, rc) - it0;
        const long long soff0 = sym_soff(r0, p.n, p.rb);
        const int gb = (int)(bt < p.grid ? bt : p.grid);
        k<<<gb, 32 * p.warps, 0, s>>>(H, M, L, p.n, eps2, range, tpart, spart, bt, p.nc, p.nrb, it0, r0, soff0);
        NB_LAUNCH_CHECK("symff_force_kernel launch");
        symff_fold_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(tpart, spart, accsum, p.n, p.rb, p.nc, it0, bt, gb, r0,
                                                            r1, soff0, b == 0);
        NB_LAUNCH_CHECK("symff_fold_kernel launch");
    }
    return NB_OK;
}

}  // namespace nb
