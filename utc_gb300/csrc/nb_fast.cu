// nb_fast.cu -- fast FP32 all-pairs force kernel for sm_103a.
//
// Replaces the reference's _computeNBodyForce_kernel / _integrateNBodySystem_
// kernel pair (benchapps/nbody/cuda/bodysystem_kernel.cu:60-138), which gives
// each thread one target, stages sources as four scalar loads per thread into
// __shared__ T[4][512] and runs one fused launch of N/256 CTAs per step.
//
// Design here (one GB300, compute-bound on the FP32 pipe):
//  * Each thread owns 2*NPAIR targets held as packed pairs, so that every
//    pair-term operation is one sm_100+ f32x2 instruction (FADD2/FMUL2/FFMA2)
//    doing two targets' work: per interaction 12 FP32 lane-operations and
//    one MUFU.RSQ, issued in 6 packed instructions plus the MUFU.  (Scalar
//    FFMA versions of this loop were measured on the same GB300 and ran
//    1-10 % slower.)
//  * Sources are staged through shared memory with each component stored
//    twice, (x, x, y, y) and (z, z, m, m), so one LDS.128 broadcast yields the
//    two packed operands a source contributes to a target pair.  The next
//    tile is prefetched into registers while the current one is consumed.
//  * Work is split stream-K style: the (target block, 32-source group)
//    iteration space is cut into `grid` equal contiguous ranges, one per
//    persistent CTA, so all SMs finish together at any N (no wave
//    quantisation).  A CTA writes one partial acceleration per target block
//    it touches; a second, bandwidth-bound kernel sums the partials of each
//    target in CTA order (deterministic) and applies the kick/drift update.
#include <algorithm>

#include "nb_internal.cuh"

namespace nb {

// Packed two-sum (Knuth): s + e == a + b exactly, s = fl(a + b).  Inline
// PTX keeps the compiler from reassociating it away.
__device__ __forceinline__ void f2_two_sum(f2 a, f2 b, f2 &s, f2 &e)
{
    s = f2_add(a, b);
    const f2 bb = f2_sub(s, a);
    e = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
}

// Each thread owns 2*NPAIR targets held as packed pairs (t + 2p*NT,
// t + (2p+1)*NT).  FLAGS: SK_COMP -- fold each tile's partial sums into a
// compensated (hi, lo) pair with a two-sum, and write both (lo at
// partial + lo_offset); SK_PHI -- also accumulate the potential
// sum_j m_j / sqrt(r^2 + eps2) in w.
// CTA blockIdx.x is CTA cta_base + blockIdx.x of a plan of grid_full CTAs,
// and works only on iterations inside [it_lo, it_hi): a launch of the CTAs
// that cover a range of target blocks computes those blocks' partial slots
// exactly as the full launch does (a shard of the targets, same bits).
template <int NT, int NPAIR, int FLAGS>
__global__ void __launch_bounds__(NT) sk_force_kernel(const float4 *__restrict__ pos, int n,
                                                      float eps2, float4 *__restrict__ partial,
                                                      long long total, int ngroups,
                                                      long long lo_offset, int cta_base, int grid_full,
                                                      long long it_lo, long long it_hi)
{
    constexpr bool COMP = (FLAGS & SK_COMP) != 0;
    constexpr bool PHI = (FLAGS & SK_PHI) != 0;
    constexpr int TB = NT * 2 * NPAIR;
    constexpr int CP_ = COMP ? NPAIR : 1;
    __shared__ __align__(16) float4 sA[NT];  // (x, x, y, y)
    __shared__ __align__(16) float4 sB[NT];  // (z, z, m, m)
    const int t = threadIdx.x;
    const int c = cta_base + blockIdx.x;
    long long it = sk_start(c, total, grid_full);
    long long end = sk_start(c + 1, total, grid_full);
    if (it < it_lo) it = it_lo;
    if (end > it_hi) end = it_hi;
    const f2 EPS2 = f2_pack(eps2, eps2);
    const f2 ZERO = f2_pack(0.f, 0.f);
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);

    while (it < end) {
        const int tb = (int)(it / ngroups);
        const long long tb_first = (long long)tb * ngroups;
        const long long seg_end = end < tb_first + ngroups ? end : tb_first + ngroups;
        const int j0 = (int)(it - tb_first) * kGroup;
        const int j1 = min((int)(seg_end - tb_first) * kGroup, n);

        f2 PX[NPAIR], PY[NPAIR], PZ[NPAIR], AX[NPAIR], AY[NPAIR], AZ[NPAIR], AP[NPAIR];
        f2 SX[CP_], SY[CP_], SZ[CP_], SP[CP_], CX[CP_], CY[CP_], CZ[CP_], CPh[CP_];
#pragma unroll
        for (int p = 0; p < NPAIR; ++p) {
            const int i0 = tb * TB + t + (2 * p) * NT;
            const int i1 = i0 + NT;
            const float4 q0 = i0 < n ? pos[i0] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 q1 = i1 < n ? pos[i1] : make_float4(0.f, 0.f, 0.f, 0.f);
            PX[p] = f2_pack(q0.x, q1.x);
            PY[p] = f2_pack(q0.y, q1.y);
            PZ[p] = f2_pack(q0.z, q1.z);
            AX[p] = AY[p] = AZ[p] = AP[p] = ZERO;
            if constexpr (COMP) SX[p] = SY[p] = SZ[p] = SP[p] = CX[p] = CY[p] = CZ[p] = CPh[p] = ZERO;
        }

        float4 nxt = (j0 + t < j1) ? pos[j0 + t] : pad;
        for (int jt = j0; jt < j1; jt += NT) {
            __syncthreads();  // the previous tile has been consumed by all warps
            sA[t] = make_float4(nxt.x, nxt.x, nxt.y, nxt.y);
            sB[t] = make_float4(nxt.z, nxt.z, nxt.w, nxt.w);
            __syncthreads();
            if (jt + NT < j1) {
                const int jn = jt + NT + t;
                nxt = jn < j1 ? pos[jn] : pad;
            }
            const int cnt = min(NT, j1 - jt);
            const int cnt4 = (cnt + 3) & ~3;  // entries past cnt are zero-mass pads
            for (int j = 0; j < cnt4; j += 4) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 a = sA[j + u];
                    const float4 b = sB[j + u];
                    const f2 X2 = f2_pack(a.x, a.y), Y2 = f2_pack(a.z, a.w);
                    const f2 Z2 = f2_pack(b.x, b.y), M2 = f2_pack(b.z, b.w);
#pragma unroll
                    for (int p = 0; p < NPAIR; ++p) {
                        const f2 rx = f2_sub(X2, PX[p]);
                        const f2 ry = f2_sub(Y2, PY[p]);
                        const f2 rz = f2_sub(Z2, PZ[p]);
                        f2 d2 = f2_fma(rx, rx, EPS2);
                        d2 = f2_fma(ry, ry, d2);
                        d2 = f2_fma(rz, rz, d2);
                        float dlo, dhi;
                        f2_unpack(d2, dlo, dhi);
                        const f2 inv = f2_pack(rsqrt_approx(dlo), rsqrt_approx(dhi));
                        const f2 inv2 = f2_mul(inv, inv);
                        const f2 mi = f2_mul(M2, inv);
                        const f2 s = f2_mul(mi, inv2);
                        AX[p] = f2_fma(rx, s, AX[p]);
                        AY[p] = f2_fma(ry, s, AY[p]);
                        AZ[p] = f2_fma(rz, s, AZ[p]);
                        if constexpr (PHI) AP[p] = f2_add(AP[p], mi);
                    }
                }
            }
            if constexpr (COMP) {
#pragma unroll
                for (int p = 0; p < NPAIR; ++p) {
                    f2 e;
                    f2_two_sum(SX[p], AX[p], SX[p], e);
                    CX[p] = f2_add(CX[p], e);
                    f2_two_sum(SY[p], AY[p], SY[p], e);
                    CY[p] = f2_add(CY[p], e);
                    f2_two_sum(SZ[p], AZ[p], SZ[p], e);
                    CZ[p] = f2_add(CZ[p], e);
                    if constexpr (PHI) {
                        f2_two_sum(SP[p], AP[p], SP[p], e);
                        CPh[p] = f2_add(CPh[p], e);
                    }
                    AX[p] = AY[p] = AZ[p] = AP[p] = ZERO;
                }
            }
        }

        float4 *dst = partial + (size_t)(c + tb) * TB;
#pragma unroll
        for (int p = 0; p < NPAIR; ++p) {
            float x0, x1, y0, y1, z0, z1, w0 = 0.f, w1 = 0.f;
            if constexpr (COMP) {
                f2_unpack(SX[p], x0, x1);
                f2_unpack(SY[p], y0, y1);
                f2_unpack(SZ[p], z0, z1);
                if constexpr (PHI) f2_unpack(SP[p], w0, w1);
            } else {
                f2_unpack(AX[p], x0, x1);
                f2_unpack(AY[p], y0, y1);
                f2_unpack(AZ[p], z0, z1);
                if constexpr (PHI) f2_unpack(AP[p], w0, w1);
            }
            dst[t + (2 * p) * NT] = make_float4(x0, y0, z0, w0);
            dst[t + (2 * p + 1) * NT] = make_float4(x1, y1, z1, w1);
            if constexpr (COMP) {
                f2_unpack(CX[p], x0, x1);
                f2_unpack(CY[p], y0, y1);
                f2_unpack(CZ[p], z0, z1);
                if constexpr (PHI) f2_unpack(CPh[p], w0, w1);
                dst[lo_offset + t + (2 * p) * NT] = make_float4(x0, y0, z0, w0);
                dst[lo_offset + t + (2 * p + 1) * NT] = make_float4(x1, y1, z1, w1);
            }
        }
        it = seg_end;
    }
}

// Sum the partial slots of each target in CTA order, then the reference's
// kick / damping / drift with unfused IEEE operations in its order
// (bodysystem_kernel.cu:115-126).  Targets i_begin <= i < i_end.
__global__ void sk_integrate_kernel(const float4 *__restrict__ pos_old, float4 *__restrict__ pos_new,
                                    float4 *__restrict__ vel, const float4 *__restrict__ partial,
                                    int i_begin, int i_end, int tbsize, long long total, int ngroups,
                                    int grid, float damping, float dt, int kick, float G,
                                    float4 *__restrict__ acc_out)
{
    const int i = i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i_end) return;
    const int tb = i / tbsize;
    const int li = i - tb * tbsize;
    const long long first = (long long)tb * ngroups;
    const int c0 = sk_owner(first, total, grid);
    const int c1 = sk_owner(first + ngroups - 1, total, grid);
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 q = partial[(size_t)(c + tb) * tbsize + li];
        ax = __fadd_rn(ax, q.x);
        ay = __fadd_rn(ay, q.y);
        az = __fadd_rn(az, q.z);
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

// ---------------------------------------------------------------------------
// dispatch over the compiled (threads per CTA, target pairs per thread) shapes
// ---------------------------------------------------------------------------
typedef void (*sk_kernel_t)(const float4 *, int, float, float4 *, long long, int, long long, int, int,
                            long long, long long);

// Compiled shapes (threads per CTA x bodies per thread): plain kernel
// 128|256 x 2|4|8; compensated and potential variants 256 x 4|8.
static sk_kernel_t sk_kernel_for(int block, int bpt, int flags)
{
#define NB_SK(NT, B, F) \
    if (block == NT && bpt == B) return sk_force_kernel<NT, B / 2, F>;
    if (flags == 0) {
        NB_SK(128, 2, 0) NB_SK(128, 4, 0) NB_SK(128, 8, 0)
        NB_SK(256, 2, 0) NB_SK(256, 4, 0) NB_SK(256, 8, 0)
    } else if (flags == SK_PHI) {
        NB_SK(256, 4, SK_PHI) NB_SK(256, 8, SK_PHI)
    } else if (flags == SK_COMP) {
        NB_SK(256, 4, SK_COMP) NB_SK(256, 8, SK_COMP)
    } else if (flags == (SK_COMP | SK_PHI)) {
        NB_SK(256, 4, SK_COMP | SK_PHI) NB_SK(256, 8, SK_COMP | SK_PHI)
    }
#undef NB_SK
    return nullptr;
}

bool fast_shape_supported(int block, int bpt, int flags)
{
    return sk_kernel_for(block, bpt, flags) != nullptr;
}

int fast_plan(int n, int block, int bpt, int ctas_per_sm, int device, SkPlan *pl, int flags)
{
    if (n < 0) return set_error(NB_ERR_INVALID, "n must be >= 0");
    if (block == 0 || bpt == 0) {
        // default shape: wide blocks for large N, finer granularity below
        if (block == 0) block = n >= 32768 ? 256 : 128;
        if (bpt == 0) bpt = n >= 8192 ? 8 : (n >= 2048 ? 4 : 2);
    }
    sk_kernel_t k = sk_kernel_for(block, bpt, flags);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "fast kernel shape (block, bodies per thread) not compiled");
    SkPlan p;
    p.n = n;
    p.block = block;
    p.bpt = bpt;
    p.tbsize = block * bpt;
    p.ntb = (n + p.tbsize - 1) / p.tbsize;
    p.ngroups = (n + kGroup - 1) / kGroup;
    p.total = (long long)p.ntb * p.ngroups;
    int sms = 0, occ = 0;
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, block, 0));
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "fast kernel does not fit on an SM");
    if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
    long long grid = (long long)sms * occ;
    if (p.total > 0 && grid > p.total) grid = p.total;
    p.grid = p.total > 0 ? (int)grid : 0;
    p.slots = p.total > 0 ? p.grid + p.ntb - 1 : 0;
    *pl = p;
    return NB_OK;
}

int fast_shard(SkPlan *p, int rank, int nranks)
{
    if (nranks < 1 || rank < 0 || rank >= nranks)
        return set_error(NB_ERR_INVALID, "shard rank must be in [0, nranks)");
    // whole target blocks per rank, the remainder to the first ranks
    const int q = p->ntb / nranks, r = p->ntb % nranks;
    const int tb0 = rank * q + (rank < r ? rank : r);
    const int tb1 = tb0 + q + (rank < r ? 1 : 0);
    p->ranged = true;
    p->it_lo = (long long)tb0 * p->ngroups;
    p->it_hi = (long long)tb1 * p->ngroups;
    p->i_lo = std::min(tb0 * p->tbsize, p->n);
    p->i_hi = std::min(tb1 * p->tbsize, p->n);
    return NB_OK;
}

int fast_force(const SkPlan &p, const float4 *pos, float eps2, float4 *partial, cudaStream_t s,
               int flags)
{
    if (p.total == 0) return NB_OK;
    sk_kernel_t k = sk_kernel_for(p.block, p.bpt, flags);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "fast kernel shape not compiled for this variant");
    const long long lo_offset = (long long)p.slots * p.tbsize;
    long long lo = 0, hi = p.total;
    int base = 0, ctas = p.grid;
    if (p.ranged) {  // only the CTAs that cover the shard's iterations
        lo = p.it_lo;
        hi = p.it_hi;
        if (hi <= lo) return NB_OK;
        base = sk_owner(lo, p.total, p.grid);
        ctas = sk_owner(hi - 1, p.total, p.grid) - base + 1;
    }
    k<<<ctas, p.block, 0, s>>>(pos, p.n, eps2, partial, p.total, p.ngroups, lo_offset, base, p.grid, lo, hi);
    NB_LAUNCH_CHECK("sk_force_kernel launch");
    return NB_OK;
}

int fast_integrate(const SkPlan &p, const float4 *pos_old, float4 *pos_new, float4 *vel,
                   const float4 *partial, float damping, float dt, int kick, float G,
                   float4 *acc_out, cudaStream_t s)
{
    const int i0 = p.ranged ? p.i_lo : 0, i1 = p.ranged ? p.i_hi : p.n;
    if (i1 <= i0) return NB_OK;
    const int bs = 256;
    sk_integrate_kernel<<<(i1 - i0 + bs - 1) / bs, bs, 0, s>>>(pos_old, pos_new, vel, partial, i0, i1,
                                                               p.tbsize, p.total, p.ngroups, p.grid,
                                                               damping, dt, kick, G, acc_out);
    NB_LAUNCH_CHECK("sk_integrate_kernel launch");
    return NB_OK;
}

// ---------------------------------------------------------------------------
// FP32 FMA peak probe: independent FMA chains on every SM.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) probe_fma2_kernel(float *out, int iters)
{
    const float base = 1.0f + 1e-6f * (float)threadIdx.x;
    f2 a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = f2_pack(base + k, base - k);
    const f2 m = f2_pack(0.999999f, 0.999998f), c = f2_pack(1e-7f, 2e-7f);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = f2_fma(a[k], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float lo, hi;
        f2_unpack(a[k], lo, hi);
        s += lo + hi;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) probe_fma1_kernel(float *out, int iters)
{
    const float base = 1.0f + 1e-6f * (float)threadIdx.x;
    float a[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = base + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) a[k] = fmaf(a[k], 0.999999f, 1e-7f);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) probe_dfma_kernel(float *out, int iters)
{
    const double base = 1.0 + 1e-9 * (double)threadIdx.x;
    double a[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = base + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) a[k] = fma(a[k], 0.999999999, 1e-10);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (float)s;
}

// packed: 0 scalar FFMA, 1 packed FFMA2, 2 FP64 DFMA
int probe_fma(int iters, int packed, double *flops, float *ms, cudaStream_t s)
{
    if (iters <= 0 || !flops || !ms) return set_error(NB_ERR_INVALID, "probe_fma arguments");
    int dev = 0, sms = 0, occ = 0;
    NB_CUDA(cudaGetDevice(&dev));
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (packed < 0 || packed > 2) return set_error(NB_ERR_INVALID, "probe_fma: packed is 0, 1 or 2");
    auto kern = packed == 2 ? probe_dfma_kernel : packed ? probe_fma2_kernel : probe_fma1_kernel;
    NB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, 0));
    const int grid = sms * std::max(occ, 1);
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = nb::dmalloc((void **)&out, sizeof(float) * grid * 256);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        kern<<<grid, 256, 0, s>>>(out, 16);  // warm-up
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) {
        kern<<<grid, 256, 0, s>>>(out, iters);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    cudaStreamSynchronize(s);  // nothing of the probe is in flight below
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    nb::dfree(out);
    if (e != cudaSuccess) return cuda_error(e, "probe_fma");
    // 16 lane-FMAs per thread per iteration either way, 2 FLOP each
    *flops = 2.0 * 16.0 * (double)iters * (double)grid * 256.0;
    return NB_OK;
}

}  // namespace nb
