// nb_adjoint.cu -- reverse-mode (adjoint) kernels of the nbody step.
//
// No counterpart in the reference (it has no gradients).  The forward step is
// the reference's update (benchapps/nbody/seq/bodysystem.cc:135-182):
//   a_i = sum_j m_j r_ij inv_ij^3,  r_ij = x_j - x_i, inv = (|r|^2+eps2)^-1/2
//   v'  = D (v + k a dt),            k_i = m_i (reference kick) or G
//   x'  = x + v' dt
// Given lx = dL/dx', lv = dL/dv' the step's vector-Jacobian product is
//   mu = lv + dt lx,  dL/dv = D mu,  g_i = D dt k_i mu_i
//   dL/dx_k = lx_k + sum_j K(r_kj) (m_k g_j - m_j g_k),
//             K(r) = inv^3 I - 3 inv^5 r r^T
//   dL/dm_k += -sum_j inv^3 (r_kj . g_j) [through a]
//              + D dt mu_k . a_k          [through k, reference kick only]
// The pair sum is evaluated as
//   out_k = m_k P - q g_k - 3 Q,  P = sum inv^3 g_j,  q = sum inv^3 m_j,
//   Q = sum inv^5 (m_k (r.g_j) - m_j (r.g_k)) r
// (26 FP32 operations and one rsqrt per pair), split stream-K over
// persistent CTAs like the forward force kernel; each CTA segment writes
// (out, dm) to its partial slot and the update kernel sums them in CTA order.
//
// The pair term of out is antisymmetric: with r = x_j - x_k,
//   T_kj = m_k inv^3 g_j - m_j inv^3 g_k - 3 inv^5 (m_k r.g_j - m_j r.g_k) r
// and T_jk = -T_kj, while the mass terms are -inv^3 r.g_j on k and
// +inv^3 r.g_k on j.  sym_vjp_kernel therefore evaluates each unordered pair
// once on the forward symmetric kernel's layout (row blocks x 32-body
// chunks, the chunk rotating through the warp with its accumulated reaction):
// 18 shared operations + 8 per side = 34 FP32 operations and one rsqrt per
// pair, 17 per ordered interaction instead of 26.
#include "nb_internal.cuh"

namespace nb {

template <int NT, int BPT>
__global__ void __launch_bounds__(NT) vjp_pair_kernel(const float4 *__restrict__ pos,
                                                      const float4 *__restrict__ gbuf, int n,
                                                      float eps2, float4 *__restrict__ partial,
                                                      long long total, int ngroups)
{
    constexpr int TB = NT * BPT;
    __shared__ __align__(16) float4 sP[NT];
    __shared__ __align__(16) float4 sG[NT];
    const int t = threadIdx.x;
    const int c = blockIdx.x;
    long long it = sk_start(c, total, gridDim.x);
    const long long end = sk_start(c + 1, total, gridDim.x);
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);

    while (it < end) {
        const int tb = (int)(it / ngroups);
        const long long tb_first = (long long)tb * ngroups;
        const long long seg_end = end < tb_first + ngroups ? end : tb_first + ngroups;
        const int j0 = (int)(it - tb_first) * kGroup;
        const int j1 = min((int)(seg_end - tb_first) * kGroup, n);

        float px[BPT], py[BPT], pz[BPT], pm[BPT], gx[BPT], gy[BPT], gz[BPT];
        float Px[BPT], Py[BPT], Pz[BPT], Q0[BPT], Q1[BPT], Q2[BPT], q[BPT], dm[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tb * TB + t + k * NT;
            const float4 a = i < n ? pos[i] : zero;
            const float4 g = i < n ? gbuf[i] : zero;
            px[k] = a.x; py[k] = a.y; pz[k] = a.z; pm[k] = a.w;
            gx[k] = g.x; gy[k] = g.y; gz[k] = g.z;
            Px[k] = Py[k] = Pz[k] = Q0[k] = Q1[k] = Q2[k] = q[k] = dm[k] = 0.f;
        }
        float4 nxp = (j0 + t < j1) ? pos[j0 + t] : pad;
        float4 nxg = (j0 + t < j1) ? gbuf[j0 + t] : zero;
        for (int jt = j0; jt < j1; jt += NT) {
            __syncthreads();
            sP[t] = nxp;
            sG[t] = nxg;
            __syncthreads();
            if (jt + NT < j1) {
                const int jn = jt + NT + t;
                nxp = jn < j1 ? pos[jn] : pad;
                nxg = jn < j1 ? gbuf[jn] : zero;
            }
            const int cnt = min(NT, j1 - jt);
            const int cnt2 = (cnt + 1) & ~1;  // entries past cnt are zero-mass, zero-g pads
            for (int j = 0; j < cnt2; j += 2) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float4 s = sP[j + u];
                    const float4 g = sG[j + u];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = s.x - px[k], ry = s.y - py[k], rz = s.z - pz[k];
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
                        q[k] = fmaf(inv3, s.w, q[k]);
                        const float rgj = fmaf(rz, g.z, fmaf(ry, g.y, rx * g.x));
                        const float rgk = fmaf(rz, gz[k], fmaf(ry, gy[k], rx * gx[k]));
                        const float cc = inv5 * fmaf(pm[k], rgj, -(s.w * rgk));
                        Q0[k] = fmaf(cc, rx, Q0[k]);
                        Q1[k] = fmaf(cc, ry, Q1[k]);
                        Q2[k] = fmaf(cc, rz, Q2[k]);
                        dm[k] = fmaf(inv3, rgj, dm[k]);
                    }
                }
            }
        }
        float4 *dst = partial + (size_t)(c + tb) * TB;
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const float ox = fmaf(pm[k], Px[k], fmaf(-q[k], gx[k], -3.f * Q0[k]));
            const float oy = fmaf(pm[k], Py[k], fmaf(-q[k], gy[k], -3.f * Q1[k]));
            const float oz = fmaf(pm[k], Pz[k], fmaf(-q[k], gz[k], -3.f * Q2[k]));
            dst[t + k * NT] = make_float4(ox, oy, oz, -dm[k]);
        }
        it = seg_end;
    }
}

template <int W, int BPT, int MINB, int U = 2>
__global__ void __launch_bounds__(32 * W, MINB) sym_vjp_kernel(const float4 *__restrict__ pos,
                                                               const float4 *__restrict__ gbuf, int n,
                                                               float eps2, float4 *__restrict__ tpart,
                                                               float4 *__restrict__ spart,
                                                               long long total, int nc, int nrb)
{
    constexpr int WB = 32 * BPT;
    constexpr int RB = W * WB;
    constexpr int RC = RB / 32;
    __shared__ __align__(16) float4 sC[32];
    __shared__ __align__(16) float4 sG[32];
    __shared__ float sF[8][W][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int c = blockIdx.x;
    long long it = sk_start(c, total, gridDim.x);
    const long long end = sk_start(c + 1, total, gridDim.x);
    const float4 pad = make_float4(kPadCoord, kPadCoord, kPadCoord, 0.f);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);

    while (it < end) {
        const int I = sym_row_of(it, nc, RC, nrb);
        const long long rfirst = sym_prefix(I, nc, RC);
        const long long rend = sym_prefix(I + 1, nc, RC);
        const long long seg_end = end < rend ? end : rend;
        const int kc0 = I * RC + (int)(it - rfirst);
        const int kc1 = I * RC + (int)(seg_end - rfirst);
        const int tbase = I * RB + wid * WB;

        // missing targets: zero mass and zero g, so every term they give is 0
        float px[BPT], py[BPT], pz[BPT], pm[BPT], gx[BPT], gy[BPT], gz[BPT];
        float Px[BPT], Py[BPT], Pz[BPT], Q0[BPT], Q1[BPT], Q2[BPT], q[BPT], dm[BPT];
#pragma unroll
        for (int k = 0; k < BPT; ++k) {
            const int i = tbase + lane + 32 * k;
            const float4 a = i < n ? pos[i] : zero;
            const float4 g = i < n ? gbuf[i] : zero;
            px[k] = a.x; py[k] = a.y; pz[k] = a.z; pm[k] = a.w;
            gx[k] = g.x; gy[k] = g.y; gz[k] = g.z;
            Px[k] = Py[k] = Pz[k] = Q0[k] = Q1[k] = Q2[k] = q[k] = dm[k] = 0.f;
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            const int jb = kc * 32;
            __syncthreads();  // previous chunk: sC/sG and sF reads are done
            if (wid == 0) {
                sC[lane] = (jb + lane < n) ? pos[jb + lane] : pad;
                sG[lane] = (jb + lane < n) ? gbuf[jb + lane] : zero;
            }
            __syncthreads();
            if (kc < (I + 1) * RC) {
                // chunk inside the own row block: directed, target side only
#pragma unroll 2
                for (int j = 0; j < 32; ++j) {
                    const float4 s = sC[j];
                    const float4 g = sG[j];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = s.x - px[k], ry = s.y - py[k], rz = s.z - pz[k];
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
                        q[k] = fmaf(inv3, s.w, q[k]);
                        const float rgj = fmaf(rz, g.z, fmaf(ry, g.y, rx * g.x));
                        const float rgk = fmaf(rz, gz[k], fmaf(ry, gy[k], rx * gx[k]));
                        const float cc = inv5 * fmaf(pm[k], rgj, -(s.w * rgk));
                        Q0[k] = fmaf(cc, rx, Q0[k]);
                        Q1[k] = fmaf(cc, ry, Q1[k]);
                        Q2[k] = fmaf(cc, rz, Q2[k]);
                        dm[k] = fmaf(inv3, rgj, dm[k]);
                    }
                }
            } else {
                // reaction on the rotating chunk body: P, q, Q of its own sum
                // and its mass gradient w = sum inv^3 r.g_k
                float rPx = 0.f, rPy = 0.f, rPz = 0.f, rq = 0.f, rQ0 = 0.f, rQ1 = 0.f, rQ2 = 0.f, rw = 0.f;
#pragma unroll(U)
                for (int r = 0; r < 32; ++r) {
                    const int idx = (lane + r) & 31;
                    const float4 s = sC[idx];
                    const float4 g = sG[idx];
#pragma unroll
                    for (int k = 0; k < BPT; ++k) {
                        const float rx = s.x - px[k], ry = s.y - py[k], rz = s.z - pz[k];
                        float d2 = fmaf(rx, rx, eps2);
                        d2 = fmaf(ry, ry, d2);
                        d2 = fmaf(rz, rz, d2);
                        const float inv = rsqrt_approx(d2);
                        const float inv2 = inv * inv;
                        const float inv3 = inv2 * inv;
                        const float inv5 = inv3 * inv2;
                        const float rgj = fmaf(rz, g.z, fmaf(ry, g.y, rx * g.x));
                        const float rgk = fmaf(rz, gz[k], fmaf(ry, gy[k], rx * gx[k]));
                        const float cc = inv5 * fmaf(pm[k], rgj, -(s.w * rgk));
                        Px[k] = fmaf(inv3, g.x, Px[k]);
                        Py[k] = fmaf(inv3, g.y, Py[k]);
                        Pz[k] = fmaf(inv3, g.z, Pz[k]);
                        q[k] = fmaf(inv3, s.w, q[k]);
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
                // lane l now holds chunk body l's reaction from this warp
                if (W > 1) {
                    sF[0][wid][lane] = rPx;
                    sF[1][wid][lane] = rPy;
                    sF[2][wid][lane] = rPz;
                    sF[3][wid][lane] = rq;
                    sF[4][wid][lane] = rQ0;
                    sF[5][wid][lane] = rQ1;
                    sF[6][wid][lane] = rQ2;
                    sF[7][wid][lane] = rw;
                    __syncthreads();
                    if (wid == 0) {
                        rPx = rPy = rPz = rq = rQ0 = rQ1 = rQ2 = rw = 0.f;
#pragma unroll
                        for (int w = 0; w < W; ++w) {
                            rPx += sF[0][w][lane];
                            rPy += sF[1][w][lane];
                            rPz += sF[2][w][lane];
                            rq += sF[3][w][lane];
                            rQ0 += sF[4][w][lane];
                            rQ1 += sF[5][w][lane];
                            rQ2 += sF[6][w][lane];
                            rw += sF[7][w][lane];
                        }
                    }
                }
                if (wid == 0 && jb + lane < n) {
                    const float4 sb = sC[lane], gb = sG[lane];
                    const float ox = fmaf(sb.w, rPx, fmaf(-rq, gb.x, -3.f * rQ0));
                    const float oy = fmaf(sb.w, rPy, fmaf(-rq, gb.y, -3.f * rQ1));
                    const float oz = fmaf(sb.w, rPz, fmaf(-rq, gb.z, -3.f * rQ2));
                    spart[sym_soff(I, n, RB) + (jb + lane - (I + 1) * RB)] = make_float4(ox, oy, oz, rw);
                }
            }
        }
        float4 *dst = tpart + (size_t)(c + I) * RB + wid * WB;
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

// g_i = D dt k_i (lv_i + dt lx_i) for the first reverse step.
__global__ void adj_g_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ lx,
                             const float4 *__restrict__ lv, float4 *__restrict__ gbuf, int n,
                             float damping, float dt, int kick, float G)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float k = kick == NB_KICK_REFERENCE ? pos[i].w : G;
    const float4 x = lx[i], v = lv[i];
    const float f = damping * dt * k;
    gbuf[i] = make_float4(f * fmaf(dt, x.x, v.x), f * fmaf(dt, x.y, v.y), f * fmaf(dt, x.z, v.z), 0.f);
}

// Directed layout: sum the partial slots of the CTAs that covered the body's
// target block (CTA order), then update.
__global__ void adj_update_kernel(const float4 *__restrict__ partial, int n, int tbsize,
                                  long long total, int ngroups, int grid,
                                  const float4 *__restrict__ pos, const float4 *__restrict__ acc,
                                  float4 *__restrict__ lx, float4 *__restrict__ lv,
                                  float *__restrict__ gm, float4 *__restrict__ gbuf, float damping,
                                  float dt, int kick, float G, int want_next_g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int tb = i / tbsize;
    const int li = i - tb * tbsize;
    const long long first = (long long)tb * ngroups;
    const int c0 = sk_owner(first, total, grid);
    const int c1 = sk_owner(first + ngroups - 1, total, grid);
    float ox = 0.f, oy = 0.f, oz = 0.f, odm = 0.f;
    for (int c = c0; c <= c1; ++c) {
        const float4 q = partial[(size_t)(c + tb) * tbsize + li];
        ox += q.x;
        oy += q.y;
        oz += q.z;
        odm += q.w;
    }
    adj_body_update(i, ox, oy, oz, odm, pos, acc, lx, lv, gm, gbuf, damping, dt, kick, G, want_next_g);
}

// Symmetric layout: target-side slots and the source-side entries of rows
// 0..I-1, then the per-body update.  Four threads share a body (thread q of
// the quad sums slots c0+q, c0+q+4, ... and rows q, q+4, ..., the quad
// combines its sums as (s0 + s1) + (s2 + s3), a fixed order): the row walk of
// the last row blocks is what bounds this kernel.
constexpr int kAdjUpdBlock = 256;

__global__ void __launch_bounds__(kAdjUpdBlock) adj_update_sym_kernel(
    const float4 *__restrict__ tpart, const float4 *__restrict__ spart, int n, int rb, int nc, int nrb,
    long long total, int grid, const float4 *__restrict__ pos, const float4 *__restrict__ acc,
    float4 *__restrict__ lx, float4 *__restrict__ lv, float *__restrict__ gm, float4 *__restrict__ gbuf,
    float damping, float dt, int kick, float G, int want_next_g)
{
    // bodies from the last one down, as in sym_integrate_kernel: the blocks
    // with the longest row walks start first
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = n - 1 - (int)(t >> 2), q = (int)(t & 3);
    const bool live = i >= 0;  // dead threads still take part in the shuffles
    float ox = 0.f, oy = 0.f, oz = 0.f, odm = 0.f;
    if (live) {
        const int rc = rb / 32;
        const int I = i / rb;
        const int c0 = sk_owner(sym_prefix(I, nc, rc), total, grid);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1, total, grid);
        const int li = i - I * rb;
        for (int c = c0 + q; c <= c1; c += 4) {
            const float4 v4 = tpart[(size_t)(c + I) * rb + li];
            ox += v4.x;
            oy += v4.y;
            oz += v4.z;
            odm += v4.w;
        }
#pragma unroll 4
        for (int r = q; r < I; r += 4) {
            const float4 v4 = spart[sym_soff(r, n, rb) + (i - (long long)(r + 1) * rb)];
            ox += v4.x;
            oy += v4.y;
            oz += v4.z;
            odm += v4.w;
        }
    }
#pragma unroll
    for (int m = 1; m <= 2; m <<= 1) {
        ox += __shfl_xor_sync(0xffffffffu, ox, m);
        oy += __shfl_xor_sync(0xffffffffu, oy, m);
        oz += __shfl_xor_sync(0xffffffffu, oz, m);
        odm += __shfl_xor_sync(0xffffffffu, odm, m);
    }
    if (!live || q != 0) return;
    adj_body_update(i, ox, oy, oz, odm, pos, acc, lx, lv, gm, gbuf, damping, dt, kick, G, want_next_g);
}

typedef void (*vjp_kernel_t)(const float4 *, const float4 *, int, float, float4 *, long long, int);

static vjp_kernel_t vjp_kernel_for(int block, int bpt)
{
    if (block == 128 && bpt == 2) return vjp_pair_kernel<128, 2>;
    if (block == 128 && bpt == 4) return vjp_pair_kernel<128, 4>;
    if (block == 256 && bpt == 2) return vjp_pair_kernel<256, 2>;
    if (block == 256 && bpt == 4) return vjp_pair_kernel<256, 4>;
    return nullptr;
}

int adj_plan(int n, int block, int bpt, int device, SkPlan *pl)
{
    if (block == 0) block = 256;
    if (bpt == 0) bpt = 4;
    vjp_kernel_t k = vjp_kernel_for(block, bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "adjoint kernel shape not compiled");
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
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "adjoint kernel does not fit on an SM");
    long long grid = (long long)sms * occ;
    if (p.total > 0 && grid > p.total) grid = p.total;
    p.grid = p.total > 0 ? (int)grid : 0;
    p.slots = p.total > 0 ? p.grid + p.ntb - 1 : 0;
    *pl = p;
    return NB_OK;
}

int adj_g(int n, const float4 *pos, const float4 *lx, const float4 *lv, float4 *gbuf, float damping,
          float dt, int kick, float G, cudaStream_t s)
{
    if (n == 0) return NB_OK;
    adj_g_kernel<<<(n + 255) / 256, 256, 0, s>>>(pos, lx, lv, gbuf, n, damping, dt, kick, G);
    NB_LAUNCH_CHECK("adj_g_kernel launch");
    return NB_OK;
}

int adj_vjp(const SkPlan &p, const float4 *pos, const float4 *gbuf, float eps2, float4 *partial,
            cudaStream_t s)
{
    if (p.total == 0) return NB_OK;
    vjp_kernel_t k = vjp_kernel_for(p.block, p.tbsize / p.block);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "adjoint kernel shape not compiled");
    k<<<p.grid, p.block, 0, s>>>(pos, gbuf, p.n, eps2, partial, p.total, p.ngroups);
    NB_LAUNCH_CHECK("vjp_pair_kernel launch");
    return NB_OK;
}

int adj_update(const SkPlan &p, const float4 *partial, const float4 *pos_prev, const float4 *acc,
               float4 *lx, float4 *lv, float *gm, float4 *gbuf, float damping, float dt, int kick,
               float G, int want_next_g, cudaStream_t s)
{
    if (p.n == 0) return NB_OK;
    adj_update_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(partial, p.n, p.tbsize, p.total, p.ngroups,
                                                       p.grid, pos_prev, acc, lx, lv, gm, gbuf,
                                                       damping, dt, kick, G, want_next_g);
    NB_LAUNCH_CHECK("adj_update_kernel launch");
    return NB_OK;
}

typedef void (*sym_vjp_kernel_t)(const float4 *, const float4 *, int, float, float4 *, float4 *,
                                 long long, int, int);

static sym_vjp_kernel_t sym_vjp_kernel_for(int w, int bpt)
{
    if (w == 1 && bpt == 10) return sym_vjp_kernel<1, 10, 8>;
    if (w == 1 && bpt == 8) return sym_vjp_kernel<1, 8, 8>;
    if (w == 1 && bpt == 12) return sym_vjp_kernel<1, 12, 8>;
    if (w == 4 && bpt == 8) return sym_vjp_kernel<4, 8, 2>;
    if (w == 8 && bpt == 8) return sym_vjp_kernel<8, 8, 1>;
    return nullptr;
}

int sym_vjp_plan(int n, int warps, int bpt, int device, SymPlan *pl)
{
    if (warps == 0 && bpt == 0) {
        // one-warp CTAs x 10 targets (row block 320; the fastest of the
        // shapes timed on GB300 at N = 16384 and 65536), then 4 x 8 (1024),
        // 8 x 8 (2048) while the source-side array is over budget
        static const int shapes[3][2] = {{1, 10}, {4, 8}, {8, 8}};
        int s = 0;
        while (s < 2 && sym_spart_entries(n, shapes[s][0] * 32 * shapes[s][1]) * (long long)sizeof(float4) >
                            kSymSpartBudget)
            ++s;
        warps = shapes[s][0];
        bpt = shapes[s][1];
    }
    sym_vjp_kernel_t k = sym_vjp_kernel_for(warps, bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "symmetric adjoint kernel shape not compiled");
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
    if (occ < 1) return set_error(NB_ERR_UNSUPPORTED, "symmetric adjoint kernel does not fit on an SM");
    long long grid = (long long)sms * occ;
    if (p.total > 0 && grid > p.total) grid = p.total;
    p.grid = p.total > 0 ? (int)grid : 0;
    p.slots = p.total > 0 ? p.grid + p.nrb - 1 : 0;
    p.spart_size = sym_spart_entries(n, p.rb);
    *pl = p;
    return NB_OK;
}

int sym_vjp(const SymPlan &p, const float4 *pos, const float4 *gbuf, float eps2, float4 *tpart,
            float4 *spart, cudaStream_t s)
{
    if (p.total == 0) return NB_OK;
    sym_vjp_kernel_t k = sym_vjp_kernel_for(p.warps, p.bpt);
    if (!k) return set_error(NB_ERR_UNSUPPORTED, "symmetric adjoint kernel shape not compiled");
    k<<<p.grid, 32 * p.warps, 0, s>>>(pos, gbuf, p.n, eps2, tpart, spart, p.total, p.nc, p.nrb);
    NB_LAUNCH_CHECK("sym_vjp_kernel launch");
    return NB_OK;
}

int adj_update_sym(const SymPlan &p, const float4 *tpart, const float4 *spart, const float4 *pos_prev,
                   const float4 *acc, float4 *lx, float4 *lv, float *gm, float4 *gbuf, float damping,
                   float dt, int kick, float G, int want_next_g, cudaStream_t s)
{
    if (p.n == 0) return NB_OK;
    const long long threads = 4ll * p.n;  // a quad of threads per body
    adj_update_sym_kernel<<<(unsigned)((threads + kAdjUpdBlock - 1) / kAdjUpdBlock), kAdjUpdBlock, 0, s>>>(
        tpart, spart, p.n, p.rb, p.nc, p.nrb, p.total, p.grid, pos_prev, acc, lx, lv, gm, gbuf, damping, dt,
        kick, G, want_next_g);
    NB_LAUNCH_CHECK("adj_update_sym_kernel launch");
    return NB_OK;
}

}  // namespace nb
