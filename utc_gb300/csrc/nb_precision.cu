// nb_precision.cu -- compensated FP32 mode with FP64 positions, the force /
// potential reduction, and the FP64 energy and momentum reduction.
//
// State of an NB_F32_COMP context:
//   pos64   double4 (x, y, z, m)   absolute positions, updated in FP64
//   pos32   float4                 working copy read by the force kernel
//   vel_hi  float4 (vx, vy, vz, w) velocity, FP32
//   vel_lo  float4                 its compensation term (v = hi + lo)
// Pair forces are FP32 (the fast kernel with SK_COMP: per-tile partial sums
// folded into a two-sum (hi, lo) pair, partial slots carry both).  FP64 is
// used on the GPU only for the absolute-position update and for the energy
// and momentum reduction.
#include "nb_internal.cuh"

namespace nb {

// host double4 state -> pos64, pos32, vel_hi, vel_lo
__global__ void comp_split_kernel(const double4 *__restrict__ pin, const double4 *__restrict__ vin,
                                  double4 *__restrict__ pos64, float4 *__restrict__ pos32,
                                  float4 *__restrict__ vhi, float4 *__restrict__ vlo, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4 p = pin[i];
    const double4 v = vin[i];
    pos64[i] = p;
    pos32[i] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
    const float hx = (float)v.x, hy = (float)v.y, hz = (float)v.z;
    vhi[i] = make_float4(hx, hy, hz, (float)v.w);
    vlo[i] = make_float4((float)(v.x - hx), (float)(v.y - hy), (float)(v.z - hz), 0.f);
}

// pos64, vel_hi + vel_lo -> double4 state
__global__ void comp_join_kernel(const double4 *__restrict__ pos64, const float4 *__restrict__ vhi,
                                 const float4 *__restrict__ vlo, double4 *__restrict__ pout,
                                 double4 *__restrict__ vout, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (pout) pout[i] = pos64[i];
    if (vout) {
        const float4 h = vhi[i], l = vlo[i];
        vout[i] = make_double4((double)h.x + (double)l.x, (double)h.y + (double)l.y,
                               (double)h.z + (double)l.z, (double)h.w);
    }
}

// Compensated sum of a target's partial slots (hi and lo blocks).
__device__ __forceinline__ void comp_slot_sum(const float4 *__restrict__ partial, long long lo_off,
                                              int tb, int li, int tbsize, long long total,
                                              int ngroups, int grid, float4 &S, float4 &C)
{
    const long long first = (long long)tb * ngroups;
    const int c0 = sk_owner(first, total, grid);
    const int c1 = sk_owner(first + ngroups - 1, total, grid);
    S = make_float4(0.f, 0.f, 0.f, 0.f);
    C = S;
    for (int c = c0; c <= c1; ++c) {
        const size_t k = (size_t)(c + tb) * tbsize + li;
        const float4 h = partial[k];
        const float4 l = partial[lo_off + k];
        float e;
        two_sum(S.x, h.x, S.x, e); C.x = __fadd_rn(C.x, __fadd_rn(e, l.x));
        two_sum(S.y, h.y, S.y, e); C.y = __fadd_rn(C.y, __fadd_rn(e, l.y));
        two_sum(S.z, h.z, S.z, e); C.z = __fadd_rn(C.z, __fadd_rn(e, l.z));
        two_sum(S.w, h.w, S.w, e); C.w = __fadd_rn(C.w, __fadd_rn(e, l.w));
    }
}

// Bare accelerations of every target, and in w the potential sum over
// j != i: the force pass sums j == i too (its term is m_i * rsqrt(eps2),
// computed here exactly as the pass computed it) and it is taken out here.
// Plain slots: float4 out; compensated slots: double4 out = hi + lo.
__global__ void sk_reduce_kernel(const float4 *__restrict__ partial, int n, int tbsize,
                                 long long total, int ngroups, int grid, long long lo_off,
                                 int comp, const float4 *__restrict__ pos32, float eps2,
                                 float4 *__restrict__ out32, double4 *__restrict__ out64)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int tb = i / tbsize;
    const int li = i - tb * tbsize;
    const float self = __fmul_rn(pos32[i].w, rsqrt_approx(eps2));
    if (comp) {
        float4 S, C;
        comp_slot_sum(partial, lo_off, tb, li, tbsize, total, ngroups, grid, S, C);
        out64[i] = make_double4((double)S.x + (double)C.x, (double)S.y + (double)C.y,
                                (double)S.z + (double)C.z,
                                ((double)S.w - (double)self) + (double)C.w);
        return;
    }
    const long long first = (long long)tb * ngroups;
    const int c0 = sk_owner(first, total, grid);
    const int c1 = sk_owner(first + ngroups - 1, total, grid);
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int c = c0; c <= c1; ++c) {
        const float4 q = partial[(size_t)(c + tb) * tbsize + li];
        a.x = __fadd_rn(a.x, q.x);
        a.y = __fadd_rn(a.y, q.y);
        a.z = __fadd_rn(a.z, q.z);
        a.w = __fadd_rn(a.w, q.w);
    }
    a.w = __fsub_rn(a.w, self);
    out32[i] = a;
}

// Compensated kick / damping (FP32 with a carried low part) and FP64 drift,
// given the acceleration as a compensated sum S + C.
__device__ __forceinline__ void comp_kick_drift(int i, float4 S, float4 C, double4 *__restrict__ pos64,
                                                float4 *__restrict__ pos32, float4 *__restrict__ vhi,
                                                float4 *__restrict__ vlo, float damping, float dt,
                                                double dt64, int kick, float G)
{
    const float ax = __fadd_rn(S.x, C.x), ay = __fadd_rn(S.y, C.y), az = __fadd_rn(S.z, C.z);
    double4 p = pos64[i];
    float4 h = vhi[i], l = vlo[i];
    const float k = kick == NB_KICK_REFERENCE ? (float)p.w : G;
    float e;
    two_sum(h.x, __fmul_rn(__fmul_rn(ax, k), dt), h.x, e); l.x = __fadd_rn(l.x, e);
    two_sum(h.y, __fmul_rn(__fmul_rn(ay, k), dt), h.y, e); l.y = __fadd_rn(l.y, e);
    two_sum(h.z, __fmul_rn(__fmul_rn(az, k), dt), h.z, e); l.z = __fadd_rn(l.z, e);
    if (damping != 1.0f) {
        h.x = __fmul_rn(h.x, damping); l.x = __fmul_rn(l.x, damping);
        h.y = __fmul_rn(h.y, damping); l.y = __fmul_rn(l.y, damping);
        h.z = __fmul_rn(h.z, damping); l.z = __fmul_rn(l.z, damping);
    }
    // renormalise (|h| >= |l|): fast two-sum
    float s;
    s = __fadd_rn(h.x, l.x); l.x = __fsub_rn(l.x, __fsub_rn(s, h.x)); h.x = s;
    s = __fadd_rn(h.y, l.y); l.y = __fsub_rn(l.y, __fsub_rn(s, h.y)); h.y = s;
    s = __fadd_rn(h.z, l.z); l.z = __fsub_rn(l.z, __fsub_rn(s, h.z)); h.z = s;
    // FP64 absolute-position update
    p.x = fma((double)h.x + (double)l.x, dt64, p.x);
    p.y = fma((double)h.y + (double)l.y, dt64, p.y);
    p.z = fma((double)h.z + (double)l.z, dt64, p.z);
    pos64[i] = p;
    pos32[i] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
    vhi[i] = h;
    vlo[i] = l;
}

__global__ void comp_integrate_kernel(const float4 *__restrict__ partial, int n, int tbsize,
                                      long long total, int ngroups, int grid, long long lo_off,
                                      double4 *__restrict__ pos64, float4 *__restrict__ pos32,
                                      float4 *__restrict__ vhi, float4 *__restrict__ vlo,
                                      float damping, float dt, double dt64, int kick, float G)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int tb = i / tbsize;
    const int li = i - tb * tbsize;
    float4 S, C;
    comp_slot_sum(partial, lo_off, tb, li, tbsize, total, ngroups, grid, S, C);
    comp_kick_drift(i, S, C, pos64, pos32, vhi, vlo, damping, dt, dt64, kick, G);
}

// Compensated symmetric partials: the target-side slots (CTA order) and the
// source-side rows 0..I-1 (row order), hi and lo halves, summed with
// two-sums; then the compensated kick / drift, or (acc_out != nullptr) the
// bare acceleration hi + lo in FP64.
__global__ void sym_comp_integrate_kernel(const float4 *__restrict__ tpart, const float4 *__restrict__ spart,
                                          long long tlo, long long slo, int n, int rb, int nc, int nrb,
                                          long long total, int grid, double4 *__restrict__ pos64,
                                          float4 *__restrict__ pos32, float4 *__restrict__ vhi,
                                          float4 *__restrict__ vlo, float damping, float dt,
                                          double dt64, int kick, float G, double4 *__restrict__ acc_out,
                                          const float4 *__restrict__ accsum)
{
    // bodies from the last one down: the longest row walks start first
    const int i = n - 1 - (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < 0) return;
    float4 S = make_float4(0.f, 0.f, 0.f, 0.f), C = S;
    if (accsum) {  // banded plan: the compensated fold's (S, C)
        S = accsum[i];
        C = accsum[(size_t)n + i];
    } else {
        const int rc = rb / 32;
        const int I = i / rb;
        const int c0 = sk_owner(sym_prefix(I, nc, rc), total, grid);
        const int c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1, total, grid);
        const int li = i - I * rb;
        float e;
        auto add = [&](const float4 h, const float4 l) {
            two_sum(S.x, h.x, S.x, e); C.x = __fadd_rn(C.x, __fadd_rn(e, l.x));
            two_sum(S.y, h.y, S.y, e); C.y = __fadd_rn(C.y, __fadd_rn(e, l.y));
            two_sum(S.z, h.z, S.z, e); C.z = __fadd_rn(C.z, __fadd_rn(e, l.z));
        };
        for (int c = c0; c <= c1; ++c) {
            const size_t k = (size_t)(c + I) * rb + li;
            add(tpart[k], tpart[tlo + k]);
        }
        long long off = (long long)i - rb;  // row r at soff(r) + i - (r + 1) rb
        for (int r = 0; r < I; ++r) {
            add(spart[off], spart[slo + off]);
            off += (long long)n - (long long)(r + 2) * rb;
        }
    }
    if (acc_out) {
        acc_out[i] = make_double4((double)S.x + (double)C.x, (double)S.y + (double)C.y,
                                  (double)S.z + (double)C.z, 0.0);
        return;
    }
    comp_kick_drift(i, S, C, pos64, pos32, vhi, vlo, damping, dt, dt64, kick, G);
}

// Energy and momentum, FP64 reduction.  Per body: kinetic 0.5 m |v|^2,
// potential -0.5 G m phi (phi over j != i, from sk_reduce_kernel), momentum
// m v.  Block partials, then one block sums them in index order
// (deterministic).
constexpr int kEnergyBlock = 256;

__global__ void energy_partial_kernel(int n, const float4 *__restrict__ pos32,
                                      const double4 *__restrict__ pos64,
                                      const float4 *__restrict__ vel32,
                                      const float4 *__restrict__ vlo,
                                      const float4 *__restrict__ phi32,
                                      const double4 *__restrict__ phi64, double G,
                                      double *__restrict__ block_out,
                                      const double4 *__restrict__ vel64)
{
    __shared__ double red[5][kEnergyBlock];
    const int i = blockIdx.x * kEnergyBlock + threadIdx.x;
    double ke = 0, pe = 0, px = 0, py = 0, pz = 0;
    if (i < n) {
        const double m = pos64 ? pos64[i].w : (double)pos32[i].w;
        double vx, vy, vz;
        if (vel64) {
            vx = vel64[i].x;
            vy = vel64[i].y;
            vz = vel64[i].z;
        } else {
            vx = vel32[i].x;
            vy = vel32[i].y;
            vz = vel32[i].z;
        }
        if (vlo) {
            vx += (double)vlo[i].x;
            vy += (double)vlo[i].y;
            vz += (double)vlo[i].z;
        }
        const double phi = phi64 ? phi64[i].w : (double)phi32[i].w;
        ke = 0.5 * m * (vx * vx + vy * vy + vz * vz);
        pe = -0.5 * G * m * phi;
        px = m * vx;
        py = m * vy;
        pz = m * vz;
    }
    red[0][threadIdx.x] = ke;
    red[1][threadIdx.x] = pe;
    red[2][threadIdx.x] = px;
    red[3][threadIdx.x] = py;
    red[4][threadIdx.x] = pz;
    __syncthreads();
    for (int w = kEnergyBlock / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int q = 0; q < 5; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 5) block_out[(size_t)blockIdx.x * 5 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void energy_final_kernel(const double *__restrict__ block_out, int nblocks,
                                    double *__restrict__ out)
{
    if (threadIdx.x >= 5) return;
    double s = 0;
    for (int b = 0; b < nblocks; ++b) s += block_out[(size_t)b * 5 + threadIdx.x];
    out[threadIdx.x] = s;
}

int comp_split(const double4 *pin, const double4 *vin, double4 *pos64, float4 *pos32,
               float4 *vhi, float4 *vlo, int n, cudaStream_t s)
{
    if (n == 0) return NB_OK;
    comp_split_kernel<<<(n + 255) / 256, 256, 0, s>>>(pin, vin, pos64, pos32, vhi, vlo, n);
    NB_LAUNCH_CHECK("comp_split_kernel launch");
    return NB_OK;
}

int comp_join(const double4 *pos64, const float4 *vhi, const float4 *vlo, double4 *pout,
              double4 *vout, int n, cudaStream_t s)
{
    if (n == 0) return NB_OK;
    comp_join_kernel<<<(n + 255) / 256, 256, 0, s>>>(pos64, vhi, vlo, pout, vout, n);
    NB_LAUNCH_CHECK("comp_join_kernel launch");
    return NB_OK;
}

int fast_reduce(const SkPlan &p, const float4 *partial, int comp, const float4 *pos32, float eps2,
                float4 *out32, double4 *out64, cudaStream_t s)
{
    if (p.n == 0) return NB_OK;
    const long long lo_off = (long long)p.slots * p.tbsize;
    sk_reduce_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(partial, p.n, p.tbsize, p.total, p.ngroups,
                                                      p.grid, lo_off, comp, pos32, eps2, out32,
                                                      out64);
    NB_LAUNCH_CHECK("sk_reduce_kernel launch");
    return NB_OK;
}

int comp_integrate(const SkPlan &p, const float4 *partial, double4 *pos64, float4 *pos32,
                   float4 *vhi, float4 *vlo, float damping, float dt, double dt64, int kick,
                   float G, cudaStream_t s)
{
    if (p.n == 0) return NB_OK;
    const long long lo_off = (long long)p.slots * p.tbsize;
    comp_integrate_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(partial, p.n, p.tbsize, p.total,
                                                           p.ngroups, p.grid, lo_off, pos64, pos32,
                                                           vhi, vlo, damping, dt, dt64, kick, G);
    NB_LAUNCH_CHECK("comp_integrate_kernel launch");
    return NB_OK;
}

int sym_comp_integrate(const SymPlan &p, const float4 *tpart, const float4 *spart, double4 *pos64,
                       float4 *pos32, float4 *vhi, float4 *vlo, float damping, float dt,
                       double dt64, int kick, float G, double4 *acc_out, cudaStream_t s, const float4 *accsum)
{
    if (p.n == 0) return NB_OK;
    if (!p.comp) return set_error(NB_ERR_INVALID, "sym_comp_integrate needs a compensated plan");
    if (p.nbands > 1 && !accsum) return set_error(NB_ERR_INVALID, "sym_comp_integrate: a banded plan needs its sums");
    sym_comp_integrate_kernel<<<(p.n + 255) / 256, 256, 0, s>>>(
        tpart, spart, (long long)p.slots * p.rb, p.spart_size, p.n, p.rb, p.nc, p.nrb, p.total,
        p.grid, pos64, pos32, vhi, vlo, damping, dt, dt64, kick, G, acc_out, p.nbands > 1 ? accsum : nullptr);
    NB_LAUNCH_CHECK("sym_comp_integrate_kernel launch");
    return NB_OK;
}

int energy_blocks(int n) { return (n + kEnergyBlock - 1) / kEnergyBlock; }

// FP64 forces and potentials of an NB_F64 state for the energy pass: one
// thread per target, sources in index order through shared memory, j == i
// left out.  Not a throughput path: it runs only when the energy is asked for.
constexpr int kPhi64Block = 256;

__global__ void __launch_bounds__(kPhi64Block) phi64_kernel(const double4 *__restrict__ pos, int n,
                                                            double eps2, double4 *__restrict__ out)
{
    __shared__ double4 sp[kPhi64Block];
    const int nt = blockDim.x;  // <= kPhi64Block
    const int i = blockIdx.x * nt + threadIdx.x;
    const double4 pi = i < n ? pos[i] : make_double4(0.0, 0.0, 0.0, 0.0);
    double ax = 0.0, ay = 0.0, az = 0.0, phi = 0.0;
    for (int jt = 0; jt < n; jt += nt) {
        __syncthreads();
        if (jt + (int)threadIdx.x < n) sp[threadIdx.x] = pos[jt + threadIdx.x];
        __syncthreads();
        const int cnt = min(nt, n - jt);
        for (int j = 0; j < cnt; ++j) {
            if (jt + j == i) continue;
            const double4 q = sp[j];
            const double rx = q.x - pi.x, ry = q.y - pi.y, rz = q.z - pi.z;
            double d2 = fma(rx, rx, eps2);
            d2 = fma(ry, ry, d2);
            d2 = fma(rz, rz, d2);
            const double inv = rsqrt64(d2);
            const double mi = q.w * inv;
            const double sc = mi * (inv * inv);
            ax = fma(rx, sc, ax);
            ay = fma(ry, sc, ay);
            az = fma(rz, sc, az);
            phi += mi;
        }
    }
    if (i < n) out[i] = make_double4(ax, ay, az, phi);
}

__global__ void widen_kernel(const float4 *__restrict__ in, double4 *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 q = in[i];
        out[i] = make_double4(q.x, q.y, q.z, q.w);
    }
}

__global__ void narrow_kernel(const double4 *__restrict__ in, float4 *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double4 q = in[i];
        out[i] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
    }
}

int widen_f32(int n, const float4 *in, double4 *out, cudaStream_t s)
{
    if (n == 0) return NB_OK;
    widen_kernel<<<(n + 255) / 256, 256, 0, s>>>(in, out, n);
    NB_LAUNCH_CHECK("widen_kernel launch");
    return NB_OK;
}

int narrow_f64(int n, const double4 *in, float4 *out, cudaStream_t s)
{
    if (n == 0) return NB_OK;
    narrow_kernel<<<(n + 255) / 256, 256, 0, s>>>(in, out, n);
    NB_LAUNCH_CHECK("narrow_kernel launch");
    return NB_OK;
}

int energy_phi_f64(int n, const double4 *pos, double eps2, double4 *out, cudaStream_t s)
{
    if (n == 0) return NB_OK;
    // one thread per body: CTAs of 256 down to 32, whichever puts the fewest
    // warps on the busiest SM (small N in large CTAs leaves SMs idle)
    int dev = 0, sms = 0;
    NB_CUDA(cudaGetDevice(&dev));
    NB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto load = [&](int b) {
        const long long grid = ((long long)n + b - 1) / b;
        return ((grid + sms - 1) / sms) * (b / 32);
    };
    int block = kPhi64Block;
    for (int b = kPhi64Block / 2; b >= 32; b /= 2)
        if (load(b) < load(block)) block = b;
    phi64_kernel<<<(n + block - 1) / block, block, 0, s>>>(pos, n, eps2, out);
    NB_LAUNCH_CHECK("phi64_kernel launch");
    return NB_OK;
}

int energy_reduce(int n, const float4 *pos32, const double4 *pos64, const float4 *vel32,
                  const float4 *vlo, const float4 *phi32, const double4 *phi64, double G,
                  double *block_tmp, double *out_dev, cudaStream_t s, const double4 *vel64)
{
    const int nb = energy_blocks(n);
    if (nb > 0) {
        energy_partial_kernel<<<nb, kEnergyBlock, 0, s>>>(n, pos32, pos64, vel32, vlo, phi32, phi64,
                                                          G, block_tmp, vel64);
        NB_LAUNCH_CHECK("energy_partial_kernel launch");
    }
    energy_final_kernel<<<1, 32, 0, s>>>(block_tmp, nb, out_dev);
    NB_LAUNCH_CHECK("energy_final_kernel launch");
    return NB_OK;
}

}  // namespace nb
