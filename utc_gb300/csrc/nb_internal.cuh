// nb_internal.cuh -- shared declarations of the GB300 nbody library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <shared_mutex>
#include <string>

#include "nbody_gb300.h"

namespace nb {

// ---------------------------------------------------------------------------
// error reporting (thread-local last error, status codes)
// ---------------------------------------------------------------------------
int set_error(int status, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);

#define NB_CUDA(call)                                              \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::nb::cuda_error(_e, #call); \
    } while (0)

#define NB_LAUNCH_CHECK(what)                                     \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::nb::cuda_error(_e, what); \
    } while (0)

// ---------------------------------------------------------------------------
// the capture gate
// ---------------------------------------------------------------------------
// A call that synchronises the whole device (cudaMalloc, cudaFree and their
// pinned-host and managed forms, cudaDeviceSynchronize, a synchronous
// cudaMemcpy) made in one host thread while another thread captures a stream
// into a graph invalidates that capture, and the synchronising call itself
// may return without having synchronised.  Several host threads that each
// step their own context (one UTC task per system) meet exactly so.  The
// library's captures hold this gate shared and its device-wide calls hold it
// exclusively, so the two never overlap within the library; a capture that
// something outside the library invalidates falls back to step-by-step
// launches (nb_step, nb_batch_run).
std::shared_mutex &capture_gate();

inline bool is_capture_error(cudaError_t e)
{
    return e >= cudaErrorStreamCaptureUnsupported && e <= cudaErrorStreamCaptureWrongThread;
}

template <class T>
inline cudaError_t dmalloc(T **p, size_t bytes)
{
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaMalloc((void **)p, bytes);
}
template <class T>
inline cudaError_t dmalloc_managed(T **p, size_t bytes)
{
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaMallocManaged((void **)p, bytes, cudaMemAttachGlobal);
}
template <class T>
inline cudaError_t hmalloc(T **p, size_t bytes)
{
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaMallocHost((void **)p, bytes);
}
inline cudaError_t dfree(void *p)
{
    if (!p) return cudaSuccess;
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaFree(p);
}
inline cudaError_t hfree(void *p)
{
    if (!p) return cudaSuccess;
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaFreeHost(p);
}
inline cudaError_t device_sync()
{
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaDeviceSynchronize();
}
inline cudaError_t dmemcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind)
{
    std::unique_lock<std::shared_mutex> g(capture_gate());
    return cudaMemcpy(dst, src, bytes, kind);
}
// graph instantiation and destruction may allocate or free device memory
inline cudaError_t graph_instantiate(cudaGraphExec_t *out, cudaGraph_t g)
{
    std::unique_lock<std::shared_mutex> lk(capture_gate());
    return cudaGraphInstantiate(out, g, 0);
}
inline cudaError_t graph_exec_destroy(cudaGraphExec_t g)
{
    if (!g) return cudaSuccess;
    std::unique_lock<std::shared_mutex> lk(capture_gate());
    return cudaGraphExecDestroy(g);
}

// ---------------------------------------------------------------------------
// packed f32x2 arithmetic (sm_100+ FFMA2 / FADD2 / FMUL2)
// ---------------------------------------------------------------------------
typedef unsigned long long f2;  // two floats in one 64-bit register pair

__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// Knuth's two-sum: s + e == a + b exactly (round-to-nearest, no FMA).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// 1/sqrt(x) in FP64: the FP64 approximate reciprocal square root refined by
// two Newton-Raphson steps, y <- y + (y/2)(1 - x y^2), each squaring the
// relative error.  x must be a normal positive FP64 number.
__device__ __forceinline__ double rsqrt64(double x)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const double r = fma(-x, y * y, 1.0);  // 1 - x y^2
        y = fma(0.5 * y, r, y);
    }
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Position used for the padding sources of a partial tile: zero mass makes
// its term exactly zero (m * finite = 0), the distance keeps d2 finite > 0.
constexpr float kPadCoord = 1.0e15f;

// ---------------------------------------------------------------------------
// stream-K plan of the fast force kernel
// ---------------------------------------------------------------------------
// The iteration space is (target block tb, source group g) with groups of
// kGroup sources; it = tb * ngroups + g.  CTA c of `grid` owns iterations
// [start(c), start(c+1)), start(c) = floor(c * total / grid), so every CTA
// gets the same number of pair evaluations up to one group.  A CTA writes
// one partial acceleration per target block it touches, into slot c + tb
// (distinct for distinct (c, tb) because CTA ranges are ordered).
constexpr int kGroup = 32;

struct SkPlan {
    int n = 0;
    int block = 0;     // threads per CTA
    int bpt = 0;       // bodies (targets) per thread
    int tbsize = 0;    // targets per block = block * bpt
    int ntb = 0;       // target blocks
    int ngroups = 0;   // source groups per target block
    long long total = 0;
    int grid = 0;      // persistent CTAs
    int slots = 0;     // grid + ntb - 1
    // a shard of the targets (fast_shard): whole target blocks; iterations
    // [it_lo, it_hi) and targets [i_lo, i_hi) of the full plan above
    bool ranged = false;
    long long it_lo = 0, it_hi = 0;
    int i_lo = 0, i_hi = 0;
};

__host__ __device__ __forceinline__ long long sk_start(long long c, long long total, int grid)
{
    return (c * total) / grid;
}
// CTA that owns iteration `it`: the largest c with start(c) <= it.
__host__ __device__ __forceinline__ int sk_owner(long long it, long long total, int grid)
{
    return (int)(((it + 1) * (long long)grid - 1) / total);
}

// Force-kernel variants: compensated (two-sum) tile accumulation writing
// (hi, lo) partials, and the potential sum carried in w.
enum : int { SK_COMP = 1, SK_PHI = 2 };

// Fast-path entry points (nb_fast.cu).  With SK_COMP the partial scratch
// holds 2 * slots * tbsize float4 (hi block, then lo block).
int fast_plan(int n, int block, int bpt, int ctas_per_sm, int device, SkPlan *plan,
              int flags = 0);
bool fast_shape_supported(int block, int bpt, int flags);
// Restrict a plan to the target blocks of shard `rank` of `nranks` (whole
// blocks each, the remainder to the first ranks).
int fast_shard(SkPlan *plan, int rank, int nranks);
int fast_force(const SkPlan &plan, const float4 *pos, float eps2, float4 *partial,
               cudaStream_t s, int flags = 0);
// Reduce the partial slots and integrate (acc_out != nullptr: write the bare
// acceleration instead of integrating).
int fast_integrate(const SkPlan &plan, const float4 *pos_old, float4 *pos_new, float4 *vel,
                   const float4 *partial, float damping, float dt, int kick, float G,
                   float4 *acc_out, cudaStream_t s);

// Precision mode, reductions and energy (nb_precision.cu)
int comp_split(const double4 *pin, const double4 *vin, double4 *pos64, float4 *pos32,
               float4 *vhi, float4 *vlo, int n, cudaStream_t s);
int comp_join(const double4 *pos64, const float4 *vhi, const float4 *vlo, double4 *pout,
              double4 *vout, int n, cudaStream_t s);
// Sum the partial slots into bare accelerations with the potential over
// j != i in w (out32 for plain slots, out64 = hi + lo for compensated ones).
int fast_reduce(const SkPlan &p, const float4 *partial, int comp, const float4 *pos32, float eps2,
                float4 *out32, double4 *out64, cudaStream_t s);
int comp_integrate(const SkPlan &p, const float4 *partial, double4 *pos64, float4 *pos32,
                   float4 *vhi, float4 *vlo, float damping, float dt, double dt64, int kick,
                   float G, cudaStream_t s);
int energy_blocks(int n);
// FP64 accelerations and potentials over j != i of an NB_F64 state, into
// out (ax, ay, az, phi) (nb_precision.cu)
// float4 <-> double4 copies (each value converted; narrowing rounds to nearest)
int widen_f32(int n, const float4 *in, double4 *out, cudaStream_t s);
int narrow_f64(int n, const double4 *in, float4 *out, cudaStream_t s);
int energy_phi_f64(int n, const double4 *pos, double eps2, double4 *out, cudaStream_t s);
// Energy and momentum in FP64 from the state (masses from pos64 if given,
// else pos32; velocities from vel64 if given, else vel32 + vlo) and the
// per-body potentials (phi64 if given, else phi32).
int energy_reduce(int n, const float4 *pos32, const double4 *pos64, const float4 *vel32,
                  const float4 *vlo, const float4 *phi32, const double4 *phi64, double G,
                  double *block_tmp, double *out_dev, cudaStream_t s,
                  const double4 *vel64 = nullptr);

// Symmetric force kernel (nb_sym.cu)
// Work layout of the symmetric kernels (nb_sym.cu, nb_adjoint.cu): row
// blocks of rb bodies paired with 32-body chunks at or after their start.
__host__ __device__ __forceinline__ long long sym_prefix(long long I, int nc, int rc)
{
    // items of rows 0..I-1: row i pairs with chunks i*rc .. nc-1
    return I * (long long)nc - (long long)rc * (I * (I - 1) / 2);
}

// Source-side array, triangular: row r keeps bodies i >= (r + 1) * rb at
// soff(r) + i - (r + 1) * rb.
__host__ __device__ __forceinline__ long long sym_soff(long long r, int n, int rb)
{
    return r * (long long)n - (long long)rb * (r * (r + 1) / 2);
}

__device__ __forceinline__ int sym_row_of(long long it, int nc, int rc, int nrb)
{
    int lo = 0, hi = nrb;  // prefix(lo) <= it < prefix(hi)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sym_prefix(mid, nc, rc) <= it) lo = mid;
        else hi = mid;
    }
    return lo;
}

struct SymPlan {
    int n = 0, warps = 0, bpt = 0;
    int comp = 0;        // compensated (hi, lo) partials: tpart and spart hold a lo block after the hi block
    int fixed = 0;       // plain plans: source side in 64-bit fixed point (sym_fx_*), spart then holds
                         // 6 n integers and a record; otherwise the triangular array
    int rb = 0;          // bodies per row block (CTA targets)
    int nc = 0;          // 32-body chunks
    int nrb = 0;         // row blocks
    long long total = 0; // (row, chunk) items
    int grid = 0;
    int slots = 0;       // grid + nrb - 1 target-side slots of rb float4
    long long spart_size = 0;  // float4 entries of the source-side array (of the largest band)
    int sms = 0;         // SMs of the device planned for
    // Triangular plans whose source-side array would pass the budget are cut
    // into bands of consecutive row blocks: the force kernel runs band by
    // band over the band's (row, chunk) items, every band's source-side
    // entries reusing one buffer, and after each band a fold kernel adds its
    // target-side slots and source-side rows into one sum per body (accsum),
    // which the integrator then reads.  nbands = 1: one pass, no fold.
    static constexpr int kMaxBands = 512;
    int nbands = 1;
    int band_row[kMaxBands + 1] = {};  // band k: row blocks [band_row[k], band_row[k + 1])
};
// float4 entries of the source-side array for row blocks of rb bodies
inline long long sym_spart_entries(int n, int rb)
{
    const int nrb = (n + rb - 1) / rb;
    return nrb > 1 ? sym_soff(nrb - 1, n, rb) : 0;
}
// Largest source-side array a default shape accepts before it moves to a
// bigger row block or to bands.
constexpr long long kSymSpartBudget = 8ll << 30;

// Bands of a triangular plan: consecutive row blocks, a new band started
// whenever the next row's entries (n - (r + 1) rb; none for the last row
// block) would take the band past cap.  Fills rows[0..k] (when rows is not
// null) and the largest band's entry count; returns the band count k, or 0
// when more than `limit` bands would be needed.
inline int sym_band_rows(int n, int rb, long long cap, int limit, int *rows, long long *max_entries)
{
    const int nrb = (n + rb - 1) / rb;
    int k = 0;
    long long acc = 0, mx = 0;
    if (rows) rows[0] = 0;
    for (int r = 0; r < nrb; ++r) {
        const long long e = r < nrb - 1 ? (long long)n - (long long)(r + 1) * rb : 0;
        if (acc > 0 && acc + e > cap) {
            if (++k >= limit) return 0;
            if (rows) rows[k] = r;
            mx = acc > mx ? acc : mx;
            acc = 0;
        }
        acc += e;
    }
    mx = acc > mx ? acc : mx;
    if (rows) rows[k + 1] = nrb;
    if (max_entries) *max_entries = mx;
    return k + 1;
}

// The bands of a plan whose source-side entries must stay within cap: as
// few as that needs, or (want > 1) as many as the smallest cap that still
// gives at most `want` bands needs, if that is more.  Returns the band
// count, or 0 beyond SymPlan::kMaxBands.
inline int sym_make_bands(int n, int rb, long long cap, int want, int *rows, long long *max_entries)
{
    if (want > 1) {
        const long long total = sym_spart_entries(n, rb);
        long long lo = (total + want - 1) / want, hi = total;
        if (lo < 1) lo = 1;
        if (hi < lo) hi = lo;
        while (lo < hi) {  // the smallest cap with at most `want` bands
            const long long mid = lo + (hi - lo) / 2;
            if (sym_band_rows(n, rb, mid, want, nullptr, nullptr) != 0) hi = mid;
            else lo = mid + 1;
        }
        if (lo < cap) cap = lo;
    }
    return sym_band_rows(n, rb, cap, SymPlan::kMaxBands, rows, max_entries);
}

// float4 entries of the fixed-point source side: 6 n 64-bit accumulators
// (hi x, y, z then lo x, y, z, each n long) and one float4 record: the sum of
// |m| over the bodies and the scale factors (sym_fx_prepare).
inline long long sym_fx_entries(int n) { return 3ll * n + 1; }

// source_side: nb_source_side (NB_SOURCE_AUTO / TRIANGULAR / FIXED), for
// plain plans; compensated plans are always triangular.  bands: 0 = bands
// only where the triangular array would pass the budget, k > 1 = k bands
// (sym_make_bands), -1 = never (the shape grows instead).
int sym_plan(int n, int warps, int bpt, int device, SymPlan *pl, int comp = 0, int source_side = 0,
             int bands = 0);
// accsum: the per-body sums of banded plans (n float4; compensated plans
// 2 n: sums, then compensations), unused otherwise
int sym_force(const SymPlan &p, const float4 *pos, float eps2, float4 *tpart, float4 *spart,
              float4 *accsum, cudaStream_t s);
// consume (fixed plans): zero the accumulators after reading them, ready for
// the next force launch; 0 leaves them for a second reader of the same
// force launch
int sym_integrate(const SymPlan &p, const float4 *pos_old, float4 *pos_new, float4 *vel,
                  const float4 *tpart, const float4 *spart, const float4 *accsum, float damping, float dt,
                  int kick, float G, float4 *acc_out, cudaStream_t s, int consume = 1);
// Fixed plans: zero the accumulators and write the record (the sum of |m| of
// pos and the scale it gives with eps2); after every new state and scratch.
int sym_fx_prepare(const SymPlan &p, const float4 *pos, float4 *spart, float eps2, cudaStream_t s);
// Fixed plans: the record's scale for a new eps2 (the masses unchanged).
int sym_fx_rescale(const SymPlan &p, float4 *spart, float eps2, cudaStream_t s);

// FP64 symmetric path (nb_sym64.cu): tpart / spart hold double4 entries.
// sym64_integrate with ffrange (the float-float path's scale record) undoes
// that path's power-of-two scaling of the sums; with accsum (banded
// float-float plans) it takes the folded per-body sums instead of the
// partials.
int sym64_plan(int n, int warps, int bpt, int device, SymPlan *pl);
int sym64_force(const SymPlan &p, const double4 *pos, double eps2, double4 *tpart, double4 *spart,
                cudaStream_t s);
int sym64_integrate(const SymPlan &p, const double4 *pos_old, double4 *pos_new, double4 *vel,
                    const double4 *tpart, const double4 *spart, double damping, double dt, int kick,
                    double G, double4 *acc_out, cudaStream_t s, const unsigned long long *ffrange = nullptr,
                    const double4 *accsum = nullptr);
// Float-float symmetric path for FP64 state (nb_symff.cu): same layout and
// double4 partials as the FP64 path; `split` holds 3 n float4 (the scaled
// three-float positions), `range` 2 unsigned long long (the scale record).
// bands as for sym_plan (0 = where the array would pass the budget, k > 1,
// -1 = never: the shape grows instead); accsum: n double4 for banded plans.
int symff_plan(int n, int warps, int bpt, int device, SymPlan *pl, int bands = 0);
int symff_force(const SymPlan &p, const double4 *pos, double eps2, float4 *split, unsigned long long *range,
                double4 *tpart, double4 *spart, double4 *accsum, cudaStream_t s, int phi = 0);
// The float-float paths' per-step preparation: range (2 unsigned long long)
// <- bits of the largest |coordinate| and |mass|; H + M + L <- the positions
// and masses scaled by those powers of two, split into three floats.
int ff_scale_split(const double4 *pos, int n, int sms, float4 *H, float4 *M, float4 *L, unsigned long long *range,
                   cudaStream_t s);

// Compensated kick / drift from compensated symmetric partials, or
// (acc_out != nullptr) the bare FP64 accelerations (nb_precision.cu);
// banded plans take accsum (2 n float4: the folded sums, then their
// compensations)
int sym_comp_integrate(const SymPlan &p, const float4 *tpart, const float4 *spart, double4 *pos64,
                       float4 *pos32, float4 *vhi, float4 *vlo, float damping, float dt,
                       double dt64, int kick, float G, double4 *acc_out, cudaStream_t s,
                       const float4 *accsum = nullptr);

// One reverse step's per-body update given the summed pair terms (o, odm):
//   lx <- lx + out;  lv <- D mu;  gm += dm (+ D dt mu.a in reference mode)
// and, when want_next_g, g for the next reverse step (at the previous state,
// whose masses are the same).
__device__ __forceinline__ void adj_body_update(int i, float ox, float oy, float oz, float odm,
                                                const float4 *__restrict__ pos,
                                                const float4 *__restrict__ acc,
                                                float4 *__restrict__ lx, float4 *__restrict__ lv,
                                                float *__restrict__ gm, float4 *__restrict__ gbuf,
                                                float damping, float dt, int kick, float G,
                                                int want_next_g)
{
    const float4 x = lx[i], v = lv[i];
    const float mux = fmaf(dt, x.x, v.x), muy = fmaf(dt, x.y, v.y), muz = fmaf(dt, x.z, v.z);
    float dmi = odm;
    if (kick == NB_KICK_REFERENCE) {
        const float4 a = acc[i];
        dmi = fmaf(damping * dt, mux * a.x + muy * a.y + muz * a.z, dmi);
    }
    gm[i] += dmi;
    const float4 nx = make_float4(x.x + ox, x.y + oy, x.z + oz, 0.f);
    const float4 nv = make_float4(damping * mux, damping * muy, damping * muz, 0.f);
    lx[i] = nx;
    lv[i] = nv;
    if (want_next_g) {
        const float k = kick == NB_KICK_REFERENCE ? pos[i].w : G;
        const float f = damping * dt * k;
        gbuf[i] = make_float4(f * fmaf(dt, nx.x, nv.x), f * fmaf(dt, nx.y, nv.y),
                              f * fmaf(dt, nx.z, nv.z), 0.f);
    }
}

// Adjoint kernels (nb_adjoint.cu)
int adj_plan(int n, int block, int bpt, int device, SkPlan *pl);
int adj_g(int n, const float4 *pos, const float4 *lx, const float4 *lv, float4 *gbuf, float damping,
          float dt, int kick, float G, cudaStream_t s);
int adj_vjp(const SkPlan &p, const float4 *pos, const float4 *gbuf, float eps2, float4 *partial,
            cudaStream_t s);
int adj_update(const SkPlan &p, const float4 *partial, const float4 *pos_prev, const float4 *acc,
               float4 *lx, float4 *lv, float *gm, float4 *gbuf, float damping, float dt, int kick,
               float G, int want_next_g, cudaStream_t s);
// Symmetric vector-Jacobian product (each unordered pair once) on the
// symmetric work layout; tpart/spart as in sym_force.
int sym_vjp_plan(int n, int warps, int bpt, int device, SymPlan *pl);
int sym_vjp(const SymPlan &p, const float4 *pos, const float4 *gbuf, float eps2, float4 *tpart,
            float4 *spart, cudaStream_t s);
int adj_update_sym(const SymPlan &p, const float4 *tpart, const float4 *spart, const float4 *pos_prev,
                   const float4 *acc, float4 *lx, float4 *lv, float *gm, float4 *gbuf, float damping,
                   float dt, int kick, float G, int want_next_g, cudaStream_t s);

// Exact-path entry points (nb_exact.cu): targets [i_begin, i_end) of n
int exact_step_f32(int n, int i_begin, int i_end, const float4 *pos_old, float4 *pos_new, float4 *vel,
                   float eps2, float damping, float dt, int kick, float G, float4 *acc_out, int block,
                   cudaStream_t s);
int exact_step_f64(int n, int i_begin, int i_end, const double4 *pos_old, double4 *pos_new,
                   double4 *vel, double eps2, double damping, double dt, int kick, double G,
                   double4 *acc_out, int block, cudaStream_t s);

// FMA peak probe (nb_fast.cu)
int probe_fma(int iters, int packed, double *flops, float *ms, cudaStream_t s);

// The adjoint's recompute stream and its three events (two "segment
// recomputed", one "buffer free"), created together or not at all
// (nb_api.cu).
int create_recompute_stream(cudaStream_t *stream, cudaEvent_t ev_rec[2], cudaEvent_t *ev_go);

}  // namespace nb
