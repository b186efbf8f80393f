/*
 * nbody_gb300.h -- C ABI of the GB300 (sm_103a) N-body all-pairs step.
 *
 * This is the drop-in boundary for the compute behind UTC's nbody GPU task.
 * In the reference the task class BodySystemSGPU<T> (benchapps/nbody/utc/
 * sgpu/body_task_sgpu.h:16-41) owns the device buffers and launches
 * _integrateNBodySystem_kernel<T> (benchapps/nbody/utc/sgpu/
 * bodysystem_kernel.cu:87-138) once per step on its task stream.  Here the
 * same work sits behind plain C entry points (pointers, sizes, status codes;
 * no C++ or torch types), which the drop-in task BodySystemGB300<T>
 * (utc_gb300/task/body_task_gb300.h) and the Python test harness call.
 *
 * Data layout (the reference's, body_task_sgpu.cu:55-58): per body 4 values
 * of the state type, position (x, y, z, m) and velocity (vx, vy, vz, w);
 * pos.w is the mass, vel.w is carried through unchanged.
 *
 * Update rule (bodysystem_kernel.cu:109-136, bodysystem.cc:135-182):
 *   a_i = sum_j m_j r_ij / (|r_ij|^2 + eps2)^(3/2),  r_ij = x_j - x_i
 *   v_i <- (v_i + (a_i * k_i) * dt) * damping
 *   x_i <- x_i + v_i * dt
 * with all a_i taken from the old positions.  k_i is pos.w of body i in
 * NB_KICK_REFERENCE mode (what the reference computes) and the constant G in
 * NB_KICK_PHYSICAL mode.
 *
 * Errors: every call returns an nb_status; nb_last_error() gives the message
 * of the last failure on the calling thread.  No call resets the device or
 * exits the process (the reference prints and calls cudaDeviceReset,
 * UTC/include/gpu/helper_cuda.h:419-442; that is deliberately not kept).
 *
 * Streams are passed as void* holding a cudaStream_t (NULL = legacy default
 * stream).  A context is used by one host thread at a time.
 */
#ifndef NBODY_GB300_H_
#define NBODY_GB300_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NB_ABI_VERSION 2

/* Largest system (and batch) size: indices stay within 32-bit arithmetic. */
#define NB_MAX_BODIES (1 << 30)

typedef enum {
    NB_OK = 0,
    NB_ERR_INVALID = 1,     /* bad argument */
    NB_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
    NB_ERR_OOM = 3,         /* device or pinned allocation failed */
    NB_ERR_STATE = 4,       /* call out of order (e.g. step before set_state) */
    NB_ERR_UNSUPPORTED = 5, /* combination not provided */
    NB_ERR_TIMEOUT = 6      /* a bounded device-side wait ran out */
} nb_status;

/* State type and arithmetic of a context. */
typedef enum {
    NB_F32 = 0,      /* float state (float4 pos/vel), float arithmetic */
    NB_F64 = 1,      /* double state (double4 pos/vel), double arithmetic */
    NB_F32_COMP = 2  /* double positions, float pair forces with compensated
                        (two-sum) accumulation; host buffers are double4 */
} nb_precision;

/* Force algorithm. */
typedef enum {
    /* Stream-K tiled kernel: packed f32x2 FMA, rsqrt.approx, deterministic
     * partial sums.  NB_F32 and NB_F32_COMP. */
    NB_ALGO_FAST = 0,
    /* IEEE arithmetic in the reference's operation order, sources summed in
     * index order: bit-identical to the reference's sequential BodySystem<T>
     * for float and double. */
    NB_ALGO_EXACT = 1,
    /* Each unordered pair evaluated once and applied to both bodies (the
     * pair term is odd in r): 16 FP32 operations and one rsqrt per two
     * interactions.  Same per-pair terms as NB_ALGO_FAST, different summation
     * order; deterministic.  NB_F32, NB_F32_COMP (compensated partial sums)
     * and NB_F64: pair terms in float-float arithmetic on the FP32 pipe
     * (positions scaled by powers of two and split on fixed grids into
     * three floats, error-free sums and products, an FP32 Newton and a
     * float-float Halley step on the FP32 rsqrt; chunk sums folded into
     * FP64), within a few 1e-15 of the FP64 reference, not bit for bit.
     * Range for NB_F64: eps2 >= 2^-100 max|x|^2 and masses >= 2^-100 of the
     * largest; coordinates within 2^-16 max|x| of zero are held to
     * 2^-69 max|x|. */
    NB_ALGO_SYM = 2,
    /* NB_F64 only: the symmetric algorithm in FP64 arithmetic throughout
     * (1/sqrt from the FP64 approximation and two Newton steps), within a
     * few 1e-16 of the FP64 reference, any range; about 1/6 the speed of
     * NB_ALGO_SYM on GB300's narrow FP64 pipe. */
    NB_ALGO_SYM_FP64 = 3
} nb_algo;

typedef enum { NB_KICK_REFERENCE = 0, NB_KICK_PHYSICAL = 1 } nb_kick;

/* Where host-visible buffers passed to set/get live. */
typedef enum { NB_HOST = 0, NB_DEVICE = 1 } nb_where;

/* Device memory kind of the context's state buffers, mirroring the
 * reference's MemType (UTC/include/gpu/GpuData.h:17-22) for the host side. */
typedef enum { NB_MEM_PAGEABLE = 0, NB_MEM_PINNED = 1, NB_MEM_UNIFIED = 2 } nb_memtype;

typedef struct nb_params {
    int n;            /* bodies, 0 <= n <= 2^30 (NB_MAX_BODIES) */
    int precision;    /* nb_precision */
    int algo;         /* nb_algo */
    int kick;         /* nb_kick */
    double eps2;      /* softening squared, as BodySystemSGPU::initImpl takes it */
    double damping;
    double dt;
    double G;         /* used in NB_KICK_PHYSICAL mode */
    int block;        /* threads per CTA (0 = tuned/auto): fast kernel; symmetric
                         kernels (warps x 32); exact kernel upper bound (it
                         takes smaller CTAs when they spread over more SMs;
                         its results do not depend on the CTA size) */
    int bpt;          /* fast kernel bodies per thread (0 = tuned/auto) */
    int ctas_per_sm;  /* fast kernel persistent CTAs per SM (0 = occupancy) */
    int memtype;      /* nb_memtype, for nb_run_host staging */
    int source_side;  /* nb_source_side: how NB_ALGO_SYM (NB_F32) sums the
                         reactions on the source bodies; other contexts and
                         batches ignore it (a value outside the enum is
                         NB_ERR_INVALID everywhere) */
    int bands;        /* NB_ALGO_SYM with the triangular source side (NB_F32,
                         NB_F32_COMP and NB_F64): 0 = cut the rows into bands
                         only where the array would pass 8 GiB; k in 2..512 =
                         k bands (fewer where there are fewer row blocks,
                         more where 8 GiB needs more): smaller scratch, for
                         tests and tight memory; other values
                         NB_ERR_INVALID; other contexts and batches ignore
                         it */
    int reserved[2];
} nb_params;

/* Source side of the symmetric FP32 kernel (nb_params.source_side).  Each
 * row block's reactions on the bodies after it are either stored in a
 * triangular array, about N^2 / (2 rb) float4 (67 MB at N = 65536, 3.4 GB at
 * N = 1M with the shapes chosen there), and summed by the integrator in row
 * order; or added at once into per-body 64-bit fixed-point accumulators with
 * integer atomics, 48 B per body, summed essentially exactly and still
 * deterministic (integer sums do not depend on their order), but measured
 * 2-10 % slower on GB300 at the same launch shape.  Where the triangular
 * array would pass 8 GiB even with 4 warps x 20 targets per lane (N above
 * about 1.66e6), it is cut into bands of consecutive row blocks, stepped
 * band by band through one 8 GiB buffer (nb_params.bands; the float-float
 * kernel of NB_F64 state does the same past N = 185k).  NB_SOURCE_AUTO
 * takes the triangular array (in bands where needed) and the fixed-point
 * side only beyond 512 bands (N above about 3.6e7).  Both are within the
 * same tolerances of the FP64 oracle. */
typedef enum { NB_SOURCE_AUTO = 0, NB_SOURCE_TRIANGULAR = 1, NB_SOURCE_FIXED = 2 } nb_source_side;

typedef struct nb_ctx nb_ctx;

/* Fill *p with defaults (F32, FAST, reference kick, eps2 0.00125,
 * damping 0.995 as BodySystem's constructor, bodysystem.cc:13-25). */
void nb_params_default(nb_params *p);

/* Create a context on the current CUDA device; allocates its state and
 * scratch buffers.  Replaces the GpuData allocations of
 * body_task_sgpu.cu:55-58. */
int nb_create(const nb_params *p, nb_ctx **out);
/* Synchronise the device, then free the context.  Distinct contexts may be
 * created, stepped and destroyed from several host threads at once (one UTC
 * task per system): the library keeps its own graph captures apart from its
 * allocations, frees and device synchronisations.  When a thread outside the
 * library is capturing a graph the device cannot be synchronised: the call
 * then returns NB_ERR_CUDA and keeps the context, to be destroyed again after
 * that capture. */
int nb_destroy(nb_ctx *ctx);

/* Load / read back the state.  pos and vel hold 4*n values of the state type
 * (double4 for NB_F32_COMP).  where = NB_HOST or NB_DEVICE.  Replaces
 * GpuData::sync / fetch (UTC/include/gpu/GpuData.h:31-354). */
int nb_set_state(nb_ctx *ctx, const void *pos, const void *vel, int where, void *stream);
int nb_get_state(nb_ctx *ctx, void *pos, void *vel, int where, void *stream);

/* Advance `steps` steps on `stream` (asynchronous).  Replaces the launch
 * loop of BodySystemSGPU::runImpl, body_task_sgpu.cu:85-127.  Bulk steps
 * (32 or more in one call) replay a captured CUDA graph; on the legacy
 * default stream, which cannot be captured, they run on a stream of the
 * context's own, after an event recorded on the caller's stream, and the
 * caller's stream waits for their end (so the call stays ordered like any
 * other work on it).  A capture that another thread's device-wide call
 * invalidates is dropped and those steps are launched one by one (same
 * results). */
int nb_step(nb_ctx *ctx, int steps, void *stream);

/* Change eps2 (the softening squared), damping, dt and G of a context (or of
 * a batch).  Replaces BodySystem<T>::setSoftening (which stores the square),
 * setDamping and the per-call deltaTime of update(deltaTime)
 * (benchapps/nbody/seq/bodysystem.h:19-29).  Takes effect for the next step;
 * drops captured step graphs and a recorded adjoint forward pass. */
int nb_set_params(nb_ctx *ctx, double eps2, double damping, double dt, double G);

/* nb_step with a CUDA event pair around every kernel it launches, on the
 * same stream.  Adds the summed device milliseconds of the force kernel and
 * of the reduce/integrate kernel to *ms_force and *ms_integrate (the exact
 * algorithm's single fused kernel counts as force).  Synchronises `stream`. */
int nb_step_timed(nb_ctx *ctx, int steps, float *ms_force, float *ms_integrate, void *stream);

/* Bare accelerations a_i (no kick factor) of the current state into a device
 * buffer of n 4-vectors of the state type (w = 0). */
int nb_accel(nb_ctx *ctx, void *acc_dev, void *stream);

/* Total energy and momentum of the current state, reduced in FP64 on the
 * GPU: out5 = {kinetic sum 0.5 m |v|^2, potential -0.5 G sum_i sum_{j!=i}
 * m_i m_j / sqrt(r^2 + eps2), momentum x, y, z}.  The pair terms are FP32
 * (compensated in NB_F32_COMP) or FP64-accurate (NB_F64: float-float with
 * NB_ALGO_SYM, FP64 arithmetic with the other algorithms).  accphi_dev
 * (may be NULL) receives per body the bare acceleration and, in w, the
 * potential sum over j != i, as n float4 (NB_F32) or double4 (NB_F32_COMP,
 * NB_F64).  NB_F32 reference-exact contexts take FP64 pair terms on their
 * float positions (scratch allocated on the first call).  Needs eps2 > 0.
 * Synchronises `stream`.  No counterpart in the reference (used by the
 * precision study). */
int nb_energy(nb_ctx *ctx, double *out5, void *accphi_dev, void *stream);

/* Adjoint (reverse mode) of `steps` steps; no counterpart in the reference.
 * nb_adj_forward advances the state like nb_step and keeps a checkpoint
 * (positions and velocities) every ckpt_every steps.  nb_adj_backward then
 * takes the cotangents of the final positions gx_T and velocities gv_T
 * (device, n float4, xyz used; gv_T may be NULL for zero) and writes
 * dL/dx0, dL/dv0 (device n float4, w = 0) and dL/dm (device n float),
 * recomputing each segment's trajectory from its checkpoint.  The recompute
 * of the next segment runs on a stream of the context's own, ordered against
 * `stream` by events: the results are complete once `stream` has reached the
 * end of the call.  NB_F32 fast or symmetric contexts; both kick modes.
 * Each nb_adj_forward gets a new generation number (from 1, increasing per
 * context), written to *generation (may be NULL).  nb_adj_backward takes the
 * generation of the forward pass whose gradients it is asked for and returns
 * NB_ERR_STATE when the context no longer holds that pass (a later
 * nb_adj_forward replaced it, or nb_set_params / nb_autotune dropped it), so
 * a caller that records several trajectories on one context gets an error
 * instead of another trajectory's gradients. */
int nb_adj_forward(nb_ctx *ctx, int steps, int ckpt_every, void *stream,
                   unsigned long long *generation);
int nb_adj_backward(nb_ctx *ctx, unsigned long long generation, const void *gx_T, const void *gv_T,
                    void *gx0, void *gv0, void *gm, void *stream);

/* The whole task run with host buffers, as BodySystemSGPU::runImpl
 * (body_task_sgpu.cu:40-137): copy pos/vel in, run `loops` steps, and after
 * every out_interval-th step copy the positions to
 * outbuffer + (step/out_interval - 1) * 4n.  pos/vel are not modified.
 * Unlike the reference (which synchronises the stream after every step and
 * copies each frame synchronously), frames are snapshotted on the GPU and
 * copied to pinned staging on a second stream while the next steps run.
 * timings (may be NULL) receives {total, kernel, copyin, copyout} seconds,
 * the reference's runtime[4] (copyout: device time of the frame copies,
 * which overlap the kernels).  Synchronises `stream` before returning. */
int nb_run_host(nb_ctx *ctx, const void *pos, const void *vel, int loops,
                int out_interval, void *outbuffer, double *timings, void *stream);

/* One fast FP32 step (force + kick/drift, NB_ALGO_FAST arithmetic) that
 * allocates nothing.  No counterpart in the reference: it exists for callers
 * that cannot call cudaMalloc -- an application whose memory manager owns
 * the GPU's memory and hands out sub-buffers itself, or a latency-critical
 * loop that cannot take the device synchronisation cudaMalloc/cudaFree may
 * cause.  The caller passes device buffers of n float4: pos_old (read),
 * pos_new (written, distinct from pos_old) and vel (updated in place).
 * The partial-force scratch is a 16 MiB array compiled into the library
 * (present on every GPU that loads it until exit), which limits n to
 * 262,144; larger n returns NB_ERR_INVALID.  The first call in each CUDA
 * context looks up that array's device address (again after cudaDeviceReset
 * or in a driver-API context of the caller's), so make it before any stream
 * capture in that context.  All calls share the array: calls whose kernels
 * overlap on the GPU race and must be serialised. */
int nb_step_f32_noalloc(const float *pos_old, float *pos_new, float *vel, int n, float eps2,
                        float damping, float dt, int kick, float G, void *stream);

/* ------------------------------------------------------------------------
 * Target partition across GPUs: replaces the multi-GPU task
 * BodySystemMGPU<T> (benchapps/nbody/utc-snode-mgpu/mgpu/body_task_mgpu.cu:
 * 14-163), whose threads each own a range of targets, copy every body's
 * positions in before each step and their own range out after it.
 *
 * nb_create_shard makes a context (on the current device) for shard `rank`
 * of `nranks`: it holds every body's state and, per step, updates only its
 * own targets against all sources.  NB_F32 with NB_ALGO_FAST: whole target
 * blocks of the directed kernel's plan per shard (the remainder to the first
 * ranks), and the shard launches exactly the CTAs of the single-GPU launch
 * that cover its blocks, so the shards' results put together equal a
 * single-GPU NB_ALGO_FAST context's bit for bit.  NB_ALGO_EXACT (NB_F32 or
 * NB_F64): the reference's split, n / nranks bodies each and one more for
 * the first n % nranks ranks; bit-identical to the sequential reference.
 * With nranks > 1, nb_step / nb_step_timed take one step per call: between
 * steps the caller brings the other shards' new positions into this
 * context's current position buffer (nb_state_ptrs; an all-gather of every
 * shard's range [first, first + count) of that buffer, e.g. by NCCL).  Velocities
 * are valid in the shard's own range only.  nb_accel, nb_energy, the adjoint,
 * nb_run_host and nb_autotune are refused (NB_ERR_UNSUPPORTED) on such a
 * shard.  nb_shard_info: {first body, body count, rank, nranks}.
 * ---------------------------------------------------------------------- */
int nb_create_shard(const nb_params *p, int rank, int nranks, nb_ctx **out);
int nb_shard_info(nb_ctx *ctx, int *info4);

/* ------------------------------------------------------------------------
 * Batches: many independent systems of uneven size advanced together, one
 * persistent launch per step for all of them.  Replaces running one
 * Task<BodySystemSGPU<T>> per system (benchapps/nbody/utc/nbody_mtask.cc:
 * 199-231).  Bodies of all systems are concatenated (system s after
 * systems 0..s-1): float4 for NB_F32 batches (NB_ALGO_SYM or NB_ALGO_FAST),
 * double4 for NB_F64 batches (NB_ALGO_SYM: float-float pair terms, the
 * multi-task app's FTYPE double; no batched adjoint).  All systems share
 * eps2, damping, dt, G and kick mode from *p (p->n is ignored; p->block /
 * p->bpt, when set, give the initial warps per CTA * 32 and bodies per
 * lane).
 * ---------------------------------------------------------------------- */
typedef struct nb_batch nb_batch;
int nb_batch_create(const nb_params *p, int nsys, const int *sizes, nb_batch **out);
int nb_batch_destroy(nb_batch *b);
int nb_batch_set_state(nb_batch *b, const void *pos, const void *vel, int where, void *stream);
int nb_batch_get_state(nb_batch *b, void *pos, void *vel, int where, void *stream);
/* `steps` steps, launched one by one. */
int nb_batch_step(nb_batch *b, int steps, void *stream);
/* `steps` steps as one CUDA graph (captured on first use for this step count
 * and parity, replayed afterwards; launched one by one when the capture does
 * not take, as nb_step); `stream` must not be the legacy default stream.
 * nb_batch_destroy behaves as nb_destroy. */
int nb_batch_run(nb_batch *b, int steps, void *stream);
/* Time every compiled launch shape on this batch and keep the fastest
 * (state preserved); cache_path (may be NULL) is a text file of earlier
 * choices keyed by device and size histogram.  chosen2 = {warps per CTA,
 * bodies per lane}. */
int nb_batch_autotune(nb_batch *b, int reps, const char *cache_path, void *stream, int *chosen2);
int nb_batch_set_shape(nb_batch *b, int warps_per_cta, int bodies_per_lane);
/* {warps per CTA, bodies per lane, grid, workers, iterations, slots} */
int nb_batch_plan_info(nb_batch *b, long long *info6);
int nb_batch_launches_per_step(nb_batch *b);
/* Baseline: each system stepped by its own plain launches (force +
 * integrate per system per step), as separate per-system tasks would. */
int nb_batch_step_per_system(nb_batch *b, int steps, void *stream);
/* Baseline in the reference's multi-task pattern (benchapps/nbody/utc/
 * nbody_mtask.cc:199-231): ntasks host threads with a stream each run their
 * systems with a stream synchronise after every step (as
 * BodySystemSGPU::runImpl does).  Synchronous. */
int nb_batch_step_tasks(nb_batch *b, int steps, int ntasks);
/* Adjoint of `steps` batched steps, same contract as nb_adj_forward /
 * nb_adj_backward over the concatenated bodies of all systems (no
 * counterpart in the reference). */
int nb_batch_set_params(nb_batch *b, double eps2, double damping, double dt, double G);
int nb_batch_adj_forward(nb_batch *b, int steps, int ckpt_every, void *stream,
                         unsigned long long *generation);
int nb_batch_adj_backward(nb_batch *b, unsigned long long generation, const void *gx_T,
                          const void *gv_T, void *gx0, void *gv0, void *gm, void *stream);

/* Seeded initial conditions generated on the GPU, one thread per body
 * (counter-based: a body's draw depends only on (seed, index)).  kind 0:
 * uniform cube, positions U[-1,1]^3, velocities U[-vmax,vmax]^3, masses
 * U[0.5,1.5]/n; kind 1: Plummer sphere of scale a, total mass M and
 * gravitational constant G (Aarseth, Henon & Wielen sampling), masses M/n,
 * centre of mass and momentum moved to zero; kinds 2, 3, 4: the reference
 * app's random, shell and expand configurations with a = clusterScale and
 * vmax = velocityScale, masses 1 (same distributions as randomizeBodies,
 * not its rand() sequence).  pos/vel: device, n 4-vectors of
 * float (NB_F32) or double (NB_F64), vel.w = 1.  scratch_dev: device buffer of
 * nb_ics_scratch_bytes(n) bytes (Plummer only).  Replaces the host-side
 * randomizeBodies (benchapps/nbody/seq/nbody.h:89-250) for large synthetic
 * inputs; the app's own initialiser stays on the host (it draws rand()). */
int nb_ics_generate(int kind, int n, unsigned long long seed, double a, double G, double M,
                    double vmax, int precision, void *pos_dev, void *vel_dev, void *scratch_dev,
                    void *stream);
size_t nb_ics_scratch_bytes(int n);

/* Device pointers of the current state (valid until the next nb_step).
 * A context with the fixed-point source side (nb_params.source_side) takes
 * the masses into its scale at nb_set_state: after changing pos.w through
 * these pointers, load the state again with nb_set_state (NB_DEVICE) before
 * stepping.  Positions and velocities may be written freely. */
int nb_state_ptrs(nb_ctx *ctx, void **pos_dev, void **vel_dev);

/* Resolved launch shape of the context's force kernel: {block, bpt, grid,
 * target block size, slots}; for the symmetric kernels block = warps per
 * CTA * 32, bpt = targets per lane and the target block is the row block. */
int nb_plan_info(nb_ctx *ctx, int *info5);

/* Source side of a symmetric context: info4 = {source side (NB_SOURCE_FIXED
 * or NB_SOURCE_TRIANGULAR), bands of the triangular array (1 = one pass),
 * MiB of scratch the source side holds (the largest band's share),
 * 0 (reserved)}.  Other contexts give {0, 1, 0, 0}. */
int nb_source_info(nb_ctx *ctx, int *info4);

/* Time every compiled launch shape of the context's force kernel on its
 * current state (`reps` steps each; the state is restored) and keep the
 * fastest; a symmetric shape whose triangular source-side array would pass
 * 8 GiB is timed in bands (skipped if it has no banded form).  cache_path
 * (may be NULL) is a text file of earlier choices keyed
 * by device, precision, algorithm and n: a hit applies the cached shape
 * without timing.  chosen2 = {threads per CTA, bodies per lane}.  Drops
 * captured step graphs and a recorded adjoint forward pass; the reference-
 * exact kernel has nothing to tune.  Synchronises `stream`.  No counterpart in
 * the reference (its block size is a command-line flag). */
int nb_autotune(nb_ctx *ctx, int reps, const char *cache_path, void *stream, int *chosen2);

/* Number of kernels nb_step launches per step for this context. */
int nb_launches_per_step(nb_ctx *ctx);

/* Peak FMA throughput probe: runs a kernel of independent FMA chains on all
 * SMs for `iters` iterations (packed 0: scalar FP32 FFMA, 1: packed FP32
 * FFMA2, 2: FP64 DFMA); *flops receives the operations issued (2 per
 * lane-FMA) and *ms the device time. */
int nb_probe_fma_peak(int iters, int packed, double *flops, float *ms, void *stream);

const char *nb_last_error(void);
int nb_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
