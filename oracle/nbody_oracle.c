/*
 * nbody_oracle.c -- CPU restatement of the UTC nbody all-pairs step.
 *
 * TEST INFRASTRUCTURE ONLY (the correctness oracle and the timed CPU
 * baseline); see nbody_oracle.h.  Compile with -O2 -ffp-contract=off.
 *
 * The arithmetic order of every float/double expression follows the
 * reference line for line so that results are bit-identical:
 *   pair term      benchapps/nbody/seq/bodysystem.h:71-96
 *   force loop     benchapps/nbody/seq/bodysystem.cc:103-133
 *   integrator     benchapps/nbody/seq/bodysystem.cc:135-182
 *   initialisers   benchapps/nbody/seq/nbody.h:89-250
 */
#include "nbody_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* host thread fan-out over target ranges                              */
/* ------------------------------------------------------------------ */
typedef void (*range_fn)(void *ctx, int lo, int hi);
typedef struct {
    range_fn fn;
    void *ctx;
    int lo, hi;
} range_job;

static void *range_thread(void *p)
{
    range_job *j = (range_job *)p;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static void parallel_for(int n, int nthreads, range_fn fn, void *ctx)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (nthreads > n) nthreads = n > 0 ? n : 1;
    if (nthreads == 1) {
        fn(ctx, 0, n);
        return;
    }
    pthread_t th[256];
    int joined[256];
    range_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = (int)(((long long)n * t) / nthreads);
        jobs[t].hi = (int)(((long long)n * (t + 1)) / nthreads);
    }
    for (int t = 1; t < nthreads; ++t) {
        joined[t] = pthread_create(&th[t], NULL, range_thread, &jobs[t]) == 0;
        /* thread creation failed: run that range on this thread instead */
        if (!joined[t]) range_thread(&jobs[t]);
    }
    range_thread(&jobs[0]);
    for (int t = 1; t < nthreads; ++t)
        if (joined[t]) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* pair term and force loop                                            */
/* ------------------------------------------------------------------ */

/* bodysystem.h:71-96 for T=float.  The reciprocal is taken in double
 * ("1.0/sqrt_T(distSqr)" with a double literal) and rounded to float. */
static inline void pair_f32(float acc[3], const float *p0, const float *p1,
                            float eps2)
{
    float r0 = p1[0] - p0[0];
    float r1 = p1[1] - p0[1];
    float r2 = p1[2] - p0[2];
    float distSqr = r0 * r0 + r1 * r1 + r2 * r2;
    distSqr += eps2;
    float invDist = (float)(1.0 / (double)sqrtf(distSqr));
    float invDistCube = invDist * invDist * invDist;
    float s = p1[3] * invDistCube;
    acc[0] += r0 * s;
    acc[1] += r1 * s;
    acc[2] += r2 * s;
}

static inline void pair_f64(double acc[3], const double *p0, const double *p1,
                            double eps2)
{
    double r0 = p1[0] - p0[0];
    double r1 = p1[1] - p0[1];
    double r2 = p1[2] - p0[2];
    double distSqr = r0 * r0 + r1 * r1 + r2 * r2;
    distSqr += eps2;
    double invDist = 1.0 / sqrt(distSqr);
    double invDistCube = invDist * invDist * invDist;
    double s = p1[3] * invDistCube;
    acc[0] += r0 * s;
    acc[1] += r1 * s;
    acc[2] += r2 * s;
}

typedef struct {
    int n;
    const float *pos;
    float eps2;
    float *acc;
} accel_f32_ctx;

static void accel_f32_range(void *vp, int lo, int hi)
{
    accel_f32_ctx *c = (accel_f32_ctx *)vp;
    for (int i = lo; i < hi; ++i) {
        float a[3] = {0.f, 0.f, 0.f};
        const float *pi = c->pos + 4 * (size_t)i;
        /* bodysystem.cc:112-125 unrolls by 4 with no remainder; the sum
         * order is plain j = 0..n-1 either way. */
        for (int j = 0; j < c->n; ++j) pair_f32(a, pi, c->pos + 4 * (size_t)j, c->eps2);
        c->acc[3 * (size_t)i + 0] = a[0];
        c->acc[3 * (size_t)i + 1] = a[1];
        c->acc[3 * (size_t)i + 2] = a[2];
    }
}

typedef struct {
    int n;
    const double *pos;
    double eps2;
    double *acc;
    const int *tidx; /* NULL: all targets */
} accel_f64_ctx;

static void accel_f64_range(void *vp, int lo, int hi)
{
    accel_f64_ctx *c = (accel_f64_ctx *)vp;
    for (int t = lo; t < hi; ++t) {
        int i = c->tidx ? c->tidx[t] : t;
        double a[3] = {0.0, 0.0, 0.0};
        const double *pi = c->pos + 4 * (size_t)i;
        for (int j = 0; j < c->n; ++j) pair_f64(a, pi, c->pos + 4 * (size_t)j, c->eps2);
        c->acc[3 * (size_t)t + 0] = a[0];
        c->acc[3 * (size_t)t + 1] = a[1];
        c->acc[3 * (size_t)t + 2] = a[2];
    }
}

int orc_accel_f32(int n, const float *pos, float eps2, float *acc, int nthreads)
{
    if (n < 0 || (n > 0 && (!pos || !acc))) return 1;
    accel_f32_ctx c = {n, pos, eps2, acc};
    parallel_for(n, nthreads, accel_f32_range, &c);
    return 0;
}

int orc_accel_f64(int n, const double *pos, double eps2, double *acc, int nthreads)
{
    if (n < 0 || (n > 0 && (!pos || !acc))) return 1;
    accel_f64_ctx c = {n, pos, eps2, acc, NULL};
    parallel_for(n, nthreads, accel_f64_range, &c);
    return 0;
}

int orc_accel_subset_f64(int n, const double *pos, int nt, const int *tidx,
                         double eps2, double *acc, int nthreads)
{
    if (n < 0 || nt < 0 || (nt > 0 && (!pos || !acc || !tidx))) return 1;
    for (int t = 0; t < nt; ++t)
        if (tidx[t] < 0 || tidx[t] >= n) return 1;
    accel_f64_ctx c = {n, pos, eps2, acc, tidx};
    parallel_for(nt, nthreads, accel_f64_range, &c);
    return 0;
}

typedef struct {
    int n;
    const double *pos;
    double eps2;
    double *acc;
    double *phi;
    const int *tidx;
} accphi_ctx;

static void accphi_range(void *vp, int lo, int hi)
{
    accphi_ctx *c = (accphi_ctx *)vp;
    for (int t = lo; t < hi; ++t) {
        int i = c->tidx[t];
        const double *pi = c->pos + 4 * (size_t)i;
        double a[3] = {0.0, 0.0, 0.0}, ph = 0.0;
        for (int j = 0; j < c->n; ++j) {
            const double *pj = c->pos + 4 * (size_t)j;
            double r0 = pj[0] - pi[0], r1 = pj[1] - pi[1], r2 = pj[2] - pi[2];
            double d2 = r0 * r0 + r1 * r1 + r2 * r2 + c->eps2;
            double inv = 1.0 / sqrt(d2);
            double mi = pj[3] * inv;
            double s = mi * inv * inv;
            a[0] += r0 * s;
            a[1] += r1 * s;
            a[2] += r2 * s;
            if (j != i) ph += mi;
        }
        c->acc[3 * (size_t)t + 0] = a[0];
        c->acc[3 * (size_t)t + 1] = a[1];
        c->acc[3 * (size_t)t + 2] = a[2];
        c->phi[t] = ph;
    }
}

int orc_accel_phi_subset_f64(int n, const double *pos, int nt, const int *tidx,
                             double eps2, double *acc, double *phi, int nthreads)
{
    if (n < 0 || nt < 0 || (nt > 0 && (!pos || !acc || !phi || !tidx))) return 1;
    for (int t = 0; t < nt; ++t)
        if (tidx[t] < 0 || tidx[t] >= n) return 1;
    accphi_ctx c = {n, pos, eps2, acc, phi, tidx};
    parallel_for(nt, nthreads, accphi_range, &c);
    return 0;
}

/* ------------------------------------------------------------------ */
/* integrator (bodysystem.cc:135-182)                                  */
/* ------------------------------------------------------------------ */
static void integrate_f32(int n, float *pos, float *vel, const float *force,
                          float damping, float dt, int kick_mode, float G)
{
    for (int i = 0; i < n; ++i) {
        size_t idx = 4 * (size_t)i, fi = 3 * (size_t)i;
        float p[3] = {pos[idx], pos[idx + 1], pos[idx + 2]};
        float k = kick_mode == ORC_KICK_REFERENCE ? pos[idx + 3] : G;
        float v[3] = {vel[idx], vel[idx + 1], vel[idx + 2]};
        for (int d = 0; d < 3; ++d) v[d] += (force[fi + d] * k) * dt;
        for (int d = 0; d < 3; ++d) v[d] *= damping;
        for (int d = 0; d < 3; ++d) p[d] += v[d] * dt;
        for (int d = 0; d < 3; ++d) {
            pos[idx + d] = p[d];
            vel[idx + d] = v[d];
        }
    }
}

static void integrate_f64(int n, double *pos, double *vel, const double *force,
                          double damping, double dt, int kick_mode, double G)
{
    for (int i = 0; i < n; ++i) {
        size_t idx = 4 * (size_t)i, fi = 3 * (size_t)i;
        double p[3] = {pos[idx], pos[idx + 1], pos[idx + 2]};
        double k = kick_mode == ORC_KICK_REFERENCE ? pos[idx + 3] : G;
        double v[3] = {vel[idx], vel[idx + 1], vel[idx + 2]};
        for (int d = 0; d < 3; ++d) v[d] += (force[fi + d] * k) * dt;
        for (int d = 0; d < 3; ++d) v[d] *= damping;
        for (int d = 0; d < 3; ++d) p[d] += v[d] * dt;
        for (int d = 0; d < 3; ++d) {
            pos[idx + d] = p[d];
            vel[idx + d] = v[d];
        }
    }
}

int orc_step_f32(int n, float *pos, float *vel, float eps2, float damping,
                 float dt, int steps, int kick_mode, float G, int nthreads)
{
    if (n < 0 || steps < 0 || (n > 0 && (!pos || !vel))) return 1;
    if (kick_mode != ORC_KICK_REFERENCE && kick_mode != ORC_KICK_PHYSICAL) return 1;
    float *force = (float *)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
    if (!force) return 2;
    for (int s = 0; s < steps; ++s) {
        orc_accel_f32(n, pos, eps2, force, nthreads);
        integrate_f32(n, pos, vel, force, damping, dt, kick_mode, G);
    }
    free(force);
    return 0;
}

int orc_step_f64(int n, double *pos, double *vel, double eps2, double damping,
                 double dt, int steps, int kick_mode, double G, int nthreads)
{
    if (n < 0 || steps < 0 || (n > 0 && (!pos || !vel))) return 1;
    if (kick_mode != ORC_KICK_REFERENCE && kick_mode != ORC_KICK_PHYSICAL) return 1;
    double *force = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    if (!force) return 2;
    for (int s = 0; s < steps; ++s) {
        orc_accel_f64(n, pos, eps2, force, nthreads);
        integrate_f64(n, pos, vel, force, damping, dt, kick_mode, G);
    }
    free(force);
    return 0;
}

/* One step of the targets [i0, i1) only, against all n sources at pos_old:
 * the part of a step one thread of the reference's multi-GPU task computes
 * (benchapps/nbody/utc-snode-mgpu/mgpu/body_task_mgpu.cu:102-151: every
 * body's positions in, the local range's new positions out).  Writes the
 * range's positions to pos_new and its velocities in place; the other
 * entries of pos_new and vel are left as they are. */
typedef struct {
    int n, i0;
    const float *pos;
    float eps2;
    float *acc;
} accel_rng_ctx;

static void accel_rng_range(void *vp, int lo, int hi)
{
    accel_rng_ctx *c = (accel_rng_ctx *)vp;
    for (int t = lo; t < hi; ++t) {
        float a[3] = {0.f, 0.f, 0.f};
        const float *pi = c->pos + 4 * (size_t)(c->i0 + t);
        for (int j = 0; j < c->n; ++j) pair_f32(a, pi, c->pos + 4 * (size_t)j, c->eps2);
        c->acc[3 * (size_t)t + 0] = a[0];
        c->acc[3 * (size_t)t + 1] = a[1];
        c->acc[3 * (size_t)t + 2] = a[2];
    }
}

int orc_step_range_f32(int n, const float *pos_old, float *pos_new, float *vel, int i0, int i1,
                       float eps2, float damping, float dt, int kick_mode, float G, int nthreads)
{
    if (n < 0 || i0 < 0 || i1 < i0 || i1 > n || (n > 0 && (!pos_old || !pos_new || !vel))) return 1;
    if (kick_mode != ORC_KICK_REFERENCE && kick_mode != ORC_KICK_PHYSICAL) return 1;
    const int m = i1 - i0;
    float *force = (float *)malloc(sizeof(float) * 3 * (size_t)(m > 0 ? m : 1));
    if (!force) return 2;
    accel_rng_ctx c = {n, i0, pos_old, eps2, force};
    parallel_for(m, nthreads, accel_rng_range, &c);
    memcpy(pos_new + 4 * (size_t)i0, pos_old + 4 * (size_t)i0, sizeof(float) * 4 * (size_t)m);
    integrate_f32(m, pos_new + 4 * (size_t)i0, vel + 4 * (size_t)i0, force, damping, dt, kick_mode, G);
    free(force);
    return 0;
}

/* ------------------------------------------------------------------ */
/* energy and momentum                                                 */
/* ------------------------------------------------------------------ */
typedef struct {
    int n;
    const double *pos;
    double eps2;
    double *phi; /* per-target sum_j!=i m_j / sqrt(r^2+eps2) */
} pot_ctx;

static void pot_range(void *vp, int lo, int hi)
{
    pot_ctx *c = (pot_ctx *)vp;
    for (int i = lo; i < hi; ++i) {
        const double *pi = c->pos + 4 * (size_t)i;
        double s = 0.0;
        for (int j = 0; j < c->n; ++j) {
            if (j == i) continue;
            const double *pj = c->pos + 4 * (size_t)j;
            double r0 = pj[0] - pi[0], r1 = pj[1] - pi[1], r2 = pj[2] - pi[2];
            double d2 = r0 * r0 + r1 * r1 + r2 * r2 + c->eps2;
            s += pj[3] / sqrt(d2);
        }
        c->phi[i] = s;
    }
}

int orc_energy_f64(int n, const double *pos, const double *vel, double eps2,
                   double G, double *out, int nthreads)
{
    if (n < 0 || !out || (n > 0 && (!pos || !vel))) return 1;
    double *phi = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!phi) return 2;
    pot_ctx c = {n, pos, eps2, phi};
    parallel_for(n, nthreads, pot_range, &c);
    double ke = 0.0, pe = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    for (int i = 0; i < n; ++i) {
        const double *p = pos + 4 * (size_t)i, *v = vel + 4 * (size_t)i;
        double m = p[3];
        ke += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        pe += -0.5 * G * m * phi[i];
        px += m * v[0];
        py += m * v[1];
        pz += m * v[2];
    }
    out[0] = ke;
    out[1] = pe;
    out[2] = px;
    out[3] = py;
    out[4] = pz;
    free(phi);
    return 0;
}

/* ------------------------------------------------------------------ */
/* FP64 reference adjoint                                               */
/* ------------------------------------------------------------------ */
/* With bare accelerations a_i = sum_j m_j r_ij inv^3 (r_ij = x_j - x_i,
 * inv = (|r|^2+eps2)^-1/2) and per-body kick factor k_i (m_i or G):
 *   v' = D (v + k a dt),  x' = x + v' dt.
 * Backward through one step, with lx = dL/dx', lv = dL/dv':
 *   mu = lv + dt lx;  dL/dv = D mu;  g_i = D dt k_i mu_i;
 *   dL/dx_k = lx_k + sum_j K(r_kj) (m_k g_j - m_j g_k),
 *             K(r) = inv^3 I - 3 inv^5 r r^T;
 *   dL/dm_k += -sum_j inv^3 (r_kj . g_j)   (through a)
 *            + D dt mu_k . a_k  when k_k = m_k (reference kick). */
typedef struct {
    int n;
    const double *pos; /* 4n at step t */
    const double *g;   /* 3n */
    double eps2;
    double *jtg; /* 3n out */
    double *dm;  /* n out (through a only) */
} vjp_ctx;

static void vjp_range(void *vp, int lo, int hi)
{
    vjp_ctx *c = (vjp_ctx *)vp;
    for (int k = lo; k < hi; ++k) {
        const double *pk = c->pos + 4 * (size_t)k;
        const double *gk = c->g + 3 * (size_t)k;
        double mk = pk[3];
        double o[3] = {0, 0, 0}, dm = 0.0;
        for (int j = 0; j < c->n; ++j) {
            if (j == k) continue;
            const double *pj = c->pos + 4 * (size_t)j;
            const double *gj = c->g + 3 * (size_t)j;
            double mj = pj[3];
            double r[3] = {pj[0] - pk[0], pj[1] - pk[1], pj[2] - pk[2]};
            double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + c->eps2;
            double inv = 1.0 / sqrt(d2);
            double inv3 = inv * inv * inv;
            double inv5 = inv3 * inv * inv;
            double w[3];
            for (int d = 0; d < 3; ++d) w[d] = mk * gj[d] - mj * gk[d];
            double rw = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
            for (int d = 0; d < 3; ++d) o[d] += inv3 * w[d] - 3.0 * inv5 * rw * r[d];
            double rg = r[0] * gj[0] + r[1] * gj[1] + r[2] * gj[2];
            dm -= inv3 * rg;
        }
        for (int d = 0; d < 3; ++d) c->jtg[3 * (size_t)k + d] = o[d];
        c->dm[k] = dm;
    }
}

static int forward_store_f64(int n, const double *pos0, const double *vel0,
                             double eps2, double damping, double dt, int steps,
                             int kick_mode, double G, double *xs, double *vs,
                             double *as, int nthreads)
{
    size_t sz = 4 * (size_t)n;
    memcpy(xs, pos0, sizeof(double) * sz);
    memcpy(vs, vel0, sizeof(double) * sz);
    for (int t = 0; t < steps; ++t) {
        double *x = xs + sz * t, *v = vs + sz * t;
        double *xn = xs + sz * (t + 1), *vn = vs + sz * (t + 1);
        double *a = as + 3 * (size_t)n * t;
        orc_accel_f64(n, x, eps2, a, nthreads);
        memcpy(xn, x, sizeof(double) * sz);
        memcpy(vn, v, sizeof(double) * sz);
        integrate_f64(n, xn, vn, a, damping, dt, kick_mode, G);
    }
    return 0;
}

int orc_loss_f64(int n, const double *pos0, const double *vel0, double eps2,
                 double damping, double dt, int steps, int kick_mode, double G,
                 const double *y, double *loss, int nthreads)
{
    if (n < 0 || steps < 0 || !loss || (n > 0 && (!pos0 || !vel0 || !y))) return 1;
    size_t sz = 4 * (size_t)(n > 0 ? n : 1);
    double *x = (double *)malloc(sizeof(double) * sz);
    double *v = (double *)malloc(sizeof(double) * sz);
    if (!x || !v) {
        free(x);
        free(v);
        return 2;
    }
    memcpy(x, pos0, sizeof(double) * 4 * (size_t)n);
    memcpy(v, vel0, sizeof(double) * 4 * (size_t)n);
    int rc = orc_step_f64(n, x, v, eps2, damping, dt, steps, kick_mode, G, nthreads);
    double L = 0.0;
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double e = x[4 * (size_t)i + d] - y[3 * (size_t)i + d];
            L += e * e;
        }
    *loss = L;
    free(x);
    free(v);
    return rc;
}

int orc_adjoint_f64(int n, const double *pos0, const double *vel0, double eps2,
                    double damping, double dt, int steps, int kick_mode,
                    double G, const double *y, double *loss, double *gx,
                    double *gv, double *gm, int nthreads)
{
    if (n <= 0 || steps < 0 || !pos0 || !vel0 || !y || !loss || !gx || !gv || !gm)
        return 1;
    if (kick_mode != ORC_KICK_REFERENCE && kick_mode != ORC_KICK_PHYSICAL) return 1;
    size_t sz = 4 * (size_t)n, n3 = 3 * (size_t)n;
    double *xs = (double *)malloc(sizeof(double) * sz * (steps + 1));
    double *vs = (double *)malloc(sizeof(double) * sz * (steps + 1));
    double *as = (double *)malloc(sizeof(double) * n3 * (steps > 0 ? steps : 1));
    double *lx = (double *)malloc(sizeof(double) * n3);
    double *lv = (double *)malloc(sizeof(double) * n3);
    double *g = (double *)malloc(sizeof(double) * n3);
    double *jtg = (double *)malloc(sizeof(double) * n3);
    double *dma = (double *)malloc(sizeof(double) * n);
    if (!xs || !vs || !as || !lx || !lv || !g || !jtg || !dma) {
        free(xs); free(vs); free(as); free(lx); free(lv); free(g); free(jtg); free(dma);
        return 2;
    }
    forward_store_f64(n, pos0, vel0, eps2, damping, dt, steps, kick_mode, G, xs,
                      vs, as, nthreads);
    const double *xT = xs + sz * steps;
    double L = 0.0;
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double e = xT[4 * (size_t)i + d] - y[3 * (size_t)i + d];
            L += e * e;
            lx[3 * (size_t)i + d] = 2.0 * e;
            lv[3 * (size_t)i + d] = 0.0;
        }
    for (int i = 0; i < n; ++i) gm[i] = 0.0;
    for (int t = steps - 1; t >= 0; --t) {
        const double *x = xs + sz * t;
        const double *a = as + n3 * t;
        for (int i = 0; i < n; ++i) {
            double k = kick_mode == ORC_KICK_REFERENCE ? x[4 * (size_t)i + 3] : G;
            double mua = 0.0;
            for (int d = 0; d < 3; ++d) {
                size_t q = 3 * (size_t)i + d;
                double mu = lv[q] + dt * lx[q];
                lv[q] = damping * mu;
                g[q] = damping * dt * k * mu;
                mua += mu * a[q];
            }
            if (kick_mode == ORC_KICK_REFERENCE) gm[i] += damping * dt * mua;
        }
        vjp_ctx c = {n, x, g, eps2, jtg, dma};
        parallel_for(n, nthreads, vjp_range, &c);
        for (size_t q = 0; q < n3; ++q) lx[q] += jtg[q];
        for (int i = 0; i < n; ++i) gm[i] += dma[i];
    }
    memcpy(gx, lx, sizeof(double) * n3);
    memcpy(gv, lv, sizeof(double) * n3);
    *loss = L;
    free(xs); free(vs); free(as); free(lx); free(lv); free(g); free(jtg); free(dma);
    return 0;
}

/* ------------------------------------------------------------------ */
/* initial conditions (nbody.h:22-250)                                 */
/* ------------------------------------------------------------------ */
typedef struct { float x, y, z; } v3f;

static float v3_normalize(v3f *v)
{
    float dist = sqrtf(v->x * v->x + v->y * v->y + v->z * v->z);
    if (dist > 1e-6) {
        v->x /= dist;
        v->y /= dist;
        v->z /= dist;
    }
    return dist;
}

static float v3_dot(v3f a, v3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

static v3f v3_cross(v3f a, v3f b)
{
    v3f r;
    r.x = a.y * b.z - a.z * b.y;
    r.y = a.z * b.x - a.x * b.z;
    r.z = a.x * b.y - a.y * b.x;
    return r;
}

static inline float urand11(void) { return rand() / (float)RAND_MAX * 2 - 1; }

void orc_srand(unsigned seed) { srand(seed); }

#define DEFINE_RANDOMIZE(NAME, T)                                                 \
int NAME(int config, T *pos, T *vel, float clusterScale, float velocityScale,     \
         int numBodies)                                                           \
{                                                                                 \
    if (numBodies < 0 || (numBodies > 0 && (!pos || !vel))) return 1;             \
    int p = 0, v = 0, i = 0;                                                      \
    if (config == 1) { /* SHELL, nbody.h:141-194 */                               \
        float scale = clusterScale;                                               \
        float vscale = scale * velocityScale;                                     \
        float inner = 2.5f * scale;                                               \
        float outer = 4.0f * scale;                                               \
        while (i < numBodies) {                                                   \
            float x = urand11(), y = urand11(), z = urand11();                    \
            v3f point = {x, y, z};                                                \
            float len = v3_normalize(&point);                                     \
            if (len > 1) continue;                                                \
            pos[p++] = point.x * (inner + (outer - inner) * rand() / (float)RAND_MAX); \
            pos[p++] = point.y * (inner + (outer - inner) * rand() / (float)RAND_MAX); \
            pos[p++] = point.z * (inner + (outer - inner) * rand() / (float)RAND_MAX); \
            pos[p++] = 1.0f;                                                      \
            v3f axis = {0.0f, 0.0f, 1.0f};                                        \
            v3_normalize(&axis);                                                  \
            if (1 - v3_dot(point, axis) < 1e-6) {                                 \
                axis.x = point.y;                                                 \
                axis.y = point.x;                                                 \
                v3_normalize(&axis);                                              \
            }                                                                     \
            v3f vv = {(float)pos[4 * i], (float)pos[4 * i + 1], (float)pos[4 * i + 2]}; \
            vv = v3_cross(vv, axis);                                              \
            vel[v++] = vv.x * vscale;                                             \
            vel[v++] = vv.y * vscale;                                             \
            vel[v++] = vv.z * vscale;                                             \
            vel[v++] = 1.0f;                                                      \
            i++;                                                                  \
        }                                                                         \
    } else if (config == 2) { /* EXPAND, nbody.h:196-233 */                       \
        float scale = clusterScale * numBodies / (1024.f);                        \
        if (scale < 1.0f) scale = clusterScale;                                   \
        float vscale = scale * velocityScale;                                     \
        while (i < numBodies) {                                                   \
            v3f point;                                                            \
            point.x = urand11();                                                  \
            point.y = urand11();                                                  \
            point.z = urand11();                                                  \
            float lenSqr = v3_dot(point, point);                                  \
            if (lenSqr > 1) continue;                                             \
            pos[p++] = point.x * scale;                                           \
            pos[p++] = point.y * scale;                                           \
            pos[p++] = point.z * scale;                                           \
            pos[p++] = 1.0f;                                                      \
            vel[v++] = point.x * vscale;                                          \
            vel[v++] = point.y * vscale;                                          \
            vel[v++] = point.z * vscale;                                          \
            vel[v++] = 1.0f;                                                      \
            i++;                                                                  \
        }                                                                         \
    } else { /* RANDOM (and default), nbody.h:95-139 */                          \
        float scale = clusterScale * (1.0f > numBodies / (1024.0f) ? 1.0f         \
                                                 : numBodies / (1024.0f));        \
        float vscale = velocityScale * scale;                                     \
        while (i < numBodies) {                                                   \
            v3f point;                                                            \
            point.x = urand11();                                                  \
            point.y = urand11();                                                  \
            point.z = urand11();                                                  \
            float lenSqr = v3_dot(point, point);                                  \
            if (lenSqr > 1) continue;                                             \
            v3f velocity;                                                         \
            velocity.x = urand11();                                               \
            velocity.y = urand11();                                               \
            velocity.z = urand11();                                               \
            lenSqr = v3_dot(velocity, velocity);                                  \
            if (lenSqr > 1) continue;                                             \
            pos[p++] = point.x * scale;                                           \
            pos[p++] = point.y * scale;                                           \
            pos[p++] = point.z * scale;                                           \
            pos[p++] = 1.0f;                                                      \
            vel[v++] = velocity.x * vscale;                                       \
            vel[v++] = velocity.y * vscale;                                       \
            vel[v++] = velocity.z * vscale;                                       \
            vel[v++] = 1.0f;                                                      \
            i++;                                                                  \
        }                                                                         \
    }                                                                             \
    return 0;                                                                     \
}

DEFINE_RANDOMIZE(orc_randomize_f32, float)
DEFINE_RANDOMIZE(orc_randomize_f64, double)

/* demoParams[] and the per-N override, seq/nbody_main.cc:57-66 and 115-144
 * (identical in utc/nbody_main.cc:57-66, 160-189). */
void orc_demo_params(int paraSelect, int n, float *dt, float *clusterScale,
                     float *velocityScale, float *softening, float *damping)
{
    static const float tbl[7][5] = {
        {0.016f, 1.54f, 8.0f, 0.1f, 1.0f},
        {0.016f, 0.68f, 20.0f, 0.1f, 1.0f},
        {0.0006f, 0.16f, 1000.0f, 1.0f, 1.0f},
        {0.0006f, 0.16f, 1000.0f, 1.0f, 1.0f},
        {0.0019f, 0.32f, 276.0f, 1.0f, 1.0f},
        {0.0016f, 0.32f, 272.0f, 0.145f, 1.0f},
        {0.016000f, 6.040000f, 0.000000f, 1.000000f, 1.000000f},
    };
    if (paraSelect > 6 || paraSelect < 0) paraSelect = 0;
    float cs = tbl[paraSelect][1], vs = tbl[paraSelect][2];
    if (n <= 1024) { cs = 1.52f; vs = 2.f; }
    else if (n <= 2048) { cs = 1.56f; vs = 2.64f; }
    else if (n <= 4096) { cs = 1.68f; vs = 2.98f; }
    else if (n <= 8192) { cs = 1.98f; vs = 2.9f; }
    else if (n <= 16384) { cs = 1.54f; vs = 8.f; }
    else if (n <= 32768) { cs = 1.44f; vs = 11.f; }
    *dt = tbl[paraSelect][0];
    *clusterScale = cs;
    *velocityScale = vs;
    *softening = tbl[paraSelect][3];
    *damping = tbl[paraSelect][4];
}
