/*
 * nbody_oracle.h -- CPU restatement of the UTC nbody all-pairs step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GB300 kernels: only the test suite, the smoke check and the benchmark's CPU
 * baseline leg load it.  The product path (utc_gb300) never links or calls it.
 *
 * Every function restates the reference's sequential algorithm with the same
 * arithmetic order, so that a float or double run is bit-identical to the
 * reference's BodySystem<T> (pinned by the tests against the reference's own
 * golden frames, benchapps/nbody/seq/nbody_outpos.txt).  Build with
 * -ffp-contract=off: the reference was compiled for x86-64 without FMA, and a
 * contracted build (the default for GNU C on aarch64) would differ in the last
 * bit.
 *
 * Reference files (paths within the UTC project, utc-0.1/):
 *   benchapps/nbody/seq/bodysystem.h:71-96   bodyBodyInteraction<T>
 *   benchapps/nbody/seq/bodysystem.cc:103-133 _computeNBodyGravitation
 *   benchapps/nbody/seq/bodysystem.cc:135-182 _integrateNBodySystem
 *   benchapps/nbody/seq/bodysystem.cc:64-73   update = forces, then integrate
 *   benchapps/nbody/seq/nbody.h:89-250        randomizeBodies (glibc rand())
 */
#ifndef NBODY_ORACLE_H_
#define NBODY_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* Kick factor applied to the accumulated acceleration sum.
 * ORC_KICK_REFERENCE: multiply by the target's own pos.w, exactly as the
 *   reference does (bodysystem.cc:149, "invMass = m_pos[index+3]").
 * ORC_KICK_PHYSICAL: multiply by the constant G (a_i = G sum_j m_j r/|r|^3). */
enum { ORC_KICK_REFERENCE = 0, ORC_KICK_PHYSICAL = 1 };

/* Accelerations (the bare sum over j of m_j r_ij / (r^2+eps2)^1.5, no kick
 * factor), acc is 3*n, pos is 4*n (x, y, z, m).  Each target sums its sources
 * in index order j = 0..n-1 as bodysystem.cc:106-125 does.  nthreads splits
 * the targets over host threads; results do not depend on it. */
int orc_accel_f32(int n, const float *pos, float eps2, float *acc, int nthreads);
int orc_accel_f64(int n, const double *pos, double eps2, double *acc, int nthreads);

/* Same sum for a subset of targets (target indices tidx[0..nt)) against all n
 * sources, in double; used as the FP64 all-pairs oracle on a subsample. */
int orc_accel_subset_f64(int n, const double *pos, int nt, const int *tidx,
                         double eps2, double *acc, int nthreads);

/* For targets tidx[0..nt): acceleration sum (as above, acc 3*nt) and the
 * potential sum phi = sum_{j != i} m_j / sqrt(r^2 + eps2) (phi nt), double. */
int orc_accel_phi_subset_f64(int n, const double *pos, int nt, const int *tidx,
                             double eps2, double *acc, double *phi, int nthreads);

/* `steps` calls of BodySystem<T>::update(dt): all forces from the old
 * positions, then kick (x kick factor), damping, drift.  pos/vel (4*n) are
 * updated in place; pos.w and vel.w pass through unchanged. */
int orc_step_f32(int n, float *pos, float *vel, float eps2, float damping,
                 float dt, int steps, int kick_mode, float G, int nthreads);
int orc_step_f64(int n, double *pos, double *vel, double eps2, double damping,
                 double dt, int steps, int kick_mode, double G, int nthreads);
/* One step of targets [i0, i1) against all n sources (a shard of the
 * multi-GPU target partition); pos_new/vel receive that range only. */
int orc_step_range_f32(int n, const float *pos_old, float *pos_new, float *vel, int i0, int i1,
                       float eps2, float damping, float dt, int kick_mode, float G, int nthreads);

/* Total energy and momentum of a state in double:
 * out[0] = kinetic  sum_i 0.5 m_i |v_i|^2
 * out[1] = potential -0.5 G sum_i sum_{j!=i} m_i m_j / sqrt(r^2 + eps2)
 * out[2..4] = momentum sum_i m_i v_i */
int orc_energy_f64(int n, const double *pos, const double *vel, double eps2,
                   double G, double *out, int nthreads);

/* Reverse-mode gradient of L = sum_i |x_T,i - y_i|^2 through `steps` double
 * steps (same update rule as orc_step_f64).  y is 3*n.  Writes the loss and
 * dL/dx0 (3n), dL/dv0 (3n), dL/dm (n).  All intermediate states are stored
 * (this is the plain reference adjoint, meant for small n). */
int orc_adjoint_f64(int n, const double *pos0, const double *vel0, double eps2,
                    double damping, double dt, int steps, int kick_mode,
                    double G, const double *y, double *loss, double *gx,
                    double *gv, double *gm, int nthreads);

/* Loss only (same definition), for finite differences. */
int orc_loss_f64(int n, const double *pos0, const double *vel0, double eps2,
                 double damping, double dt, int steps, int kick_mode, double G,
                 const double *y, double *loss, int nthreads);

/* randomizeBodies restated (nbody.h:89-250).  config: 0 RANDOM, 1 SHELL,
 * 2 EXPAND.  Uses the C library's rand(); call orc_srand(1) first to start
 * from the state a fresh process has.  vel gets 4 values per body (the
 * reference's vec4vel=true).  The colour stream of the reference is not drawn:
 * it comes after positions and velocities and does not change them. */
void orc_srand(unsigned seed);
int orc_randomize_f32(int config, float *pos, float *vel, float clusterScale,
                      float velocityScale, int n);
int orc_randomize_f64(int config, double *pos, double *vel, float clusterScale,
                      float velocityScale, int n);

/* The app's per-N preset of cluster and velocity scale
 * (seq/nbody_main.cc:115-144), for demo parameter set `paraSelect`. */
void orc_demo_params(int paraSelect, int n, float *dt, float *clusterScale,
                     float *velocityScale, float *softening, float *damping);

#ifdef __cplusplus
}
#endif
#endif
