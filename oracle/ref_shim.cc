/*
 * ref_shim.cc -- C entry points around the reference's own sequential nbody
 * code, compiled from the reference sources where they lie (see
 * oracle/Makefile).  Only the build recipe's output, oracle/_ref/libnbref.so,
 * contains reference code; this file holds none.
 *
 * TEST INFRASTRUCTURE ONLY: it lets the tests check the oracle restatement
 * (nbody_oracle.c) against the reference's BodySystem<T>
 * (benchapps/nbody/seq/bodysystem.cc) and randomizeBodies
 * (benchapps/nbody/seq/nbody.h:89-250) bit for bit.
 */
#include <cstdlib>
#include <cstring>

#include "bodysystem.h"
#include "nbody.h"

template <typename T>
static int run_impl(int n, T *pos, T *vel, T softening, T damping, T dt, int steps)
{
    /* bodysystem.cc:112-125 unrolls the source loop by 4 and reads past the
     * end unless n is a multiple of 4 */
    if (n <= 0 || (n % 4) != 0 || steps < 0 || !pos || !vel) return 1;
    BodySystem<T> nbody((unsigned)n);
    nbody.setDamping(damping);
    nbody.setSoftening(softening); /* squares it, bodysystem.h:21-23 */
    nbody.setPosArray(pos);
    nbody.setVelArray(vel);
    for (int s = 0; s < steps; ++s) nbody.update(dt);
    std::memcpy(pos, nbody.getPosArray(), sizeof(T) * 4 * (size_t)n);
    std::memcpy(vel, nbody.getVelArray(), sizeof(T) * 4 * (size_t)n);
    return 0;
}

extern "C" {

void ref_srand(unsigned seed) { srand(seed); }

int ref_randomize_f32(int config, float *pos, float *vel, float clusterScale,
                      float velocityScale, int n)
{
    randomizeBodies((NBodyConfig)config, pos, vel, (float *)0, clusterScale,
                    velocityScale, n, true);
    return 0;
}

int ref_randomize_f64(int config, double *pos, double *vel, float clusterScale,
                      float velocityScale, int n)
{
    randomizeBodies((NBodyConfig)config, pos, vel, (float *)0, clusterScale,
                    velocityScale, n, true);
    return 0;
}

int ref_run_f32(int n, float *pos, float *vel, float softening, float damping,
                float dt, int steps)
{
    return run_impl<float>(n, pos, vel, softening, damping, dt, steps);
}

int ref_run_f64(int n, double *pos, double *vel, double softening,
                double damping, double dt, int steps)
{
    return run_impl<double>(n, pos, vel, softening, damping, dt, steps);
}

} /* extern "C" */
