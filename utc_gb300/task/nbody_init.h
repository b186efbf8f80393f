/*
 * nbody_init.h -- the app's body initialisers and frame writer as UTC tasks.
 *
 * NbodyInit<T>::runImpl restates randomizeBodies (benchapps/nbody/utc/
 * task.cc:10-169, identical to seq/nbody.h:89-250): RANDOM, SHELL and EXPAND
 * configurations drawn from the C library's rand() in the same order and
 * with the same float arithmetic, so a fresh process produces the
 * reference's bodies exactly.  Output<T>::runImpl writes one text frame as
 * task.cc:172-181 does.  The preset table is seq/nbody_main.cc:57-66 with
 * the per-N override of utc/nbody_main.cc:160-189.
 */
#ifndef UTC_GB300_NBODY_INIT_H_
#define UTC_GB300_NBODY_INIT_H_

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "utc_standin.h"

enum NBodyConfig { NBODY_CONFIG_RANDOM, NBODY_CONFIG_SHELL, NBODY_CONFIG_EXPAND, NBODY_NUM_CONFIGS };

struct NBodyParams {
    float m_timestep, m_clusterScale, m_velocityScale, m_softening, m_damping;
};

inline NBodyParams nbody_demo_params(int paraSelect, int numBodies)
{
    static const NBodyParams demo[7] = {
        {0.016f, 1.54f, 8.0f, 0.1f, 1.0f},      {0.016f, 0.68f, 20.0f, 0.1f, 1.0f},
        {0.0006f, 0.16f, 1000.0f, 1.0f, 1.0f},  {0.0006f, 0.16f, 1000.0f, 1.0f, 1.0f},
        {0.0019f, 0.32f, 276.0f, 1.0f, 1.0f},   {0.0016f, 0.32f, 272.0f, 0.145f, 1.0f},
        {0.016f, 6.04f, 0.0f, 1.0f, 1.0f},
    };
    if (paraSelect > 6 || paraSelect < 0) paraSelect = 0;
    NBodyParams p = demo[paraSelect];
    const struct { int n; float cs, vs; } over[] = {
        {1024, 1.52f, 2.f}, {2048, 1.56f, 2.64f}, {4096, 1.68f, 2.98f},
        {8192, 1.98f, 2.9f}, {16384, 1.54f, 8.f}, {32768, 1.44f, 11.f},
    };
    for (const auto &o : over)
        if (numBodies <= o.n) {
            p.m_clusterScale = o.cs;
            p.m_velocityScale = o.vs;
            break;
        }
    return p;
}

namespace nbinit {
struct v3 { float x, y, z; };
inline float normalize(v3 &v)
{
    float d = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    if (d > 1e-6) {
        v.x /= d;
        v.y /= d;
        v.z /= d;
    }
    return d;
}
inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline v3 cross(v3 a, v3 b)
{
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float urand11() { return rand() / (float)RAND_MAX * 2 - 1; }
}  // namespace nbinit

template <typename T>
class NbodyInit : public UserTaskBase {
public:
    void initImpl() {}
    void runImpl(NBodyConfig config, T *pos, T *vel, float *color, float clusterScale,
                 float velocityScale, int numBodies, bool vec4vel)
    {
        using namespace nbinit;
        int p = 0, v = 0, i = 0;
        if (config == NBODY_CONFIG_SHELL) {
            float scale = clusterScale, vscale = scale * velocityScale;
            float inner = 2.5f * scale, outer = 4.0f * scale;
            while (i < numBodies) {
                float x = urand11(), y = urand11(), z = urand11();
                v3 point = {x, y, z};
                if (normalize(point) > 1) continue;
                pos[p++] = point.x * (inner + (outer - inner) * rand() / (float)RAND_MAX);
                pos[p++] = point.y * (inner + (outer - inner) * rand() / (float)RAND_MAX);
                pos[p++] = point.z * (inner + (outer - inner) * rand() / (float)RAND_MAX);
                pos[p++] = 1.0f;
                v3 axis = {0.0f, 0.0f, 1.0f};
                normalize(axis);
                if (1 - dot(point, axis) < 1e-6) {
                    axis.x = point.y;
                    axis.y = point.x;
                    normalize(axis);
                }
                v3 vv = {(float)pos[4 * i], (float)pos[4 * i + 1], (float)pos[4 * i + 2]};
                vv = cross(vv, axis);
                vel[v++] = vv.x * vscale;
                vel[v++] = vv.y * vscale;
                vel[v++] = vv.z * vscale;
                if (vec4vel) vel[v++] = 1.0f;
                i++;
            }
        } else if (config == NBODY_CONFIG_EXPAND) {
            float scale = clusterScale * numBodies / (1024.f);
            if (scale < 1.0f) scale = clusterScale;
            float vscale = scale * velocityScale;
            while (i < numBodies) {
                v3 point = {urand11(), 0, 0};
                point.y = urand11();
                point.z = urand11();
                if (dot(point, point) > 1) continue;
                pos[p++] = point.x * scale;
                pos[p++] = point.y * scale;
                pos[p++] = point.z * scale;
                pos[p++] = 1.0f;
                vel[v++] = point.x * vscale;
                vel[v++] = point.y * vscale;
                vel[v++] = point.z * vscale;
                if (vec4vel) vel[v++] = 1.0f;
                i++;
            }
        } else {
            float scale = clusterScale * (1.0f > numBodies / (1024.0f) ? 1.0f : numBodies / (1024.0f));
            float vscale = velocityScale * scale;
            while (i < numBodies) {
                v3 point = {urand11(), 0, 0};
                point.y = urand11();
                point.z = urand11();
                if (dot(point, point) > 1) continue;
                v3 velocity = {urand11(), 0, 0};
                velocity.y = urand11();
                velocity.z = urand11();
                if (dot(velocity, velocity) > 1) continue;
                pos[p++] = point.x * scale;
                pos[p++] = point.y * scale;
                pos[p++] = point.z * scale;
                pos[p++] = 1.0f;
                vel[v++] = velocity.x * vscale;
                vel[v++] = velocity.y * vscale;
                vel[v++] = velocity.z * vscale;
                if (vec4vel) vel[v++] = 1.0f;
                i++;
            }
        }
        if (color) {
            int c = 0;
            for (int k = 0; k < numBodies; k++) {
                color[c++] = rand() / (float)RAND_MAX;
                color[c++] = rand() / (float)RAND_MAX;
                color[c++] = rand() / (float)RAND_MAX;
                color[c++] = 1.0f;
            }
        }
    }
};

template <typename T>
class Output : public UserTaskBase {
public:
    void initImpl() {}
    void runImpl(FILE **fp, T *buffer, float timestamp, int numBodies)
    {
        std::fprintf(*fp, "%f\n", timestamp);
        for (int j = 0; j < numBodies; j++) {
            std::fprintf(*fp, "%.5f ", (double)buffer[j * 4 + 0]);
            std::fprintf(*fp, "%.5f ", (double)buffer[j * 4 + 1]);
            std::fprintf(*fp, "%.5f ", (double)buffer[j * 4 + 2]);
            std::fprintf(*fp, "%.5f\n", (double)buffer[j * 4 + 3]);
        }
    }
};

#endif
