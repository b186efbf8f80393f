"""Host restatement of the GPU initial-condition generator -- TEST
INFRASTRUCTURE ONLY (imported by tests/test_ics.py).

It restates, in numpy FP64, the counter-based scheme of
utc_gb300/csrc/nb_ics.cu (nb_ics_generate) so that the generator's output can
be compared with an independent computation rather than only with
distribution shapes:

* stream k of body i under seed s is splitmix64(s ^ splitmix64(256 i + k)),
  SplitMix64 being the finaliser of Steele, Lea & Flood (2014) with its
  published increment and multipliers (pinned by the published known-answer
  sequence in tests/test_ics.py); u01 takes its top 53 bits;
* kind 0, uniform cube: x = 2u - 1 from streams 0-2, v = vmax (2u - 1) from
  4-6, m = (0.5 + u_3) / n;
* kind 1, Plummer sphere (Aarseth, Henon & Wielen 1974): radius from stream
  0, direction from 1 and 2, speed fraction q by rejection (streams 8 + 2t,
  9 + 2t, 64 tries, falling back to sqrt(2/9)), velocity direction from 3
  and 4, masses M / n; then the mass-weighted centre and mean velocity,
  summed in FP64 from the stored (possibly float) values, are subtracted;
* kinds 2, 3, 4: the reference app's random, shell and expand
  configurations (benchapps/nbody/seq/nbody.h:89-250: same arithmetic
  structure, with the counter streams in place of rand()): a point of the
  unit ball by rejection from the cube (3 streams per try from stream 8,
  40 tries; random draws its velocity point from stream 128 on), shell radii
  from streams 128-130 and the velocity pos x axis with axis z, or (y, x, 1)
  normalised next to the pole.

Where the GPU and numpy evaluate the same IEEE operations (products, sums,
divisions and square roots without a fused multiply-add) the results are
equal bit for bit: the cube, random and expand configurations.  The shell
normalisation and velocity (which the compiler may fuse into multiply-adds),
and the Plummer sampler (CUDA's rcbrt, rsqrt and sincospi against numpy's
cbrt, sqrt and sin/cos of pi x) agree to a few units in the last place.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(z):
    """The SplitMix64 output function of state z (uint64 array or scalar):
    add the golden-ratio increment, then the two xor-shift-multiply rounds."""
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def u01(seed, ids, k):
    """Uniform doubles in [0, 1): stream k of bodies `ids` under `seed`."""
    ids = np.asarray(ids, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = splitmix64(np.uint64(seed) ^ splitmix64(ids * np.uint64(256) + np.uint64(k)))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _ball_point(seed, ids, k0):
    """Point of the unit ball by rejection from the cube, 40 tries of 3
    streams from k0; the last candidate is pulled to radius 0.5 if all
    miss."""
    n = ids.size
    x = np.zeros(n)
    y = np.zeros(n)
    z = np.zeros(n)
    ln = np.zeros(n)
    todo = np.ones(n, dtype=bool)
    for t in range(40):
        idx = np.nonzero(todo)[0]
        if idx.size == 0:
            break
        sub = ids[idx]
        cx = 2.0 * u01(seed, sub, k0 + 3 * t) - 1.0
        cy = 2.0 * u01(seed, sub, k0 + 3 * t + 1) - 1.0
        cz = 2.0 * u01(seed, sub, k0 + 3 * t + 2) - 1.0
        cl = np.sqrt(cx * cx + cy * cy + cz * cz)
        x[idx], y[idx], z[idx], ln[idx] = cx, cy, cz, cl
        todo[idx[cl <= 1.0]] = False
    if todo.any():
        idx = np.nonzero(todo)[0]
        s = 0.5 / ln[idx]
        x[idx] *= s
        y[idx] *= s
        z[idx] *= s
        ln[idx] = 0.5
    return x, y, z, ln


def _store(a, precision):
    """The kernel's store into float4 (round to nearest) or double4."""
    return a.astype(np.float32) if precision == "f32" else a


def generate(kind, n, seed, a=1.0, G=1.0, M=1.0, vmax=0.01, precision="f32"):
    """(pos, vel) as the GPU generator stores them: (n, 4) float32 or float64.
    kind: "cube", "plummer", "random", "shell" or "expand"."""
    ids = np.arange(n, dtype=np.uint64)
    pos = np.zeros((n, 4))
    vel = np.zeros((n, 4))
    vel[:, 3] = 1.0
    if kind == "cube":
        for c in range(3):
            pos[:, c] = 2.0 * u01(seed, ids, c) - 1.0
            vel[:, c] = vmax * (2.0 * u01(seed, ids, 4 + c) - 1.0)
        pos[:, 3] = (0.5 + u01(seed, ids, 3)) / n
        return _store(pos, precision), _store(vel, precision)
    if kind in ("random", "expand"):
        x, y, z, _ = _ball_point(seed, ids, 8)
        pos[:, 3] = 1.0
        if kind == "expand":
            s = a * (n / 1024.0)
            if s < 1.0:
                s = a
            pos[:, 0], pos[:, 1], pos[:, 2] = x * s, y * s, z * s
            vel[:, 0], vel[:, 1], vel[:, 2] = x * s * vmax, y * s * vmax, z * s * vmax
            return _store(pos, precision), _store(vel, precision)
        s = a * max(1.0, n / 1024.0)
        vx, vy, vz, _ = _ball_point(seed, ids, 128)
        pos[:, 0], pos[:, 1], pos[:, 2] = x * s, y * s, z * s
        vel[:, 0], vel[:, 1], vel[:, 2] = vx * s * vmax, vy * s * vmax, vz * s * vmax
        return _store(pos, precision), _store(vel, precision)
    if kind == "shell":
        x, y, z, ln = _ball_point(seed, ids, 8)
        big = ln > 1e-6
        il = np.where(big, 1.0 / np.where(big, ln, 1.0), 1.0)
        x, y, z = np.where(big, x * il, x), np.where(big, y * il, y), np.where(big, z * il, z)
        inner, outer = 2.5 * a, 4.0 * a
        px = x * (inner + (outer - inner) * u01(seed, ids, 128))
        py = y * (inner + (outer - inner) * u01(seed, ids, 129))
        pz = z * (inner + (outer - inner) * u01(seed, ids, 130))
        ax, ay, az = np.zeros(n), np.zeros(n), np.ones(n)
        pole = (1.0 - z) < 1e-6
        if pole.any():
            ilp = 1.0 / np.sqrt(y[pole] * y[pole] + x[pole] * x[pole] + 1.0)
            ax[pole], ay[pole], az[pole] = y[pole] * ilp, x[pole] * ilp, ilp
        vs = a * vmax
        pos[:, 0], pos[:, 1], pos[:, 2], pos[:, 3] = px, py, pz, 1.0
        vel[:, 0] = (py * az - pz * ay) * vs
        vel[:, 1] = (pz * ax - px * az) * vs
        vel[:, 2] = (px * ay - py * ax) * vs
        return _store(pos, precision), _store(vel, precision)
    if kind != "plummer":
        raise ValueError(kind)
    x1 = np.maximum(0.999 * u01(seed, ids, 0), 1e-300)
    c1 = 1.0 / np.cbrt(x1)
    r = a / np.sqrt(c1 * c1 - 1.0)
    ct = 2.0 * u01(seed, ids, 1) - 1.0
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = np.pi * (2.0 * u01(seed, ids, 2))
    pos[:, 0], pos[:, 1], pos[:, 2] = r * st * np.cos(ph), r * st * np.sin(ph), r * ct
    pos[:, 3] = M / n
    q = np.full(n, 0.4714045207910317)
    todo = np.ones(n, dtype=bool)
    for t in range(64):
        idx = np.nonzero(todo)[0]
        if idx.size == 0:
            break
        qq = u01(seed, ids[idx], 8 + 2 * t)
        yy = 0.1 * u01(seed, ids[idx], 9 + 2 * t)
        t1 = 1.0 - qq * qq
        ok = yy < qq * qq * (t1 * t1 * t1 * np.sqrt(t1))
        q[idx[ok]] = qq[ok]
        todo[idx[ok]] = False
    vesc = np.sqrt(2.0 * G * M) / np.sqrt(np.sqrt(r * r + a * a))
    ct = 2.0 * u01(seed, ids, 3) - 1.0
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = np.pi * (2.0 * u01(seed, ids, 4))
    v = q * vesc
    vel[:, 0], vel[:, 1], vel[:, 2] = v * st * np.cos(ph), v * st * np.sin(ph), v * ct
    pos, vel = _store(pos, precision), _store(vel, precision)
    # recentre: FP64 moments of the stored values, subtracted in FP64 and
    # stored again
    m = pos[:, 3].astype(np.float64)
    mt = m.sum()
    mt = mt if mt > 0 else 1.0
    for c in range(3):
        cp = (m * pos[:, c].astype(np.float64)).sum() / mt
        cv = (m * vel[:, c].astype(np.float64)).sum() / mt
        pos[:, c] = pos[:, c].astype(np.float64) - cp
        vel[:, c] = vel[:, c].astype(np.float64) - cv
    return pos, vel
