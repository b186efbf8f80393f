"""Seeded random parity sweep: random mode, N, kick mode, eps2, damping, dt,
G and step count; positions and velocities after the steps against the
oracle's steps from the same start, at each mode's tolerance (the exact
kernels bit for bit against the oracle in their own precision)."""
import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu

MODES = [("f32", "fast"), ("f32", "sym"), ("f32", "exact"), ("f64", "exact"), ("f64", "sym"), ("f64", "sym64"),
         ("f32comp", "fast"), ("f32comp", "sym")]
# relative tolerance on |x_gpu - x_oracle| / (|x| + 0.1) after the steps
TOL = {("f32", "fast"): 1e-5, ("f32", "sym"): 1e-5, ("f64", "sym"): 1e-12, ("f64", "sym64"): 1e-12,
       ("f32comp", "fast"): 1e-8, ("f32comp", "sym"): 1e-8}


def cases(count=48, seed=2024):
    rng = np.random.default_rng(seed)
    for k in range(count):
        prec, algo = MODES[k % len(MODES)]
        n = int(np.exp(rng.uniform(0, np.log(6000))))
        yield dict(k=k, prec=prec, algo=algo, n=n, kick=["reference", "physical"][int(rng.integers(2))],
                   eps2=float(10 ** rng.uniform(-4, -1)), damping=float(rng.choice([1.0, 0.999, 0.995])),
                   dt=float(10 ** rng.uniform(-4, -2)), G=float(rng.uniform(0.5, 2.0)),
                   steps=int(rng.integers(1, 4)), ic=["plummer", "cube"][int(rng.integers(2))],
                   seed=int(rng.integers(1 << 30)))


@pytest.mark.parametrize("c", list(cases()), ids=lambda c: f"{c['k']}-{c['prec']}-{c['algo']}-n{c['n']}")
def test_random_case(cuda, c):
    prec, algo, n = c["prec"], c["algo"], c["n"]
    p, v = (ics.plummer if c["ic"] == "plummer" else ics.uniform_cube)(n, seed=c["seed"])
    f32 = prec == "f32"
    T = np.float32 if f32 else np.float64
    pos, vel = (ics.f32(p), ics.f32(v)) if f32 else (p, v)
    eps2, damp, dt, G = (T(c["eps2"]), T(c["damping"]), T(c["dt"]), T(c["G"]))
    km = oracle.KICK_REFERENCE if c["kick"] == "reference" else oracle.KICK_PHYSICAL
    with NBodySystem(n, prec, algo, kick=c["kick"], eps2=eps2, damping=damp, dt=dt, G=G) as s:
        s.set_state(pos, vel)
        s.step(c["steps"])
        gp, gv = s.get_state()
    if algo == "exact":  # bit for bit against the oracle in the state precision
        wp, wv = oracle.step(pos, vel, eps2, damp, dt, c["steps"], kick_mode=km, G=G)
        assert gp.tobytes() == wp.tobytes() and gv.tobytes() == wv.tobytes()
        return
    wp, wv = oracle.step(np.asarray(pos, np.float64), np.asarray(vel, np.float64), float(eps2), float(damp),
                         float(dt), c["steps"], kick_mode=km, G=float(G))
    rel = np.linalg.norm(np.asarray(gp, np.float64)[:, :3] - wp[:, :3], axis=1) / (
        np.linalg.norm(wp[:, :3], axis=1) + 0.1)
    assert rel.max() <= TOL[(prec, algo)], rel.max()
    # the displacement, which a tiny dt makes small, carries the forces
    dx = np.asarray(gp, np.float64)[:, :3] - np.asarray(pos, np.float64)[:, :3]
    wdx = wp[:, :3] - np.asarray(pos, np.float64)[:, :3]
    scale = np.abs(wdx).max() + 1e-300
    dtol = {"f32": 1e-3, "f32comp": 1e-6, "f64": 1e-10}[prec]
    assert np.abs(dx - wdx).max() <= dtol * scale + 4 * np.finfo(T).eps * (np.abs(wp[:, :3]).max())
