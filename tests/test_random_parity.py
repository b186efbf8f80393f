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


def cases_more(count=24, seed=4049):
    """A second sweep over the paths added later: the fixed-point source side
    of the symmetric kernel, and target partitions of 2 to 5 shards (the
    directed kernel's and the reference-exact ones, float and double)."""
    rng = np.random.default_rng(seed)
    modes = [("symfx", "f32"), ("shard-fast", "f32"), ("shard-exact", "f32"), ("shard-exact", "f64")]
    for k in range(count):
        mode, prec = modes[k % len(modes)]
        yield dict(k=k, mode=mode, prec=prec, n=int(np.exp(rng.uniform(0, np.log(6000)))),
                   nranks=int(rng.integers(2, 6)), kick=["reference", "physical"][int(rng.integers(2))],
                   eps2=float(10 ** rng.uniform(-4, -1)), damping=float(rng.choice([1.0, 0.999, 0.995])),
                   dt=float(10 ** rng.uniform(-4, -2)), G=float(rng.uniform(0.5, 2.0)),
                   steps=int(rng.integers(1, 5)), ic=["plummer", "cube"][int(rng.integers(2))],
                   seed=int(rng.integers(1 << 30)))


@pytest.mark.parametrize("c", list(cases_more()), ids=lambda c: f"{c['k']}-{c['mode']}-{c['prec']}-n{c['n']}")
def test_random_case_more(cuda, c):
    from test_shard_gpu import run_shards

    n, T = c["n"], np.float64 if c["prec"] == "f64" else np.float32
    p, v = (ics.plummer if c["ic"] == "plummer" else ics.uniform_cube)(n, seed=c["seed"])
    pos, vel = p.astype(T), v.astype(T)
    eps2, damp, dt, G = T(c["eps2"]), T(c["damping"]), T(c["dt"]), T(c["G"])
    km = oracle.KICK_REFERENCE if c["kick"] == "reference" else oracle.KICK_PHYSICAL
    kw = dict(kick=c["kick"], eps2=float(eps2), damping=float(damp), dt=float(dt))
    if c["mode"] == "symfx":
        with NBodySystem(n, "f32", "sym", G=float(G), source_side="fixed", **kw) as s:
            s.set_state(pos, vel)
            s.step(c["steps"])
            gp, _ = s.get_state()
        wp, _ = oracle.step(np.asarray(pos, np.float64), np.asarray(vel, np.float64), float(eps2), float(damp),
                            float(dt), c["steps"], kick_mode=km, G=float(G))
        rel = np.linalg.norm(np.asarray(gp, np.float64)[:, :3] - wp[:, :3], axis=1) / (
            np.linalg.norm(wp[:, :3], axis=1) + 0.1)
        assert rel.max() <= 1e-5, rel.max()
        return
    algo = "fast" if c["mode"] == "shard-fast" else "exact"
    if c["kick"] == "physical" and float(G) != 1.0:
        kw["kick"] = "reference"  # the shard helper takes no G; the reference kick needs none
        km = oracle.KICK_REFERENCE
    gp, gv, _ = run_shards(n, c["nranks"], c["steps"], c["prec"], algo, pos, vel, **kw)
    if algo == "exact":
        wp, wv = oracle.step(pos, vel, eps2, damp, dt, c["steps"], kick_mode=km)
    else:
        with NBodySystem(n, "f32", "fast", **kw) as s:
            s.set_state(pos, vel)
            s.step(c["steps"])
            wp, wv = s.get_state()
    assert gp.tobytes() == wp.tobytes() and gv.tobytes() == wv.tobytes()


def cases_bands(count=18, seed=4051):
    """A third sweep: the symmetric kernels with their triangular array in
    2 to 8 bands (float, compensated and float-float double state), against
    the same context stepped in one pass and, for float state, the FP64
    oracle."""
    rng = np.random.default_rng(seed)
    precs = ["f32", "f64", "f32comp"]
    for k in range(count):
        yield dict(k=k, prec=precs[k % 3], n=int(np.exp(rng.uniform(np.log(600), np.log(9000)))),
                   bands=int(rng.integers(2, 9)), kick=["reference", "physical"][int(rng.integers(2))],
                   eps2=float(10 ** rng.uniform(-4, -1)), damping=float(rng.choice([1.0, 0.999, 0.995])),
                   dt=float(10 ** rng.uniform(-4, -2)), G=float(rng.uniform(0.5, 2.0)),
                   steps=int(rng.integers(1, 5)), ic=["plummer", "cube"][int(rng.integers(2))],
                   seed=int(rng.integers(1 << 30)))


@pytest.mark.parametrize("c", list(cases_bands()), ids=lambda c: f"{c['k']}-{c['prec']}-n{c['n']}-b{c['bands']}")
def test_random_case_bands(cuda, c):
    n, prec = c["n"], c["prec"]
    T = np.float32 if prec == "f32" else np.float64
    p, v = (ics.plummer if c["ic"] == "plummer" else ics.uniform_cube)(n, seed=c["seed"])
    pos, vel = p.astype(T), v.astype(T)
    eps2, damp, dt, G = (float(T(c[k])) for k in ("eps2", "damping", "dt", "G"))
    out = []
    for bands in (0, c["bands"]):
        with NBodySystem(n, prec, "sym", kick=c["kick"], eps2=eps2, damping=damp, dt=dt, G=G, bands=bands) as s:
            s.set_state(pos, vel)
            s.step(c["steps"])
            out.append((s.get_state()[0], s.source_info()))
    assert c["bands"] == 0 or out[1][1]["bands"] >= 1
    (a, _), (b, _) = out
    scale = np.linalg.norm(np.asarray(a, np.float64)[:, :3], axis=1) + 0.1
    rel = np.linalg.norm(np.asarray(b, np.float64)[:, :3] - np.asarray(a, np.float64)[:, :3], axis=1) / scale
    assert rel.max() <= {"f32": 1e-5, "f32comp": 1e-9, "f64": 1e-13}[prec], rel.max()
    if prec == "f32":
        km = oracle.KICK_REFERENCE if c["kick"] == "reference" else oracle.KICK_PHYSICAL
        wp, _ = oracle.step(np.asarray(pos, np.float64), np.asarray(vel, np.float64), eps2, damp, dt, c["steps"],
                            kick_mode=km, G=G)
        rel = np.linalg.norm(np.asarray(b, np.float64)[:, :3] - wp[:, :3], axis=1) / (
            np.linalg.norm(wp[:, :3], axis=1) + 0.1)
        assert rel.max() <= 1e-5, rel.max()
