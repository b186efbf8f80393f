"""Initial conditions drawn on the GPU (nb_ics_generate): equal to the host
restatement of the generator (oracle/ics.py) -- bit for bit for the cube,
random and expand configurations, within a few units in the last place for
the shell and the Plummer sphere, whose arithmetic the compiler may fuse or
whose cbrt/rsqrt/sincospi differ from numpy's -- deterministic per seed, and
distributed as specified (the analytic Plummer mass profile and the virial
ratio, the cube's ranges).  The restatement's SplitMix64 is pinned by the
published known-answer sequence."""
import numpy as np
import pytest

import oracle
from oracle import ics as ics_oracle
from utc_gb300.nbody import NBodySystem, gpu_initial_conditions

gpu = pytest.mark.gpu


def test_splitmix64_known_answers():
    """SplitMix64 from state 1234567: the first five outputs of the published
    reference sequence (each output mixes the state after one increment)."""
    want = [6457827717110365317, 3203168211198807973, 9817491932198370423,
            4593380528125082431, 16408922859458223821]
    state = 1234567
    got = []
    for _ in range(5):
        got.append(int(ics_oracle.splitmix64(np.uint64(state))))
        state = (state + 0x9E3779B97F4A7C15) % (1 << 64)
    assert got == want


def test_restatement_streams_are_per_body():
    """A body's draws depend only on (seed, index, stream): the restated
    cube of 1000 bodies is the head of the one of 3000 (masses aside)."""
    a, _ = ics_oracle.generate("cube", 1000, seed=5, precision="f64")
    b, _ = ics_oracle.generate("cube", 3000, seed=5, precision="f64")
    assert np.array_equal(a[:, :3], b[:1000, :3])
    u = ics_oracle.u01(9, np.arange(100000, dtype=np.uint64), 3)
    assert 0.0 <= u.min() and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01


def _ulps_close(got, want, rel):
    """Per body: |got - want| <= rel * (|want| + median |want|), all four
    components."""
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    scale = np.abs(want) + np.median(np.abs(want))
    return float((np.abs(got - want) / scale).max()) <= rel


@gpu
@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("kind", ["cube", "random", "expand", "shell", "plummer"])
@pytest.mark.parametrize("n,seed", [(100003, 7), (4099, (1 << 63) + 5)])
def test_gpu_generator_matches_restatement(cuda, kind, precision, n, seed):
    a, vmax = (1.0, 0.01) if kind in ("cube", "plummer") else (1.54, 8.0)
    gp, gv = [t.cpu().numpy() for t in gpu_initial_conditions(kind, n, seed=seed, a=a, vmax=vmax,
                                                               precision=precision)]
    wp, wv = ics_oracle.generate(kind, n, seed, a=a, vmax=vmax, precision=precision)
    if kind in ("cube", "random", "expand"):
        assert gp.tobytes() == wp.tobytes() and gv.tobytes() == wv.tobytes()
        return
    # shell: fused multiply-adds in the radius and velocity; Plummer: CUDA's
    # rcbrt / rsqrt / sincospi against numpy's cbrt / sqrt / sin(pi x), then
    # the recentring.  FP64 within 1e-12; float within two float ulps, since
    # a double near a rounding midpoint may round either way
    rel = 1e-12 if precision == "f64" else 2.5e-7
    assert _ulps_close(gp, wp, rel) and _ulps_close(gv, wv, rel)
    assert np.array_equal(gp[:, 3], wp[:, 3]) and np.array_equal(gv[:, 3], wv[:, 3])


@gpu
def test_deterministic_and_seeded(cuda):
    a = gpu_initial_conditions("plummer", 5000, seed=3)
    b = gpu_initial_conditions("plummer", 5000, seed=3)
    c = gpu_initial_conditions("plummer", 5000, seed=4)
    assert all((x.cpu().numpy().tobytes() == y.cpu().numpy().tobytes()) for x, y in zip(a, b))
    assert a[0].cpu().numpy().tobytes() != c[0].cpu().numpy().tobytes()
    # a body's coordinates do not depend on how many bodies are drawn (its
    # mass does: U[0.5,1.5]/n)
    d = gpu_initial_conditions("cube", 1000, seed=5)[0].cpu().numpy()
    e = gpu_initial_conditions("cube", 3000, seed=5)[0].cpu().numpy()
    assert d[:, :3].tobytes() == e[:1000, :3].tobytes()


@gpu
def test_cube_ranges(cuda):
    n = 20000
    p, v = [t.cpu().numpy() for t in gpu_initial_conditions("cube", n, seed=1, vmax=0.01)]
    assert np.abs(p[:, :3]).max() <= 1.0 and np.abs(v[:, :3]).max() <= 0.01
    assert (p[:, 3] >= 0.5 / n).all() and (p[:, 3] <= 1.5 / n).all()
    assert abs(p[:, :3].mean()) < 0.02 and abs(p[:, 3].sum() - 1.0) < 0.01
    assert np.all(v[:, 3] == 1.0)


@gpu
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_plummer_profile_and_virial(cuda, precision):
    n = 100000
    p, v = [t.cpu().numpy().astype(np.float64) for t in gpu_initial_conditions("plummer", n, seed=2,
                                                                                 precision=precision)]
    com = (p[:, :3] * p[:, 3:4]).sum(0)
    mom = (v[:, :3] * p[:, 3:4]).sum(0)
    assert np.abs(com).max() < 1e-6 and np.abs(mom).max() < 1e-6
    r = np.linalg.norm(p[:, :3], axis=1)
    for rr in (0.5, 1.0, 2.0, 5.0):
        want = rr ** 3 / (rr * rr + 1) ** 1.5 / 0.999  # truncated at X <= 0.999
        assert abs((r < rr).mean() - min(want, 1.0)) < 0.01
    # virial ratio -K / W ~ 0.5 (potential from the GPU energy pass, small softening)
    with NBodySystem(n, "f32", "fast", kick="physical", eps2=np.float32(1e-6)) as s:
        s.set_state(p.astype(np.float32), v.astype(np.float32))
        e = s.energy()
    assert abs(-e[0] / e[1] - 0.5) < 0.03


@gpu
@pytest.mark.parametrize("kind", ["random", "shell", "expand"])
def test_reference_configurations(cuda, kind):
    """The reference app's three initial configurations drawn on the GPU:
    the support and structure of each distribution (randomizeBodies,
    benchapps/nbody/seq/nbody.h:89-250), with clusterScale 1.54 and
    velocityScale 8 (the app's first preset)."""
    n, cs, vs = 5000, 1.54, 8.0
    p, v = [t.cpu().numpy().astype(np.float64) for t in
            gpu_initial_conditions(kind, n, seed=2, a=cs, vmax=vs)]
    assert (p[:, 3] == 1.0).all() and (v[:, 3] == 1.0).all()
    r = np.linalg.norm(p[:, :3], axis=1)
    if kind == "random":
        s = cs * max(1.0, n / 1024)
        assert r.max() <= s * (1 + 1e-6)
        assert np.linalg.norm(v[:, :3], axis=1).max() <= s * vs * (1 + 1e-6)
        # uniform in the ball: the fraction inside half the radius is 1/8
        assert abs((r < 0.5 * s).mean() - 0.125) < 0.02
    elif kind == "shell":
        assert r.min() >= 2.5 * cs * (1 - 1e-6) and r.max() <= 4.0 * cs * (1 + 1e-6)
        # velocity = (pos x z) cs vs: perpendicular to z and to pos
        assert np.abs(v[:, 2]).max() <= 1e-4 * np.abs(v[:, :3]).max()
        assert np.abs((p[:, :3] * v[:, :3]).sum(1)).max() <= 1e-3 * (r * np.linalg.norm(v[:, :3], axis=1)).max()
        assert np.allclose(v[:, 0], p[:, 1] * cs * vs, rtol=1e-5, atol=1e-5)
    else:
        s = cs * n / 1024
        assert r.max() <= s * (1 + 1e-6)
        assert np.allclose(v[:, :3], p[:, :3] * vs, rtol=1e-5, atol=1e-6)
