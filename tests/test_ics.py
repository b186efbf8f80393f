"""Initial conditions drawn on the GPU (nb_ics_generate): deterministic per
seed, and distributed as specified (checked against the analytic Plummer
mass profile and the virial ratio, and the cube's ranges)."""
import numpy as np
import pytest

import oracle
from utc_gb300.nbody import NBodySystem, gpu_initial_conditions

pytestmark = pytest.mark.gpu


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


def test_cube_ranges(cuda):
    n = 20000
    p, v = [t.cpu().numpy() for t in gpu_initial_conditions("cube", n, seed=1, vmax=0.01)]
    assert np.abs(p[:, :3]).max() <= 1.0 and np.abs(v[:, :3]).max() <= 0.01
    assert (p[:, 3] >= 0.5 / n).all() and (p[:, 3] <= 1.5 / n).all()
    assert abs(p[:, :3].mean()) < 0.02 and abs(p[:, 3].sum() - 1.0) < 0.01
    assert np.all(v[:, 3] == 1.0)


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
