"""Batches of FP64 state (the reference multi-task app's FTYPE double,
benchapps/nbody/utc/nbody_mtask.cc): one float-float symmetric launch per
step over many uneven systems.

Checks: every system's accelerations against the FP64 oracle to 1e-13 at
every compiled launch shape; several steps against the oracle's FP64 steps;
the CUDA-graph run equals step-by-step launches bitwise; the per-system
baseline equals independent NB_F64 symmetric contexts bitwise, and the
task-pattern baseline equals the per-system one bitwise; the batched run
agrees with the per-system run to 1e-13; autotuning keeps the results; the
adjoint is refused.
"""
import numpy as np
import pytest

import oracle
from utc_gb300 import _native as N
from utc_gb300 import ics
from utc_gb300.nbody import NBodyBatch, NBodySystem

pytestmark = pytest.mark.gpu

EPS2, DT = 1e-3, 1e-3
SIZES = [1, 2, 31, 33, 128, 300, 1024, 5000, 77]


def make_batch(sizes, seed=0):
    ps, vs = [], []
    for k, n in enumerate(sizes):
        p, v = ics.plummer(int(n), seed=seed + k)
        ps.append(p)
        vs.append(v)
    return np.concatenate(ps), np.concatenate(vs)


def per_system(arr, sizes):
    off = np.concatenate([[0], np.cumsum(sizes)])
    return [arr[off[i]:off[i + 1]] for i in range(len(sizes))]


def close(got, want, tol):
    d = np.linalg.norm(np.asarray(got, np.float64) - want, axis=1)
    w = np.linalg.norm(want, axis=1)
    return bool((d <= tol * (w + w.mean())).all())


@pytest.mark.parametrize("shape", [(1, 2), (1, 4), (2, 2), (2, 4), (4, 2), (4, 4)])
def test_f64_batch_accelerations_vs_oracle(cuda, shape):
    """One reference-kick step from zero velocity with masses 1: the new
    velocity is a * dt exactly up to FP64 rounding of the product."""
    pos, _ = make_batch(SIZES, seed=10)
    vel = np.zeros_like(pos)
    with NBodyBatch(SIZES, kick="physical", eps2=EPS2, dt=DT, warps_per_cta=shape[0], bodies_per_lane=shape[1],
                    precision="f64") as b:
        info = b.plan_info()
        assert (info["warps_per_cta"], info["bodies_per_lane"]) == shape
        b.set_state(pos, vel)
        b.step(1)
        _, v1 = b.get_state()
    for p, v in zip(per_system(pos, SIZES), per_system(v1, SIZES)):
        assert close(v[:, :3] / DT, oracle.accel(p, EPS2), 1e-13)


@pytest.mark.parametrize("kick", ["physical", "reference"])
def test_f64_batch_steps_vs_oracle(cuda, kick):
    sizes = [3, 200, 1500, 64]
    pos, vel = make_batch(sizes, seed=4)
    km = oracle.KICK_REFERENCE if kick == "reference" else oracle.KICK_PHYSICAL
    with NBodyBatch(sizes, kick=kick, eps2=EPS2, damping=0.999, dt=DT, precision="f64") as b:
        b.set_state(pos, vel)
        b.step(10)
        got, gv = b.get_state()
    for p, v, g in zip(per_system(pos, sizes), per_system(vel, sizes), per_system(got, sizes)):
        want, _ = oracle.step(p, v, EPS2, 0.999, DT, 10, kick_mode=km)
        rel = np.linalg.norm(g[:, :3] - want[:, :3], axis=1) / (np.linalg.norm(want[:, :3], axis=1) + 0.1)
        assert rel.max() <= 1e-13


def test_f64_graph_run_equals_step_launches(cuda):
    import torch

    sizes = ics.batch_sizes(40, lo=128, hi=2048, seed=3)
    pos, vel = make_batch(sizes, seed=1)
    stream = torch.cuda.Stream()
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, precision="f64") as b:
        b.set_state(pos, vel)
        b.step(7)
        want = b.get_state()
        with torch.cuda.stream(stream):
            b.set_state(pos, vel, stream=stream.cuda_stream)
            b.run(7, stream.cuda_stream)
            stream.synchronize()
            got = b.get_state(stream=stream.cuda_stream)
    assert got[0].tobytes() == want[0].tobytes() and got[1].tobytes() == want[1].tobytes()


def test_f64_per_system_baselines_equal_independent_contexts(cuda):
    sizes = [64, 1000, 3, 4096, 77]
    pos, vel = make_batch(sizes, seed=7)
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, precision="f64") as b:
        b.set_state(pos, vel)
        b.step_per_system(3)
        got, _ = b.get_state()
        b.set_state(pos, vel)
        b.step_tasks(3, 3)
        got_tasks, _ = b.get_state()
    assert got.tobytes() == got_tasks.tobytes()
    for p, v, g in zip(per_system(pos, sizes), per_system(vel, sizes), per_system(got, sizes)):
        with NBodySystem(p.shape[0], "f64", "sym", kick="physical", eps2=EPS2, damping=1.0, dt=DT) as s:
            s.set_state(p, v)
            s.step(3)
            want, _ = s.get_state()
        assert g.tobytes() == want.tobytes()


def test_f64_batched_matches_per_system_and_autotune(cuda, tmp_path):
    """The batch scales all systems by one pair of powers of two, a system on
    its own by its own: the results differ by rounding only."""
    sizes = ics.batch_sizes(24, lo=128, hi=4096, seed=5)
    pos, vel = make_batch(sizes, seed=2)
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, precision="f64") as b:
        b.set_state(pos, vel)
        b.step_per_system(5)
        ref, _ = b.get_state()
        b.set_state(pos, vel)
        b.step(5)
        bat, _ = b.get_state()
        shape = b.autotune(reps=1, cache_path=str(tmp_path / "tune.txt"))
        assert shape in [(1, 2), (1, 4), (2, 2), (2, 4), (4, 2), (4, 4)]
        b.set_state(pos, vel)
        b.step(5)
        tuned, _ = b.get_state()
    for got in (bat, tuned):
        d = np.linalg.norm(got[:, :3] - ref[:, :3], axis=1)
        assert (d <= 1e-13 * (np.linalg.norm(ref[:, :3], axis=1) + 0.1)).all()


def test_f64_batch_refuses_adjoint_and_exact(cuda):
    with NBodyBatch([10, 20], precision="f64") as b:
        b.set_state(*make_batch([10, 20]))
        assert b.lib.nb_batch_adj_forward(b.handle, 4, 2, None, None) == N.NB_ERR_UNSUPPORTED
    with pytest.raises(RuntimeError):
        NBodyBatch([10, 20], precision="f64", algo="exact")
