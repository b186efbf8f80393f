"""Batched systems: one persistent launch per step over many uneven systems.

Checks: every system's accelerations (one step from zero velocity) against
the FP64 oracle at the fast-path tolerance; the CUDA-graph run equals
step-by-step launches bitwise; the per-system baseline equals independent
NBodySystem contexts bitwise; every compiled launch shape and the autotuner
(with its cache file) keep the results within tolerance.
"""
import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem, NBodyBatch

pytestmark = pytest.mark.gpu

EPS2, DT = np.float32(1e-3), np.float32(1e-3)


def make_batch(sizes, seed=0):
    ps, vs = [], []
    for k, n in enumerate(sizes):
        p, v = ics.plummer(int(n), seed=seed + k)
        ps.append(ics.f32(p))
        vs.append(ics.f32(v))
    return np.concatenate(ps), np.concatenate(vs)


def per_system(arr, sizes):
    off = np.concatenate([[0], np.cumsum(sizes)])
    return [arr[off[i]:off[i + 1]] for i in range(len(sizes))]


SIZES = [1, 2, 31, 33, 128, 300, 1024, 5000, 77]


@pytest.mark.parametrize("algo,shape", [("fast", s) for s in [(2, 4), (2, 8), (4, 2), (4, 4), (4, 8), (8, 2),
                                                                (8, 4), (8, 8)]] +
                         [("sym", s) for s in [(1, 8), (1, 12), (1, 16), (2, 8), (2, 16), (4, 8), (4, 16)]])
def test_batch_accelerations_vs_oracle(cuda, algo, shape):
    pos, _ = make_batch(SIZES, seed=10)
    vel = np.zeros_like(pos)
    with NBodyBatch(SIZES, eps2=EPS2, dt=DT, warps_per_cta=shape[0], bodies_per_lane=shape[1],
                    algo=algo) as b:
        assert b.plan_info()["warps_per_cta"] == shape[0]
        b.set_state(pos, vel)
        b.step(1)
        _, v1 = b.get_state()
    for p, v in zip(per_system(pos, SIZES), per_system(v1, SIZES)):
        a = v[:, :3].astype(np.float64) / float(DT)
        ref = oracle.accel(p.astype(np.float64), float(EPS2))
        d = np.linalg.norm(a - ref, axis=1)
        w = np.linalg.norm(ref, axis=1)
        assert (d <= 2e-5 * (w + w.mean())).all()


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_graph_run_equals_step_launches(cuda, algo):
    import torch

    sizes = ics.batch_sizes(40, lo=128, hi=2048, seed=3)
    pos, vel = make_batch(sizes, seed=1)
    stream = torch.cuda.Stream()
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, algo=algo) as b:
        b.set_state(pos, vel)
        b.step(7)
        want = b.get_state()
        with torch.cuda.stream(stream):
            b.set_state(pos, vel, stream=stream.cuda_stream)
            b.run(7, stream.cuda_stream)
            stream.synchronize()
            got = b.get_state(stream=stream.cuda_stream)
            # second replay continues from the advanced state (odd step count)
            b.run(7, stream.cuda_stream)
            b.run(7, stream.cuda_stream)
            stream.synchronize()
        b.set_state(pos, vel)
        b.step(21)
        want3 = b.get_state()
        with torch.cuda.stream(stream):
            got3 = b.get_state(stream=stream.cuda_stream)
    assert got[0].tobytes() == want[0].tobytes() and got[1].tobytes() == want[1].tobytes()
    assert got3[0].tobytes() == want3[0].tobytes()


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_per_system_baseline_equals_independent_contexts(cuda, algo):
    sizes = [64, 1000, 3, 4096]
    pos, vel = make_batch(sizes, seed=7)
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, algo=algo) as b:
        b.set_state(pos, vel)
        b.step_per_system(3)
        got, _ = b.get_state()
    for p, v, g in zip(per_system(pos, sizes), per_system(vel, sizes), per_system(got, sizes)):
        with NBodySystem(p.shape[0], "f32", algo, kick="physical", eps2=EPS2, damping=1.0, dt=DT) as s:
            s.set_state(p, v)
            s.step(3)
            want, _ = s.get_state()
        assert g.tobytes() == want.tobytes()


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_batched_matches_per_system_within_tolerance(cuda, algo):
    sizes = ics.batch_sizes(24, lo=128, hi=4096, seed=5)
    pos, vel = make_batch(sizes, seed=2)
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, algo=algo) as b:
        b.set_state(pos, vel)
        b.step(5)
        bat, _ = b.get_state()
        b.set_state(pos, vel)
        b.step_per_system(5)
        ref, _ = b.get_state()
    d = np.linalg.norm(bat[:, :3].astype(np.float64) - ref[:, :3], axis=1)
    w = np.linalg.norm(ref[:, :3].astype(np.float64), axis=1)
    assert (d <= 1e-5 * (w + 0.1)).all()


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_autotune_and_cache(cuda, tmp_path, algo):
    sizes = ics.batch_sizes(64, lo=128, hi=4096, seed=11)
    pos, vel = make_batch(sizes, seed=4)
    cache = str(tmp_path / "tune.txt")
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, algo=algo) as b:
        b.set_state(pos, vel)
        w, k = b.autotune(reps=1, cache_path=cache)
        info = b.plan_info()
        assert (info["warps_per_cta"], info["bodies_per_lane"]) == (w, k)
        p0, _ = b.get_state()
        assert p0.tobytes() == pos.tobytes()  # tuning left the state as it was
        b.step(2)
        tuned, _ = b.get_state()
    lines = open(cache).read().strip().splitlines()
    assert len(lines) == 1 and lines[0].endswith(f"{w} {k}")
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, algo=algo) as b2:
        b2.set_state(pos, vel)
        assert b2.autotune(reps=1, cache_path=cache) == (w, k)  # served from the cache
        assert len(open(cache).read().strip().splitlines()) == 1
        b2.step(2)
        again, _ = b2.get_state()
    assert tuned.tobytes() == again.tobytes()


@pytest.mark.parametrize("algo", ["fast", "sym"])
@pytest.mark.parametrize("kick", ["physical", "reference"])
def test_batched_adjoint_matches_per_system_adjoint(cuda, kick, algo):
    import torch

    sizes = [1, 40, 300, 129, 1000]
    steps, every = 12, 5
    ps, vs, ys = [], [], []
    for k, n in enumerate(sizes):
        p, v = ics.uniform_cube(n, seed=20 + k)
        if kick == "reference":
            p[:, 3] *= n
        ps.append(ics.f32(p))
        vs.append(ics.f32(v))
        ys.append(ics.gaussian_targets(n, seed=40 + k))
    pos, vel, y = np.concatenate(ps), np.concatenate(vs), np.concatenate(ys)
    eps2, dt = np.float32(1e-2), np.float32(1e-3)
    with NBodyBatch(sizes, kick=kick, eps2=eps2, dt=dt, algo=algo) as b:
        b.set_state(pos, vel)
        b.adj_forward(steps, every)
        pT, _ = b.get_state()
        gx = torch.zeros((b.nbody, 4), device="cuda")
        gx[:, :3] = torch.tensor(2 * (pT[:, :3].astype(np.float64) - y), dtype=torch.float32, device="cuda")
        bx, bv, bm = [t.cpu().numpy() for t in b.adj_backward(gx)]
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k, n in enumerate(sizes):
        sl = slice(off[k], off[k + 1])
        L, rx, rv, rm = oracle.adjoint(ps[k].astype(np.float64), vs[k].astype(np.float64), ys[k],
                                       float(eps2), 1.0, float(dt), steps,
                                       kick_mode=oracle.KICK_PHYSICAL if kick == "physical" else oracle.KICK_REFERENCE)
        for got, want in ((bx[sl, :3], rx), (bv[sl, :3], rv), (bm[sl], rm)):
            assert np.linalg.norm(got - want) <= 1e-4 * np.linalg.norm(want) + 1e-12


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_task_pattern_baseline_equals_per_system(cuda, algo):
    sizes = [64, 1000, 3, 4096, 77, 500]
    pos, vel = make_batch(sizes, seed=9)
    with NBodyBatch(sizes, eps2=EPS2, dt=DT, algo=algo) as b:
        b.set_state(pos, vel)
        b.step_per_system(3)
        want, _ = b.get_state()
        b.set_state(pos, vel)
        b.step_tasks(3, 4)
        got, _ = b.get_state()
    assert got.tobytes() == want.tobytes()


@pytest.mark.parametrize("algo", ["fast", "sym"])
@pytest.mark.parametrize("kick", ["physical", "reference"])
def test_batched_second_backward_recomputes_every_segment(cuda, algo, kick):
    """The batched forward leaves the last segment's states in place for the
    first backward; a second backward recomputes it and gives the same bits."""
    import torch

    sizes = [3, 200, 64, 700]
    p, v = make_batch(sizes, seed=30)
    if kick == "reference":
        p[:, 3] *= 100
    with NBodyBatch(sizes, kick=kick, eps2=np.float32(1e-2), dt=np.float32(1e-3), damping=0.999,
                    algo=algo) as b:
        b.set_state(p, v)
        b.adj_forward(13, 4)
        gx = torch.randn((b.nbody, 4), device="cuda")
        first = [t.cpu().numpy() for t in b.adj_backward(gx)]
        second = [t.cpu().numpy() for t in b.adj_backward(gx)]
    for x, y in zip(first, second):
        assert x.tobytes() == y.tobytes()
