"""nb_autotune, the single-system autotuner: in every mode it restores the
state it timed on, reports the shape nb_plan_info then shows, and the tuned
context steps bit for bit like a fresh context created with that shape; the
cache file gives the same choice to the next context."""
import numpy as np
import pytest

from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu

# "symfx": the symmetric FP32 kernel with its fixed-point source side;
# "symband": the symmetric kernel with its triangular array in three bands
MODES = [("f32", "sym"), ("f32", "symfx"), ("f32", "symband"), ("f32", "fast"), ("f32comp", "sym"),
         ("f32comp", "fast"), ("f64", "sym"), ("f64", "symband"), ("f64", "sym64"), ("f32", "exact")]


def system(n, prec, algo, **kw):
    if algo == "symfx":
        return NBodySystem(n, prec, "sym", source_side="fixed", **kw)
    if algo == "symband":
        return NBodySystem(n, prec, "sym", bands=3, **kw)
    return NBodySystem(n, prec, algo, **kw)


def state(prec, n):
    p, v = ics.plummer(n, seed=31)
    if prec == "f32":
        return ics.f32(p), ics.f32(v)
    return p, v


@pytest.mark.parametrize("prec,algo", MODES)
def test_autotune_every_mode(cuda, tmp_path, prec, algo):
    n = 5000
    pos, vel = state(prec, n)
    eps2 = np.float32(1e-3) if prec == "f32" else 1e-3
    dt = np.float32(1e-3) if prec == "f32" else 1e-3
    cache = str(tmp_path / "tune.txt")
    kw = dict(kick="physical", eps2=eps2, damping=1.0, dt=dt)
    with system(n, prec, algo, **kw) as s:
        s.set_state(pos, vel)
        before = s.get_state()
        shape = s.autotune(reps=1, cache_path=cache)
        after = s.get_state()
        assert before[0].tobytes() == after[0].tobytes() and before[1].tobytes() == after[1].tobytes()
        if algo == "exact":
            return
        info = s.plan_info()
        assert (info["block"], info["bpt"]) == shape
        s.step(3)
        tuned = s.get_state()
    with system(n, prec, algo, block=shape[0], bpt=shape[1], **kw) as f:
        f.set_state(pos, vel)
        f.step(3)
        fresh = f.get_state()
    assert tuned[0].tobytes() == fresh[0].tobytes() and tuned[1].tobytes() == fresh[1].tobytes()
    # the cache gives the next context the same shape
    with system(n, prec, algo, **kw) as s2:
        s2.set_state(pos, vel)
        assert s2.autotune(reps=1, cache_path=cache) == shape
    assert len(open(cache).read().splitlines()) == 1
    if algo == "sym" and prec == "f32":
        # a context with the other source side keeps its own cache entry
        with system(n, prec, "symfx", **kw) as s3:
            s3.set_state(pos, vel)
            w, b = s3.autotune(reps=1, cache_path=cache)
        assert w == 32 and b in (4, 8, 16)
        assert len(open(cache).read().splitlines()) == 2


def test_autotune_drops_a_recorded_adjoint_forward(cuda):
    import torch

    from utc_gb300 import _native as N

    n = 2000
    pos, vel = state("f32", n)
    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-3), damping=1.0,
                     dt=np.float32(1e-3)) as s:
        s.set_state(pos, vel)
        s.adj_forward(4, 2)
        s.autotune(reps=1)
        with pytest.raises(N.NbError):
            s.adj_backward(torch.zeros((n, 4), device="cuda"))
