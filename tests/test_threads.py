"""Contexts and batches used from several host threads at once, as the UTC
app's one-task-per-system pattern does (benchapps/nbody/utc/nbody_mtask.cc:
one Task per system, each on its own thread and stream): while some threads
capture their step graphs, others create, step and destroy their own
contexts.  The library keeps its captures apart from its allocations, frees
and device synchronisations, so every thread's result equals the same run made
alone, bit for bit, and no call fails."""
import threading

import numpy as np
import pytest

from utc_gb300 import ics
from utc_gb300.nbody import NBodyBatch, NBodySystem

pytestmark = pytest.mark.gpu

# (precision, algo, n): each steps 64 steps (the bulk of them as replayed
# step graphs, which nb_step captures at first use)
JOBS = [("f32", "sym", 3000), ("f64", "sym", 2000), ("f32", "fast", 2500), ("f64", "sym64", 1500),
        ("f32comp", "sym", 1800), ("f32", "exact", 1024), ("f64", "exact", 700), ("f32", "sym", 4096)]
STEPS = 64


def start(prec, n, seed):
    p, v = ics.plummer(n, seed=seed)
    if prec == "f32":
        return ics.f32(p), ics.f32(v)
    return p, v


def run_single(prec, algo, n, seed, stream):
    pos, vel = start(prec, n, seed)
    eps2 = np.float32(1e-3) if prec == "f32" else 1e-3
    dt = np.float32(1e-3) if prec == "f32" else 1e-3
    with NBodySystem(n, prec, algo, kick="physical", eps2=eps2, damping=1.0, dt=dt) as s:
        s.set_state(pos, vel, stream=stream)
        s.step(STEPS, stream=stream)
        return s.get_state(stream=stream)


def run_batch(sizes, seed, stream, graph):
    ps, vs = zip(*(start("f32", n, seed + k) for k, n in enumerate(sizes)))
    with NBodyBatch(sizes, eps2=1e-3, dt=1e-3) as b:
        b.set_state(np.concatenate(ps), np.concatenate(vs), stream=stream)
        if graph:
            b.run(STEPS, stream)
        else:
            b.step(STEPS, stream=stream)
        return b.get_state(stream=stream)


def threaded(fns, rounds):
    """Run every fn(stream) on its own thread and stream, `rounds` times over;
    returns the last round's results and the errors seen."""
    import torch

    results, errors = [None] * len(fns), []

    def worker(k):
        try:
            st = torch.cuda.Stream()
            for _ in range(rounds):
                results[k] = fns[k](int(st.cuda_stream))
        except Exception as e:  # reported below, with the job it came from
            errors.append((k, repr(e)))

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(len(fns))]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in ts), "a worker thread did not finish"
    return results, errors


def test_threads_step_graphs_while_others_allocate(cuda):
    import torch

    fns = [lambda s, j=j, k=k: run_single(*j, seed=40 + k, stream=s) for k, j in enumerate(JOBS)]
    fns.append(lambda s: run_batch([700, 1300, 512], 90, s, graph=True))
    fns.append(lambda s: run_batch([900, 300], 95, s, graph=False))
    alone = []
    st = torch.cuda.Stream()
    for f in fns:
        alone.append(f(int(st.cuda_stream)))
    together, errors = threaded(fns, rounds=3)
    assert not errors, errors
    for k, (a, t) in enumerate(zip(alone, together)):
        assert a[0].tobytes() == t[0].tobytes() and a[1].tobytes() == t[1].tobytes(), k


def test_threads_many_small_contexts(cuda):
    # sixteen threads each cycling create -> 64 steps -> destroy, so that
    # allocations and frees keep landing inside other threads' captures
    fns = [lambda s, k=k: run_single("f32" if k % 2 else "f64", "sym", 512 + 64 * k, 7 + k, s) for k in range(16)]
    import torch

    st = torch.cuda.Stream()
    alone = [f(int(st.cuda_stream)) for f in fns]
    together, errors = threaded(fns, rounds=4)
    assert not errors, errors
    for a, t in zip(alone, together):
        assert a[0].tobytes() == t[0].tobytes() and a[1].tobytes() == t[1].tobytes()


def test_destroy_keeps_the_context_while_another_thread_captures(cuda):
    # a thread outside the library captures a graph in global mode; the
    # device cannot be synchronised meanwhile, so nb_destroy refuses and
    # keeps the context, which stays usable and is destroyed afterwards
    import torch

    from utc_gb300 import _native as N

    n = 1024
    pos, vel = start("f32", n, 3)
    s = NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-3), damping=1.0, dt=np.float32(1e-3))
    s.set_state(pos, vel)
    started, release = threading.Event(), threading.Event()
    seen = []

    def capture():
        st = torch.cuda.Stream()
        x = torch.zeros(16, device="cuda")
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(st):
            g.capture_begin(capture_error_mode="global")
            x.add_(1)
            started.set()
            release.wait(30)
            try:
                g.capture_end()
            except Exception as e:  # a refused call elsewhere may void the capture
                seen.append(repr(e))

    t = threading.Thread(target=capture)
    t.start()
    assert started.wait(30)
    rc = s.lib.nb_destroy(s.handle)
    msg = s.lib.nb_last_error().decode()
    release.set()
    t.join(60)
    if rc == N.NB_OK:
        s.handle = None  # destroyed after all: nothing of it may be used below
    assert rc == N.NB_ERR_CUDA and "captures a graph" in msg, (rc, msg)
    s.step(2)  # kept and usable
    s.get_state()
    s.close()
