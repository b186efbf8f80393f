"""Edge cases across every precision and algorithm: empty and one-body
systems, invalid arguments answered with status codes (never a device
fault), rejected combinations, and the batch API's argument checks."""
import ctypes as C

import numpy as np
import pytest

import oracle
from utc_gb300 import _native as N
from utc_gb300 import ics
from utc_gb300.nbody import NBodyBatch, NBodySystem

pytestmark = pytest.mark.gpu

# "symfx": the symmetric FP32 kernel with its fixed-point source side;
# "symband": the symmetric kernel with its triangular array in three bands
MODES = [("f32", "fast"), ("f32", "sym"), ("f32", "symfx"), ("f32", "symband"), ("f32", "exact"), ("f64", "exact"),
         ("f64", "sym"), ("f64", "symband"), ("f64", "sym64"), ("f32comp", "fast"), ("f32comp", "sym"),
         ("f32comp", "symband")]


def system(n, prec, algo, **kw):
    if algo == "symfx":
        return NBodySystem(n, prec, "sym", source_side="fixed", **kw)
    if algo == "symband":
        return NBodySystem(n, prec, "sym", bands=3, **kw)
    return NBodySystem(n, prec, algo, **kw)


def dtype_of(prec):
    return np.float64 if prec in ("f64", "f32comp") else np.float32


@pytest.mark.parametrize("prec,algo", MODES)
def test_empty_system_every_mode(cuda, prec, algo):
    dt = dtype_of(prec)
    with system(0, prec, algo) as s:
        s.set_state(np.zeros((0, 4), dt), np.zeros((0, 4), dt))
        s.step(3)
        p, v = s.get_state()
        assert p.shape == (0, 4) and v.shape == (0, 4)
        assert s.launches_per_step() == 0


@pytest.mark.parametrize("prec,algo", MODES)
def test_one_body_drifts_freely(cuda, prec, algo):
    """A lone body feels no force (its self term is r = 0): after k steps of
    the physical kick it has moved by k dt v exactly as the oracle says."""
    dt_ = dtype_of(prec)
    pos = np.array([[0.25, -0.5, 0.125, 2.0]], dt_)
    vel = np.array([[0.5, 0.25, -1.0, 1.0]], dt_)
    with system(1, prec, algo, kick="physical", eps2=1e-2, damping=1.0, dt=1e-3) as s:
        s.set_state(pos, vel)
        s.step(5)
        p, v = s.get_state()
    want_p, want_v = oracle.step(pos.astype(np.float64), vel.astype(np.float64), 1e-2, 1.0, 1e-3, 5,
                                 kick_mode=oracle.KICK_PHYSICAL)
    assert np.allclose(p[:, :3], want_p[:, :3], rtol=1e-6, atol=1e-7)
    assert np.allclose(v[:, :3], want_v[:, :3], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("prec,algo", MODES)
def test_status_codes_every_mode(cuda, prec, algo):
    with system(64, prec, algo) as s:
        assert s.lib.nb_step(s.handle, 1, None) == N.NB_ERR_STATE
        assert s.lib.nb_accel(s.handle, None, None) == N.NB_ERR_STATE
        assert s.lib.nb_step(s.handle, -1, None) == N.NB_ERR_INVALID
        dt_ = dtype_of(prec)
        p, v = ics.plummer(64, seed=1)
        p, v = p.astype(dt_), v.astype(dt_)
        s.set_state(p, v)
        assert s.lib.nb_accel(s.handle, None, None) == N.NB_ERR_INVALID
        assert s.lib.nb_set_state(s.handle, p.ctypes.data_as(C.c_void_p), None, 0, None) == N.NB_ERR_INVALID
        assert s.lib.nb_set_state(s.handle, p.ctypes.data_as(C.c_void_p),
                                  v.ctypes.data_as(C.c_void_p), 7, None) == N.NB_ERR_INVALID
        s.step(1)  # the context is still usable after the refusals


@pytest.mark.parametrize("prec,algo", [("f64", "fast"), ("f32comp", "exact")])
def test_rejected_combinations(cuda, prec, algo):
    with pytest.raises(N.NbError) as e:
        system(16, prec, algo)
    assert e.value.status == N.NB_ERR_UNSUPPORTED


@pytest.mark.parametrize("prec,algo", [("f32", "exact"), ("f64", "exact"), ("f64", "sym"),
                                       ("f32comp", "fast"), ("f32comp", "sym")])
def test_adjoint_needs_a_float_fast_context(cuda, prec, algo):
    dt_ = dtype_of(prec)
    p, v = ics.plummer(32, seed=2)
    with system(32, prec, algo) as s:
        s.set_state(p.astype(dt_), v.astype(dt_))
        assert s.lib.nb_adj_forward(s.handle, 4, 2, None, None) == N.NB_ERR_UNSUPPORTED


def test_batch_argument_checks(cuda):
    lib = N.lib()
    prm = N.NbParams()
    lib.nb_params_default(C.byref(prm))
    h = C.c_void_p()
    sizes = np.array([4, 0, 9], np.int32)  # a system without bodies
    assert lib.nb_batch_create(C.byref(prm), 3, sizes.ctypes.data_as(C.c_void_p), C.byref(h)) == N.NB_ERR_INVALID
    sizes = np.array([4, 9], np.int32)
    prm.algo = N.NB_ALGO_EXACT
    assert lib.nb_batch_create(C.byref(prm), 2, sizes.ctypes.data_as(C.c_void_p), C.byref(h)) == N.NB_ERR_UNSUPPORTED
    prm.algo = N.NB_ALGO_FAST  # FP64 batches run the (float-float) symmetric algorithm only
    prm.precision = N.NB_F64
    assert lib.nb_batch_create(C.byref(prm), 2, sizes.ctypes.data_as(C.c_void_p), C.byref(h)) == N.NB_ERR_UNSUPPORTED
    with NBodyBatch([4, 9]) as b:
        assert b.lib.nb_batch_step(b.handle, 1, None) == N.NB_ERR_STATE
        with pytest.raises(N.NbError):
            b.set_shape(3, 5)  # shape not compiled


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_batch_of_single_bodies(cuda, algo):
    """Systems of one body each: no forces, free drift, every system apart."""
    sizes = [1] * 37
    p, v = ics.uniform_cube(37, seed=4)
    p32, v32 = ics.f32(p), ics.f32(v)
    with NBodyBatch(sizes, eps2=np.float32(1e-3), dt=np.float32(1e-3), algo=algo) as b:
        b.set_state(p32, v32)
        b.step(4)
        got, gv = b.get_state()
    assert np.array_equal(gv, v32)
    want = p32.copy()
    for _ in range(4):
        want[:, :3] = want[:, :3] + v32[:, :3] * np.float32(1e-3)
    assert np.allclose(got, want, rtol=0, atol=1e-7)


@pytest.mark.parametrize("prec,algo", MODES)
@pytest.mark.parametrize("where", ["side", "legacy"])
def test_graph_replay_equals_single_steps(cuda, prec, algo, where):
    """nb_step replays a captured graph of steps, on a non-default stream
    directly and from the legacy default stream through the context's own
    stream (ordered by events both ways, so the calls around it on the legacy
    stream need no synchronisation); the result must equal stepping one
    launch pair at a time, from either ping-pong buffer."""
    import torch

    dt_ = dtype_of(prec)
    n = 700
    p, v = ics.plummer(n, seed=5)
    p, v = p.astype(dt_), v.astype(dt_)
    side = torch.cuda.Stream()
    with system(n, prec, algo, kick="physical", eps2=1e-3, damping=1.0, dt=1e-3) as s:
        s.set_state(p, v)
        for _ in range(71):
            s.step(1)
        want = s.get_state()
        s.set_state(p, v)
        s.step(1)  # odd start: the graph begins from the second buffer
        if where == "side":
            torch.cuda.synchronize()
            with torch.cuda.stream(side):
                s.step(70, stream=side.cuda_stream)
                side.synchronize()
        else:
            s.step(70, stream=0)
        got = s.get_state()
    assert got[0].tobytes() == want[0].tobytes() and got[1].tobytes() == want[1].tobytes()


def test_graph_replay_speeds_up_small_systems(cuda, capsys):
    """Calls of fewer than 32 steps launch kernel by kernel; longer ones
    replay graphs, on a non-default stream and from the legacy one."""
    import torch

    n, steps = 1024, 320
    p, v = ics.plummer(n, seed=6)
    side = torch.cuda.Stream()
    legacy = torch.cuda.default_stream()
    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-3), dt=np.float32(1e-3)) as s:
        s.set_state(ics.f32(p), ics.f32(v))
        times = {}
        for name, st, per_call in (("launches", legacy, 16), ("graph", side, steps),
                                   ("graph_legacy", legacy, steps)):
            with torch.cuda.stream(st):
                h = 0 if st is legacy else st.cuda_stream
                s.step(steps, stream=h)  # warm-up (captures the graph)
                st.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                for _ in range(steps // per_call):
                    s.step(per_call, stream=h)
                b.record(st)
                b.synchronize()
                times[name] = a.elapsed_time(b) / steps
    with capsys.disabled():
        print(f"\n[small N] N={n}: {times['launches'] * 1e3:.1f} us/step launched, "
              f"{times['graph'] * 1e3:.1f} us/step from the graph, "
              f"{times['graph_legacy'] * 1e3:.1f} from the legacy stream")
    assert times["graph"] < times["launches"]
    assert times["graph_legacy"] < times["launches"]


@pytest.mark.parametrize("prec,algo", MODES)
def test_set_params_equals_a_fresh_context(cuda, prec, algo):
    """nb_set_params (setSoftening / setDamping / update(dt)) mid-run: the
    steps after it equal those of a context created with the new values,
    also through a graph captured before the change."""
    import torch

    dt_ = dtype_of(prec)
    n = 500
    p, v = ics.plummer(n, seed=8)
    p, v = p.astype(dt_), v.astype(dt_)
    side = torch.cuda.Stream()
    kw = dict(kick="physical", eps2=1e-3, damping=1.0, dt=1e-3)
    with system(n, prec, algo, **kw) as s:
        s.set_state(p, v)
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            s.step(40, stream=side.cuda_stream)  # captures a graph with the old values
            side.synchronize()
        mid = s.get_state()
        s.set_params(2e-3, 0.99, 5e-4)
        with torch.cuda.stream(side):
            s.step(40, stream=side.cuda_stream)
            side.synchronize()
        got = s.get_state()
    with system(n, prec, algo, kick="physical", eps2=2e-3, damping=0.99, dt=5e-4) as f:
        f.set_state(*mid)
        for _ in range(40):
            f.step(1)
        want = f.get_state()
    assert got[0].tobytes() == want[0].tobytes() and got[1].tobytes() == want[1].tobytes()


def test_set_params_rejects_non_finite(cuda):
    with NBodySystem(16, "f32", "sym") as s:
        assert s.lib.nb_set_params(s.handle, float("nan"), 1.0, 1e-3, 1.0) == N.NB_ERR_INVALID
        assert s.lib.nb_set_params(None, 1e-3, 1.0, 1e-3, 1.0) == N.NB_ERR_INVALID


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_batch_set_params(cuda, algo):
    import torch

    sizes = [5, 300, 64]
    p, v = ics.uniform_cube(369, seed=3)
    p32, v32 = ics.f32(p), ics.f32(v)
    side = torch.cuda.Stream()
    with NBodyBatch(sizes, eps2=np.float32(1e-3), dt=np.float32(1e-3), algo=algo) as b:
        b.set_state(p32, v32)
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            b.run(6, side.cuda_stream)
            side.synchronize()
        mid = b.get_state()
        b.set_params(np.float32(2e-3), 1.0, np.float32(5e-4))
        with torch.cuda.stream(side):
            b.run(6, side.cuda_stream)  # the old graph was dropped
            side.synchronize()
        got = b.get_state()
    with NBodyBatch(sizes, eps2=np.float32(2e-3), dt=np.float32(5e-4), algo=algo) as f:
        f.set_state(*mid)
        f.step(6)
        want = f.get_state()
    assert got[0].tobytes() == want[0].tobytes()


def test_step_inside_a_callers_graph_capture(cuda):
    """A caller capturing its own stream into a CUDA graph can put nb_step in
    it: nb_step then launches step by step into that capture instead of
    capturing a graph of its own."""
    import torch

    n = 300
    p, v = ics.plummer(n, seed=9)
    p32, v32 = ics.f32(p), ics.f32(v)
    side = torch.cuda.Stream()
    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-3), dt=np.float32(1e-3)) as s:
        s.set_state(p32, v32)
        for _ in range(40):
            s.step(1)
        want = s.get_state()
        s.set_state(p32, v32)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            s.step(40, stream=torch.cuda.current_stream().cuda_stream)
        g.replay()
        torch.cuda.synchronize()
        got = s.get_state()
    assert got[0].tobytes() == want[0].tobytes() and got[1].tobytes() == want[1].tobytes()


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_batch_run_inside_a_callers_graph_capture(cuda, algo):
    import torch

    sizes = [3, 250, 64]
    p, v = ics.uniform_cube(317, seed=11)
    p32, v32 = ics.f32(p), ics.f32(v)
    side = torch.cuda.Stream()
    with NBodyBatch(sizes, eps2=np.float32(1e-3), dt=np.float32(1e-3), algo=algo) as b:
        b.set_state(p32, v32)
        b.step(6)
        want = b.get_state()
        b.set_state(p32, v32)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            b.run(6, torch.cuda.current_stream().cuda_stream)
        g.replay()
        torch.cuda.synchronize()
        got = b.get_state()
    assert got[0].tobytes() == want[0].tobytes()


def test_python_layer_checks_device_buffers(cuda):
    """Device tensors of the wrong shape are refused before any copy (the C
    ABI copies whole buffers by the context's size); a tensor of another
    dtype is converted and gives the same state as the exact dtype."""
    import torch

    n = 300
    p64, v64 = ics.plummer(n, seed=11)
    with NBodySystem(n, "f64", "sym", kick="physical", eps2=1e-3, damping=1.0, dt=1e-3) as s:
        s.set_state(torch.from_numpy(p64).cuda(), torch.from_numpy(v64).cuda())
        want = s.get_state()
        s.set_state(torch.from_numpy(p64).float().cuda(), torch.from_numpy(v64).float().cuda())
        got = s.get_state()
        assert np.array_equal(got[0], p64.astype(np.float32).astype(np.float64))
        with pytest.raises(ValueError):
            s.set_state(torch.zeros((n - 1, 4), dtype=torch.float64, device="cuda"),
                        torch.zeros((n - 1, 4), dtype=torch.float64, device="cuda"))
        with pytest.raises(ValueError):
            s.get_state_device(torch.empty((n, 4), dtype=torch.float32, device="cuda"),
                               torch.empty((n, 4), dtype=torch.float32, device="cuda"))
        pt = torch.empty((n, 4), dtype=torch.float64, device="cuda")
        vt = torch.empty_like(pt)
        s.set_state(torch.from_numpy(p64).cuda(), torch.from_numpy(v64).cuda())
        s.get_state_device(pt, vt)
        torch.cuda.synchronize()
        assert np.array_equal(pt.cpu().numpy(), want[0])
    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-3), damping=1.0,
                     dt=np.float32(1e-3)) as s:
        s.set_state(ics.f32(p64), ics.f32(v64))
        s.adj_forward(4, 2)
        g = torch.randn((n, 4), device="cuda") * 1e-3
        a = [t.clone() for t in s.adj_backward(g)]
        b = s.adj_backward(g.double())
        assert all(torch.equal(x, y) for x, y in zip(a, b))
        with pytest.raises(ValueError):
            s.adj_backward(torch.zeros((n, 3), device="cuda"))
        with pytest.raises(ValueError):
            s.adj_backward(g.cpu())


@pytest.mark.parametrize("prec,algo", MODES)
def test_coincident_bodies_every_mode(cuda, prec, algo):
    """Bodies at the same point (every body has a twin, three share one
    point): with eps2 > 0 their pair terms are exactly 0 (r = 0) and every
    acceleration stays finite and equal to the oracle's."""
    base, _ = ics.plummer(300, seed=21)
    pos = np.concatenate([base, base])
    pos[7, :3] = pos[8, :3] = pos[9, :3]
    pos[:, 3] = 1.0 / pos.shape[0]
    dt = dtype_of(prec)
    host = pos.astype(dt)
    eps2 = 1e-3 if dt == np.float64 else np.float32(1e-3)
    with system(pos.shape[0], prec, algo, kick="physical", eps2=eps2, damping=1.0) as s:
        s.set_state(host, np.zeros_like(host))
        a = s.accel().astype(np.float64)
    want = oracle.accel(host.astype(np.float64), float(eps2))
    assert np.isfinite(a).all()
    tol = 1e-12 if prec == "f64" else 1e-5
    d = np.linalg.norm(a - want, axis=1)
    w = np.linalg.norm(want, axis=1)
    assert (d <= tol * (w + w.mean())).all()


@pytest.mark.parametrize("prec,algo", MODES)
def test_zero_softening_is_nan_like_the_reference(cuda, prec, algo):
    """The reference sums over every j including i (bodysystem.cc:115-125,
    bodysystem_kernel.cu:60-85), so with eps2 = 0 the self term is 0 * inf
    and every acceleration is NaN; each mode gives the same."""
    p, _ = ics.plummer(64, seed=1)
    dt = dtype_of(prec)
    host = p.astype(dt)
    assert np.isnan(oracle.accel(host, 0.0)).all()
    with system(64, prec, algo, kick="physical", eps2=0.0, damping=1.0) as s:
        s.set_state(host, np.zeros_like(host))
        assert np.isnan(s.accel()).all()


TOL = {("f32", "fast"): 2e-5, ("f32", "sym"): 2e-5, ("f32", "symfx"): 2e-5, ("f32", "symband"): 2e-5,
       ("f32", "exact"): 2e-5, ("f64", "exact"): 1e-14, ("f64", "sym"): 1e-13, ("f64", "symband"): 1e-13,
       ("f64", "sym64"): 1e-13, ("f32comp", "fast"): 2e-6, ("f32comp", "sym"): 2e-6, ("f32comp", "symband"): 2e-6}


@pytest.mark.parametrize("prec,algo", MODES)
@pytest.mark.parametrize("n", [1, 3, 4, 5, 127, 128, 129])
def test_small_sizes_every_mode(cuda, prec, algo, n):
    """The small sizes of the test plan (tails of every tile and warp): the
    accelerations against the oracle at each mode's tolerance, and one step's
    positions against the oracle's step."""
    p, v = ics.plummer(n, seed=50 + n)
    dt = dtype_of(prec)
    pos = p.astype(np.float32).astype(dt) if prec == "f32" else p.astype(dt)
    vel = v.astype(np.float32).astype(dt) if prec == "f32" else v.astype(dt)
    eps2 = 1e-2 if dt == np.float64 else np.float32(1e-2)
    with system(n, prec, algo, kick="physical", eps2=eps2, damping=1.0, dt=1e-3 if dt == np.float64
                     else np.float32(1e-3)) as s:
        s.set_state(pos, vel)
        a = np.asarray(s.accel(), np.float64)
        s.step(1)
        p1, _ = s.get_state()
    want = oracle.accel(np.asarray(pos, np.float64), float(eps2))
    d = np.linalg.norm(a - want, axis=1)
    w = np.linalg.norm(want, axis=1)
    assert (d <= TOL[(prec, algo)] * (w + w.mean())).all()
    wp, _ = oracle.step(np.asarray(pos, np.float64), np.asarray(vel, np.float64), float(eps2), 1.0,
                        float(np.float32(1e-3)) if dt != np.float64 else 1e-3, 1, kick_mode=oracle.KICK_PHYSICAL)
    rel = np.linalg.norm(np.asarray(p1, np.float64)[:, :3] - wp[:, :3], axis=1) / (
        np.linalg.norm(wp[:, :3], axis=1) + 0.1)
    assert rel.max() <= 1e-6


@pytest.mark.parametrize("prec,algo", MODES)
@pytest.mark.parametrize("n", [0, 1, 2])
def test_energy_tiny_systems_every_mode(cuda, prec, algo, n):
    """nb_energy in every mode on 0, 1 and 2 bodies: zeros for none, no
    potential for one (the sum runs over j != i), the oracle's values for
    two."""
    dt = dtype_of(prec)
    p, v = ics.plummer(max(n, 1), seed=7)
    pos, vel = p[:n].astype(dt), v[:n].astype(dt)
    eps2 = 1e-2 if dt == np.float64 else np.float32(1e-2)
    with system(n, prec, algo, kick="physical", eps2=eps2) as s:
        s.set_state(pos, vel)
        e = s.energy()
    if n == 0:
        assert np.array_equal(e, np.zeros(5))
        return
    ref = np.array(oracle.energy(np.asarray(pos, np.float64), np.asarray(vel, np.float64), float(eps2)))
    assert np.allclose(e, ref, rtol=1e-5, atol=1e-12)
    if n == 1:
        assert e[1] == 0.0
