"""GPU parity of the C-ABI kernels against the CPU oracle.

Tolerances (float32 fast path; the exact path is checked bit for bit):
  * accelerations: per body |a_gpu - a_ref| <= 2e-5 * (|a_ref| + mean|a_ref|)
    against the FP64 oracle on the same float32 positions (rsqrt.approx is
    within 2 ulp and the partial sums run in a different order than the
    reference's sequential loop);
  * positions after the stated steps: per body |x_gpu - x_orc| <= 1e-5 *
    (|x_orc| + 0.1);
  * displacement x_T - x_0: per body within 1e-5 relative plus 4 float ulps
    of the position (the storage granularity of float positions).
"""
import json
import os

import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel_body_err(got, want):
    d = np.linalg.norm(np.asarray(got, np.float64) - np.asarray(want, np.float64), axis=1)
    w = np.linalg.norm(np.asarray(want, np.float64), axis=1)
    return d, w


def assert_accel_close(got, want, tol=2e-5):
    d, w = rel_body_err(got, want)
    bound = tol * (w + w.mean())
    bad = np.nonzero(d > bound)[0]
    assert bad.size == 0, f"{bad.size} bodies off, worst ratio {np.max(d / np.maximum(bound, 1e-300))}"


def cube_f32(n, seed=0):
    p, v = ics.uniform_cube(n, seed=seed)
    return ics.f32(p), ics.f32(v)


# ---------------------------------------------------------------------------
# exact algorithm: bit-identical to the reference's sequential BodySystem<T>
# ---------------------------------------------------------------------------
def test_exact_f32_reproduces_reference_golden_frames(cuda):
    kat = json.load(open(os.path.join(GOLD, "kat_shell_n1024.json")))
    sc = kat["scenario"]
    dt, cs, vs, soft, damp = oracle.demo_params(sc["para_select"], sc["n"])
    pos, vel = oracle.randomize(1, sc["n"], np.float32, seed=sc["rand_seed"])
    eps2 = np.float32(soft) * np.float32(soft)
    with NBodySystem(sc["n"], "f32", "exact", eps2=eps2, damping=damp, dt=dt) as s:
        s.set_state(pos, vel)
        s.step(sc["steps"])
        p1, _ = s.get_state()
    import hashlib

    text = oracle.format_frames([pos, p1], dt)
    assert hashlib.sha256(text.encode()).hexdigest() == kat["seq_outpos_sha256"]


@pytest.mark.parametrize("n", [1, 2, 3, 5, 31, 127, 129, 1000])
@pytest.mark.parametrize("kick", ["reference", "physical"])
def test_exact_f32_bitwise(cuda, n, kick):
    pos, vel = cube_f32(n, seed=n)
    km = oracle.KICK_REFERENCE if kick == "reference" else oracle.KICK_PHYSICAL
    want_p, want_v = oracle.step(pos, vel, np.float32(1e-2), np.float32(0.999), np.float32(1e-3), 6,
                                 kick_mode=km, G=np.float32(0.7))
    with NBodySystem(n, "f32", "exact", kick=kick, eps2=np.float32(1e-2), damping=np.float32(0.999),
                     dt=np.float32(1e-3), G=np.float32(0.7), block=64) as s:
        s.set_state(pos, vel)
        s.step(6)
        p, v = s.get_state()
    assert p.tobytes() == want_p.tobytes() and v.tobytes() == want_v.tobytes()


@pytest.mark.parametrize("n", [1, 4, 100, 513])
def test_exact_f64_bitwise(cuda, n):
    pos, vel = ics.uniform_cube(n, seed=n + 1)
    want_p, want_v = oracle.step(pos, vel, 1e-2, 0.995, 1e-3, 5)
    with NBodySystem(n, "f64", "exact", eps2=1e-2, damping=0.995, dt=1e-3) as s:
        s.set_state(pos, vel)
        s.step(5)
        p, v = s.get_state()
    assert p.tobytes() == want_p.tobytes() and v.tobytes() == want_v.tobytes()


# ---------------------------------------------------------------------------
# fast algorithm
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("kick", ["reference", "physical"])
def test_fast_plain_cpu_scale_workload(cuda, kick):
    """N=4096 uniform cube, masses U[0.5,1.5]/N, eps2=1e-2, dt=1e-3,
    damping 1, 10 steps, seed 0: positions, per-step accelerations and the
    displacement against the oracle."""
    n, steps = 4096, 10
    pos, vel = cube_f32(n, seed=0)
    km = oracle.KICK_REFERENCE if kick == "reference" else oracle.KICK_PHYSICAL
    eps2, dt = np.float32(1e-2), np.float32(1e-3)
    with NBodySystem(n, "f32", "fast", kick=kick, eps2=eps2, damping=1.0, dt=dt, G=1.0) as s:
        s.set_state(pos, vel)
        cur_p, cur_v = pos, vel
        for _ in range(steps):
            a_gpu = s.accel()
            a_ref = oracle.accel(cur_p.astype(np.float64), float(eps2))
            assert_accel_close(a_gpu, a_ref)
            s.step(1)
            cur_p, cur_v = oracle.step(cur_p, cur_v, eps2, 1.0, dt, 1, kick_mode=km)
        p, v = s.get_state()
    d, w = rel_body_err(p[:, :3], cur_p[:, :3])
    assert (d <= 1e-5 * (w + 0.1)).all(), d.max()
    disp_gpu = p[:, :3].astype(np.float64) - pos[:, :3]
    disp_orc = cur_p[:, :3].astype(np.float64) - pos[:, :3]
    ulp = np.spacing(np.abs(cur_p[:, :3]).astype(np.float32)).astype(np.float64)
    assert (np.abs(disp_gpu - disp_orc) <= 1e-5 * np.abs(disp_orc) + 4 * ulp).all()
    assert np.array_equal(p[:, 3], pos[:, 3]) and np.array_equal(v[:, 3], vel[:, 3])


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_fast_kat_within_reference_gpu_envelope(cuda, algo):
    """The golden scenario (SHELL, N=1024, 100 chaotic steps) on the directed
    and symmetric paths stays within the envelope the reference's own GPU run
    shows around the sequential frames."""
    kat = json.load(open(os.path.join(GOLD, "kat_shell_n1024.json")))
    env = kat["gpu_vs_seq_final_frame"]
    dt, cs, vs, soft, damp = oracle.demo_params(0, 1024)
    pos, vel = oracle.randomize(1, 1024, np.float32)
    eps2 = np.float32(soft) * np.float32(soft)
    want, _ = oracle.step(pos, vel, eps2, damp, dt, 100)
    with NBodySystem(1024, "f32", algo, eps2=eps2, damping=damp, dt=dt) as s:
        s.set_state(pos, vel)
        s.step(100)
        got, _ = s.get_state()
    d = np.abs(got[:, :3].astype(np.float64) - want[:, :3])
    assert np.median(d) <= 10 * env["median_abs"]
    assert d.max() <= 10 * env["max_abs"]


@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 127, 128, 129, 255, 257, 1000, 2047, 2049, 4097])
def test_fast_accel_ragged_sizes(cuda, n):
    pos, _ = cube_f32(n, seed=100 + n)
    vel = np.zeros_like(pos)
    with NBodySystem(n, "f32", "fast", eps2=np.float32(1e-2)) as s:
        s.set_state(pos, vel)
        a = s.accel()
    assert_accel_close(a, oracle.accel(pos.astype(np.float64), float(np.float32(1e-2))))


@pytest.mark.parametrize("block,bpt", [(128, 2), (128, 4), (128, 8), (256, 2), (256, 4), (256, 8)])
@pytest.mark.parametrize("ctas", [0, 1])
def test_fast_launch_shapes(cuda, block, bpt, ctas):
    n = 3001
    pos, _ = cube_f32(n, seed=7)
    vel = np.zeros_like(pos)
    with NBodySystem(n, "f32", "fast", eps2=np.float32(1e-3), block=block, bpt=bpt,
                     ctas_per_sm=ctas) as s:
        s.set_state(pos, vel)
        a = s.accel()
        info = s.plan_info()
    assert info["block"] == block and info["bpt"] == bpt
    assert_accel_close(a, oracle.accel(pos.astype(np.float64), float(np.float32(1e-3))))


def test_fast_deterministic(cuda):
    n = 5000
    pos, vel = cube_f32(n, seed=11)
    outs = []
    for _ in range(2):
        with NBodySystem(n, "f32", "fast", kick="physical", eps2=np.float32(1e-2), damping=1.0,
                         dt=np.float32(1e-3)) as s:
            s.set_state(pos, vel)
            s.step(20)
            outs.append(s.get_state())
    assert outs[0][0].tobytes() == outs[1][0].tobytes()
    assert outs[0][1].tobytes() == outs[1][1].tobytes()


def test_fast_gpu_scale_plummer_properties(cuda):
    """N=65536 Plummer, masses 1/N, eps2=1e-4, dt=1e-4, 100 steps at full size:
    accelerations on a 512-body subsample against the FP64 oracle, momentum
    balance of the force sum, rerun determinism."""
    n = 65536
    p64, v64 = ics.plummer(n, seed=0)
    pos, vel = ics.f32(p64), ics.f32(v64)
    eps2, dt = np.float32(1e-4), np.float32(1e-4)
    with NBodySystem(n, "f32", "fast", kick="physical", eps2=eps2, damping=1.0, dt=dt) as s:
        s.set_state(pos, vel)
        a = s.accel()
        tidx = np.random.default_rng(0).choice(n, 512, replace=False).astype(np.int32)
        ref = oracle.accel_subset_f64(pos.astype(np.float64), tidx, float(eps2))
        assert_accel_close(a[tidx], ref)
        m = pos[:, 3].astype(np.float64)
        f = (a.astype(np.float64) * m[:, None])
        assert np.linalg.norm(f.sum(0)) <= 1e-4 * np.abs(f).sum()
        s.step(100)
        p1, v1 = s.get_state()
    with NBodySystem(n, "f32", "fast", kick="physical", eps2=eps2, damping=1.0, dt=dt) as s:
        s.set_state(pos, vel)
        s.step(100)
        p2, v2 = s.get_state()
    assert np.isfinite(p1).all() and p1.tobytes() == p2.tobytes() and v1.tobytes() == v2.tobytes()


# ---------------------------------------------------------------------------
# boundary: host runs, drop-in task, errors, empty input
# ---------------------------------------------------------------------------
def test_run_host_frames_match_stepping(cuda):
    n = 2048
    pos, vel = oracle.randomize(1, n, np.float32)
    with NBodySystem(n, "f32", "fast", eps2=np.float32(0.01), damping=1.0, dt=np.float32(0.016)) as s:
        frames, t = s.run_host(pos, vel, 12, 4)
        s.set_state(pos, vel)
        want = []
        for _ in range(3):
            s.step(4)
            want.append(s.get_state()[0])
    assert frames.shape == (3, n, 4)
    for k in range(3):
        assert frames[k].tobytes() == want[k].tobytes()
    assert t[0] > 0 and t[1] > 0 and t[2] >= 0 and t[3] >= 0


@pytest.mark.parametrize("memtype", [0, 1, 2])
def test_drop_in_task_f32(cuda, memtype):
    import ctypes as C

    from utc_gb300 import _native as N

    n, loops, oi = 1024, 20, 5
    pos, vel = oracle.randomize(1, n, np.float32)
    dt, _, _, soft, damp = oracle.demo_params(0, n)
    eps2 = np.float32(soft) * np.float32(soft)
    out = np.zeros((loops // oi, n, 4), np.float32)
    rt = (C.c_double * 4)()
    p_in, v_in = pos.copy(), vel.copy()
    rc = N.task_lib().nbt_run_f32(n, eps2, np.float32(damp), p_in.ctypes.data_as(C.c_void_p),
                                  v_in.ctypes.data_as(C.c_void_p), rt, loops, oi, 256,
                                  np.float32(dt), out.ctypes.data_as(C.c_void_p), memtype, -1, 0)
    assert rc == 0
    assert p_in.tobytes() == pos.tobytes()  # the task does not write its inputs
    with NBodySystem(n, "f32", "sym", eps2=eps2, damping=damp, dt=dt) as s:
        frames, _ = s.run_host(pos, vel, loops, oi)
    assert out.tobytes() == frames.tobytes()
    assert rt[0] > 0 and rt[1] > 0


def test_drop_in_task_f64_exact_matches_oracle(cuda):
    import ctypes as C

    from utc_gb300 import _native as N

    n, loops, oi = 512, 6, 3
    pos, vel = oracle.randomize(1, n, np.float64)
    dt, _, _, soft, damp = oracle.demo_params(0, n)
    s64 = float(np.float32(soft))
    eps2 = s64 * s64
    out = np.zeros((loops // oi, n, 4), np.float64)
    rt = (C.c_double * 4)()
    rc = N.task_lib().nbt_run_f64(n, eps2, float(np.float32(damp)), pos.ctypes.data_as(C.c_void_p),
                                  vel.ctypes.data_as(C.c_void_p), rt, loops, oi, 128,
                                  float(np.float32(dt)), out.ctypes.data_as(C.c_void_p), 0, 1, 0)
    assert rc == 0
    p, v = pos, vel
    for k in range(loops // oi):
        p, v = oracle.step(p, v, eps2, float(np.float32(damp)), float(np.float32(dt)), oi)
        assert out[k].tobytes() == p.tobytes()


@pytest.mark.parametrize("memtype", [0, 1, 2])
def test_drop_in_task_f64_default_symmetric(cuda, memtype):
    """The double task's default algorithm (the float-float symmetric kernel)
    against the FP64 oracle, frames every 4 steps, pageable / pinned / unified
    staging: positions within 1e-12 relative in every frame."""
    import ctypes as C

    from utc_gb300 import _native as N

    n, loops, oi = 1024, 8, 4
    pos, vel = oracle.randomize(1, n, np.float64)
    dt, _, _, soft, damp = oracle.demo_params(0, n)
    eps2 = float(np.float32(soft)) ** 2
    out = np.zeros((loops // oi, n, 4), np.float64)
    rt = (C.c_double * 4)()
    rc = N.task_lib().nbt_run_f64(n, eps2, float(np.float32(damp)), pos.ctypes.data_as(C.c_void_p),
                                  vel.ctypes.data_as(C.c_void_p), rt, loops, oi, 128,
                                  float(np.float32(dt)), out.ctypes.data_as(C.c_void_p), memtype, -1, 0)
    assert rc == 0
    p, v = pos, vel
    for k in range(loops // oi):
        p, v = oracle.step(p, v, eps2, float(np.float32(damp)), float(np.float32(dt)), oi)
        rel = np.linalg.norm(out[k][:, :3] - p[:, :3], axis=1) / (np.linalg.norm(p[:, :3], axis=1) + 1e-3)
        assert rel.max() <= 1e-12


def test_status_codes_on_device(cuda):
    import ctypes as C

    from utc_gb300 import _native as N

    with NBodySystem(64, "f32", "fast") as s:
        assert s.lib.nb_step(s.handle, 1, None) == N.NB_ERR_STATE
        assert s.lib.nb_get_state(s.handle, None, None, 0, None) == N.NB_ERR_STATE
        assert s.lib.nb_step(s.handle, -1, None) == N.NB_ERR_INVALID
        assert s.lib.nb_run_host(s.handle, None, None, 1, 0, None, None, None) == N.NB_ERR_INVALID
        pos, vel = cube_f32(64)
        s.set_state(pos, vel)
        assert s.lib.nb_accel(s.handle, None, None) == N.NB_ERR_INVALID
        assert s.lib.nb_set_state(s.handle, pos.ctypes.data_as(C.c_void_p), None, 0, None) == N.NB_ERR_INVALID
        assert s.launches_per_step() == 2


def test_empty_system(cuda):
    with NBodySystem(0, "f32", "fast") as s:
        s.set_state(np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32))
        s.step(3)
        p, v = s.get_state()
        assert p.shape == (0, 4)
        assert s.launches_per_step() == 0


def test_app_driver_reproduces_golden_file(cuda, tmp_path):
    """The app driver (the reference's flags; bodies from NbodyInit's SHELL
    initialiser on rand(); Task<BodySystemGB300<float>> with the exact
    algorithm; frames through Task<Output<float>>) writes the reference's
    golden output file byte for byte."""
    import hashlib
    import subprocess

    kat = json.load(open(os.path.join(GOLD, "kat_shell_n1024.json")))
    app = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "utc_gb300", "nbody_main")
    out = tmp_path / "outpos.txt"
    r = subprocess.run([app, "-F", "-a", "1", "-n", "1024", "-i", "0", "-l", "100", "-o", "100",
                        "-O", str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    data = out.read_bytes()
    assert len(data) == kat["seq_outpos_bytes"]
    assert hashlib.sha256(data).hexdigest() == kat["seq_outpos_sha256"]
    # the default (symmetric) run of the same scenario stays within the
    # envelope of the reference's own GPU run
    out2 = tmp_path / "outpos_sym.txt"
    r = subprocess.run([app, "-F", "-n", "1024", "-i", "0", "-l", "100", "-o", "100", "-O", str(out2)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    a = np.array(data.decode().split(), dtype=np.float64)
    b = np.array(out2.read_text().split(), dtype=np.float64)
    assert a.shape == b.shape
    d = np.abs(a - b)
    assert d.max() <= 10 * kat["gpu_vs_seq_final_frame"]["max_abs"]
