"""The drop-in task (BodySystemGB300<T> on the UTC task stand-in) run on the
CPU against a host-only mock of the C ABI (tests/mock_abi.cc: nb_run_host
steps with the oracle; the stand-in's four CUDA runtime calls hand out a
recognisable fake stream).  Checks the task's plumbing without a GPU:
initImpl keeps the caller's pointers and runImpl reads them at run time,
frames land at outbuffer + f * 4N, runtime[4] is filled, the parameters and
the worker's own stream reach the C ABI, the input arrays are not updated,
and a failing C-ABI call comes back as the task's status.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def mock_task(tmp_path_factory):
    oracle.build(ref=False)
    out = str(tmp_path_factory.mktemp("taskmock") / "libtaskmock.so")
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    odir = os.path.join(REPO, "oracle")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-o", out,
           os.path.join(REPO, "utc_gb300", "task", "body_task_gb300.cc"),
           os.path.join(REPO, "utc_gb300", "task", "body_task_mgpu_gb300.cc"), os.path.join(REPO, "tests", "mock_abi.cc"),
           "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "utc_gb300", "task"), "-I", odir,
           "-I", os.path.join(cuda_home, "include"), "-L", odir, "-loracle", "-Wl,-rpath," + odir, "-lpthread",
           # bind the library's calls to its own mock definitions even when a real CUDA runtime (torch's)
           # is already in the process's global symbol scope
           "-Wl,-Bsymbolic"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = C.CDLL(out)
    vp, I, D = C.c_void_p, C.c_int, C.c_double
    lib.nbt_run_f64.argtypes = [C.c_uint, D, D, vp, vp, vp, I, I, I, D, vp, I, I, I]
    lib.nbt_run_f32.argtypes = [C.c_uint, C.c_float, C.c_float, vp, vp, vp, I, I, I, C.c_float, vp, I, I, I]
    lib.mock_fake_stream.restype = vp
    lib.mock_record.argtypes = [C.POINTER(vp), vp, vp]
    lib.nbt_mgpu_run_f32.argtypes = [C.c_uint, C.c_float, C.c_float, vp, vp, vp, I, I, I, C.c_float, vp, I, I]
    lib.nbt_mgpu_run_f64.argtypes = [C.c_uint, D, D, vp, vp, vp, I, I, I, D, vp, I, I]
    lib.path = out
    return lib


def record(lib):
    s = C.c_void_p()
    ints = np.zeros(9, np.int32)
    dbl = np.zeros(3, np.float64)
    lib.mock_record(C.byref(s), ints.ctypes.data_as(C.c_void_p), dbl.ctypes.data_as(C.c_void_p))
    return s.value, ints, dbl


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_task_plumbing_on_the_mock(mock_task, dtype):
    n, loops, oi = 96, 12, 4
    pos, vel = oracle.randomize(1, n, dtype)
    pos0, vel0 = pos.copy(), vel.copy()
    eps2, damp, dt = 0.01, 0.999, 0.005
    frames = np.full((loops // oi + 1, n, 4), -7.0, dtype)  # one spare frame stays untouched
    rt = np.zeros(4, np.float64)
    run = mock_task.nbt_run_f64 if dtype == np.float64 else mock_task.nbt_run_f32
    rc = run(n, eps2, damp, pos.ctypes.data, vel.ctypes.data, rt.ctypes.data, loops, oi, 128, dt,
             frames.ctypes.data, 1, -1, 0)
    assert rc == 0
    # the caller's arrays are read, not updated (body_task_sgpu.cu:20-26)
    assert np.array_equal(pos, pos0) and np.array_equal(vel, vel0)
    # frames f = 0.. at outbuffer + f * 4N, each after (f + 1) * oi steps
    p, v = pos0, vel0
    for f in range(loops // oi):
        p, v = oracle.step(p, v, dtype(eps2), dtype(damp), dtype(dt), oi)
        assert np.array_equal(frames[f], p)
    assert (frames[-1] == -7.0).all()
    assert list(rt) == [1.0, 2.0, 3.0, 4.0]
    stream, ints, dbl = record(mock_task)
    calls, rn, rloops, roi, prec, algo, memtype, made, destroyed = ints
    assert stream == mock_task.mock_fake_stream()  # launched on the worker's own stream
    assert (rn, rloops, roi) == (n, loops, oi)
    assert prec == (1 if dtype == np.float64 else 0)  # NB_F64 / NB_F32
    assert algo == 2  # NB_ALGO_SYM, the task's default for both state types
    assert memtype == 1  # NB_MEM_PINNED passed through
    np.testing.assert_allclose(dbl, [float(dtype(eps2)), float(dtype(damp)), float(dtype(dt))])
    assert made >= 1 and destroyed >= 1  # the worker made and released its stream


def test_task_reports_a_failing_call(mock_task):
    n = 3  # the mock refuses this size
    pos, vel = oracle.randomize(1, 4, np.float64)
    frames = np.full((2, 4, 4), -7.0)
    rt = np.zeros(4, np.float64)
    rc = mock_task.nbt_run_f64(n, 0.01, 1.0, pos.ctypes.data, vel.ctypes.data, rt.ctypes.data, 2, 1, 128, 0.01,
                               frames.ctypes.data, 0, -1, 0)
    assert rc == 1  # NB_ERR_INVALID from nb_create, kept as the task's status
    assert (frames == -7.0).all() and (rt == 0).all()


# ---- BodyTaskGroup: tasks whose runs go as one batch ----

def group_run(lib, dtype, sizes, eps2s, loops, oi, members=None, timeout=30.0, damping=0.999, dt=0.005):
    n_sys = len(sizes)
    states = [oracle.randomize(1, n, dtype, seed=1 + k) for k, n in enumerate(sizes)]
    pos = [p for p, _ in states]
    vel = [v for _, v in states]
    frames = [np.full((loops // oi + 1, n, 4), -7.0, dtype) for n in sizes]  # one spare frame each
    ptr = C.c_void_p * n_sys
    st = np.full(n_sys, -1, np.int32)
    rt = np.zeros((n_sys, 4), np.float64)
    fn = lib.nbt_group_run_f64 if dtype == np.float64 else lib.nbt_group_run_f32
    T = C.c_double if dtype == np.float64 else C.c_float
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, T, T, C.c_int, C.c_int,
                   C.c_int, C.c_double, C.c_void_p, C.c_void_p]
    sz = np.asarray(sizes, np.int32)
    e = np.asarray(eps2s, dtype)
    lib.mock_batch_reset()
    rc = fn(n_sys, sz.ctypes.data, ptr(*[p.ctypes.data for p in pos]), ptr(*[v.ctypes.data for v in vel]),
            ptr(*[f.ctypes.data for f in frames]), e.ctypes.data, damping, dt, loops, oi,
            members or n_sys, timeout, st.ctypes.data, rt.ctypes.data)
    return rc, st, pos, vel, frames, rt


def batch_record(lib):
    ints = np.zeros(6, np.int32)
    s = C.c_void_p()
    lib.mock_batch_record(ints.ctypes.data_as(C.c_void_p), C.byref(s))
    return ints, s.value


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_group_runs_every_member_as_one_batch(mock_task, dtype):
    sizes, loops, oi = [64, 100, 36], 12, 4
    rc, st, pos, vel, frames, rt = group_run(mock_task, dtype, sizes, [0.01] * 3, loops, oi)
    assert rc == 0 and list(st) == [0, 0, 0]
    for k, n in enumerate(sizes):
        p, v = oracle.randomize(1, n, dtype, seed=1 + k)
        assert np.array_equal(pos[k], p) and np.array_equal(vel[k], v)  # inputs not updated
        for f in range(loops // oi):
            p, v = oracle.step(p, v, dtype(0.01), dtype(0.999), dtype(0.005), oi)
            assert np.array_equal(frames[k][f], p), (k, f)
        assert (frames[k][-1] == -7.0).all()
    (creates, runs, nsys, destroys, prec, algo), stream = batch_record(mock_task)
    assert (creates, runs, nsys, destroys) == (1, loops // oi, 3, 1)  # one batch, one run per frame
    assert prec == (1 if dtype == np.float64 else 0) and algo == 2
    assert stream == mock_task.mock_fake_stream()  # the batch's own stream
    # every member gets the batch's timers: 3 frames x 1 ms kernel, 1 ms copy-in, 3 x 1 ms copy-out
    for r in rt:
        assert r[0] > 0 and np.allclose(r[1:], [3e-3, 1e-3, 3e-3])


def test_group_refuses_members_that_differ(mock_task):
    rc, st, _, _, frames, _ = group_run(mock_task, np.float64, [64, 64], [0.01, 0.02], 8, 4)
    assert list(st) == [1, 1]  # NB_ERR_INVALID for every member
    assert all((f == -7.0).all() for f in frames)
    assert batch_record(mock_task)[0][0] == 0  # no batch made


def test_group_reports_a_failing_batch_to_every_member(mock_task):
    rc, st, _, _, frames, _ = group_run(mock_task, np.float32, [64, 3, 40], [0.01] * 3, 8, 4)
    assert list(st) == [1, 1, 1]  # the planted nb_batch_create failure
    assert all((f == -7.0).all() for f in frames)


def test_group_that_does_not_fill_times_out(mock_task):
    # a group of three with two tasks: the round ends at the timeout
    rc, st, _, _, frames, _ = group_run(mock_task, np.float64, [64, 64], [0.01] * 2, 8, 4, members=3, timeout=0.3)
    assert list(st) == [4, 4]  # NB_ERR_STATE
    assert all((f == -7.0).all() for f in frames)
    assert batch_record(mock_task)[0][0] == 0


def test_group_refuses_a_null_outbuffer(mock_task):
    sizes = [64, 64]
    states = [oracle.randomize(1, n, np.float64, seed=5 + k) for k, n in enumerate(sizes)]
    good = np.full((3, 64, 4), -7.0)
    ptr = C.c_void_p * 2
    st = np.full(2, -1, np.int32)
    e = np.full(2, 0.01)
    fn = mock_task.nbt_group_run_f64
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                   C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p]
    mock_task.mock_batch_reset()
    fn(2, np.asarray(sizes, np.int32).ctypes.data, ptr(*[p.ctypes.data for p, _ in states]),
       ptr(*[v.ctypes.data for _, v in states]), ptr(good.ctypes.data, None), e.ctypes.data, 0.999, 0.005,
       8, 4, 2, 30.0, st.ctypes.data, None)
    assert list(st) == [1, 1] and (good == -7.0).all()
    assert batch_record(mock_task)[0][0] == 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("nthreads", [1, 3, 4])
def test_mgpu_task_on_the_mock(mock_task, dtype, nthreads):
    """The multi-GPU task (BodySystemMGPU_GB300<T>) with `nthreads` threads on
    the mock: each thread steps its own range of targets (the reference's
    split, uneven here), pushes it into the other threads' position buffers
    after every step and writes its range of each frame; the frames equal
    the oracle's run of the whole system bit for bit, the caller's arrays
    are not updated and every thread fills its row of runtime."""
    n, loops, oi = 101, 12, 4
    pos, vel = oracle.randomize(1, n, dtype)
    pos0, vel0 = pos.copy(), vel.copy()
    eps2, damp, dt = 0.01, 0.999, 0.005
    frames = np.full((loops // oi + 1, n, 4), -7.0, dtype)
    rt = np.full((nthreads, 4), -1.0)
    run = mock_task.nbt_mgpu_run_f64 if dtype == np.float64 else mock_task.nbt_mgpu_run_f32
    rc = run(n, eps2, damp, pos.ctypes.data, vel.ctypes.data, rt.ctypes.data, loops, oi, 128, dt,
             frames.ctypes.data, nthreads, -1)
    assert rc == 0
    assert np.array_equal(pos, pos0) and np.array_equal(vel, vel0)
    p, v = pos0, vel0
    for f in range(loops // oi):
        p, v = oracle.step(p, v, dtype(eps2), dtype(damp), dtype(dt), oi)
        assert np.array_equal(frames[f], p), f
    assert (frames[-1] == -7.0).all()
    assert (rt >= 0).all()


def test_mgpu_task_failures_end_every_thread(mock_task):
    """A thread whose shard cannot be made (n = 5: shard 1 refused), or whose
    fifth step fails (n = 7), ends the run for every thread at the same
    barrier: the call returns the failing status instead of hanging, and a
    later run of the same task object works.  Run in a child process with a
    time limit, so that a deadlock fails the test."""
    import sys

    code = f"""
import ctypes as C, numpy as np
lib = C.CDLL({mock_task.path!r})
vp, I = C.c_void_p, C.c_int
lib.nbt_mgpu_run_f32.argtypes = [C.c_uint, C.c_float, C.c_float, vp, vp, vp, I, I, I, C.c_float, vp, I, I]
out = []
for n in (5, 7, 8):
    pos = np.zeros((n, 4), np.float32); pos[:, 0] = np.arange(n); pos[:, 3] = 1
    vel = np.zeros((n, 4), np.float32)
    frames = np.full((4, n, 4), -7.0, np.float32)
    rt = np.zeros((3, 4))
    rc = lib.nbt_mgpu_run_f32(n, 0.01, 1.0, pos.ctypes.data, vel.ctypes.data, rt.ctypes.data, 9, 3, 128, 0.001,
                              frames.ctypes.data, 3, -1)
    out.append((rc, bool((frames[0] == -7).all()), bool((frames[1] == -7).all())))
print(out)
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    res = eval(r.stdout.strip().splitlines()[-1])
    # n=5: refused at set-up, nothing written; n=7: the first frame (step 3)
    # is out, the failure at step 5 stops the second; n=8 runs clean
    assert res[0] == (1, True, True)
    assert res[1][0] == 2 and res[1][1] is False and res[1][2] is True
    assert res[2] == (0, False, False)
