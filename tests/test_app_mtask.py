"""The multi-task app driver (utc_gb300/nbody_mtask, the reference's
benchapps/nbody/utc/nbody_mtask.cc flags): T systems through one batched
launch per step (default) or one GPU task per system (-B 0, the reference's
pattern); both write every system's frames with -O, and they agree to the
printed precision in double (the app's FTYPE) and float state."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

APP = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "utc_gb300", "nbody_mtask")


def frames_of(path, ntasks, n, nframes):
    lines = open(path).read().splitlines()
    assert len(lines) == ntasks * nframes * (n + 1)
    vals = []
    for k in range(ntasks * nframes):
        block = lines[k * (n + 1):(k + 1) * (n + 1)]
        float(block[0])  # the frame's time line
        vals.append(np.array([[float(x) for x in ln.split()] for ln in block[1:]]))
    return np.array(vals).reshape(ntasks, nframes, n, 4)


@pytest.mark.parametrize("state", ["double", "float"])
def test_mtask_batched_equals_per_task(cuda, tmp_path, state):
    n, ntasks, loops, oi = 256, 4, 10, 5
    extra = ["-F"] if state == "float" else []
    out = {}
    for mode in ("1", "0"):
        path = str(tmp_path / f"out{mode}.txt")
        r = subprocess.run([APP, "-v", "-n", str(n), "-T", str(ntasks), "-l", str(loops), "-o", str(oi),
                            "-O", path, "-B", mode] + extra, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "Test complete !!!" in r.stdout and f"Number of tasks: {ntasks}" in r.stdout
        out[mode] = frames_of(path, ntasks, n, loops // oi + 1)
    batched, tasks = out["1"], out["0"]
    # frame 0 is every system's start; the systems differ (one rand() stream)
    assert np.array_equal(batched[:, 0], tasks[:, 0])
    assert not np.array_equal(tasks[0, 0], tasks[1, 0])
    tol = 2e-5 if state == "double" else 1e-4 * (np.abs(tasks).max() + 1)
    assert np.abs(batched - tasks).max() <= tol


@pytest.mark.parametrize("state", ["double", "float"])
def test_mtask_many_tasks_at_once(cuda, state):
    # sixteen tasks, each on its own thread, create, capture their step graphs
    # (50 steps per frame), copy and destroy at the same time; every run ends
    # cleanly and every task reports success
    extra = ["-F"] if state == "float" else []
    for _ in range(3):
        r = subprocess.run([APP, "-v", "-n", "1024", "-T", "16", "-l", "100", "-o", "50", "-B", "0"] + extra,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        assert "status" not in r.stderr and "Test complete !!!" in r.stdout


@pytest.mark.parametrize("state", ["double", "float"])
def test_mtask_grouped_tasks_equal_the_batch(cuda, tmp_path, state):
    # -B 2: one task per system, the tasks joined in one BodyTaskGroup, whose
    # run is the same batch as -B 1: the frames agree bit for bit
    n, ntasks, loops, oi = 512, 6, 40, 20
    extra = ["-F"] if state == "float" else []
    out = {}
    for mode in ("1", "2"):
        path = str(tmp_path / f"out{mode}.txt")
        r = subprocess.run([APP, "-v", "-n", str(n), "-T", str(ntasks), "-l", str(loops), "-o", str(oi),
                            "-O", path, "-B", mode] + extra, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "Test complete !!!" in r.stdout
        out[mode] = open(path).read()
    assert out["1"] == out["2"]


@pytest.mark.parametrize("algo", ["0", "1"])
def test_mtask_algorithm_flag_reaches_the_tasks(cuda, tmp_path, algo):
    # -a goes to every task with -B 0 and -B 2.  A group runs the directed
    # kernel (-a 0) as one batch and the reference-exact one (-a 1, no
    # batched form) system after system; either way its frames equal the
    # lone tasks' frames
    out = {}
    for mode in ("0", "2"):
        path = str(tmp_path / f"out{mode}.txt")
        r = subprocess.run([APP, "-F", "-n", "256", "-T", "3", "-l", "10", "-o", "5", "-O", path, "-B", mode,
                            "-a", algo], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        out[mode] = frames_of(path, 3, 256, 3)
        assert np.isfinite(out[mode]).all()
    if algo == "1":  # the same single-system exact runs: byte for byte
        assert out["0"].tobytes() == out["2"].tobytes()
    else:  # the directed batch against the directed single-system kernel
        assert np.abs(out["0"] - out["2"]).max() <= 1e-4 * (np.abs(out["0"]).max() + 1)
