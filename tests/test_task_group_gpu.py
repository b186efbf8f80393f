"""BodyTaskGroup on the GPU: tasks of ragged sizes (one per system, as the
reference's multi-task app, benchapps/nbody/utc/nbody_mtask.cc:199-231) whose
runs meet in one group go as one nb_batch, so every task's frames equal the
same batch run through the C ABI bit for bit, and follow the oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle
from utc_gb300 import _native as N
from utc_gb300.nbody import NBodyBatch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_group_frames_equal_the_batch(cuda, dtype):
    import torch

    sizes, loops, oi = [300, 1000, 64, 2048], 24, 8
    eps2, damp, dt = dtype(0.01), dtype(0.999), dtype(0.005)
    states = [oracle.randomize(1, n, dtype, seed=11 + k) for k, n in enumerate(sizes)]
    frames = [np.full((loops // oi, n, 4), -7.0, dtype) for n in sizes]
    ptr = C.c_void_p * len(sizes)
    st = np.full(len(sizes), -1, np.int32)
    rt = np.zeros((len(sizes), 4))
    fn = N.task_lib().nbt_group_run_f64 if dtype == np.float64 else N.task_lib().nbt_group_run_f32
    e = np.full(len(sizes), eps2, dtype)
    rc = fn(len(sizes), np.asarray(sizes, np.int32).ctypes.data, ptr(*[p.ctypes.data for p, _ in states]),
            ptr(*[v.ctypes.data for _, v in states]), ptr(*[f.ctypes.data for f in frames]), e.ctypes.data,
            damp, dt, loops, oi, len(sizes), 60.0, st.ctypes.data, rt.ctypes.data)
    assert rc == 0 and (st == 0).all()
    assert (rt[:, 0] > 0).all() and (rt[:, 1] > 0).all()
    # the same batch through the C ABI
    s = torch.cuda.Stream()
    prec = "f64" if dtype == np.float64 else "f32"
    with NBodyBatch(sizes, kick="reference", eps2=float(eps2), damping=float(damp), dt=float(dt),
                    precision=prec) as b:
        b.set_state(np.concatenate([p for p, _ in states]), np.concatenate([v for _, v in states]),
                    stream=int(s.cuda_stream))
        off = np.concatenate([[0], np.cumsum(sizes)])
        for f in range(loops // oi):
            b.run(oi, int(s.cuda_stream))
            pos, _ = b.get_state(stream=int(s.cuda_stream))
            for k in range(len(sizes)):
                assert frames[k][f].tobytes() == pos[off[k]:off[k + 1]].tobytes(), (k, f)
    # and the oracle, in FP64, from the same start
    for k, (p, v) in enumerate(states):
        wp, _ = oracle.step(p.astype(np.float64), v.astype(np.float64), float(eps2), float(damp), float(dt),
                            loops)
        tol = 1e-9 if dtype == np.float64 else 1e-3
        assert np.abs(frames[k][-1].astype(np.float64) - wp).max() <= tol * (np.abs(wp).max() + 1)
