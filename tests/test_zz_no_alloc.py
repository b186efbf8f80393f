"""nb_step_f32_noalloc, the step for callers that cannot allocate device
memory (an application whose memory manager owns the GPU's memory, or a
latency-critical loop that cannot take cudaMalloc's synchronisation), checked
through the C ABI against the regular fast entry point on two calls in a row.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  It passes alone in a fresh
process as well as after the other tests (the first call on the device sets
up the scratch address itself).
"""
import ctypes as C

import numpy as np
import pytest

from utc_gb300 import _native as N
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem, current_stream_handle

pytestmark = pytest.mark.gpu


def close_per_body(got, want, tol=1e-5):
    d = np.linalg.norm(got[:, :3].astype(np.float64) - want[:, :3], axis=1)
    w = np.linalg.norm(want[:, :3].astype(np.float64), axis=1)
    return bool((d <= tol * (w + max(w.mean(), 0.1))).all())


@pytest.mark.parametrize("n", [3000, 65536])
def test_noalloc_matches_regular_step_on_two_calls(cuda, n):
    import torch

    p64, v64 = ics.plummer(n, seed=3)
    pos, vel = ics.f32(p64), ics.f32(v64)
    eps2, dt = np.float32(1e-4), np.float32(1e-4)
    with NBodySystem(n, "f32", "fast", kick="physical", eps2=eps2, damping=1.0, dt=dt) as s:
        s.set_state(pos, vel)
        s.step(1)
        ref = [s.get_state()]
        s.step(1)
        ref.append(s.get_state())
    lib = N.lib()
    bufs = [torch.from_numpy(pos).cuda(), torch.zeros((n, 4), dtype=torch.float32, device="cuda")]
    vt = torch.from_numpy(vel).cuda()
    stream = C.c_void_p(current_stream_handle())
    for k in range(2):
        rc = lib.nb_step_f32_noalloc(C.c_void_p(bufs[k % 2].data_ptr()),
                                     C.c_void_p(bufs[(k + 1) % 2].data_ptr()),
                                     C.c_void_p(vt.data_ptr()), n, eps2, 1.0, dt,
                                     N.NB_KICK_PHYSICAL, 1.0, stream)
        assert rc == N.NB_OK, lib.nb_last_error()
        torch.cuda.synchronize()
        p = bufs[(k + 1) % 2].cpu().numpy()
        v = vt.cpu().numpy()
        assert close_per_body(p, ref[k][0]), f"positions differ after call {k + 1}"
        assert close_per_body(v, ref[k][1]), f"velocities differ after call {k + 1}"
        assert np.array_equal(p[:, 3], pos[:, 3])


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    lib = N.lib()
    rc = lib.nb_step_f32_noalloc(None, None, None, 262145, 1e-4, 1.0, 1e-4,
                                 N.NB_KICK_PHYSICAL, 1.0, None)
    assert rc == N.NB_ERR_INVALID
    assert b"262144" in lib.nb_last_error()
