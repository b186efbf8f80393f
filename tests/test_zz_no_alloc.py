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


# The entry point's fixed launch shape and scratch size (nb_noalloc.cu): 128
# threads x 8 bodies per thread, 2^20 float4 of partial-force slots.
NOALLOC_BLOCK, NOALLOC_BPT, NOALLOC_SLOTS_FLOAT4 = 128, 8, 1 << 20


def close_per_body(got, want, tol=1e-5):
    d = np.linalg.norm(got[:, :3].astype(np.float64) - want[:, :3], axis=1)
    w = np.linalg.norm(want[:, :3].astype(np.float64), axis=1)
    return bool((d <= tol * (w + max(w.mean(), 0.1))).all())


def grid_is_capped(plan):
    """True when the regular plan's partial slots (slots x tbsize float4)
    would not fit the fixed scratch array, so that the no-alloc step runs
    fewer persistent CTAs than the regular step with the same shape (its
    partial sums then split differently and the results differ in rounding
    only)."""
    return plan["slots"] * plan["tbsize"] > NOALLOC_SLOTS_FLOAT4


@pytest.mark.parametrize("n,kick", [(3000, "physical"), (3000, "reference"), (65536, "physical"),
                                    (250000, "reference"), (262144, "physical")])
def test_noalloc_matches_regular_step_on_two_calls(cuda, n, kick):
    """Against the regular fast step with the same launch shape: bit for bit
    while the plan fits the scratch array as it is; within 1e-5 per body
    where the entry point had to lower the grid.  On GB300 the shape runs 4
    CTAs per SM (608 CTAs), so slots = 608 + n/1024 - 1 fit the array's 1024
    slots up to the size limit, and every size here compares bit for bit;
    the cap matters on GPUs with more resident CTAs."""
    import torch

    p64, v64 = ics.plummer(n, seed=3)
    if kick == "reference":
        p64[:, 3] *= 4.0  # kick x pos.w: heavier bodies so the factor matters
    pos, vel = ics.f32(p64), ics.f32(v64)
    eps2, dt, damping = np.float32(1e-4), np.float32(1e-4), np.float32(0.999)
    km = N.NB_KICK_PHYSICAL if kick == "physical" else N.NB_KICK_REFERENCE
    with NBodySystem(n, "f32", "fast", kick=kick, eps2=eps2, damping=damping, dt=dt,
                     block=NOALLOC_BLOCK, bpt=NOALLOC_BPT) as s:
        plan = s.plan_info()
        s.set_state(pos, vel)
        s.step(1)
        ref = [s.get_state()]
        s.step(1)
        ref.append(s.get_state())
    capped = grid_is_capped(plan)
    if n == 3000:
        assert not capped
    lib = N.lib()
    bufs = [torch.from_numpy(pos).cuda(), torch.zeros((n, 4), dtype=torch.float32, device="cuda")]
    vt = torch.from_numpy(vel).cuda()
    stream = C.c_void_p(current_stream_handle())
    for k in range(2):
        rc = lib.nb_step_f32_noalloc(C.c_void_p(bufs[k % 2].data_ptr()),
                                     C.c_void_p(bufs[(k + 1) % 2].data_ptr()),
                                     C.c_void_p(vt.data_ptr()), n, eps2, damping, dt, km, 1.0, stream)
        assert rc == N.NB_OK, lib.nb_last_error()
        torch.cuda.synchronize()
        p = bufs[(k + 1) % 2].cpu().numpy()
        v = vt.cpu().numpy()
        if capped:
            assert close_per_body(p, ref[k][0]), f"positions differ after call {k + 1}"
            assert close_per_body(v, ref[k][1]), f"velocities differ after call {k + 1}"
        else:
            assert np.array_equal(p, ref[k][0]), f"positions differ after call {k + 1}"
            assert np.array_equal(v, ref[k][1]), f"velocities differ after call {k + 1}"
        assert np.array_equal(p[:, 3], pos[:, 3])


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    lib = N.lib()
    rc = lib.nb_step_f32_noalloc(None, None, None, 262145, 1e-4, 1.0, 1e-4,
                                 N.NB_KICK_PHYSICAL, 1.0, None)
    assert rc == N.NB_ERR_INVALID
    assert b"262144" in lib.nb_last_error()


def _driver():
    """The CUDA driver API through ctypes (only what the next test uses)."""
    cu = C.CDLL("libcuda.so.1")
    u64, vp = C.c_uint64, C.c_void_p
    for name, args in [("cuInit", [C.c_uint]), ("cuDeviceGet", [C.POINTER(C.c_int), C.c_int]),
                       ("cuCtxCreate_v4", [C.POINTER(vp), vp, C.c_uint, C.c_int]),
                       ("cuCtxPopCurrent_v2", [C.POINTER(vp)]), ("cuCtxDestroy_v2", [vp]),
                       ("cuCtxSynchronize", []), ("cuMemAlloc_v2", [C.POINTER(u64), C.c_size_t]),
                       ("cuMemFree_v2", [u64]), ("cuMemcpyHtoD_v2", [u64, vp, C.c_size_t]),
                       ("cuMemcpyDtoH_v2", [vp, u64, C.c_size_t])]:
        f = getattr(cu, name)
        f.argtypes, f.restype = args, C.c_int
    return cu


def test_noalloc_in_a_driver_api_context(cuda):
    """The scratch array's address belongs to a CUDA context: a call made
    while a caller's own driver-API context is current looks it up in that
    context, and the next call in the primary context uses the primary
    context's address again.  Both give the step bit for bit."""
    import torch

    n = 3000
    p64, v64 = ics.plummer(n, seed=5)
    pos, vel = ics.f32(p64), ics.f32(v64)
    lib = N.lib()
    eps2, dt = np.float32(1e-4), np.float32(1e-4)

    def step_in_primary():
        p0, p1 = torch.from_numpy(pos).cuda(), torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        v = torch.from_numpy(vel).cuda()
        rc = lib.nb_step_f32_noalloc(C.c_void_p(p0.data_ptr()), C.c_void_p(p1.data_ptr()),
                                     C.c_void_p(v.data_ptr()), n, eps2, 1.0, dt, N.NB_KICK_PHYSICAL, 1.0,
                                     C.c_void_p(current_stream_handle()))
        assert rc == N.NB_OK, lib.nb_last_error()
        torch.cuda.synchronize()
        return p1.cpu().numpy(), v.cpu().numpy()

    want_p, want_v = step_in_primary()

    cu = _driver()
    assert cu.cuInit(0) == 0
    dev = C.c_int()
    assert cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
    ctx = C.c_void_p()
    assert cu.cuCtxCreate_v4(C.byref(ctx), None, 0, dev) == 0  # current from here on
    nbytes = n * 16
    ptrs = []
    try:
        for _ in range(3):
            d = C.c_uint64()
            assert cu.cuMemAlloc_v2(C.byref(d), nbytes) == 0
            ptrs.append(d.value)
        p0, p1, v = ptrs
        assert cu.cuMemcpyHtoD_v2(p0, pos.ctypes.data, nbytes) == 0
        assert cu.cuMemcpyHtoD_v2(v, vel.ctypes.data, nbytes) == 0
        rc = lib.nb_step_f32_noalloc(C.c_void_p(p0), C.c_void_p(p1), C.c_void_p(v), n, eps2, 1.0, dt,
                                     N.NB_KICK_PHYSICAL, 1.0, None)
        assert rc == N.NB_OK, lib.nb_last_error()
        assert cu.cuCtxSynchronize() == 0
        got_p, got_v = np.empty_like(pos), np.empty_like(vel)
        assert cu.cuMemcpyDtoH_v2(got_p.ctypes.data, p1, nbytes) == 0
        assert cu.cuMemcpyDtoH_v2(got_v.ctypes.data, v, nbytes) == 0
    finally:
        for d in ptrs:
            cu.cuMemFree_v2(d)
        popped = C.c_void_p()
        cu.cuCtxPopCurrent_v2(C.byref(popped))
        cu.cuCtxDestroy_v2(ctx)
    assert np.array_equal(got_p, want_p) and np.array_equal(got_v, want_v)

    again_p, again_v = step_in_primary()
    assert np.array_equal(again_p, want_p) and np.array_equal(again_v, want_v)
