"""Hand-written adjoint through the C ABI against the FP64 reference adjoint
(itself checked against FP64 central differences in test_oracle.py).

Tolerance: norm-wise relative error of each gradient (x0, v0, m) against the
FP64 adjoint <= 1e-4, the target stated for the adjoint; FP32 kernels, FP64
reference.
"""
import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / (np.linalg.norm(b) + 1e-300))


def system(n, algo, **kw):
    """algo "fast": directed forward and VJP kernels; "sym": symmetric ones;
    "symfx": symmetric ones, the forward with its fixed-point source side;
    "symband": symmetric ones, the forward's triangular array in three bands
    (what large N runs)."""
    if algo == "symfx":
        return NBodySystem(n, "f32", "sym", source_side="fixed", **kw)
    if algo == "symband":
        return NBodySystem(n, "f32", "sym", bands=3, **kw)
    return NBodySystem(n, "f32", algo, **kw)


def gpu_grads(pos32, vel32, y, kick, eps2, dt, damping, steps, every, G=1.0, algo="fast"):
    import torch

    n = pos32.shape[0]
    with system(n, algo, kick=kick, eps2=eps2, damping=damping, dt=dt, G=G) as s:
        s.set_state(pos32, vel32)
        s.adj_forward(steps, every)
        pT, _ = s.get_state()
        gx = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        gx[:, :3] = torch.from_numpy(2.0 * (pT[:, :3].astype(np.float64) - y)).float().cuda()
        gx0, gv0, gm = s.adj_backward(gx)
        torch.cuda.synchronize()
        return pT, gx0[:, :3].cpu().numpy(), gv0[:, :3].cpu().numpy(), gm.cpu().numpy()


@pytest.mark.parametrize("algo", ["fast", "sym", "symfx", "symband"])
@pytest.mark.parametrize("kick", ["physical", "reference"])
@pytest.mark.parametrize("n,steps,every", [(96, 30, 7), (1000, 20, 20), (257, 12, 1), (3000, 6, 4)])
def test_adjoint_matches_fp64_reference(cuda, algo, kick, n, steps, every):
    p64, v64 = ics.uniform_cube(n, seed=n)
    if kick == "reference":
        p64[:, 3] *= n  # O(1) masses so the kick x pos.w is not negligible
    y = ics.gaussian_targets(n, seed=n + 1)
    p32, v32 = ics.f32(p64), ics.f32(v64)
    eps2, dt = np.float32(1e-2), np.float32(1e-3)
    _, gx, gv, gm = gpu_grads(p32, v32, y, kick, eps2, dt, 1.0, steps, every, algo=algo)
    km = oracle.KICK_PHYSICAL if kick == "physical" else oracle.KICK_REFERENCE
    L, rx, rv, rm = oracle.adjoint(p32.astype(np.float64), v32.astype(np.float64), y, float(eps2), 1.0,
                                   float(dt), steps, kick_mode=km)
    assert rel(gx, rx) <= 1e-4
    assert rel(gv, rv) <= 1e-4
    assert rel(gm, rm) <= 1e-4


@pytest.mark.parametrize("algo", ["fast", "sym", "symfx", "symband"])
def test_checkpoint_interval_does_not_change_gradients(cuda, algo):
    n, steps = 300, 24
    p64, v64 = ics.uniform_cube(n, seed=3)
    y = ics.gaussian_targets(n, seed=4)
    p32, v32 = ics.f32(p64), ics.f32(v64)
    outs = [gpu_grads(p32, v32, y, "physical", np.float32(1e-2), np.float32(1e-3), 1.0, steps, k,
                      algo=algo) for k in (1, 5, 24)]
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.asarray(a).tobytes() == np.asarray(b).tobytes()


def test_autograd_function_loss_gradients(cuda):
    """loss = sum |x_T - y|^2 through torch autograd: gradients equal the FP64
    adjoint's within 1e-4; adding 0.5 sum |v_T|^2 feeds a velocity cotangent
    and matches nb_adj_backward called with (2 (x_T - y), v_T) directly."""
    import torch

    from utc_gb300.autograd import trajectory

    n, steps, every = 128, 16, 4
    p64, v64 = ics.uniform_cube(n, seed=8)
    p32, v32 = ics.f32(p64), ics.f32(v64)
    y = ics.gaussian_targets(n, seed=9)
    yt = torch.tensor(y, dtype=torch.float32, device="cuda")
    kw = dict(kick="physical", eps2=np.float32(1e-2), damping=1.0, dt=np.float32(1e-3))

    def leaves():
        return (torch.tensor(p32[:, :3], device="cuda", requires_grad=True),
                torch.tensor(v32[:, :3], device="cuda", requires_grad=True),
                torch.tensor(p32[:, 3], device="cuda", requires_grad=True))

    x0, v0, m = leaves()
    with NBodySystem(n, "f32", "fast", **kw) as s:
        xT, _ = trajectory(x0, v0, m, s, steps, every)
        loss = ((xT - yt) ** 2).sum()
        loss.backward()
    L, rx, rv, rm = oracle.adjoint(p32.astype(np.float64), v32.astype(np.float64), y, 1e-2, 1.0,
                                   float(np.float32(1e-3)), steps)
    assert abs(loss.item() - L) <= 1e-4 * L
    assert rel(x0.grad.cpu().numpy(), rx) <= 1e-4
    assert rel(v0.grad.cpu().numpy(), rv) <= 1e-4
    assert rel(m.grad.cpu().numpy(), rm) <= 1e-4

    x0, v0, m = leaves()
    with NBodySystem(n, "f32", "fast", **kw) as s:
        xT, vT = trajectory(x0, v0, m, s, steps, every)
        (((xT - yt) ** 2).sum() + 0.5 * (vT ** 2).sum()).backward()
        gx = torch.zeros((n, 4), device="cuda")
        gv = torch.zeros((n, 4), device="cuda")
        gx[:, :3] = 2 * (xT.detach() - yt)
        gv[:, :3] = vT.detach()
        s.set_state(p32, v32)
        s.adj_forward(steps, every)
        dx, dv, dm = s.adj_backward(gx, gv)
    assert torch.equal(x0.grad, dx[:, :3]) and torch.equal(v0.grad, dv[:, :3])
    assert torch.equal(m.grad, dm)


@pytest.mark.parametrize("algo", ["fast", "sym", "symfx", "symband"])
@pytest.mark.parametrize("kick", ["physical", "reference"])
def test_second_backward_recomputes_every_segment(cuda, algo, kick):
    """The forward pass leaves the last segment's states in place and the first
    backward uses them; a second backward after the same forward recomputes
    that segment too and must give the same bits."""
    import torch

    n, steps, every = 700, 17, 5
    p64, v64 = ics.uniform_cube(n, seed=21)
    if kick == "reference":
        p64[:, 3] *= n
    p32, v32 = ics.f32(p64), ics.f32(v64)
    with system(n, algo, kick=kick, eps2=np.float32(1e-2), damping=0.999, dt=np.float32(1e-3)) as s:
        s.set_state(p32, v32)
        s.adj_forward(steps, every)
        gx = torch.randn((n, 4), device="cuda")
        gv = torch.randn((n, 4), device="cuda")
        a = [t.cpu().numpy() for t in s.adj_backward(gx, gv)]
        b = [t.cpu().numpy() for t in s.adj_backward(gx, gv)]
    for x, y in zip(a, b):
        assert x.tobytes() == y.tobytes()


def test_stale_forward_pass_is_refused(cuda):
    """Two trajectories recorded on one system before the first backward: the
    first graph's backward raises (NB_ERR_STATE) instead of returning the
    second trajectory's gradients; the second graph's backward still gives
    the gradients of its own trajectory.  The same check through the C ABI
    with explicit generation numbers."""
    import torch

    from utc_gb300 import _native as N
    from utc_gb300.autograd import trajectory

    n, steps, every = 128, 8, 4
    p64, v64 = ics.uniform_cube(n, seed=30)
    p32, v32 = ics.f32(p64), ics.f32(v64)
    y = torch.tensor(ics.gaussian_targets(n, seed=31), dtype=torch.float32, device="cuda")
    kw = dict(kick="physical", eps2=np.float32(1e-2), damping=1.0, dt=np.float32(1e-3))

    def leaves(scale):
        return (torch.tensor(p32[:, :3] * scale, device="cuda", requires_grad=True),
                torch.tensor(v32[:, :3], device="cuda", requires_grad=True),
                torch.tensor(p32[:, 3], device="cuda", requires_grad=True))

    with NBodySystem(n, "f32", "sym", **kw) as s:
        a = leaves(1.0)
        b = leaves(0.5)
        xa, _ = trajectory(*a, s, steps, every)
        xb, _ = trajectory(*b, s, steps, every)
        with pytest.raises(RuntimeError, match="no longer holds"):
            ((xa - y) ** 2).sum().backward()
        ((xb - y) ** 2).sum().backward()
        got = b[0].grad.cpu().numpy()
    with NBodySystem(n, "f32", "sym", **kw) as s2:
        c = leaves(0.5)
        xc, _ = trajectory(*c, s2, steps, every)
        ((xc - y) ** 2).sum().backward()
    assert np.array_equal(got, c[0].grad.cpu().numpy())

    with NBodySystem(n, "f32", "fast", **kw) as s:
        s.set_state(p32, v32)
        g1 = s.adj_forward(steps, every)
        g2 = s.adj_forward(steps, every)
        assert g2 == g1 + 1
        gx = torch.randn((n, 4), device="cuda")
        z = [torch.zeros((n, 4), device="cuda"), torch.zeros((n, 4), device="cuda"),
             torch.zeros((n,), device="cuda")]
        import ctypes as C
        rc = s.lib.nb_adj_backward(s.handle, C.c_ulonglong(g1), C.c_void_p(gx.data_ptr()), None,
                                   *[C.c_void_p(t.data_ptr()) for t in z], None)
        assert rc == N.NB_ERR_STATE
        s.set_params(np.float32(2e-2), 1.0, np.float32(1e-3))
        with pytest.raises(RuntimeError):
            s.adj_backward(gx, generation=g2)  # nb_set_params dropped the pass


def test_batch_stale_forward_pass_is_refused(cuda):
    import torch

    from utc_gb300.nbody import NBodyBatch

    sizes = np.array([64, 100, 37], dtype=np.int32)
    ps, vs = zip(*[ics.uniform_cube(int(k), seed=40 + i) for i, k in enumerate(sizes)])
    pos, vel = ics.f32(np.concatenate(ps)), ics.f32(np.concatenate(vs))
    with NBodyBatch(sizes, kick="physical", eps2=np.float32(1e-2), dt=np.float32(1e-3)) as b:
        b.set_state(pos, vel)
        g1 = b.adj_forward(6, 3)
        gx = torch.randn((b.nbody, 4), device="cuda")
        first = [t.cpu().numpy() for t in b.adj_backward(gx, generation=g1)]
        b.set_state(pos, vel)
        g2 = b.adj_forward(6, 3)
        with pytest.raises(RuntimeError, match="no longer holds"):
            b.adj_backward(gx, generation=g1)
        again = [t.cpu().numpy() for t in b.adj_backward(gx, generation=g2)]
    for x, y in zip(first, again):
        assert x.tobytes() == y.tobytes()
