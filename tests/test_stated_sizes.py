"""The extension workloads at their stated sizes, each against the FP64
oracle (or an FP64-accurate GPU run pinned to it at smaller sizes), with the
tolerance its target states.

* Precision study: N=1,048,576 Plummer sphere, 20 steps of dt=1e-4,
  eps2=1e-4.  Compensated FP32 pair forces with FP64 positions
  (NB_F32_COMP, symmetric kernel): forces on a 4096-body subsample within
  1e-5 per body (median 1e-7) of FP64 all-pairs sums over the million
  sources at steps 0, 10 and 20; potentials within 1e-6; energy drift over
  the 20 steps within 1e-8; positions within 1e-9 (|x| + 0.1) of an
  FP64-accurate run.  Plain FP32 (the default symmetric kernel, the N=1M
  forward target): positions within 1e-5 (|x| + 0.1) of the same run, and a
  median force error at least ten times the compensated one.  The FP64
  trajectory of a million bodies is out of the CPU oracle's reach (1.1e12
  pair terms a step), so it comes from the float-float symmetric kernel for
  FP64 state, held to 1e-13 of the FP64 oracle in test_sym.py.
* Adjoint: N=16384 uniform cube, 200 steps, checkpoints every 20, loss
  sum |x_T - y|^2 with Gaussian targets (sigma 0.5): gradients to x0, v0 and
  m from the symmetric and the directed kernels within 1e-4 (norm-wise) of
  the FP64 reference adjoint, and the directional derivative along 64 random
  coordinates of x0 and v0 within 1e-4 of an FP64 central difference
  (h = 1e-6).
* Batched: 512 Plummer systems, N log-uniform in [128, 16384], eps2 = dt =
  1e-3, 50 steps, autotuned shape, CUDA graph: every system within
  1e-5 (|x| + 0.1) of its own per-system launches; eight systems against the
  FP64 oracle's trajectories; the batched adjoint of the adjoint workload's
  loss against the FP64 reference adjoint on the same eight systems.
"""
import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodyBatch, NBodySystem

pytestmark = pytest.mark.gpu


def _rel_pos(got, want, floor=0.1):
    got = np.asarray(got, np.float64)[:, :3]
    want = np.asarray(want, np.float64)[:, :3]
    return np.linalg.norm(got - want, axis=1) / (np.linalg.norm(want, axis=1) + floor)


def _body_rel(got, want):
    d = np.linalg.norm(np.asarray(got, np.float64)[:, :3] - want, axis=1)
    return d / np.linalg.norm(want, axis=1)


def test_precision_study_n1m(cuda, capsys):
    n, steps, eps2, dt = 1 << 20, 20, 1e-4, 1e-4
    p, v = ics.plummer(n, seed=0)
    p32, v32 = ics.f32(p), ics.f32(v)
    # every run starts from the float-rounded state so that one FP64-accurate
    # trajectory serves both FP32 modes
    p0, v0 = p32.astype(np.float64), v32.astype(np.float64)
    e2, d = float(np.float32(eps2)), float(np.float32(dt))
    tidx = np.sort(np.random.default_rng(7).choice(n, 4096, replace=False)).astype(np.int32)

    with NBodySystem(n, "f64", "sym", kick="physical", eps2=e2, damping=1.0, dt=d) as s:
        s.set_state(p0, v0)
        s.step(steps)
        want, want_v = s.get_state()

    report = {}
    with NBodySystem(n, "f32comp", "sym", kick="physical", eps2=e2, damping=1.0, dt=d) as s:
        s.set_state(p0, v0)
        errs, E = [], []
        for t in range(steps + 1):
            if t in (0, steps // 2, steps):
                e, bodies = s.energy(with_bodies=True)
                E.append(e[0] + e[1])
                a = np.asarray(s.accel(), np.float64)
                pos, _ = s.get_state()
                ref_a, ref_phi = oracle.accel_phi_subset_f64(np.asarray(pos, np.float64), tidx, e2)
                fa = _body_rel(a[tidx], ref_a)
                fp = np.abs(np.asarray(bodies, np.float64)[tidx, 3] - ref_phi) / np.abs(ref_phi)
                errs.append((t, float(np.median(fa)), float(fa.max()), float(fp.max())))
            if t < steps:
                s.step(1)
        got, got_v = s.get_state()
    comp_med0 = errs[0][1]
    for t, med, mx, phi in errs:
        assert mx <= 1e-5 and med <= 1e-7 and phi <= 1e-6, (t, med, mx, phi)
    drift = abs((E[-1] - E[0]) / E[0])
    assert drift <= 1e-8
    rc = _rel_pos(got, want)
    assert rc.max() <= 1e-9
    vd = np.linalg.norm(np.asarray(got_v, np.float64)[:, :3] - want_v[:, :3], axis=1)
    assert (vd <= 1e-7 * (np.linalg.norm(want_v[:, :3], axis=1) + 0.01)).all()
    report["compensated"] = (errs, drift, rc.max())

    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(eps2), damping=1.0,
                     dt=np.float32(dt)) as s:
        s.set_state(p32, v32)
        a = np.asarray(s.accel(), np.float64)
        ref_a = oracle.accel_subset_f64(p0, tidx, e2)
        plain_med0 = float(np.median(_body_rel(a[tidx], ref_a)))
        s.step(steps)
        gp, _ = s.get_state()
    rp = _rel_pos(gp, want)
    assert rp.max() <= 1e-5
    assert plain_med0 >= 10 * comp_med0
    with capsys.disabled():
        print(f"\n[precision N=1M, 20 steps] compensated: force err (step, median, max, phi max) "
              f"{[(t, f'{m:.1e}', f'{x:.1e}', f'{q:.1e}') for t, m, x, q in errs]}, energy drift "
              f"{drift:.1e}, positions {rc.max():.1e} of the FP64-accurate run; plain FP32: median force "
              f"err {plain_med0:.1e}, positions {rp.max():.1e}")


def test_adjoint_workload_full_size(cuda, capsys):
    import torch

    n, T, K = 16384, 200, 20
    eps2, dt = np.float32(1e-2), np.float32(1e-3)
    p64, v64 = ics.uniform_cube(n, seed=0)
    y = ics.gaussian_targets(n, seed=1, sigma=0.5)
    p32, v32 = ics.f32(p64), ics.f32(v64)
    yt = torch.tensor(y, dtype=torch.float32, device="cuda")
    grads = {}
    for algo in ("sym", "fast"):
        with NBodySystem(n, "f32", algo, kick="physical", eps2=eps2, damping=1.0, dt=dt) as s:
            s.set_state(p32, v32)
            gen = s.adj_forward(T, K)
            pT = torch.empty((n, 4), device="cuda")
            vT = torch.empty((n, 4), device="cuda")
            s.get_state_device(pT, vT)
            gx = torch.zeros((n, 4), device="cuda")
            gx[:, :3] = 2.0 * (pT[:, :3] - yt)
            g = s.adj_backward(gx, generation=gen)
            torch.cuda.synchronize()
            grads[algo] = [t.cpu().numpy() for t in g]
    pd, vd = p32.astype(np.float64), v32.astype(np.float64)
    L, rx, rv, rm = oracle.adjoint(pd, vd, y, float(eps2), 1.0, float(dt), T, kick_mode=oracle.KICK_PHYSICAL)

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

    errs = {}
    for algo, (gx0, gv0, gm) in grads.items():
        errs[algo] = (rel(gx0[:, :3], rx), rel(gv0[:, :3], rv), rel(gm, rm))
        assert max(errs[algo]) <= 1e-4, (algo, errs[algo])
    # directional FP64 central difference over 64 random coordinates of x0, v0
    rng = np.random.default_rng(5)
    which = rng.integers(0, 2, 64)
    body = rng.choice(n, 64, replace=False)
    comp = rng.integers(0, 3, 64)
    sign = rng.choice([-1.0, 1.0], 64)
    h = 1e-6

    def perturbed(eps):
        pp, vv = pd.copy(), vd.copy()
        for w, i, c, sg in zip(which, body, comp, sign):
            (pp if w == 0 else vv)[i, c] += eps * sg
        return pp, vv

    lp = oracle.loss(*perturbed(h), y, float(eps2), 1.0, float(dt), T)
    lm = oracle.loss(*perturbed(-h), y, float(eps2), 1.0, float(dt), T)
    fd = (lp - lm) / (2 * h)
    gx0, gv0, _ = grads["sym"]
    an = sum(sg * (gx0 if w == 0 else gv0)[i, c] for w, i, c, sg in zip(which, body, comp, sign))
    an64 = sum(sg * (rx if w == 0 else rv)[i, c] for w, i, c, sg in zip(which, body, comp, sign))
    assert abs(an - fd) <= 1e-4 * abs(fd)
    assert abs(an64 - fd) <= 1e-4 * abs(fd)
    with capsys.disabled():
        print(f"\n[adjoint N=16384, 200 steps, K=20] gradient error vs the FP64 adjoint (x0, v0, m): "
              f"sym {errs['sym'][0]:.1e} {errs['sym'][1]:.1e} {errs['sym'][2]:.1e}, fast "
              f"{errs['fast'][0]:.1e} {errs['fast'][1]:.1e} {errs['fast'][2]:.1e}; directional derivative "
              f"{an:.6e} vs FP64 central difference {fd:.6e} (rel {abs(an - fd) / abs(fd):.1e})")


def test_batched_workload_full_size(cuda, capsys):
    import torch

    sizes = ics.batch_sizes(512, lo=128, hi=16384, seed=0)
    steps, eps2, dt = 50, np.float32(1e-3), np.float32(1e-3)
    ps, vs = [], []
    for k, nn in enumerate(sizes):
        p, v = ics.plummer(int(nn), seed=1000 + k)
        ps.append(ics.f32(p))
        vs.append(ics.f32(v))
    pos, vel = np.concatenate(ps), np.concatenate(vs)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    # eight systems for the FP64 checks: the two smallest, the rest drawn
    # among those of at most 2048 bodies (the FP64 adjoint's cost)
    order = np.argsort(sizes, kind="stable")
    small = [int(k) for k in np.nonzero(sizes <= 2048)[0]]
    rng = np.random.default_rng(3)
    pick = sorted(set([int(order[0]), int(order[1])] +
                      [int(k) for k in rng.choice(small, 6, replace=False)]))
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    with torch.cuda.stream(stream), NBodyBatch(sizes, kick="physical", eps2=eps2, dt=dt) as b:
        b.set_state(pos, vel, stream=sh)
        shape = b.autotune(reps=1, stream=sh)
        b.set_state(pos, vel, stream=sh)
        b.run(steps, sh)
        stream.synchronize()
        got, _ = b.get_state(stream=sh)
        b.set_state(pos, vel, stream=sh)
        b.step_per_system(steps, sh)
        stream.synchronize()
        per, _ = b.get_state(stream=sh)
        # adjoint of the adjoint workload's loss, every system at once
        ys = [ics.gaussian_targets(int(nn), seed=2000 + k) for k, nn in enumerate(sizes)]
        y = np.concatenate(ys)
        b.set_state(pos, vel, stream=sh)
        gen = b.adj_forward(steps, 10, stream=sh)
        stream.synchronize()
        pT, _ = b.get_state(stream=sh)
        gx = torch.zeros((b.nbody, 4), device="cuda")
        gx[:, :3] = torch.tensor(2.0 * (pT[:, :3].astype(np.float64) - y), dtype=torch.float32,
                                 device="cuda")
        bx, bv, bm = [t.cpu().numpy() for t in b.adj_backward(gx, stream=sh, generation=gen)]
    rper = _rel_pos(got, per)
    assert rper.max() <= 1e-5
    worst_pos, worst_grad = 0.0, 0.0
    for k in pick:
        sl = slice(int(off[k]), int(off[k + 1]))
        want, _ = oracle.step(ps[k].astype(np.float64), vs[k].astype(np.float64), float(eps2), 1.0,
                              float(dt), steps, kick_mode=oracle.KICK_PHYSICAL)
        r = _rel_pos(got[sl], want).max()
        worst_pos = max(worst_pos, r)
        assert r <= 1e-5, (k, int(sizes[k]), r)
        L, rx, rv, rm = oracle.adjoint(ps[k].astype(np.float64), vs[k].astype(np.float64), ys[k],
                                       float(eps2), 1.0, float(dt), steps, kick_mode=oracle.KICK_PHYSICAL)
        for g, w in ((bx[sl, :3], rx), (bv[sl, :3], rv), (bm[sl], rm)):
            e = float(np.linalg.norm(g - w) / (np.linalg.norm(w) + 1e-300))
            worst_grad = max(worst_grad, e)
            assert e <= 1e-4, (k, int(sizes[k]), e)
    with capsys.disabled():
        print(f"\n[batched 512 systems, {int(sizes.sum())} bodies, 50 steps, shape {shape}] max "
              f"|dx|/(|x|+0.1) vs per-system launches {rper.max():.1e}; vs FP64 oracle on systems "
              f"{[int(sizes[k]) for k in pick]}: positions {worst_pos:.1e}, adjoint gradients {worst_grad:.1e}")
