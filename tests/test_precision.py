"""Precision mode (NB_F32_COMP): FP32 pair forces with compensated (two-sum)
accumulation, FP64 absolute positions, FP64 energy/momentum reduction.

Tolerances: compensated accelerations per body within 2e-6 (|a| + mean|a|)
of the FP64 oracle (the rsqrt.approx error of each pair term bounds it);
energies within 1e-6 relative of the FP64 oracle; positions after the
stated steps within 1e-9 relative (FP64 positions, 1e-9 covers the float
velocity increments).
"""
import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu


def body_err(got, want):
    """Per-body error relative to |a| + mean|a| (0 where both are exactly 0)."""
    d = np.linalg.norm(np.asarray(got, np.float64) - want, axis=1)
    w = np.linalg.norm(want, axis=1)
    scale = w + w.mean()
    return np.where(scale > 0, d / np.where(scale > 0, scale, 1.0), d)


def test_state_roundtrip(cuda):
    p, v = ics.plummer(1000, seed=2)
    with NBodySystem(1000, "f32comp", "fast", eps2=1e-3) as s:
        s.set_state(p, v)
        p2, v2 = s.get_state()
    assert p2.tobytes() == p.tobytes()
    assert np.abs(v2[:, :3] - v[:, :3]).max() <= 1e-14 * np.abs(v[:, :3]).max()
    assert np.array_equal(v2[:, 3], v[:, 3])


@pytest.mark.parametrize("algo", ["fast", "sym"])
@pytest.mark.parametrize("n", [1, 7, 383, 385, 1000, 4097])
def test_compensated_accel_vs_fp64(cuda, n, algo):
    p, _ = ics.plummer(n, seed=n)
    v = np.zeros_like(p)
    with NBodySystem(n, "f32comp", algo, eps2=1e-4) as s:
        s.set_state(p, v)
        a = s.accel()
    p32 = p.astype(np.float32).astype(np.float64)  # the pair terms read float positions
    ref = oracle.accel(p32, float(np.float32(1e-4)))
    assert body_err(a, ref).max() <= 2e-6


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_compensated_beats_plain_at_scale(cuda, algo):
    n = 65536
    p, _ = ics.plummer(n, seed=5)
    v = np.zeros_like(p)
    tidx = np.random.default_rng(1).choice(n, 256, replace=False).astype(np.int32)
    p32 = p.astype(np.float32)
    ref = oracle.accel_subset_f64(p32.astype(np.float64), tidx, float(np.float32(1e-4)))
    with NBodySystem(n, "f32comp", algo, eps2=1e-4) as s:
        s.set_state(p, v)
        ac = s.accel()[tidx]
    with NBodySystem(n, "f32", "fast", eps2=np.float32(1e-4)) as s:
        s.set_state(p32, v.astype(np.float32))
        ap = s.accel()[tidx]
    ec, ep = body_err(ac, ref).max(), body_err(ap, ref).max()
    assert ec <= 2e-6
    assert ec < ep


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_compensated_steps_vs_fp64_oracle(cuda, algo):
    n, steps = 2048, 10
    p, v = ics.plummer(n, seed=9)
    p32 = p.astype(np.float32).astype(np.float64)
    p[:, :3] = p32[:, :3]  # same starting positions as the float working copy
    with NBodySystem(n, "f32comp", algo, kick="physical", eps2=1e-3, damping=1.0, dt=1e-3) as s:
        s.set_state(p, v)
        s.step(steps)
        pg, vg = s.get_state()
    pr, vr = oracle.step(p, v, 1e-3, 1.0, 1e-3, steps, kick_mode=oracle.KICK_PHYSICAL)
    rel = np.linalg.norm(pg[:, :3] - pr[:, :3], axis=1) / (np.linalg.norm(pr[:, :3], axis=1) + 0.1)
    assert rel.max() <= 1e-9, rel.max()
    dv = np.linalg.norm(vg[:, :3] - vr[:, :3], axis=1) / (np.linalg.norm(vr[:, :3], axis=1) + 1e-3)
    assert dv.max() <= 1e-6, dv.max()


@pytest.mark.parametrize("precision,algo", [("f32", "fast"), ("f32", "sym"), ("f32", "exact"), ("f32comp", "fast"),
                                            ("f32comp", "sym"), ("f64", "sym"), ("f64", "symband"),
                                            ("f64", "sym64"), ("f64", "exact")])
def test_energy_momentum_vs_fp64(cuda, precision, algo):
    """"symband": the float-float energy pass with its triangular array in
    three bands (the potential folded with the forces)."""
    n = 4096
    p, v = ics.plummer(n, seed=4)
    if precision == "f32":
        p, v = p.astype(np.float32), v.astype(np.float32)
    eps2 = np.float32(1e-3)
    kw = {"bands": 3} if algo == "symband" else {}
    with NBodySystem(n, precision, algo.replace("symband", "sym"), kick="physical", eps2=eps2, **kw) as s:
        s.set_state(p, v)
        e, bodies = s.energy(with_bodies=True)
    p64 = np.asarray(p, np.float64)
    if precision == "f32comp":
        p64 = p64.astype(np.float32).astype(np.float64)  # pair terms read float positions
    ref = oracle.energy(p64, np.asarray(v, np.float64), float(eps2))
    tol = {"f32comp": 1e-6, "f32": 2e-5, "f64": 1e-12}[precision]
    assert abs(e[0] - ref[0]) <= 1e-12 * abs(ref[0]) + 1e-300
    assert abs(e[1] - ref[1]) <= tol * abs(ref[1])
    pmag = np.abs(p64[:, 3] * np.linalg.norm(v[:, :3], axis=1)).sum()
    assert np.abs(e[2:] - ref[2:]).max() <= 1e-12 * pmag
    tidx = np.arange(0, n, 16, dtype=np.int32)
    acc, phi = oracle.accel_phi_subset_f64(p64, tidx, float(eps2))
    assert np.abs(bodies[tidx, 3] - phi).max() <= tol * np.abs(phi).max()
    if precision == "f64":
        assert np.abs(bodies[tidx, :3] - acc).max() <= 1e-12 * np.abs(acc).max()


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_energy_conserved_by_small_steps(cuda, algo):
    n = 4096
    p, v = ics.plummer(n, seed=6)
    with NBodySystem(n, "f32comp", algo, kick="physical", eps2=1e-2, damping=1.0, dt=1e-4) as s:
        s.set_state(p, v)
        e0 = s.energy()
        s.step(50)
        e1 = s.energy()
    E0, E1 = e0[0] + e0[1], e1[0] + e1[1]
    assert abs(E1 - E0) <= 1e-5 * abs(E0)


@pytest.mark.parametrize("algo", ["fast", "sym"])
def test_compensated_run_host_frames(cuda, algo):
    n = 1500
    p, v = ics.plummer(n, seed=12)
    with NBodySystem(n, "f32comp", algo, kick="physical", eps2=1e-3, damping=1.0, dt=1e-3) as s:
        frames, t = s.run_host(p, v, 9, 2)
        s.set_state(p, v)
        want = []
        for _ in range(4):
            s.step(2)
            want.append(s.get_state()[0])
    assert frames.shape == (4, n, 4) and frames.dtype == np.float64
    for k in range(4):
        assert frames[k].tobytes() == want[k].tobytes()


@pytest.mark.parametrize("n,shape,bands", [(65536, (32, 12), 1), (1048576, (128, 12), 2)])
def test_compensated_sym_default_shape(cuda, n, shape, bands):
    """Compensated symmetric plan: one-warp CTAs x 12 targets unless the
    source-side array's hi and lo halves would pass 8 GiB, then 4 warps x 12,
    in bands of at most 8 GiB beyond that (11.5 GB in two bands at N = 2^20)."""
    with NBodySystem(n, "f32comp", "sym") as s:
        info, src = s.plan_info(), s.source_info()
    assert (info["block"], info["bpt"]) == shape
    assert src["bands"] == bands and src["mib"] <= 8192, src


@pytest.mark.parametrize("n", [3000, 20000])
@pytest.mark.parametrize("bands", [2, 5])
def test_compensated_sym_bands(cuda, n, bands):
    """The compensated kernel in bands: the fold keeps each body's (sum,
    compensation) pair as the compensated integrator does, so accelerations
    stay within the compensated tolerance of the FP64 oracle, and steps
    agree with the one-pass plan to float rounding."""
    p, v = ics.plummer(n, seed=n + 5)
    eps2 = 1e-3
    # the pair terms read float positions
    want = oracle.accel(p.astype(np.float32).astype(np.float64), float(np.float32(eps2)))
    outs = []
    for kw in ({}, {"bands": bands}):
        with NBodySystem(n, "f32comp", "sym", kick="physical", eps2=eps2, damping=1.0, dt=1e-3, **kw) as s:
            s.set_state(p, v)
            a = s.accel()
            s.step(8)
            outs.append((a, s.get_state()[0], s.source_info()))
    assert outs[1][2]["bands"] > 1
    for a, _, _ in outs:
        assert body_err(a, want).max() <= 2e-6
    rel = np.linalg.norm(outs[0][1][:, :3] - outs[1][1][:, :3], axis=1) / (np.linalg.norm(outs[0][1][:, :3], axis=1) + 0.1)
    assert rel.max() <= 1e-6


def test_f64_energy_paths_agree_and_timing(cuda, capsys):
    """FP64 state: the float-float energy pass (symmetric kernel with the
    potential, NB_ALGO_SYM) and the FP64 one (NB_ALGO_SYM_FP64) agree to
    1e-13 per body in (acc, phi) and in the totals; both timed."""
    import time

    import torch

    n = 16384
    p, v = ics.plummer(n, seed=8)
    out = {}
    for algo in ("sym", "sym64"):
        with NBodySystem(n, "f64", algo, kick="physical", eps2=1e-4) as s:
            s.set_state(p, v)
            s.energy()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e, bodies = s.energy(with_bodies=True)
            out[algo] = (e, bodies, time.perf_counter() - t0)
    (ea, ba, ta), (eb, bb, tb) = out["sym"], out["sym64"]
    assert np.abs(ea - eb).max() <= 1e-13 * np.abs(eb).max()
    scale = np.abs(bb).max(axis=0)
    assert (np.abs(ba - bb) <= 1e-13 * scale).all()
    with capsys.disabled():
        print(f"\n[energy f64] N={n}: float-float pass {ta * 1e3:.2f} ms, FP64 pass {tb * 1e3:.2f} ms")
