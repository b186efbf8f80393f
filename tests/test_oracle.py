"""The oracle is pinned before it is trusted (CPU only).

* It reproduces the reference's own golden frames
  (benchapps/nbody/seq/nbody_outpos.txt) byte for byte.
* It reproduces every digest in tests/golden/ref_runs.json, recorded from the
  reference's BodySystem<T> compiled from its sources.
* Where oracle/_ref/libnbref.so is present, it matches the reference
  bit for bit on further random cases.
* The FP64 adjoint agrees with central finite differences.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def sha(b):
    return hashlib.sha256(b).hexdigest()


@pytest.fixture(scope="module")
def orc(built):
    return oracle


def kat_text(orc_mod):
    kat = json.load(open(os.path.join(GOLD, "kat_shell_n1024.json")))
    sc = kat["scenario"]
    dt, cs, vs, soft, damp = orc_mod.demo_params(sc["para_select"], sc["n"])
    pos, vel = orc_mod.randomize(1, sc["n"], np.float32, seed=sc["rand_seed"])
    eps2 = np.float32(soft) * np.float32(soft)
    p1, _ = orc_mod.step(pos, vel, eps2, damp, dt, sc["steps"])
    return kat, orc_mod.format_frames([pos, p1], dt), (pos, vel, eps2, damp, dt)


def test_kat_reproduces_reference_golden_frames(orc):
    kat, text, _ = kat_text(orc)
    assert len(text.encode()) == kat["seq_outpos_bytes"]
    assert sha(text.encode()) == kat["seq_outpos_sha256"]


@pytest.mark.parametrize("nthreads", [1, 3, 8])
def test_thread_count_does_not_change_bits(orc, nthreads):
    pos, vel = orc.randomize(0, 300, np.float32)
    a, va = orc.step(pos, vel, np.float32(0.01), 1.0, 0.01, 3, nthreads=1)
    b, vb = orc.step(pos, vel, np.float32(0.01), 1.0, 0.01, 3, nthreads=nthreads)
    assert a.tobytes() == b.tobytes() and va.tobytes() == vb.tobytes()


def test_reference_run_digests(orc):
    cases = json.load(open(os.path.join(GOLD, "ref_runs.json")))["cases"]
    assert len(cases) >= 8
    for c in cases:
        dtype = np.float32 if c["dtype"] == "f32" else np.float64
        dt, cs, vs, soft, damp = orc.demo_params(c["para_select"], c["n"])
        pos = np.zeros((c["n"], 4), dtype)
        vel = np.zeros((c["n"], 4), dtype)
        orc.lib().orc_srand(1)
        fn = orc.lib().orc_randomize_f32 if dtype == np.float32 else orc.lib().orc_randomize_f64
        assert fn(c["config"], pos.reshape(-1), vel.reshape(-1), cs, vs, c["n"]) == 0
        assert sha(pos.tobytes() + vel.tobytes()) == c["init_sha256"], c
        if dtype == np.float32:
            eps2, d, h = np.float32(soft) * np.float32(soft), np.float32(damp), np.float32(dt)
        else:
            s64 = float(np.float32(soft))
            eps2, d, h = s64 * s64, float(np.float32(damp)), float(np.float32(dt))
        p1, v1 = orc.step(pos, vel, eps2, d, h, c["steps"])
        assert sha(p1.tobytes() + v1.tobytes()) == c["final_sha256"], c


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("n,dtype,steps", [(4, np.float32, 7), (64, np.float32, 12),
                                           (252, np.float64, 5), (1000, np.float32, 3),
                                           (96, np.float64, 9)])
def test_restatement_matches_reference_build(orc, n, dtype, steps):
    r = orc.ref_lib()
    rng = np.random.default_rng(n)
    pos = np.empty((n, 4), dtype)
    pos[:, :3] = rng.uniform(-2, 2, (n, 3))
    pos[:, 3] = rng.uniform(0.5, 1.5, n)
    vel = np.zeros((n, 4), dtype)
    vel[:, :3] = rng.uniform(-0.1, 0.1, (n, 3))
    vel[:, 3] = 1
    soft, damp, dt = dtype(0.05), dtype(0.999), dtype(0.003)
    rp, rv = pos.copy(), vel.copy()
    if dtype == np.float32:
        assert r.ref_run_f32(n, rp.reshape(-1), rv.reshape(-1), soft, damp, dt, steps) == 0
    else:
        assert r.ref_run_f64(n, rp.reshape(-1), rv.reshape(-1), soft, damp, dt, steps) == 0
    mp, mv = orc.step(pos, vel, soft * soft, damp, dt, steps)
    assert mp.tobytes() == rp.tobytes()
    assert mv.tobytes() == rv.tobytes()


def test_padding_with_zero_mass_bodies_is_exact(orc):
    """The reference's 4x-unrolled source loop needs n % 4 == 0; zero-mass
    bodies appended to reach it change no other body's result."""
    pos, vel = orc.randomize(1, 13, np.float32)
    pad_p = np.zeros((16, 4), np.float32)
    pad_v = np.zeros((16, 4), np.float32)
    pad_p[:13], pad_v[:13] = pos, vel
    pad_p[13:, :3] = 1e3
    a, va = orc.step(pos, vel, np.float32(0.01), 1.0, 0.016, 4)
    b, vb = orc.step(pad_p, pad_v, np.float32(0.01), 1.0, 0.016, 4)
    assert a.tobytes() == b[:13].tobytes() and va.tobytes() == vb[:13].tobytes()


def test_accel_f64_matches_numpy(orc):
    rng = np.random.default_rng(3)
    n = 50
    pos = np.empty((n, 4))
    pos[:, :3] = rng.normal(size=(n, 3))
    pos[:, 3] = rng.uniform(0.5, 1.5, n)
    eps2 = 1e-2
    r = pos[None, :, :3] - pos[:, None, :3]
    inv3 = (np.sum(r * r, -1) + eps2) ** -1.5
    want = np.einsum("ij,ijk->ik", inv3 * pos[None, :, 3], r)
    got = orc.accel(pos, eps2)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14)
    sub = orc.accel_subset_f64(pos, np.array([0, 7, 49], np.int32), eps2)
    np.testing.assert_array_equal(sub, got[[0, 7, 49]])


@pytest.mark.parametrize("kick", [oracle.KICK_PHYSICAL, oracle.KICK_REFERENCE])
def test_adjoint_f64_matches_finite_differences(orc, kick):
    from utc_gb300 import ics

    n, steps = 24, 15
    pos, vel = ics.uniform_cube(n, seed=5)
    y = ics.gaussian_targets(n, seed=6)
    kw = dict(eps2=1e-2, damping=0.999, dt=1e-2, steps=steps, kick_mode=kick, G=1.0)
    L, gx, gv, gm = orc.adjoint(pos, vel, y, **kw)
    assert np.isclose(L, orc.loss(pos, vel, y, **kw), rtol=1e-14)
    rng = np.random.default_rng(0)
    h = 1e-6
    for _ in range(12):
        which = rng.integers(0, 3)
        i = rng.integers(0, n)
        d = rng.integers(0, 3)
        p2, v2 = pos.copy(), vel.copy()
        tgt = {0: (p2, d), 1: (v2, d), 2: (p2, 3)}[which]
        arr, col = tgt
        arr[i, col] += h
        lp = orc.loss(p2, v2, y, **kw)
        arr[i, col] -= 2 * h
        lm = orc.loss(p2, v2, y, **kw)
        fd = (lp - lm) / (2 * h)
        an = {0: gx[i, d], 1: gv[i, d], 2: gm[i]}[which]
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (which, i, d, fd, an)


def test_energy_momentum_definition(orc):
    pos = np.array([[0, 0, 0, 2.0], [1, 0, 0, 3.0]])
    vel = np.array([[0, 1, 0, 1.0], [0, 0, 2, 1.0]])
    ke, pe, px, py, pz = orc.energy(pos, vel, eps2=0.0, G=1.0)
    assert np.isclose(ke, 0.5 * 2 * 1 + 0.5 * 3 * 4)
    assert np.isclose(pe, -2 * 3 / 1.0)
    assert np.allclose([px, py, pz], [0, 2, 6])
