"""NB_ALGO_SYM: each unordered pair evaluated once, applied to both bodies.

Same tolerances as the directed fast path (tests/test_gpu_parity.py):
accelerations per body within 2e-5 (|a| + mean|a|) of the FP64 oracle,
positions within 1e-5 (|x| + 0.1); reruns bitwise identical.
"""
import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu


def close(got, want, tol=2e-5):
    d = np.linalg.norm(np.asarray(got, np.float64) - want, axis=1)
    w = np.linalg.norm(want, axis=1)
    return bool((d <= tol * (w + w.mean())).all())


@pytest.mark.parametrize("n", [1, 2, 31, 33, 255, 256, 257, 1000, 2047, 2048, 2049, 4097, 9000])
@pytest.mark.parametrize("shape", [(0, 0), (32, 16), (32, 20), (32, 8), (32, 4), (64, 16), (128, 20),
                                   (256, 24), (256, 8), (256, 4), (128, 8), (256, -8), (128, -8), (256, -4)])
def test_sym_accel_vs_fp64(cuda, n, shape):
    p, _ = ics.plummer(n, seed=n)
    pos = ics.f32(p)
    with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-3), block=shape[0], bpt=shape[1]) as s:
        s.set_state(pos, np.zeros_like(pos))
        a = s.accel()
    assert close(a, oracle.accel(pos.astype(np.float64), float(np.float32(1e-3))))


def test_sym_full_size_subsample_and_determinism(cuda):
    n = 65536
    p, v = ics.plummer(n, seed=0)
    pos, vel = ics.f32(p), ics.f32(v)
    outs = []
    for _ in range(2):
        with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-4), damping=1.0,
                         dt=np.float32(1e-4)) as s:
            s.set_state(pos, vel)
            a = s.accel()
            s.step(20)
            outs.append(s.get_state())
    tidx = np.random.default_rng(3).choice(n, 512, replace=False).astype(np.int32)
    ref = oracle.accel_subset_f64(pos.astype(np.float64), tidx, float(np.float32(1e-4)))
    assert close(a[tidx], ref)
    assert outs[0][0].tobytes() == outs[1][0].tobytes() and outs[0][1].tobytes() == outs[1][1].tobytes()


@pytest.mark.parametrize("kick", ["reference", "physical"])
def test_sym_steps_vs_oracle(cuda, kick):
    n, steps = 4096, 10
    p, v = ics.uniform_cube(n, seed=0)
    pos, vel = ics.f32(p), ics.f32(v)
    km = oracle.KICK_REFERENCE if kick == "reference" else oracle.KICK_PHYSICAL
    with NBodySystem(n, "f32", "sym", kick=kick, eps2=np.float32(1e-2), damping=1.0,
                     dt=np.float32(1e-3)) as s:
        s.set_state(pos, vel)
        s.step(steps)
        got, _ = s.get_state()
    want, _ = oracle.step(pos, vel, np.float32(1e-2), 1.0, np.float32(1e-3), steps, kick_mode=km)
    d = np.linalg.norm(got[:, :3].astype(np.float64) - want[:, :3], axis=1)
    w = np.linalg.norm(want[:, :3].astype(np.float64), axis=1)
    assert (d <= 1e-5 * (w + 0.1)).all()


def test_sym_adjoint_matches_directed_adjoint(cuda):
    import torch

    n, steps = 600, 12
    p, v = ics.uniform_cube(n, seed=2)
    y = ics.gaussian_targets(n, seed=3)
    pos, vel = ics.f32(p), ics.f32(v)
    grads = []
    for algo in ("fast", "sym"):
        with NBodySystem(n, "f32", algo, kick="physical", eps2=np.float32(1e-2), damping=1.0,
                         dt=np.float32(1e-3)) as s:
            s.set_state(pos, vel)
            s.adj_forward(steps, 5)
            pT, _ = s.get_state()
            gx = torch.zeros((n, 4), device="cuda")
            gx[:, :3] = torch.tensor(2 * (pT[:, :3].astype(np.float64) - y), dtype=torch.float32,
                                     device="cuda")
            grads.append([t.cpu().numpy() for t in s.adj_backward(gx)])
    for a, b in zip(grads[0], grads[1]):
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b)


@pytest.mark.parametrize("n,shape,bands", [(65536, (32, 16), 1), (1048576, (128, 20), 1), (1024, (32, 4), 1),
                                           (4096, (32, 8), 1), (16384, (32, 16), 1), (1600000, (128, 20), 1),
                                           (1700000, (128, 20), 2), (2097152, (128, 20), 2),
                                           (6000000, (128, 20), 14)])
def test_sym_default_shape(cuda, n, shape, bands):
    """One-warp CTAs x 16 targets unless the triangular source-side array
    (about N^2 / (2 rb) float4) would pass 8 GiB, then 4 warps x 20 targets;
    small systems drop to 8 or 4 targets per lane to keep four (row, chunk)
    items per SM.  Once the 4 x 20 array would pass 8 GiB too (N above about
    1.66e6: 8.0 GB at 1.6e6, 9.0 GB at 1.7e6), it is cut into bands of at
    most 8 GiB (112 GB in 14 bands at N = 6e6), so the context stays within
    about 9 GB.  With the fixed-point source side: one warp x 16 at any size
    (48 B per body whatever the row block)."""
    import torch

    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    with NBodySystem(n, "f32", "sym") as s:
        info = s.plan_info()
        src = s.source_info()
        used = free0 - torch.cuda.mem_get_info()[0]
    assert (info["block"], info["bpt"]) == shape
    assert src["side"] == "triangular" and src["bands"] == bands, src
    assert src["mib"] <= 8192
    assert used < 10 << 30, used
    with NBodySystem(n, "f32", "sym", source_side="fixed") as s:
        info = s.plan_info()
    assert (info["block"], info["bpt"]) == (32, min(shape[1], 16))


@pytest.mark.parametrize("n", [700, 4097, 20000])
@pytest.mark.parametrize("bands", [2, 3, 7])
@pytest.mark.parametrize("shape", [(0, 0), (128, 20), (32, 8)])
def test_sym_bands_vs_fp64(cuda, n, bands, shape):
    """The triangular source side cut into bands (nb_params.bands): the
    force kernel runs band by band and a fold kernel adds each band's
    target-side slots and source-side rows into one sum per body.
    Accelerations within 2e-5 of the FP64 oracle for every banded shape;
    reruns and a second context give the same bits; the scratch of the
    source side shrinks with the band count."""
    p, _ = ics.plummer(n, seed=n + 11)
    pos = ics.f32(p)
    z = np.zeros_like(pos)
    want = oracle.accel(pos.astype(np.float64), float(np.float32(1e-3)))
    outs = []
    for _ in range(2):
        with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-3), block=shape[0], bpt=shape[1],
                         bands=bands) as s:
            info = s.source_info()
            rb = s.plan_info()["tbsize"]
            s.set_state(pos, z)
            a = s.accel()
            assert a.tobytes() == s.accel().tobytes()
            outs.append(a)
    nrb = -(-n // rb)
    # about `bands` bands: whole row blocks each, so a few more where rows are long
    assert info["side"] == "triangular" and 1 <= info["bands"] <= nrb, info
    if nrb > bands:
        assert info["bands"] > 1, info
    assert close(outs[0], want)
    assert outs[0].tobytes() == outs[1].tobytes()


@pytest.mark.parametrize("kick", ["reference", "physical"])
def test_sym_bands_steps_vs_oracle(cuda, kick):
    """Leapfrog steps with a banded plan (graph replay included) against the
    FP64 oracle, as test_sym_steps_vs_oracle does for one pass."""
    n, steps = 4096, 40
    p, v = ics.uniform_cube(n, seed=7)
    pos, vel = ics.f32(p), ics.f32(v)
    km = oracle.KICK_REFERENCE if kick == "reference" else oracle.KICK_PHYSICAL
    with NBodySystem(n, "f32", "sym", kick=kick, eps2=np.float32(1e-2), damping=1.0, dt=np.float32(1e-3),
                     bands=4) as s:
        assert s.source_info()["bands"] > 1
        s.set_state(pos, vel)
        s.step(steps)
        got, _ = s.get_state()
    want, _ = oracle.step(pos.astype(np.float64), vel.astype(np.float64), float(np.float32(1e-2)), 1.0,
                          float(np.float32(1e-3)), steps, kick_mode=km)
    rel = np.linalg.norm(got[:, :3] - want[:, :3], axis=1) / (np.linalg.norm(want[:, :3], axis=1) + 0.1)
    assert rel.max() <= 1e-5


@pytest.mark.parametrize("n,bands", [(65536, 1), (185000, 1), (190000, 2), (300000, 3)])
def test_sym_f64_default_plan(cuda, n, bands):
    """FP64 state: one warp x 2 targets at every size, the triangular array
    (N^2 / 4 bytes) cut into bands of at most 8 GiB past N = 185k."""
    import torch

    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    with NBodySystem(n, "f64", "sym") as s:
        info, src = s.plan_info(), s.source_info()
        used = free0 - torch.cuda.mem_get_info()[0]
    assert (info["block"], info["bpt"]) == (32, 2)
    assert src["bands"] == bands and src["mib"] <= 8192, src
    assert used < 10 << 30, used


@pytest.mark.parametrize("n", [4096, 65536])
def test_sym_fixed_point_source_side_is_exact_and_deterministic(cuda, n):
    """The source side summed in fixed point (NB_SOURCE_FIXED): accelerations
    of every fixed-point shape within 2e-5 of the FP64 oracle, and the
    median error within twice the triangular array's (the pair terms'
    rsqrt.approx error dominates both); a second context (a different CTA order
    at run time) gives the same bits; so do two calls of one context, and
    steps after nb_set_state with heavier masses (a new scale record)."""
    p, _ = ics.plummer(n, seed=n + 3)
    p32 = ics.f32(p)
    v = np.zeros_like(p32)
    tidx = np.random.default_rng(2).choice(n, 256, replace=False).astype(np.int32)
    ref = oracle.accel_subset_f64(p32.astype(np.float64), tidx, float(np.float32(1e-4)))
    outs = []
    for shape in [(32, 16), (32, 16), (32, 8), (32, 4)]:
        with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-4), block=shape[0], bpt=shape[1],
                         source_side="fixed") as s:
            s.set_state(p32, v)
            a = s.accel()
            again = s.accel()
            assert a.tobytes() == again.tobytes()
            outs.append(a)
        d = np.linalg.norm(a[tidx].astype(np.float64) - ref, axis=1)
        w = np.linalg.norm(ref, axis=1)
        assert (d <= 2e-5 * (w + w.mean())).all(), shape
    assert outs[0].tobytes() == outs[1].tobytes()
    with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-4), source_side="triangular") as s:
        s.set_state(p32, v)
        tri = s.accel()
    w = np.linalg.norm(ref, axis=1)
    e_fx = np.linalg.norm(outs[0][tidx].astype(np.float64) - ref, axis=1) / w
    e_tri = np.linalg.norm(tri[tidx].astype(np.float64) - ref, axis=1) / w
    assert np.median(e_fx) <= 2 * np.median(e_tri)
    heavy = p32.copy()
    heavy[:, 3] *= 1e6
    with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-4), source_side="fixed") as s:
        s.set_state(heavy, v)
        a = s.accel()
    ref_h = oracle.accel_subset_f64(heavy.astype(np.float64), tidx, float(np.float32(1e-4)))
    d = np.linalg.norm(a[tidx].astype(np.float64) - ref_h, axis=1)
    w = np.linalg.norm(ref_h, axis=1)
    assert (d <= 2e-5 * (w + w.mean())).all()


# float-float pair arithmetic (its triangular array in one pass, or in three
# bands); FP64 arithmetic throughout
F64_SYM = ["sym", "symband", "sym64"]


def f64sys(n, algo, **kw):
    if algo == "symband":
        return NBodySystem(n, "f64", "sym", bands=3, **kw)
    return NBodySystem(n, "f64", algo, **kw)


@pytest.mark.parametrize("algo", F64_SYM)
@pytest.mark.parametrize("n", [1, 2, 33, 255, 256, 257, 1000, 2049, 5000])
def test_sym_f64_accel_vs_oracle(cuda, n, algo):
    """Symmetric kernels for FP64 state: accelerations within 1e-13
    (|a| + mean|a|) of the FP64 oracle -- the float-float kernel (exact
    three-float position differences, error-free sums and products, a Halley
    step on the FP32 rsqrt) and the FP64 one (FP64 rsqrt approximation and two
    Newton steps)."""
    p, _ = ics.plummer(n, seed=n)
    with f64sys(n, algo, eps2=1e-3) as s:
        s.set_state(p, np.zeros_like(p))
        a = s.accel()
    assert close(a, oracle.accel(p, 1e-3), tol=1e-13)


@pytest.mark.parametrize("algo,shape", [("sym", s) for s in [(32, 2), (32, 4), (128, 4), (256, 4), (256, 8)]] +
                         [("symband", s) for s in [(32, 2), (32, 4)]] +
                         [("sym64", s) for s in [(32, 8), (32, 4), (128, 8), (256, 8)]])
@pytest.mark.parametrize("n", [1000, 4097])
def test_sym_f64_every_shape_vs_oracle(cuda, algo, shape, n):
    """Every compiled shape of both FP64-state symmetric kernels, including
    the multi-warp ones the default plan only picks for large N (their
    reactions are summed across the CTA's warps through shared memory)."""
    p, _ = ics.plummer(n, seed=n + 1)
    with f64sys(n, algo, eps2=1e-3, block=shape[0], bpt=shape[1]) as s:
        info = s.plan_info()
        assert (info["block"], info["bpt"]) == shape
        s.set_state(p, np.zeros_like(p))
        a = s.accel()
        e, bodies = s.energy(with_bodies=True)
    want = oracle.accel(p, 1e-3)
    assert close(a, want, tol=1e-13)
    assert close(bodies[:, :3], want, tol=1e-13)


@pytest.mark.parametrize("algo", F64_SYM)
def test_sym_f64_close_pairs_far_from_origin(cuda, algo):
    """A dense core (radius 0.05) inside a halo, both 3.6e3 from the origin:
    r = x_j - x_i of close pairs cancels all but the last 20 bits of the
    coordinates, which a two-float position split would lose; the three-float
    split keeps them."""
    n = 4096
    rng = np.random.default_rng(5)
    p = np.empty((n, 4))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    rad = np.where(np.arange(n) % 4 == 0, 0.05, 1.0) * rng.random(n) ** (1 / 3)
    p[:, :3] = np.array([3.0e3, -2.0e3, 5.0e2]) + u * rad[:, None]
    p[:, 3] = rng.uniform(0.5, 1.5, n) / n
    with f64sys(n, algo, eps2=1e-4) as s:
        s.set_state(p, np.zeros_like(p))
        a = s.accel()
    assert close(a, oracle.accel(p, 1e-4), tol=1e-13)


@pytest.mark.parametrize("algo", F64_SYM)
def test_sym_f64_tight_binaries(cuda, algo):
    """Tight binaries (separation 1e-4, softening 1e-5 of it): each body's
    acceleration is dominated by its partner's single pair term, so the pair
    term's own accuracy is the result's -- checked per body, without the
    mean-magnitude cushion, to 5e-14."""
    nb = 600
    rng = np.random.default_rng(12)
    c = rng.normal(size=(nb, 3))
    d = rng.normal(size=(nb, 3))
    d *= 1e-4 / np.linalg.norm(d, axis=1, keepdims=True)
    p = np.empty((2 * nb, 4))
    p[0::2, :3] = c - d / 2
    p[1::2, :3] = c + d / 2
    p[:, 3] = rng.uniform(0.5, 1.5, 2 * nb)
    with f64sys(2 * nb, algo, eps2=1e-18) as s:
        s.set_state(p, np.zeros_like(p))
        a = s.accel()
    want = oracle.accel(p, 1e-18)
    rel = np.linalg.norm(a - want, axis=1) / np.linalg.norm(want, axis=1)
    assert rel.max() <= 5e-14, rel.max()


@pytest.mark.parametrize("algo", F64_SYM)
def test_sym_f64_si_units(cuda, algo):
    """Planetary magnitudes in SI units (positions ~1e11 m, masses ~1e24 to
    1e30 kg, eps2 = (1e7 m)^2): unscaled, the float-float kernel's inv^3
    would underflow the float range; it scales positions and masses by powers
    of two on the device each step and undoes that exactly."""
    n = 1000
    rng = np.random.default_rng(9)
    p = np.empty((n, 4))
    p[:, :3] = rng.normal(size=(n, 3)) * 1.5e11
    p[:, 3] = 10.0 ** rng.uniform(24, 30, n)
    with f64sys(n, algo, eps2=1e14, G=6.674e-11) as s:
        s.set_state(p, np.zeros_like(p))
        a = s.accel()
    assert close(a, oracle.accel(p, 1e14), tol=1e-13)


@pytest.mark.parametrize("algo", F64_SYM)
def test_sym_f64_power_of_two_scale_invariance(cuda, algo):
    """Positions x 2^10, masses x 2^5 and eps2 x 2^20 give the accelerations
    x 2^-15 bit for bit: the float-float kernel works in units normalized by
    powers of two, the FP64 kernel scales exactly."""
    n = 777
    p, _ = ics.plummer(n, seed=4)
    q = p.copy()
    q[:, :3] *= 2.0 ** 10
    q[:, 3] *= 2.0 ** 5
    out = []
    for x, e in ((p, 1e-3), (q, 1e-3 * 2.0 ** 20)):
        with f64sys(n, algo, eps2=e) as s:
            s.set_state(x, np.zeros_like(x))
            out.append(s.accel())
    assert np.array_equal(out[1], out[0] * 2.0 ** -15)


@pytest.mark.parametrize("algo", F64_SYM)
@pytest.mark.parametrize("kick", ["reference", "physical"])
def test_sym_f64_steps_vs_oracle(cuda, kick, algo):
    n, steps = 3000, 10
    p, v = ics.uniform_cube(n, seed=1)
    km = oracle.KICK_REFERENCE if kick == "reference" else oracle.KICK_PHYSICAL
    with f64sys(n, algo, kick=kick, eps2=1e-2, damping=0.999, dt=1e-3) as s:
        s.set_state(p, v)
        s.step(steps)
        got, gv = s.get_state()
        s.set_state(p, v)
        s.step(steps)
        again, _ = s.get_state()
    want, wv = oracle.step(p, v, 1e-2, 0.999, 1e-3, steps, kick_mode=km)
    rel = np.linalg.norm(got[:, :3] - want[:, :3], axis=1) / (np.linalg.norm(want[:, :3], axis=1) + 0.1)
    assert rel.max() <= 1e-13
    assert got.tobytes() == again.tobytes()


def test_gpu_scale_positions_after_100_steps_vs_fp64(cuda, capsys):
    """The GPU-scale workload as the bench runs it (N=65536 Plummer,
    eps2 = dt = 1e-4, 100 leapfrog steps): float positions from the symmetric
    kernel (both source sides) and the directed kernel within 1e-5 (|x| + 0.1)
    of an FP64 run of the same float-rounded start.  The FP64 run is the
    float-float symmetric kernel for FP64 state, itself held to 1e-13 of the
    FP64 oracle (test_sym_f64_*); the CPU oracle would need 4-8 minutes for
    the 4.3e11 FP64 pair terms of this run."""
    n, steps = 65536, 100
    p, v = ics.plummer(n, seed=0)
    p32, v32 = ics.f32(p), ics.f32(v)
    with NBodySystem(n, "f64", "sym", kick="physical", eps2=float(np.float32(1e-4)), damping=1.0,
                     dt=float(np.float32(1e-4))) as s:
        s.set_state(p32.astype(np.float64), v32.astype(np.float64))
        s.step(steps)
        want, _ = s.get_state()
    scale = np.linalg.norm(want[:, :3], axis=1) + 0.1
    worst = {}
    for algo, side in (("sym", "auto"), ("sym", "fixed"), ("fast", "auto")):
        with NBodySystem(n, "f32", algo, kick="physical", eps2=np.float32(1e-4), damping=1.0,
                         dt=np.float32(1e-4), source_side=side) as s:
            s.set_state(p32, v32)
            s.step(steps)
            got, _ = s.get_state()
        rel = np.linalg.norm(got[:, :3].astype(np.float64) - want[:, :3], axis=1) / scale
        worst[f"{algo}/{side}"] = float(rel.max())
        assert rel.max() <= 1e-5, (algo, side, rel.max())
    with capsys.disabled():
        print("\n[N=65536, 100 steps] max |dx|/(|x|+0.1) against the FP64-accurate run: "
              + ", ".join(f"{k} {v:.1e}" for k, v in worst.items()))


def test_sym_fixed_point_steps_and_new_eps2(cuda):
    """Steps with the fixed-point source side: positions after 40 steps within
    1e-5 (|x| + 0.1) of the FP64 oracle, bitwise reruns through the captured
    graph and step by step, and nb_set_params to a new eps2 (its scale is
    rewritten before the next force launch) equal to a fresh context made
    with that eps2."""
    n, steps = 3000, 40
    p, v = ics.plummer(n, seed=17)
    p32, v32 = ics.f32(p), ics.f32(v)
    kw = dict(kick="physical", damping=1.0, dt=np.float32(1e-4), source_side="fixed")
    with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-4), **kw) as s:
        s.set_state(p32, v32)
        s.step(steps)
        got, _ = s.get_state()
        s.set_state(p32, v32)
        for _ in range(steps):
            s.step(1)
        again, _ = s.get_state()
        s.set_params(np.float32(1e-2), 1.0, np.float32(1e-4))
        s.set_state(p32, v32)
        s.step(3)
        newe, _ = s.get_state()
        s.set_state(p32, v32)
        s.set_params(np.float32(1e-3), 1.0, np.float32(1e-4))
        s.step(3)
        mid, _ = s.get_state()
    with NBodySystem(n, "f32", "sym", eps2=np.float32(1e-3), **kw) as s:
        s.set_state(p32, v32)
        s.step(3)
        fresh, _ = s.get_state()
    want, _ = oracle.step(p32.astype(np.float64), v32.astype(np.float64), float(np.float32(1e-4)), 1.0,
                          float(np.float32(1e-4)), steps, kick_mode=oracle.KICK_PHYSICAL)
    rel = np.linalg.norm(got[:, :3].astype(np.float64) - want[:, :3], axis=1) / (
        np.linalg.norm(want[:, :3], axis=1) + 0.1)
    assert rel.max() <= 1e-5
    assert got.tobytes() == again.tobytes()
    assert mid.tobytes() == fresh.tobytes()
    assert newe.tobytes() != mid.tobytes()
