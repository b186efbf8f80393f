"""The reference's CUDA kernel, compiled unchanged for sm_103a, as the GPU
baseline: it agrees with the oracle, and the fast kernel is timed against it
on the GPU-scale workload (N=65536 Plummer, eps2=1e-4, dt=1e-4)."""
import os

import numpy as np
import pytest

import oracle
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_kernel(cuda):
    if not os.path.exists(oracle.REF_CUBIN):
        pytest.skip("reference cubin not built (needs the reference checkout at build time)")
    from ref_gpu import RefKernel

    k = RefKernel()
    yield k
    k.close()


def run_ref(ref_kernel, pos, vel, steps, dt, eps2, block=256):
    import torch

    s = torch.cuda.current_stream()
    bufs = [torch.from_numpy(pos).cuda(), torch.empty_like(torch.from_numpy(pos)).cuda()]
    v = torch.from_numpy(vel).cuda()
    n = pos.shape[0]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for i in range(steps):
        ref_kernel.step(bufs[i % 2].data_ptr(), bufs[(i + 1) % 2].data_ptr(), v.data_ptr(), n, dt,
                        eps2, 1.0, block, s.cuda_stream)
    e1.record(s)
    e1.synchronize()
    return bufs[steps % 2].cpu().numpy(), v.cpu().numpy(), e0.elapsed_time(e1)


def test_reference_kernel_matches_oracle(ref_kernel):
    n = 2048
    pos, vel = oracle.randomize(1, n, np.float32)
    dt, _, _, soft, _ = oracle.demo_params(0, n)
    eps2 = np.float32(soft) * np.float32(soft)
    p, _, _ = run_ref(ref_kernel, pos, vel, 3, dt, eps2)
    want, _ = oracle.step(pos, vel, eps2, 1.0, dt, 3)
    assert np.abs(p - want).max() < 1e-4


def test_fast_kernel_beats_reference_kernel(ref_kernel, capsys):
    import torch

    n, steps = 65536, 10
    p64, v64 = ics.plummer(n, seed=0)
    pos, vel = ics.f32(p64), ics.f32(v64)
    run_ref(ref_kernel, pos, vel, 2, 1e-4, 1e-4)  # warm-up
    p_ref, _, ms_ref = run_ref(ref_kernel, pos, vel, steps, 1e-4, 1e-4)
    rate_ref = n * n * steps / (ms_ref * 1e-3) / 1e9
    for algo in ("fast", "sym"):
        with NBodySystem(n, "f32", algo, kick="reference", eps2=1e-4, damping=1.0, dt=1e-4) as s:
            s.set_state(pos, vel)
            s.step(2)
            s.set_state(pos, vel)
            f, g = s.step_timed(steps)
            p_ours, _ = s.get_state()
        torch.cuda.synchronize()
        # both run the reference's update rule (kick x pos.w) on the same input
        assert np.abs(p_ours - p_ref).max() < 1e-5
        rate_ours = n * n * steps / ((f + g) * 1e-3) / 1e9
        with capsys.disabled():
            print(f"\n[gpu baseline] N={n}: reference kernel (sm_103a build) {rate_ref:.1f} G interactions/s, "
                  f"{ms_ref / steps:.3f} ms/step; {algo} kernel {rate_ours:.1f} G interactions/s, "
                  f"{(f + g) / steps:.3f} ms/step; speed-up {rate_ours / rate_ref:.2f}x")
        assert rate_ours > rate_ref


def test_batch_vs_reference_kernel_per_system(ref_kernel, capsys):
    """The batched workload (512 Plummer systems, N log-uniform in
    [128, 16384], eps2 = dt = 1e-3, 50 steps) three ways on the same GPU: the
    reference's kernel launched once per system per step (its own launch
    shape: block 128, one target per thread; sizes rounded up to a multiple
    of 128 as the reference app rounds N, so all three run those sizes), this
    library's plain per-system launches, and the autotuned batched launch in
    a CUDA graph.  The reference's update rule (kick x pos.w) throughout."""
    import torch

    from utc_gb300.nbody import NBodyBatch

    sizes = (ics.batch_sizes(512, lo=128, hi=16384, seed=0) + 127) // 128 * 128
    steps = 50
    ps, vs = [], []
    for k, nn in enumerate(sizes):
        p, v = ics.plummer(int(nn), seed=1000 + k)
        ps.append(ics.f32(p))
        vs.append(ics.f32(v))
    pos, vel = np.concatenate(ps), np.concatenate(vs)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    bufs = [torch.from_numpy(pos).cuda(), torch.from_numpy(pos).cuda()]
    vt = torch.from_numpy(vel).cuda()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def ref_steps(nsteps):
        for t in range(nsteps):
            for k, nn in enumerate(sizes):
                o = int(off[k]) * 16
                ref_kernel.step(bufs[t % 2].data_ptr() + o, bufs[(t + 1) % 2].data_ptr() + o,
                                vt.data_ptr() + o, int(nn), 1e-3, 1e-3, 1.0, 128, sh)

    torch.cuda.synchronize()
    ref_steps(2)  # warm-up, on `stream`
    stream.synchronize()  # before the default stream rewrites its buffers
    bufs[0].copy_(torch.from_numpy(pos))
    vt.copy_(torch.from_numpy(vel))
    torch.cuda.synchronize()
    e0.record(stream)
    ref_steps(steps)
    e1.record(stream)
    e1.synchronize()
    ms_ref = e0.elapsed_time(e1)
    p_ref = bufs[steps % 2].cpu().numpy()
    times = {}
    with torch.cuda.stream(stream), NBodyBatch(sizes, kick="reference", eps2=np.float32(1e-3),
                                               dt=np.float32(1e-3)) as b:
        b.set_state(pos, vel, stream=sh)
        shape = b.autotune(reps=1, stream=sh)
        for name, fn in (("graph", lambda: b.run(steps, sh)),
                         ("per_system", lambda: b.step_per_system(steps, sh))):
            b.set_state(pos, vel, stream=sh)
            fn()  # warm-up (captures the graph)
            b.set_state(pos, vel, stream=sh)
            stream.synchronize()
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            times[name] = e0.elapsed_time(e1)
            got, _ = b.get_state(stream=sh)
            assert np.abs(got - p_ref).max() < 1e-4, name
    pairs = float(np.sum(sizes.astype(np.float64) ** 2)) * steps
    with capsys.disabled():
        print(f"\n[batch baseline] {len(sizes)} systems ({int(sizes.sum())} bodies), {steps} steps: reference "
              f"kernel per system {ms_ref:.1f} ms ({pairs / ms_ref / 1e6:.0f} G interactions/s); this library's "
              f"per-system launches {times['per_system']:.1f} ms; batched graph (shape {shape}) "
              f"{times['graph']:.1f} ms ({pairs / times['graph'] / 1e6:.0f} G interactions/s); speed-up "
              f"{ms_ref / times['graph']:.1f}x over the reference kernel per system, "
              f"{times['per_system'] / times['graph']:.2f}x over own per-system launches")
    assert times["graph"] < ms_ref


def test_reference_kernel_f64_vs_exact_f64(ref_kernel, capsys):
    """The app's default state type is double: the reference's kernel in
    double against the reference-exact FP64 kernel, same input, same update
    rule (reference kick).  Agreement to FP64 rounding; both timed."""
    import torch

    n, steps, block = 16384, 3, 256
    p64, v64 = ics.plummer(n, seed=3)
    s = torch.cuda.current_stream()
    bufs = [torch.from_numpy(p64).cuda(), torch.empty_like(torch.from_numpy(p64)).cuda()]
    vt = torch.from_numpy(v64).cuda()
    ref_kernel.step(bufs[0].data_ptr(), bufs[1].data_ptr(), vt.data_ptr(), n, 1e-4, 1e-4, 1.0, block,
                    s.cuda_stream, double=True)  # warm-up
    bufs[0].copy_(torch.from_numpy(p64))
    vt.copy_(torch.from_numpy(v64))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for i in range(steps):
        ref_kernel.step(bufs[i % 2].data_ptr(), bufs[(i + 1) % 2].data_ptr(), vt.data_ptr(), n, 1e-4, 1e-4,
                        1.0, block, s.cuda_stream, double=True)
    e1.record(s)
    e1.synchronize()
    ms_ref = e0.elapsed_time(e1)
    p_ref = bufs[steps % 2].cpu().numpy()
    r_ref = n * n * steps / (ms_ref * 1e-3) / 1e9
    for algo in ("exact", "sym", "sym64"):
        with NBodySystem(n, "f64", algo, kick="reference", eps2=1e-4, damping=1.0, dt=1e-4) as sy:
            sy.set_state(p64, v64)
            sy.step(1)
            sy.set_state(p64, v64)
            f, g = sy.step_timed(steps)
            p_ours, _ = sy.get_state()
        assert np.abs(p_ours - p_ref).max() <= 1e-12 * np.abs(p_ref).max()
        r_ours = n * n * steps / ((f + g) * 1e-3) / 1e9
        with capsys.disabled():
            print(f"\n[gpu baseline f64] N={n}: reference kernel (double, sm_103a build) {r_ref:.2f} "
                  f"G interactions/s; {algo} FP64 kernel {r_ours:.2f} G interactions/s; "
                  f"ratio {r_ours / r_ref:.2f}x")
    from utc_gb300.nbody import probe_fma_peak

    peak64, _ = probe_fma_peak(2000, packed=2)
    with capsys.disabled():
        print(f"[gpu baseline f64] measured FP64 DFMA peak {peak64 / 1e12:.3f} TFLOP/s")
    assert peak64 > 0
