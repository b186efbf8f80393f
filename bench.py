"""Benchmark of the nbody all-pairs step on GB300.

Workload (one bench "step"): the GPU-scale plain forward run -- N=65536
Plummer sphere (a=1, isotropic distribution-function velocities, equal masses
1/N), eps2=1e-4, dt=1e-4, 100 leapfrog steps from the same initial state.
Metric: G body-interactions/s = N^2 * leapfrog steps / t / 1e9 (self pairs
count, as in the reference).  FP32-pipe % uses the reference's 20 FLOP per
interaction (benchapps/nbody/seq/bodysystem.h:75-95).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs an independent replica of the workload
(weak scaling, no data-path collective); rank 0 prints one JSON line.
`e2e` times nb_run_host (the C-ABI call the task makes) from pinned host
buffers; `e2e.through_task` times the drop-in UTC task itself
(BodySystemGB300<float>: init, run, wait, from pageable arrays).

Extension workloads, one JSON line each (not the headline):
  --workload precision  N=1,048,576 Plummer, 20 steps of dt=1e-4, plain FP32
                        vs compensated FP32 + FP64 positions: per-step force
                        and energy error against the FP64 oracle on a
                        4096-body subsample; forward throughput at N=1M
  --workload adjoint    N=16384 uniform cube, 200 steps, checkpoints every 20:
                        adjoint/forward time ratio; gradient error against the
                        FP64 reference adjoint (full size) and FP64 central
                        differences (64 coordinates, N=2048 replica)
  --workload batched    512 Plummer systems, N log-uniform in [128, 16384],
                        eps2=1e-3, dt=1e-3, 50 steps: autotuned persistent
                        launch in a CUDA graph vs per-system launches
  --workload double     the app's default state type: N=16384 Plummer in
                        FP64, reference kick, eps2=dt=1e-4, 10 steps, through
                        the float-float symmetric kernel (default), the FP64
                        symmetric kernel and the reference-exact FP64 kernel:
                        throughput, force error against the FP64 oracle
                        (512-body subsample), final positions against the
                        reference-exact run
  --workload frames     N=65536, 200 steps through nb_run_host with a frame
                        every 200, 20, 5 and 1 steps, pageable and pinned
                        host memory: wall time against one frame
  --workload ics        initial conditions drawn on the GPU (cube, Plummer,
                        the app's shell) at N=2^20 and 2^24: bodies/s and
                        store bandwidth, beside the host generator
  --workload sharded    one N=1,048,576 system split over the ranks (the
                        multi-GPU target partition, one all-gather per step),
                        10 leapfrog steps per bench step: strong scaling
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_BODIES = 65536
LEAPFROG_STEPS = 100
EPS2 = 1e-4
DT = 1e-4
FLOP_PER_INTERACTION = 20
METRIC = "G body-interactions/s"
UNIT = "G interactions/s"
WORKLOAD = (f"plain forward, Plummer N={N_BODIES}, {LEAPFROG_STEPS} leapfrog steps per bench step, "
            f"eps2={EPS2}, dt={DT}, masses 1/N, kick G=1")
L2_FLUSH_BYTES = 256 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, world, device=None):
    """Max of a per-rank float over all ranks (the timing rule: the slowest
    rank's time).  Uses the initialised process group (NCCL on GPUs, gloo on
    CPU); identity for one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_state():
    from utc_gb300 import ics

    p, v = ics.plummer(N_BODIES, seed=0)
    return ics.f32(p), ics.f32(v)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def integrate_bytes(n, algo, plan):
    """Bytes the integrate kernel has to move per launch: the state read and
    written (pos and vel, 64 B per body) plus every partial-sum entry it adds,
    16 B each: the target-side slots of the CTAs that worked on the body's
    block and, on the symmetric path (triangular source side), one
    source-side entry per earlier row block."""
    grid, rb = plan["grid"], plan["tbsize"]
    nblk = (n + rb - 1) // rb
    if algo == "sym":
        nc, rc = (n + 31) // 32, rb // 32

        def first(b):
            return b * nc - rc * (b * (b - 1) // 2)
        total = first(nblk)
    else:
        ng = (n + 31) // 32

        def first(b):
            return b * ng
        total = nblk * ng

    def owner(it):
        return ((it + 1) * grid - 1) // total
    entries = 0
    for b in range(nblk):
        rows = min(rb, n - b * rb)
        entries += (owner(first(b + 1) - 1) - owner(first(b)) + 1) * rows
        if algo == "sym":
            entries += b * rows  # source-side rows 0..b-1
    return 64.0 * n + 16.0 * entries


def committed_traffic():
    """Per-launch DRAM bytes and pipe counters of the top kernels from the
    committed ncu summaries (profiles/traffic.json)."""
    try:
        return json.load(open(os.path.join(REPO, "profiles", "traffic.json")))
    except (OSError, ValueError):
        return {}


# Algorithmic bytes of the integrator per body (FP32, split integrator
# kernel): read pos 16 + vel 16 + acceleration 16, write pos 16 + vel 16.
INTEGRATOR_BYTES_PER_BODY = 80


def _device_free_bytes():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def sub_n1m_forward(peak_flops, source_side="auto"):
    """The forward target at N=1,048,576 (Plummer, eps2 = dt = 1e-4): the
    FP32 symmetric kernel (its default triangular source side, or the
    fixed-point one), 3 leapfrog steps after one untimed step, per-kernel
    CUDA events; the context's device footprint beside it."""
    from utc_gb300 import ics
    from utc_gb300.nbody import NBodySystem

    n = 1 << 20
    p, v = ics.plummer(n, seed=0)
    p32, v32 = ics.f32(p), ics.f32(v)
    free0 = _device_free_bytes()
    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(EPS2), damping=1.0,
                     dt=np.float32(DT), source_side=source_side) as s:
        footprint = free0 - _device_free_bytes()
        s.set_state(p32, v32)
        s.step(1)
        s.set_state(p32, v32)
        steps = 3
        f, g = s.step_timed(steps)
        plan = s.plan_info()
    inter = float(n) ** 2 * steps
    return {"workload": f"plain forward, Plummer N={n}, {steps} leapfrog steps, eps2={EPS2}, dt={DT}",
            "G_interactions_per_s": inter / ((f + g) * 1e-3) / 1e9,
            "force_kernel_G_interactions_per_s": inter / (f * 1e-3) / 1e9,
            "force_ms_per_launch": f / steps, "integrate_ms_per_launch": g / steps,
            "tflops_20flop": FLOP_PER_INTERACTION * inter / (f * 1e-3) / 1e12,
            "frac_of_fp32_peak_20flop": FLOP_PER_INTERACTION * inter / (f * 1e-3) / peak_flops,
            "device_footprint_bytes": int(footprint), "plan": plan,
            "source_side": "triangular array" if source_side == "auto" else "fixed-point accumulators"}


def sub_adjoint(reps=3):
    """The adjoint workload (N=16384 uniform cube, 200 steps, checkpoints
    every 20, default symmetric kernels): medians of the plain forward, the
    checkpointed forward and the backward (recompute + VJP)."""
    import torch

    from utc_gb300 import ics
    from utc_gb300.nbody import NBodySystem

    n, T, K = 16384, 200, 20
    p64, v64 = ics.uniform_cube(n, seed=0)
    y = torch.tensor(ics.gaussian_targets(n, seed=1, sigma=0.5), dtype=torch.float32, device="cuda")
    p32, v32 = ics.f32(p64), ics.f32(v64)
    stream = torch.cuda.current_stream()

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    ts = {"forward": [], "adj_forward": [], "adj_backward": []}
    with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-2), damping=1.0,
                     dt=np.float32(1e-3)) as s:
        pT = torch.empty((n, 4), device="cuda")
        vT = torch.empty((n, 4), device="cuda")
        for r in range(reps + 1):
            s.set_state(p32, v32)
            tf = timed(lambda: s.step(T))
            s.set_state(p32, v32)
            ta = timed(lambda: s.adj_forward(T, K))
            s.get_state_device(pT, vT)
            gx = torch.zeros((n, 4), device="cuda")
            gx[:, :3] = 2.0 * (pT[:, :3] - y)
            tb = timed(lambda: s.adj_backward(gx))
            if r:  # the first round is the warm-up
                ts["forward"].append(tf)
                ts["adj_forward"].append(ta)
                ts["adj_backward"].append(tb)
    med = {k: float(np.median(v)) for k, v in ts.items()}
    return {"workload": f"adjoint, uniform cube N={n}, {T} steps, checkpoints every {K}, symmetric kernels",
            "ms_median": med,
            "backward_over_forward": med["adj_backward"] / med["forward"],
            "backward_plus_ckpt_forward_over_forward": (med["adj_backward"] + med["adj_forward"]) / med["forward"]}


def sub_batched():
    """The batched workload (512 Plummer systems, N log-uniform in
    [128, 16384], eps2 = dt = 1e-3, 50 steps): the autotuned batched launch
    in a CUDA graph against this library's plain per-system launches."""
    import torch

    from utc_gb300 import ics
    from utc_gb300.nbody import NBodyBatch

    sizes = ics.batch_sizes(512, lo=128, hi=16384, seed=0)
    steps = 50
    ps, vs = [], []
    for k, nn in enumerate(sizes):
        p, v = ics.plummer(int(nn), seed=1000 + k)
        ps.append(ics.f32(p))
        vs.append(ics.f32(v))
    pos, vel = np.concatenate(ps), np.concatenate(vs)
    pairs = float(np.sum(sizes.astype(np.float64) ** 2)) * steps
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    res = {}
    with torch.cuda.stream(stream), NBodyBatch(sizes, kick="physical", eps2=np.float32(1e-3),
                                               dt=np.float32(1e-3)) as b:
        b.set_state(pos, vel, stream=sh)
        shape = b.autotune(reps=1, stream=sh)
        for name, fn in (("graph", lambda: b.run(steps, sh)),
                         ("per_system", lambda: b.step_per_system(steps, sh))):
            b.set_state(pos, vel, stream=sh)
            fn()  # warm-up (captures the graph)
            b.set_state(pos, vel, stream=sh)
            stream.synchronize()
            a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            c.record(stream)
            c.synchronize()
            res[name] = a.elapsed_time(c)
    return {"workload": f"batched, {sizes.size} Plummer systems N in [128, 16384] ({int(sizes.sum())} "
                        f"bodies), {steps} steps, eps2=dt=1e-3",
            "autotuned_shape": list(shape), "ms_batched_graph": res["graph"],
            "ms_per_system_launches": res["per_system"],
            "speedup_vs_per_system": res["per_system"] / res["graph"],
            "G_interactions_per_s_batched": pairs / (res["graph"] * 1e-3) / 1e9,
            "G_interactions_per_s_per_system": pairs / (res["per_system"] * 1e-3) / 1e9,
            "reference_kernel_per_system": "timed in tests/test_reference_gpu_kernel.py "
                                           "(the reference's kernel is test infrastructure)"}


# ---------------------------------------------------------------------------
# CPU baseline (oracle port of the reference's sequential BodySystem<float>)
# ---------------------------------------------------------------------------
def cpu_single_thread(pos, vel):
    """One leapfrog step of the workload by the oracle port on ONE host
    thread, as the reference's sequential nbody runs
    (benchapps/nbody/seq/nbody_main.cc:177-190, bodysystem.cc:103-133)."""
    import oracle

    t0 = time.perf_counter()
    oracle.step(pos, vel, np.float32(EPS2), np.float32(1.0), np.float32(DT), 1,
                kick_mode=oracle.KICK_PHYSICAL, G=np.float32(1.0), nthreads=1)
    dt = time.perf_counter() - t0
    return {"value": float(N_BODIES) ** 2 / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
            "nproc": os.cpu_count(),
            "sample": f"1 of the {LEAPFROG_STEPS} leapfrog steps at N={N_BODIES} ({dt:.1f} s on 1 host "
                      f"thread of {os.cpu_count()}; the reference's CPU nbody is sequential)"}


def cpu_baseline(pos, vel, min_seconds=10.0, max_steps=3, threads=None):
    import oracle

    threads = threads or (os.cpu_count() or 1)
    kind = "port"
    t0 = time.perf_counter()
    steps = 0
    p, v = pos, vel
    while steps < max_steps:
        p, v = oracle.step(p, v, np.float32(EPS2), np.float32(1.0), np.float32(DT), 1,
                           kick_mode=oracle.KICK_PHYSICAL, G=np.float32(1.0), nthreads=threads)
        steps += 1
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    rate = float(N_BODIES) ** 2 * steps / dt / 1e9
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{steps} of the {LEAPFROG_STEPS} leapfrog steps at N={N_BODIES} "
                      f"({dt:.1f} s on {threads} host threads; oracle restatement of "
                      f"BodySystem<float>, targets split across threads, bit-identical per body)",
            "threads_1": cpu_single_thread(pos, vel)}


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle

    oracle.build(ref=False)
    pos, vel = workload_state()
    threads = os.cpu_count() or 1
    # one bounded sample per bench step: one leapfrog step of the workload
    for _ in range(args.warmup):
        oracle.step(pos, vel, np.float32(EPS2), np.float32(1.0), np.float32(DT), 1,
                    kick_mode=oracle.KICK_PHYSICAL, G=np.float32(1.0), nthreads=threads)
    t0 = time.perf_counter()
    p, v = pos, vel
    for _ in range(args.steps):
        p, v = oracle.step(p, v, np.float32(EPS2), np.float32(1.0), np.float32(DT), 1,
                           kick_mode=oracle.KICK_PHYSICAL, G=np.float32(1.0), nthreads=threads)
    el = time.perf_counter() - t0
    val = float(N_BODIES) ** 2 * args.steps / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Plummer sphere)",
        "config": {"workload": WORKLOAD + "; reference arm: one leapfrog step per bench step",
                   "n": N_BODIES, "parallelism": "host threads"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} single leapfrog steps at N={N_BODIES} on "
                                   f"{threads} host threads (reference sequential algorithm, "
                                   f"oracle restatement; the compiled reference is x86-only here)",
                         "threads_1": cpu_single_thread(pos, vel)},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    from utc_gb300 import _native as N
    from utc_gb300.nbody import NBodySystem, probe_fma_peak

    N.lib()
    pos, vel = workload_state()
    stream = torch.cuda.current_stream()
    sh = int(stream.cuda_stream)
    pos_d = torch.from_numpy(pos).to(dev)
    vel_d = torch.from_numpy(vel).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    sysm = NBodySystem(N_BODIES, "f32", args.algo, kick="physical", eps2=EPS2, damping=1.0, dt=DT, G=1.0)
    plan = sysm.plan_info()
    launches_per_leapfrog = sysm.launches_per_step()

    def one_step(timed=False):
        sysm.set_state(pos_d, vel_d, stream=sh)
        if timed:
            return sysm.step_timed(LEAPFROG_STEPS, stream=sh)
        sysm.step(LEAPFROG_STEPS, stream=sh)
        return None

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    t_wall0 = time.perf_counter()
    dev_ms = 0.0
    force_ms = 0.0
    integ_ms = 0.0
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        flush.zero_()  # evict L2 between timed steps (outside the event pair)
        ev0.record(stream)
        f, g = one_step(timed=True)
        ev1.record(stream)
        ev1.synchronize()
        dev_ms += ev0.elapsed_time(ev1)
        force_ms += f
        integ_ms += g
    barrier()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()

    dev_ms_max = max_over_ranks(dev_ms, world, dev)
    interactions = float(N_BODIES) ** 2 * LEAPFROG_STEPS * args.steps * world
    value = interactions / (dev_ms_max * 1e-3) / 1e9

    # end to end through the C ABI with host buffers (pinned), copies timed
    pos_h = torch.from_numpy(pos).pin_memory()
    vel_h = torch.from_numpy(vel).pin_memory()
    out_h = torch.empty((1, N_BODIES, 4), dtype=torch.float32).pin_memory()
    import ctypes as C

    e2e_times = []
    tim = (C.c_double * 4)()
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(sysm.lib.nb_run_host(sysm.handle, C.c_void_p(pos_h.data_ptr()),
                                     C.c_void_p(vel_h.data_ptr()), LEAPFROG_STEPS, LEAPFROG_STEPS,
                                     C.c_void_p(out_h.data_ptr()), tim, C.c_void_p(sh)),
                "nb_run_host")
        if k >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    e2e_val = interactions / max_over_ranks(sum(e2e_times), world, dev) / 1e9

    # the same K bench steps through nb_step as the product runs them: the
    # captured CUDA graph of steps, no per-kernel events (device time by one
    # event pair per bench step, L2 flushed between steps as above)
    graph_ms = 0.0
    gstream = torch.cuda.Stream()  # graphs need a stream other than the legacy default one
    gsh = int(gstream.cuda_stream)
    for k in range(args.warmup + args.steps):
        flush.zero_()
        gstream.wait_stream(stream)
        sysm.set_state(pos_d, vel_d, stream=gsh)
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(gstream)
        sysm.step(LEAPFROG_STEPS, stream=gsh)
        g1.record(gstream)
        g1.synchronize()
        if k >= args.warmup:
            graph_ms += g0.elapsed_time(g1)
    graph_ms_max = max_over_ranks(graph_ms, world, dev)
    state_bytes = N_BODIES * 16

    # the same workload through the drop-in UTC task (BodySystemGB300<float>:
    # its own worker thread and stream, nb_create + nb_run_host + nb_destroy
    # per run, pageable host arrays as the reference app passes them by
    # default; the task's reference kick costs the same as the physical one)
    tl = N.task_lib()
    pos_np = np.ascontiguousarray(pos, np.float32)
    vel_np = np.ascontiguousarray(vel, np.float32)
    frame_np = np.empty((1, N_BODIES, 4), np.float32)
    task_times = []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(tl.nbt_run_f32(N_BODIES, np.float32(EPS2), np.float32(1.0), pos_np.ctypes.data_as(C.c_void_p),
                               vel_np.ctypes.data_as(C.c_void_p), tim, LEAPFROG_STEPS, LEAPFROG_STEPS, 256,
                               np.float32(DT), frame_np.ctypes.data_as(C.c_void_p), N.NB_MEM_PAGEABLE,
                               N.NB_ALGO_SYM if args.algo == "sym" else N.NB_ALGO_FAST, local),
                "nbt_run_f32")
        if k >= args.warmup:
            task_times.append(time.perf_counter() - t0)
    e2e_task_val = interactions / max_over_ranks(sum(task_times), world, dev) / 1e9

    line = None
    if rank == 0:
        peaks = measured_peaks()
        fp32_flops, _ = probe_fma_peak(iters=20000, packed=True)
        fp32_peak_tf = fp32_flops / 1e12
        launches = args.steps * LEAPFROG_STEPS
        force_avg_s = force_ms / launches * 1e-3
        integ_avg_s = integ_ms / launches * 1e-3
        force_flops = FLOP_PER_INTERACTION * float(N_BODIES) ** 2
        achieved_tf = force_flops / force_avg_s / 1e12
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        nominal_tf = sms * 128 * 2 * (clk.get("sm_max_mhz") or 2070.0) * 1e6 / 1e12
        traffic = committed_traffic()
        integ_bytes = INTEGRATOR_BYTES_PER_BODY * N_BODIES
        integ_moved = integrate_bytes(N_BODIES, args.algo, plan)
        integ_traffic = traffic.get("integrate_bytes_per_launch") if args.algo == "sym" else None
        hbm = peaks.get("hbm_gbs")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Plummer sphere, float32)",
            "config": {"workload": WORKLOAD, "n": N_BODIES, "leapfrog_steps": LEAPFROG_STEPS,
                       "algo": args.algo,
                       "kick": "physical (G=1)", "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "flushed between timed steps (256 MB write outside the event pair)",
                       "plan": plan},
            "fp32_pct_20flop_convention": 100.0 * achieved_tf / fp32_peak_tf,
            "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": fp32_peak_tf,
                         "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak_tf,
                         "traffic": traffic.get("force_bytes_per_launch" if args.algo == "sym"
                                                else "directed_force_bytes_per_launch"),
                         "kernel": "sym_force_kernel" if args.algo == "sym" else "sk_force_kernel",
                         "flop_per_launch": force_flops,
                         "avg_launch_ms": force_avg_s * 1e3,
                         "peak_source": "packed-FMA probe measured in this run "
                                        "(MEASURED_PEAKS.json has no FP32 figure)",
                         "nominal_peak": nominal_tf,
                         "flop_convention": "20 FLOP per interaction (bodysystem.h:75-95); the "
                                            "symmetric kernel issues 16 FP32 operations per PAIR of "
                                            "interactions, so this rate can exceed the pipe's own use",
                         "ncu_fma_pipe_active": traffic.get("force_fma_pipe_active")
                         if args.algo == "sym" else traffic.get("directed_force_fma_pipe_active"),
                         "ncu_issue_active": traffic.get("force_issue_active")
                         if args.algo == "sym" else traffic.get("directed_force_issue_active"),
                         "ncu_source": traffic.get("force_source") if args.algo == "sym"
                         else traffic.get("directed_force_source")},
            "roofline_integrator": {"bound": "hbm",
                                    "kernel": "sym_integrate_kernel" if args.algo == "sym" else "sk_integrate_kernel",
                                    "achieved": integ_bytes / integ_avg_s / 1e9, "peak": hbm,
                                    "unit": "GB/s",
                                    "frac": (integ_bytes / integ_avg_s / 1e9) / hbm if hbm else None,
                                    "algorithmic_bytes_per_launch": integ_bytes,
                                    "avg_launch_ms": integ_avg_s * 1e3,
                                    "traffic": integ_traffic,
                                    "traffic_over_algorithmic": integ_traffic / integ_bytes if integ_traffic else None,
                                    "bytes_moved_per_launch": integ_moved,
                                    "moved_rate_GB_per_s": integ_moved / integ_avg_s / 1e9,
                                    "note": f"algorithmic: {INTEGRATOR_BYTES_PER_BODY} B/body (pos, vel, acc "
                                            "read; pos, vel written); moved: the state plus every partial "
                                            "entry the kernel adds (16 B each), here mostly the triangular "
                                            "source-side array (see n1m_forward_fixed_source for the O(N) "
                                            "alternative)"},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 2 * state_bytes,
                    "d2h_bytes_per_step": state_bytes,
                    "through_task": {"value": e2e_task_val, "unit": UNIT,
                                     "how": "BodySystemGB300<float> UTC task (init/run/wait), pageable host "
                                            "arrays, context made and freed per run, reference kick"},
                    "how": "nb_run_host (C ABI) from pinned host buffers, 100 leapfrog steps, "
                           "final positions read back, host wall clock"},
            "gpu_launches": launches * launches_per_leapfrog,
            "clocks": clk,
            "wall_s_timed_region": wall,
            "graph_replay": {"value": interactions / (graph_ms_max * 1e-3) / 1e9, "unit": UNIT,
                             "ms_per_step": graph_ms_max / args.steps,
                             "how": "the same bench steps through nb_step on a non-default stream (replayed "
                                    "CUDA graphs of 16 steps), measured after the timed region; `value` "
                                    "itself is timed step by step with CUDA events around every kernel, "
                                    "which the force roofline needs"},
        }
        if world == 1 and not args.no_extras:
            # the other stated targets, measured in the same run (outside the
            # timed region above; each has its own CUDA-event timing)
            line["n1m_forward"] = sub_n1m_forward(fp32_flops)
            line["n1m_forward_fixed_source"] = sub_n1m_forward(fp32_flops, "fixed")
            line["adjoint_n16384"] = sub_adjoint()
            line["batched_512"] = sub_batched()
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(pos, vel)
        print(json.dumps(line), flush=True)
    sysm.close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# extension workloads
# ---------------------------------------------------------------------------
def _body_rel(got, want):
    d = np.linalg.norm(np.asarray(got, np.float64) - want, axis=1)
    w = np.linalg.norm(want, axis=1)
    return d / np.maximum(w, 1e-300)


def run_precision(args):
    import torch

    import oracle
    from utc_gb300 import ics
    from utc_gb300.nbody import NBodySystem, probe_fma_peak

    n = args.n or 1048576
    steps = args.steps if args.steps_given else 20
    eps2, dt = 1e-4, 1e-4
    p64, v64 = ics.plummer(n, seed=0)
    tidx = np.sort(np.random.default_rng(7).choice(n, min(4096, n), replace=False)).astype(np.int32)
    out = {"workload": "precision", "n": n, "steps": steps, "eps2": eps2, "dt": dt,
           "subsample": int(tidx.size), "modes": {}}
    # mode: (precision, algorithm); "fast" = directed kernels, "sym" = each
    # unordered pair once
    modes = {"f32": ("f32", "fast"), "f32sym": ("f32", "sym"), "f32comp": ("f32comp", "fast"),
             "f32comp_sym": ("f32comp", "sym")}
    final_pos = {}
    for mode, (prec, algo) in modes.items():
        sysm = NBodySystem(n, prec, algo, kick="physical", eps2=np.float32(eps2), damping=1.0,
                           dt=np.float32(dt))
        if prec == "f32":
            sysm.set_state(ics.f32(p64), ics.f32(v64))
        else:
            sysm.set_state(p64, v64)
        per_step = []
        force_ms = 0.0
        E0 = None
        for t in range(steps + 1):
            e, bodies = sysm.energy(with_bodies=True)
            if algo == "sym":
                # the energy pass uses the directed kernel; take this mode's
                # own accelerations for the force error
                bodies = np.array(bodies, dtype=np.float64)
                bodies[:, :3] = np.asarray(sysm.accel(), np.float64)[:, :3]
            pos, vel = sysm.get_state()
            # FP64 forces at the state the GPU holds (float positions in plain
            # mode, FP64 absolute positions in the compensated mode)
            ref_a, ref_phi = oracle.accel_phi_subset_f64(np.asarray(pos, np.float64), tidx, eps2)
            fa = _body_rel(bodies[tidx, :3], ref_a)
            fp = np.abs(bodies[tidx, 3].astype(np.float64) - ref_phi) / np.abs(ref_phi)
            E = e[0] + e[1]
            E0 = E if E0 is None else E0
            per_step.append({"t": t, "force_rel_median": float(np.median(fa)),
                             "force_rel_p99": float(np.quantile(fa, 0.99)),
                             "force_rel_max": float(fa.max()),
                             "phi_rel_max": float(fp.max()),
                             "energy": float(E), "energy_drift": float((E - E0) / abs(E0))})
            if t < steps:
                f, g = sysm.step_timed(1)
                force_ms += f
        final_pos[mode] = np.asarray(pos, np.float64)[:, :3]
        rate = float(n) ** 2 * steps / (force_ms * 1e-3) / 1e9
        out["modes"][mode] = {
            "force_kernel_G_interactions_per_s": rate,
            "force_rel_max_over_steps": max(r["force_rel_max"] for r in per_step),
            "force_rel_median_over_steps": float(np.median([r["force_rel_median"] for r in per_step])),
            "phi_rel_max_over_steps": max(r["phi_rel_max"] for r in per_step),
            "energy_drift_final": per_step[-1]["energy_drift"],
            "per_step": per_step,
        }
        sysm.close()
    # final positions against the compensated symmetric run (FP64 positions,
    # forces within 1.7e-6 of FP64): |dx| / (|x| + 0.1), max over bodies
    ref = final_pos["f32comp_sym"]
    scale = np.linalg.norm(ref, axis=1) + 0.1
    for mode in modes:
        out["modes"][mode]["pos_rel_max_vs_compensated_symmetric"] = float(
            (np.linalg.norm(final_pos[mode] - ref, axis=1) / scale).max())
    peak, _ = probe_fma_peak(20000, True)
    out["forward_N1M"] = {}
    for mode in modes:
        r = out["modes"][mode]["force_kernel_G_interactions_per_s"]
        out["forward_N1M"][mode] = {"G_interactions_per_s": r, "tflops_20flop": r * 20 / 1e3,
                                    "frac_of_fp32_peak": r * 20e9 / peak}
    out["fp32_peak_tflops_probe"] = peak / 1e12
    print(json.dumps(out), flush=True)
    return 0


# FP32 pipe instructions per unordered pair of the float-float kernel (and
# one rsqrt approximation): exact grid differences 30, |r|^2 + eps2 39,
# Newton and Halley steps 18, inv^3 11, weights 8, six float-float
# accumulations 90
FF_OPS_PER_PAIR = 196


def run_double(args):
    import oracle
    from utc_gb300 import ics
    from utc_gb300.nbody import NBodySystem, probe_fma_peak

    n = args.n or 16384
    steps = args.steps if args.steps_given else 10
    eps2, dt = 1e-4, 1e-4
    p64, v64 = ics.plummer(n, seed=3)
    tidx = np.sort(np.random.default_rng(11).choice(n, min(512, n), replace=False)).astype(np.int32)
    ref_a = oracle.accel_subset_f64(p64, tidx, eps2)
    out = {"workload": "double", "n": n, "steps": steps, "eps2": eps2, "dt": dt, "kick": "reference",
           "data": "synthetic (seeded Plummer sphere, float64)", "modes": {}}
    final = {}
    for algo in ("sym", "sym64", "exact"):
        with NBodySystem(n, "f64", algo, kick="reference", eps2=eps2, damping=1.0, dt=dt) as s:
            s.set_state(p64, v64)
            a = s.accel()
            s.step(2)  # warm-up
            s.set_state(p64, v64)
            f, g = s.step_timed(steps)
            final[algo] = s.get_state()[0]
            info = s.plan_info() if algo != "exact" else None
        rate = float(n) ** 2 * steps / ((f + g) * 1e-3) / 1e9
        fe = _body_rel(a[tidx], ref_a)
        out["modes"][algo] = {"G_interactions_per_s": rate, "force_ms_per_step": f / steps,
                              "integrate_ms_per_step": g / steps,
                              "force_rel_max_vs_fp64_oracle": float(fe.max()),
                              "force_rel_median_vs_fp64_oracle": float(np.median(fe)), "plan": info}
    ex = final["exact"][:, :3]
    scale = np.linalg.norm(ex, axis=1) + 0.1
    for algo in ("sym", "sym64"):
        out["modes"][algo]["pos_rel_max_vs_exact"] = float(
            (np.linalg.norm(final[algo][:, :3] - ex, axis=1) / scale).max())
    out["modes"]["sym"]["kernel"] = "symff_force_kernel (float-float on the FP32 pipe)"
    out["modes"]["sym64"]["kernel"] = "sym64_force_kernel (FP64 pipe)"
    out["modes"]["exact"]["kernel"] = "exact_step_kernel<double> (reference operation order)"
    peak32, _ = probe_fma_peak(20000, True)
    peak64, _ = probe_fma_peak(2000, packed=2)
    ms = out["modes"]["sym"]["force_ms_per_step"]
    # unordered pairs across row blocks, ordered pairs inside each row block
    rb = out["modes"]["sym"]["plan"]["tbsize"]  # the row block
    pairs = float(n) * n / 2 + float(n) * rb / 2
    out["roofline"] = {"kernel": "symff_force_kernel", "bound": "fp32",
                       "achieved": pairs * FF_OPS_PER_PAIR / (ms * 1e-3) / 1e12,
                       "peak": peak32 / 2 / 1e12, "unit": "T FP32 instructions/s",
                       "frac": pairs * FF_OPS_PER_PAIR / (ms * 1e-3) / (peak32 / 2),
                       "ops_per_pair": FF_OPS_PER_PAIR,
                       "note": "force ms per step includes the scale reduction and split kernels; peak = "
                               "FP32 FMA probe rate in instructions (FLOP/2)"}
    out["fp64_dfma_peak_tflops_probe"] = peak64 / 1e12
    out["speedup_sym_vs_sym64"] = out["modes"]["sym"]["G_interactions_per_s"] / out["modes"]["sym64"][
        "G_interactions_per_s"]
    print(json.dumps(out), flush=True)
    return 0


def run_adjoint(args):
    import torch

    import oracle
    from utc_gb300 import ics
    from utc_gb300.nbody import NBodySystem

    n = args.n or 16384
    T, K = 200, 20
    eps2, dt = np.float32(1e-2), np.float32(1e-3)
    p64, v64 = ics.uniform_cube(n, seed=0)
    y = ics.gaussian_targets(n, seed=1, sigma=0.5)
    p32, v32 = ics.f32(p64), ics.f32(v64)
    yt = torch.tensor(y, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    def measure(algo):
        """Median times of the plain forward, the checkpointed forward and the
        backward (recompute + VJP) with one algorithm's kernels."""
        sysm = NBodySystem(n, "f32", algo, kick="physical", eps2=eps2, damping=1.0, dt=dt)
        pT = torch.empty((n, 4), device="cuda")
        vT = torch.empty((n, 4), device="cuda")
        for _ in range(args.warmup):
            sysm.set_state(p32, v32)
            sysm.adj_forward(T, K)
            sysm.get_state_device(pT, vT)
            sysm.adj_backward(torch.zeros((n, 4), device="cuda"))
        torch.cuda.synchronize()
        ts = {"forward": [], "adj_forward": [], "adj_backward": []}
        res = {}
        for _ in range(max(args.steps, 3)):
            sysm.set_state(p32, v32)
            ts["forward"].append(timed(lambda: sysm.step(T)))
            sysm.set_state(p32, v32)
            ts["adj_forward"].append(timed(lambda: sysm.adj_forward(T, K)))
            sysm.get_state_device(pT, vT)
            gx = torch.zeros((n, 4), device="cuda")
            gx[:, :3] = 2.0 * (pT[:, :3] - yt)
            ts["adj_backward"].append(timed(lambda: res.update(g=sysm.adj_backward(gx))))
        sysm.close()
        med = {k: float(np.median(v)) for k, v in ts.items()}
        return med, [t.cpu().numpy() for t in res["g"]]

    algo = args.algo
    other = "fast" if algo == "sym" else "sym"
    med, (gx0, gv0, gm) = measure(algo)
    med_o, g_o = measure(other)
    out = {"workload": "adjoint", "n": n, "steps": T, "ckpt_every": K, "eps2": float(eps2),
           "dt": float(dt), "kick": "physical (G=1)", "algo": algo, "ms_median": med,
           "adjoint_over_forward": med["adj_backward"] / med["forward"],
           "adjoint_incl_ckpt_forward_over_forward": (med["adj_backward"] + med["adj_forward"]) / med["forward"],
           "other_algo": {"algo": other, "ms_median": med_o,
                          "adjoint_over_forward": med_o["adj_backward"] / med_o["forward"],
                          "adjoint_over_default_forward": med_o["adj_backward"] / med["forward"]}}
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        L, rx, rv, rm = oracle.adjoint(p32.astype(np.float64), v32.astype(np.float64), y, float(eps2),
                                       1.0, float(dt), T, kick_mode=oracle.KICK_PHYSICAL)
        def rel(a, b):
            return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))
        out["vs_fp64_reference_adjoint"] = {"dx0": rel(gx0[:, :3], rx), "dv0": rel(gv0[:, :3], rv),
                                            "dm": rel(gm, rm), "cpu_s": time.perf_counter() - t0}
        out["other_algo"]["vs_fp64_reference_adjoint"] = {"dx0": rel(g_o[0][:, :3], rx),
                                                          "dv0": rel(g_o[1][:, :3], rv), "dm": rel(g_o[2], rm)}
        # FP64 central differences on 64 coordinates, on an N=2048 replica
        nf = 2048
        pf, vf = ics.uniform_cube(nf, seed=3)
        yf = ics.gaussian_targets(nf, seed=4, sigma=0.5)
        pf32, vf32 = ics.f32(pf), ics.f32(vf)
        with NBodySystem(nf, "f32", algo, kick="physical", eps2=eps2, damping=1.0, dt=dt) as s2:
            s2.set_state(pf32, vf32)
            s2.adj_forward(T, K)
            q, _ = s2.get_state()
            g2 = torch.zeros((nf, 4), device="cuda")
            g2[:, :3] = torch.tensor(2.0 * (q[:, :3].astype(np.float64) - yf), dtype=torch.float32, device="cuda")
            ax, av, am = [t.cpu().numpy() for t in s2.adj_backward(g2)]
        rng = np.random.default_rng(5)
        base_p, base_v = pf32.astype(np.float64), vf32.astype(np.float64)
        errs, h = [], 1e-6
        for _ in range(64):
            which, i, d = int(rng.integers(0, 3)), int(rng.integers(0, nf)), int(rng.integers(0, 3))
            arr_p, arr_v = base_p.copy(), base_v.copy()
            arr, col = {0: (arr_p, d), 1: (arr_v, d), 2: (arr_p, 3)}[which]
            arr[i, col] += h
            lp = oracle.loss(arr_p, arr_v, yf, float(eps2), 1.0, float(dt), T)
            arr[i, col] -= 2 * h
            lm = oracle.loss(arr_p, arr_v, yf, float(eps2), 1.0, float(dt), T)
            fd = (lp - lm) / (2 * h)
            an = {0: ax[i, d], 1: av[i, d], 2: am[i]}[which]
            errs.append(abs(an - fd) / max(abs(fd), 1e-12))
        out["vs_fp64_central_differences"] = {"n": nf, "coords": 64, "h": h,
                                              "rel_err_median": float(np.median(errs)),
                                              "rel_err_max": float(np.max(errs))}
    print(json.dumps(out), flush=True)
    return 0


def run_batched(args):
    import torch

    from utc_gb300 import ics
    from utc_gb300.nbody import NBodyBatch

    sizes = ics.batch_sizes(512, lo=128, hi=16384, seed=0)
    steps = 50
    ps, vs = [], []
    for k, nn in enumerate(sizes):
        p, v = ics.plummer(int(nn), seed=1000 + k)
        ps.append(p)
        vs.append(v)
    pos64, vel64 = np.concatenate(ps), np.concatenate(vs)
    pos, vel = ics.f32(pos64), ics.f32(vel64)
    pairs = float(np.sum(sizes.astype(np.float64) ** 2))
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    cache = os.path.join(REPO, "_build", "batch_autotune.txt")
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    out = {"workload": "batched", "systems": int(sizes.size), "bodies": int(sizes.sum()),
           "n_min": int(sizes.min()), "n_max": int(sizes.max()), "interactions_per_step": pairs,
           "steps": steps, "eps2": 1e-3, "dt": 1e-3}
    out["algo"] = args.algo
    other = "fast" if args.algo == "sym" else "sym"

    def graph_and_per_system(algo):
        """Graph time and per-system time with the other algorithm's kernels."""
        with torch.cuda.stream(stream), NBodyBatch(sizes, kick="physical", eps2=np.float32(1e-3),
                                                   dt=np.float32(1e-3), algo=algo) as b:
            b.set_state(pos, vel, stream=sh)
            tune = b.autotune(reps=2, cache_path=cache, stream=sh)
            res = {}
            for name, fn in (("graph", lambda: b.run(steps, sh)),
                             ("per_system", lambda: b.step_per_system(steps, sh))):
                b.set_state(pos, vel, stream=sh)
                fn()  # warm-up
                b.set_state(pos, vel, stream=sh)
                stream.synchronize()
                a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                c.record(stream)
                c.synchronize()
                res[name] = a.elapsed_time(c)
            return {"algo": algo, "autotune": tune, "ms_batched_graph": res["graph"],
                    "ms_per_system_launches": res["per_system"],
                    "speedup_vs_per_system": res["per_system"] / res["graph"],
                    "G_interactions_per_s_batched": pairs * steps / (res["graph"] * 1e-3) / 1e9}

    with torch.cuda.stream(stream), NBodyBatch(sizes, kick="physical", eps2=np.float32(1e-3),
                                               dt=np.float32(1e-3), algo=args.algo) as b:
        b.set_state(pos, vel, stream=sh)
        out["autotune"] = b.autotune(reps=2, cache_path=cache, stream=sh)
        out["plan"] = b.plan_info()

        def timed(fn, reps):
            ts = []
            for _ in range(reps):
                b.set_state(pos, vel, stream=sh)
                stream.synchronize()
                a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                c.record(stream)
                c.synchronize()
                ts.append(a.elapsed_time(c))
            return float(np.median(ts))

        t_graph = timed(lambda: b.run(steps, sh), 1 + max(args.steps, 3))
        pb, _ = b.get_state(stream=sh)
        t_launch = timed(lambda: b.step(steps, sh), 3)
        t_base = timed(lambda: b.step_per_system(steps, sh), 2)
        pr, _ = b.get_state(stream=sh)
        ntasks = min(16, os.cpu_count() or 1)
        b.set_state(pos, vel, stream=sh)
        stream.synchronize()
        t0 = time.perf_counter()
        b.step_tasks(steps, ntasks)
        t_tasks = (time.perf_counter() - t0) * 1e3
        pt, _ = b.get_state(stream=sh)
        # batched adjoint: checkpointed forward (every 10 steps) and the
        # reverse pass for all systems, against the plain batched forward
        gx = torch.randn((b.nbody, 4), device="cuda", generator=torch.Generator("cuda").manual_seed(3)) * 1e-3
        adj = {"forward_ckpt": [], "backward": []}
        for _ in range(2):
            b.set_state(pos, vel, stream=sh)
            stream.synchronize()
            for name, fn in (("forward_ckpt", lambda: b.adj_forward(steps, 10, stream=sh)),
                             ("backward", lambda: b.adj_backward(gx, stream=sh))):
                a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                c.record(stream)
                c.synchronize()
                adj[name].append(a.elapsed_time(c))
        t_adjf, t_adjb = min(adj["forward_ckpt"]), min(adj["backward"])
    d = np.linalg.norm(pb[:, :3].astype(np.float64) - pr[:, :3], axis=1)
    w = np.linalg.norm(pr[:, :3].astype(np.float64), axis=1)
    out.update({
        "ms_batched_graph": t_graph, "ms_batched_launches": t_launch, "ms_per_system_launches": t_base,
        "speedup_vs_per_system": t_base / t_graph,
        "ms_per_system_tasks": t_tasks, "tasks": ntasks,
        "speedup_vs_per_system_tasks": t_tasks / t_graph,
        "tasks_note": "reference multi-task pattern: one host thread + stream per task, "
                      "stream synchronise after every system step (nbody_mtask.cc, body_task_sgpu.cu)",
        "G_interactions_per_s_batched": pairs * steps / (t_graph * 1e-3) / 1e9,
        "G_interactions_per_s_per_system": pairs * steps / (t_base * 1e-3) / 1e9,
        "final_pos_rel_diff_max_vs_per_system": float((d / (w + 0.1)).max()),
        "tasks_equal_per_system_bitwise": bool(pt.tobytes() == pr.tobytes()),
        "adjoint": {"ckpt_every": 10, "ms_forward_ckpt": t_adjf, "ms_backward": t_adjb,
                    "backward_over_forward": t_adjb / t_launch,
                    "note": "reverse pass over all systems (recompute + VJP) vs the batched forward "
                            "launched step by step"},
    })
    out["other_algo"] = graph_and_per_system(other)

    # FP64 state (the reference multi-task app's FTYPE double): the
    # float-float batched kernel against per-system float-float launches and
    # the reference's task pattern, same systems, 10 steps
    f64_steps = 10
    with torch.cuda.stream(stream), NBodyBatch(sizes, kick="physical", eps2=1e-3, dt=1e-3,
                                               precision="f64") as b:
        b.set_state(pos64, vel64, stream=sh)
        tune64 = b.autotune(reps=1, cache_path=cache, stream=sh)
        res = {}
        for name, fn in (("graph", lambda: b.run(f64_steps, sh)),
                         ("per_system", lambda: b.step_per_system(f64_steps, sh))):
            b.set_state(pos64, vel64, stream=sh)
            fn()  # warm-up
            b.set_state(pos64, vel64, stream=sh)
            stream.synchronize()
            a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            c.record(stream)
            c.synchronize()
            res[name] = a.elapsed_time(c)
        b.set_state(pos64, vel64, stream=sh)
        stream.synchronize()
        t0 = time.perf_counter()
        b.step_tasks(f64_steps, ntasks)
        res["tasks"] = (time.perf_counter() - t0) * 1e3
    out["f64"] = {"steps": f64_steps, "kernel": "bksff_force_kernel (float-float, FP64 state)",
                  "autotune": tune64, "ms_batched_graph": res["graph"],
                  "ms_per_system_launches": res["per_system"], "ms_per_system_tasks": res["tasks"],
                  "speedup_vs_per_system": res["per_system"] / res["graph"],
                  "speedup_vs_per_system_tasks": res["tasks"] / res["graph"],
                  "G_interactions_per_s_batched": pairs * f64_steps / (res["graph"] * 1e-3) / 1e9}
    out["speedup_vs_other_algo_per_system"] = out["other_algo"]["ms_per_system_launches"] / t_graph
    print(json.dumps(out), flush=True)
    return 0


def run_sharded(args):
    """One system split over the ranks (the target partition: directed
    shards, one all-gather of positions per step, `utc_gb300/shard.py`):
    N=1,048,576 Plummer, eps2 = dt = 1e-4, 10 leapfrog steps per bench step,
    timed across ranks (barrier, max over ranks).  Strong scaling: the total
    work is fixed as ranks are added.  On one GPU the exchange is empty."""
    import torch
    import torch.distributed as dist

    from utc_gb300 import ics
    from utc_gb300.shard import ShardedNBodySystem

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    os.environ.setdefault("NCCL_NVLS_ENABLE", "0")
    if not dist.is_initialized():
        if world > 1:
            dist.init_process_group("nccl", device_id=dev)
        else:
            dist.init_process_group("nccl", init_method="tcp://127.0.0.1:29561", rank=0, world_size=1)
    n = args.n or (1 << 20)
    leap = 10
    p, v = ics.plummer(n, seed=0)
    p32, v32 = ics.f32(p), ics.f32(v)
    with ShardedNBodySystem(n, "f32", "fast", kick="physical", eps2=float(np.float32(EPS2)), damping=1.0,
                            dt=float(np.float32(DT))) as s:
        for _ in range(args.warmup):
            s.set_state(p32, v32)
            s.step(leap)
        torch.cuda.synchronize()
        dist.barrier()
        stream = torch.cuda.current_stream()
        ms = 0.0
        for _ in range(args.steps):
            s.set_state(p32, v32)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.step(leap)
            b.record(stream)
            b.synchronize()
            ms += a.elapsed_time(b)
        dist.barrier()
        ms_max = max_over_ranks(ms, world, dev)
        counts = [c for _, c in s.ranges]
    val = float(n) ** 2 * leap * args.steps / (ms_max * 1e-3) / 1e9
    if rank == 0:
        print(json.dumps({"workload": "sharded", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
                          "n": n, "leapfrog_steps_per_bench_step": leap, "steps": args.steps,
                          "ms_per_step": ms_max / args.steps, "scaling": "strong",
                          "bodies_per_rank": counts, "kernel": "sk_force_kernel shards + all-gather"}),
              flush=True)
    dist.destroy_process_group()
    return 0


def run_frames(args):
    """Frame copy-out (body_task_sgpu.cu:116-125): nb_run_host with a frame
    every `oi` steps, pageable and pinned host memory, against the same run
    with one frame at the end.  Each frame is a device snapshot copied to the
    host on a second stream while the next steps run."""
    from utc_gb300 import _native as N
    from utc_gb300 import ics
    from utc_gb300.nbody import NBodySystem

    n = args.n or 65536
    loops = 200
    p, v = ics.plummer(n, seed=0)
    pos, vel = ics.f32(p), ics.f32(v)
    frame_bytes = n * 16
    out = {"workload": "frames", "n": n, "loops": loops, "algo": "sym", "eps2": 1e-4, "dt": 1e-4,
           "data": "synthetic (seeded Plummer sphere, float32)", "runs": []}
    for mname, mt in (("pageable", N.NB_MEM_PAGEABLE), ("pinned", N.NB_MEM_PINNED)):
        with NBodySystem(n, "f32", "sym", kick="physical", eps2=np.float32(1e-4), damping=1.0,
                         dt=np.float32(1e-4), memtype=mt) as s:
            s.run_host(pos, vel, 20, 20)  # warm-up: graphs, staging, snapshots
            base = None
            for oi in (loops, 20, 5, 1):
                reps = []
                for _ in range(3):
                    t0 = time.perf_counter()
                    frames, t = s.run_host(pos, vel, loops, oi)
                    reps.append(time.perf_counter() - t0)
                wall = statistics.median(reps)
                if oi == loops:
                    base = wall
                k = loops // oi
                out["runs"].append({"memtype": mname, "out_interval": oi, "frames": k, "wall_ms": wall * 1e3,
                                    "G_interactions_per_s": float(n) ** 2 * loops / wall / 1e9,
                                    "frame_GB_per_s": k * frame_bytes / wall / 1e9,
                                    "slowdown_vs_one_frame": wall / base})
    out["note"] = ("wall clock of nb_run_host from host arrays (state in, frames out); slowdown_vs_one_frame "
                   "near 1 means the copies hide behind the steps")
    print(json.dumps(out))
    return 0


def run_ics(args):
    """Initial conditions drawn on the GPU (nb_ics_generate, randomizeBodies at
    nbody.h:89-250 for large inputs): bodies per second and the store rate
    against the measured HBM copy bandwidth, beside the host generator
    (numpy, FP64) on the same sizes."""
    import torch

    from utc_gb300 import ics
    from utc_gb300.nbody import gpu_initial_conditions

    peaks = measured_peaks()
    out = {"workload": "ics", "data": "synthetic (seeded counter-based draws)", "runs": []}
    for n in (1 << 20, 1 << 24):
        for kind in ("cube", "plummer", "shell"):
            gpu_initial_conditions(kind, n, seed=1)  # warm-up, allocator
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 5
            e0.record()
            for r in range(reps):
                gpu_initial_conditions(kind, n, seed=2 + r)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            stored = 32.0 * n  # pos and vel, float4 each
            run = {"kind": kind, "n": n, "ms": ms, "G_bodies_per_s": n / ms / 1e6,
                   "store_GB_per_s": stored / ms / 1e6,
                   "hbm_frac": (stored / ms / 1e6) / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None}
            if n == 1 << 20 and kind in ("cube", "plummer"):
                t0 = time.perf_counter()
                (ics.uniform_cube if kind == "cube" else ics.plummer)(n, seed=2)
                run["host_numpy_ms"] = (time.perf_counter() - t0) * 1e3
            out["runs"].append(run)
    out["note"] = ("ms per call by CUDA events over 5 calls (each call also allocates its outputs from "
                   "torch's cache); plummer and shell add an FP64 recentering reduction")
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the N=1M, adjoint and batched sub-records of the default line")
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "precision", "adjoint", "batched", "double", "frames", "ics", "sharded"])
    ap.add_argument("--algo", default="sym", choices=["fast", "sym"],
                    help="force algorithm (plain, adjoint and batched workloads)")
    ap.add_argument("--n", type=int, default=0, help="body count override for extension workloads")
    args = ap.parse_args()
    args.steps_given = "--steps" in sys.argv
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "double":
        return run_double(args)
    if args.workload == "frames":
        return run_frames(args)
    if args.workload == "ics":
        return run_ics(args)
    if args.workload == "sharded":
        return run_sharded(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
