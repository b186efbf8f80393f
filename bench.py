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


def committed_traffic():
    """Per-launch DRAM bytes of the top kernels from the committed ncu summary."""
    try:
        return json.load(open(os.path.join(REPO, "profiles", "traffic.json")))
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
# CPU baseline (oracle port of the reference's sequential BodySystem<float>)
# ---------------------------------------------------------------------------
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
                      f"BodySystem<float>, targets split across threads, bit-identical per body)"}


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
                                   f"oracle restatement; the compiled reference is x86-only here)"},
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

    sysm = NBodySystem(N_BODIES, "f32", "fast", kick="physical", eps2=EPS2, damping=1.0, dt=DT, G=1.0)
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

    t_max = torch.tensor([dev_ms], dtype=torch.float64, device=dev)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    dev_ms_max = float(t_max.item())
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
    e2e_t = torch.tensor([sum(e2e_times)], dtype=torch.float64, device=dev)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
    e2e_val = interactions / float(e2e_t.item()) / 1e9
    state_bytes = N_BODIES * 16

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
        integ_bytes = 80.0 * N_BODIES
        hbm = peaks.get("hbm_gbs")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Plummer sphere, float32)",
            "config": {"workload": WORKLOAD, "n": N_BODIES, "leapfrog_steps": LEAPFROG_STEPS,
                       "kick": "physical (G=1)", "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "flushed between timed steps (256 MB write outside the event pair)",
                       "plan": plan},
            "fp32_pipe_pct": 100.0 * achieved_tf / fp32_peak_tf,
            "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": fp32_peak_tf,
                         "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak_tf,
                         "traffic": traffic.get("force_bytes_per_launch"),
                         "kernel": "sk_force_kernel",
                         "flop_per_launch": force_flops,
                         "avg_launch_ms": force_avg_s * 1e3,
                         "peak_source": "packed-FMA probe measured in this run "
                                        "(MEASURED_PEAKS.json has no FP32 figure)",
                         "nominal_peak": nominal_tf},
            "roofline_integrator": {"bound": "hbm", "kernel": "sk_integrate_kernel",
                                    "achieved": integ_bytes / integ_avg_s / 1e9, "peak": hbm,
                                    "unit": "GB/s",
                                    "frac": (integ_bytes / integ_avg_s / 1e9) / hbm if hbm else None,
                                    "bytes_per_launch": integ_bytes,
                                    "avg_launch_ms": integ_avg_s * 1e3,
                                    "traffic": traffic.get("integrate_bytes_per_launch"),
                                    "note": "80 B/body algorithmic; at N=65536 the state is L2-resident"},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 2 * state_bytes,
                    "d2h_bytes_per_step": state_bytes,
                    "how": "nb_run_host (C ABI) from pinned host buffers, 100 leapfrog steps, "
                           "final positions read back, host wall clock"},
            "gpu_launches": launches * launches_per_leapfrog,
            "clocks": clk,
            "wall_s_timed_region": wall,
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(pos, vel)
        print(json.dumps(line), flush=True)
    sysm.close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
