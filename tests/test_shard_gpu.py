"""Shard contexts of the target partition (nb_create_shard) on one GPU.

The shards of a partition run here as contexts of one process on one GPU,
stepped one after the other with the positions exchanged between steps by
device copies (no kernel waits on another).  Their states put together
equal a single-GPU context's bit for bit: the directed kernel's shards
against an NB_ALGO_FAST context, the reference-exact shards (float and
double) against the oracle.  ShardedNBodySystem, the torch.distributed host
side, runs on a one-rank NCCL group against the single-GPU context; its
exchange with more ranks is covered on CPU (tests/test_shard.py).
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from utc_gb300 import _native as N
from utc_gb300 import ics
from utc_gb300.nbody import NBodySystem, current_stream_handle
from utc_gb300.shard import ShardedNBodySystem, _DeviceRows, block_split, reference_split

pytestmark = pytest.mark.gpu


class Shard:
    def __init__(self, n, rank, nranks, precision, algo, **kw):
        self.lib = N.lib()
        p = N.NbParams()
        self.lib.nb_params_default(C.byref(p))
        p.n, p.precision = n, {"f32": N.NB_F32, "f64": N.NB_F64}[precision]
        p.algo = {"fast": N.NB_ALGO_FAST, "exact": N.NB_ALGO_EXACT}[algo]
        p.kick = N.NB_KICK_PHYSICAL if kw.get("kick") == "physical" else N.NB_KICK_REFERENCE
        p.eps2, p.damping, p.dt = kw["eps2"], kw["damping"], kw["dt"]
        self.h = C.c_void_p()
        N.check(self.lib.nb_create_shard(C.byref(p), rank, nranks, C.byref(self.h)), "nb_create_shard")
        info = (C.c_int * 4)()
        N.check(self.lib.nb_shard_info(self.h, info), "nb_shard_info")
        self.first, self.count = info[0], info[1]
        assert (info[2], info[3]) == (rank, nranks)
        self.n = n
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.typestr = "<f8" if precision == "f64" else "<f4"

    def rows(self, which):
        import torch

        pos, vel = C.c_void_p(), C.c_void_p()
        N.check(self.lib.nb_state_ptrs(self.h, C.byref(pos), C.byref(vel)), "nb_state_ptrs")
        return torch.as_tensor(_DeviceRows(pos.value if which == "pos" else vel.value, self.n, self.typestr),
                               device="cuda")

    def close(self):
        N.check(self.lib.nb_destroy(self.h), "nb_destroy")


def run_shards(n, nranks, steps, precision, algo, pos, vel, **kw):
    import torch

    shards = [Shard(n, r, nranks, precision, algo, **kw) for r in range(nranks)]
    s = C.c_void_p(current_stream_handle())
    try:
        for sh in shards:
            N.check(sh.lib.nb_set_state(sh.h, pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p),
                                        N.NB_HOST, s), "nb_set_state")
        for _ in range(steps):
            for sh in shards:
                N.check(sh.lib.nb_step(sh.h, 1, s), "nb_step")
            views = [sh.rows("pos") for sh in shards]
            for a, sa in zip(views, shards):
                for b, sb in zip(views, shards):
                    if sb is not sa and sb.count:
                        a[sb.first:sb.first + sb.count].copy_(b[sb.first:sb.first + sb.count])
        torch.cuda.synchronize()
        got_p = shards[0].rows("pos").cpu().numpy()
        got_v = np.empty_like(got_p)
        for sh in shards:
            got_v[sh.first:sh.first + sh.count] = sh.rows("vel").cpu().numpy()[sh.first:sh.first + sh.count]
        for sh in shards[1:]:
            assert sh.rows("pos").cpu().numpy().tobytes() == got_p.tobytes()
        return got_p, got_v, [(sh.first, sh.count) for sh in shards]
    finally:
        for sh in shards:
            sh.close()


@pytest.mark.parametrize("n", [1000, 65536, 100003])
@pytest.mark.parametrize("nranks", [2, 3])
def test_fast_shards_equal_the_single_gpu_run(cuda, n, nranks):
    p64, v64 = ics.plummer(n, seed=n)
    pos, vel = ics.f32(p64), ics.f32(v64)
    kw = dict(kick="physical", eps2=float(np.float32(1e-4)), damping=1.0, dt=float(np.float32(1e-4)))
    got_p, got_v, ranges = run_shards(n, nranks, 3, "f32", "fast", pos, vel, **kw)
    with NBodySystem(n, "f32", "fast", **kw) as s:
        tb = s.plan_info()["tbsize"]
        s.set_state(pos, vel)
        s.step(3)
        want_p, want_v = s.get_state()
    assert ranges == block_split(n, tb, nranks)
    assert got_p.tobytes() == want_p.tobytes()
    assert got_v.tobytes() == want_v.tobytes()


@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("n,nranks", [(1024, 2), (1001, 3)])
def test_exact_shards_equal_the_oracle(cuda, precision, n, nranks):
    dtype = np.float64 if precision == "f64" else np.float32
    pos, vel = oracle.randomize(1, n, dtype)
    eps2, damping, dt = dtype(0.01), dtype(0.999), dtype(0.016)
    got_p, got_v, ranges = run_shards(n, nranks, 4, precision, "exact", pos, vel, eps2=float(eps2),
                                      damping=float(damping), dt=float(dt))
    assert ranges == reference_split(n, nranks)
    want_p, want_v = oracle.step(pos, vel, eps2, damping, dt, 4)
    assert got_p.tobytes() == want_p.tobytes()
    assert got_v.tobytes() == want_v.tobytes()


@pytest.mark.parametrize("algo,precision", [("fast", "f32"), ("exact", "f32"), ("exact", "f64")])
@pytest.mark.parametrize("n,nranks", [(2, 3), (1, 2), (5, 8)])
def test_more_shards_than_bodies(cuda, algo, precision, n, nranks):
    """Shards left without targets step nothing and still take part in the
    exchange; the partition equals the single run bit for bit."""
    dtype = np.float64 if precision == "f64" else np.float32
    p, v = ics.plummer(n, seed=31 + n)
    pos, vel = p.astype(dtype), v.astype(dtype)
    kw = dict(kick="physical", eps2=float(dtype(1e-2)), damping=1.0, dt=float(dtype(1e-3)))
    got_p, got_v, ranges = run_shards(n, nranks, 3, precision, algo, pos, vel, **kw)
    assert sum(c for _, c in ranges) == n and any(c == 0 for _, c in ranges)
    with NBodySystem(n, precision, algo, **kw) as s:
        s.set_state(pos, vel)
        s.step(3)
        want_p, want_v = s.get_state()
    assert got_p.tobytes() == want_p.tobytes() and got_v.tobytes() == want_v.tobytes()


def test_shard_refusals(cuda):
    lib = N.lib()
    p = N.NbParams()
    lib.nb_params_default(C.byref(p))
    p.n, p.algo = 4096, N.NB_ALGO_SYM
    h = C.c_void_p()
    assert lib.nb_create_shard(C.byref(p), 0, 2, C.byref(h)) == N.NB_ERR_UNSUPPORTED
    p.algo = N.NB_ALGO_FAST
    assert lib.nb_create_shard(C.byref(p), 2, 2, C.byref(h)) == N.NB_ERR_INVALID
    assert lib.nb_create_shard(C.byref(p), 1, 2, C.byref(h)) == N.NB_OK
    try:
        pos, vel = ics.uniform_cube(4096, seed=1)
        pos, vel = ics.f32(pos), ics.f32(vel)
        assert lib.nb_set_state(h, pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p),
                                N.NB_HOST, None) == N.NB_OK
        assert lib.nb_step(h, 2, None) == N.NB_ERR_INVALID
        assert lib.nb_step(h, 1, None) == N.NB_OK
        out5 = (C.c_double * 5)()
        assert lib.nb_energy(h, out5, None, None) == N.NB_ERR_UNSUPPORTED
        assert b"shard" in lib.nb_last_error()
    finally:
        lib.nb_destroy(h)


def test_sharded_system_on_a_one_rank_nccl_group(cuda):
    import torch.distributed as dist

    os.environ.setdefault("NCCL_NVLS_ENABLE", "0")
    n, steps = 20000, 4
    p64, v64 = ics.plummer(n, seed=9)
    pos, vel = ics.f32(p64), ics.f32(v64)
    kw = dict(kick="physical", eps2=float(np.float32(1e-4)), damping=1.0, dt=float(np.float32(1e-4)))
    dist.init_process_group("nccl", init_method="tcp://127.0.0.1:29551", rank=0, world_size=1)
    try:
        with ShardedNBodySystem(n, "f32", "fast", **kw) as s:
            assert (s.first, s.count) == (0, n)
            s.set_state(pos, vel)
            s.step(steps)
            got_p, got_v = s.get_state()
    finally:
        dist.destroy_process_group()
    with NBodySystem(n, "f32", "fast", **kw) as s:
        s.set_state(pos, vel)
        s.step(steps)
        want_p, want_v = s.get_state()
    assert got_p.tobytes() == want_p.tobytes() and got_v.tobytes() == want_v.tobytes()


APP = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "utc_gb300", "nbody_main")
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _app(*args, timeout=300):
    import subprocess

    r = subprocess.run([APP, *args], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("threads", [2, 3])
def test_mgpu_task_reproduces_the_golden_file(cuda, tmp_path, threads):
    """The multi-GPU drop-in task (Task<BodySystemMGPU_GB300<float>> with
    `threads` threads, here all on the one GPU, reference-exact shards with
    the reference's split) writes the reference's golden output file byte
    for byte, like the one-thread task."""
    import hashlib
    import json

    kat = json.load(open(os.path.join(GOLD, "kat_shell_n1024.json")))
    out = tmp_path / "outpos.txt"
    _app("-t", str(threads), "-F", "-a", "1", "-n", "1024", "-i", "0", "-l", "100", "-o", "100", "-O", str(out))
    assert hashlib.sha256(out.read_bytes()).hexdigest() == kat["seq_outpos_sha256"]


@pytest.mark.parametrize("flags", [["-F", "-a", "0"], ["-a", "1"], []])
def test_mgpu_task_frames_equal_the_single_gpu_task(cuda, tmp_path, flags):
    """Every frame of a 3-thread run equals the one-thread run of the same
    algorithm byte for byte: the directed kernel's block shards against the
    one-GPU directed kernel (float), the exact shards against the exact
    kernel (double, the app's default state type and the multi-GPU task's
    default algorithm)."""
    one, three = tmp_path / "one.txt", tmp_path / "three.txt"
    algo = flags if flags else ["-a", "1"]  # the one-thread task's default is the symmetric kernel
    common = ["-n", "5000", "-i", "2", "-l", "12", "-o", "4", "-v"]
    _app("-t", "1", *(flags or algo), *common, "-O", str(one))
    text = _app("-t", "3", *flags, *common, "-O", str(three))
    assert "kernel time" in text
    assert one.read_bytes() == three.read_bytes()
