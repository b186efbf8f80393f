"""Target partition of one N-body system across GPUs, one process per GPU.

The reference's multi-GPU task BodySystemMGPU<T> (benchapps/nbody/
utc-snode-mgpu/mgpu/body_task_mgpu.cu:14-163) gives each of its threads a
range of target bodies (body_task_mgpu.cu:41-49); every step each thread
copies all N positions to its GPU (:109), advances its own range (:113-146),
copies that range back to a shared host buffer (:151) and waits at a barrier
(:154).  Here each rank holds a shard context (nb_create_shard): all N
positions stay in its own HBM, each step updates only its targets, and the
ranks exchange the new positions with one all-gather per step (NCCL on
GPUs, any torch.distributed backend), instead of going through host memory.

Shards of the directed kernel (NB_F32, algo "fast") own whole target blocks
of the single-GPU plan, so the shards' results together equal a single-GPU
"fast" context's bit for bit; reference-exact shards (algo "exact", float or
double) split the bodies as the reference does.

ShardExchange is the exchange alone (ranges, padding, the collective); it
works on any (n, 4) tensor, so the host logic also runs on CPU tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .nbody import _ALGO, _KICK, _PREC, current_stream_handle


def reference_split(n, nranks):
    """[(first, count)] per rank: n // nranks bodies each, one more for the
    first n % nranks ranks (body_task_mgpu.cu:41-49)."""
    q, r = divmod(int(n), int(nranks))
    out = []
    for k in range(nranks):
        first = k * (q + 1) if k < r else k * q + r
        out.append((first, q + (1 if k < r else 0)))
    return out


def block_split(n, tbsize, nranks):
    """[(first, count)] per rank for whole target blocks of tbsize bodies:
    ntb // nranks blocks each, one more for the first ntb % nranks ranks
    (what nb_create_shard does for the directed kernel)."""
    ntb = (int(n) + tbsize - 1) // tbsize
    q, r = divmod(ntb, int(nranks))
    out = []
    for k in range(nranks):
        b0 = k * q + min(k, r)
        b1 = b0 + q + (1 if k < r else 0)
        lo, hi = min(b0 * tbsize, n), min(b1 * tbsize, n)
        out.append((lo, hi - lo))
    return out


class ShardExchange:
    """All-gather of every rank's range of an (n, 4) array, in place.

    Ranges may differ in length: each rank sends its range padded to the
    longest, one all_gather brings every padded range to every rank, and the
    ranks' rows are copied to where they belong."""

    def __init__(self, ranges, rank, group=None, dtype=None, device=None):
        import torch

        self.ranges = [(int(f), int(c)) for f, c in ranges]
        self.rank = int(rank)
        self.group = group
        self.cap = max(1, max(c for _, c in self.ranges))
        world = len(self.ranges)
        self.send = torch.zeros((self.cap, 4), dtype=dtype, device=device)
        self.recv = torch.zeros((world * self.cap, 4), dtype=dtype, device=device)
        self.parts = list(self.recv.split(self.cap))

    def all_gather(self, arr):
        """arr: (n, 4) tensor whose rows [first, first + count) of this rank
        are new; afterwards every rank's rows are."""
        import torch.distributed as dist

        f, c = self.ranges[self.rank]
        if c:
            self.send[:c].copy_(arr[f:f + c])
        dist.all_gather(self.parts, self.send, group=self.group)
        for r, (fr, cr) in enumerate(self.ranges):
            if r != self.rank and cr:
                arr[fr:fr + cr].copy_(self.parts[r][:cr])


class _DeviceRows:
    """A device buffer of (n, 4) values seen by torch without a copy."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n, 4), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2, "strides": None}


class ShardedNBodySystem:
    """This rank's shard of an N-body system partitioned over the ranks of
    `group` (torch.distributed, initialised by the caller; one GPU per rank,
    the current CUDA device).  Every rank loads the whole state; step()
    advances all ranks in lockstep, exchanging positions after each step."""

    def __init__(self, n, precision="f32", algo="fast", kick="reference", eps2=0.00125, damping=0.995,
                 dt=0.016, G=1.0, group=None):
        import torch
        import torch.distributed as dist

        self.lib = N.lib()
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        p = N.NbParams()
        self.lib.nb_params_default(C.byref(p))
        p.n, p.precision, p.algo, p.kick = int(n), _PREC[precision], _ALGO[algo], _KICK[kick]
        p.eps2, p.damping, p.dt, p.G = float(eps2), float(damping), float(dt), float(G)
        self.n = int(n)
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.tdtype = torch.float64 if precision == "f64" else torch.float32
        self.typestr = "<f8" if precision == "f64" else "<f4"
        h = C.c_void_p()
        N.check(self.lib.nb_create_shard(C.byref(p), self.rank, self.world, C.byref(h)), "nb_create_shard")
        self.handle = h
        info = (C.c_int * 4)()
        N.check(self.lib.nb_shard_info(h, info), "nb_shard_info")
        self.first, self.count = int(info[0]), int(info[1])
        mine = torch.tensor([self.first, self.count], dtype=torch.int64, device="cuda")
        every = [torch.zeros_like(mine) for _ in range(self.world)]
        dist.all_gather(every, mine, group=group)
        self.ranges = [(int(t[0]), int(t[1])) for t in every]
        self.exchange = ShardExchange(self.ranges, self.rank, group, self.tdtype, "cuda")

    def close(self):
        if getattr(self, "handle", None):
            N.check(self.lib.nb_destroy(self.handle), "nb_destroy")
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _rows(self, which):
        import torch

        pos, vel = C.c_void_p(), C.c_void_p()
        N.check(self.lib.nb_state_ptrs(self.handle, C.byref(pos), C.byref(vel)), "nb_state_ptrs")
        ptr = pos.value if which == "pos" else vel.value
        return torch.as_tensor(_DeviceRows(ptr, self.n, self.typestr), device="cuda")

    def set_state(self, pos, vel):
        """Every body's state, host arrays (n, 4), on every rank."""
        a = np.ascontiguousarray(pos, dtype=self.dtype).reshape(self.n, 4)
        b = np.ascontiguousarray(vel, dtype=self.dtype).reshape(self.n, 4)
        N.check(self.lib.nb_set_state(self.handle, a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                                      N.NB_HOST, C.c_void_p(current_stream_handle())), "nb_set_state")

    def step(self, steps=1):
        s = C.c_void_p(current_stream_handle())
        for _ in range(int(steps)):
            N.check(self.lib.nb_step(self.handle, 1, s), "nb_step")
            if self.world > 1 and self.n:
                self.exchange.all_gather(self._rows("pos"))

    def get_state(self):
        """(positions, velocities) of every body as host arrays; the
        velocities are gathered from their owners."""
        import torch

        pos = self._rows("pos").clone()
        vel = self._rows("vel").clone()
        if self.world > 1 and self.n:
            self.exchange.all_gather(vel)
        torch.cuda.current_stream().synchronize()
        return pos.cpu().numpy(), vel.cpu().numpy()
