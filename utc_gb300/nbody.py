"""Python face of the C ABI: an NBodySystem owning one nb_ctx.

State arrays are (n, 4): positions (x, y, z, m) and velocities
(vx, vy, vz, w), float32 for precision "f32" and float64 for "f64", the
layout of the reference's GpuData buffers (benchapps/nbody/utc/sgpu/
body_task_sgpu.cu:55-58).  numpy arrays are host buffers; torch CUDA tensors
are device buffers (used in place, no host round trip).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

_PREC = {"f32": N.NB_F32, "f64": N.NB_F64, "f32comp": N.NB_F32_COMP}
_ALGO = {"fast": N.NB_ALGO_FAST, "exact": N.NB_ALGO_EXACT, "sym": N.NB_ALGO_SYM, "sym64": N.NB_ALGO_SYM_FP64}
_KICK = {"reference": N.NB_KICK_REFERENCE, "physical": N.NB_KICK_PHYSICAL}


def _torch():
    import torch
    return torch


def current_stream_handle():
    """cudaStream_t of torch's current stream as an int (0 = legacy default)."""
    torch = _torch()
    if torch.cuda.is_available():
        return int(torch.cuda.current_stream().cuda_stream)
    return 0


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _device_buffer(x, shape, dtype, name):
    """x as a contiguous CUDA tensor of exactly `shape` and `dtype` (converted
    if only the dtype or the layout differ).  The C ABI copies whole buffers
    by the context's size: a tensor of another size would be read or written
    past its end, so that is refused here."""
    torch = _torch()
    if not _is_torch(x) or not x.is_cuda:
        raise ValueError(f"{name}: needs a CUDA tensor")
    if tuple(x.shape) != tuple(shape):
        raise ValueError(f"{name}: needs shape {tuple(shape)}, got {tuple(x.shape)}")
    return x.to(dtype).contiguous()


class NBodySystem:
    def __init__(self, n, precision="f32", algo="fast", kick="reference", eps2=0.00125,
                 damping=0.995, dt=0.016, G=1.0, block=0, bpt=0, ctas_per_sm=0,
                 memtype=N.NB_MEM_PAGEABLE, source_side="auto", bands=0):
        self.lib = N.lib()
        p = N.NbParams()
        self.lib.nb_params_default(C.byref(p))
        p.n = int(n)
        p.precision = _PREC[precision]
        p.algo = _ALGO[algo]
        p.kick = _KICK[kick]
        p.eps2, p.damping, p.dt, p.G = float(eps2), float(damping), float(dt), float(G)
        p.block, p.bpt, p.ctas_per_sm, p.memtype = int(block), int(bpt), int(ctas_per_sm), int(memtype)
        # symmetric FP32 kernel: "triangular" array or "fixed"-point accumulators
        p.source_side = {"auto": N.NB_SOURCE_AUTO, "triangular": N.NB_SOURCE_TRIANGULAR,
                         "fixed": N.NB_SOURCE_FIXED}[source_side]
        # symmetric kernels with the triangular array: 0 = bands only where it
        # would pass 8 GiB, k > 1 = k bands (at most as many as row blocks)
        p.bands = int(bands)
        self.params = p
        self.n = int(n)
        self.precision = precision
        # host-side state type: double4 for f64 and for the compensated mode
        self.dtype = np.float64 if precision in ("f64", "f32comp") else np.float32
        h = C.c_void_p()
        N.check(self.lib.nb_create(C.byref(p), C.byref(h)), "nb_create")
        self.handle = h

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "handle", None):
            # a refused destroy (another thread is capturing a graph) keeps the
            # context, and the handle with it, for a later close()
            N.check(self.lib.nb_destroy(self.handle), "nb_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def _torch_dtype(self):
        torch = _torch()
        return torch.float64 if self.dtype == np.float64 else torch.float32

    def _buf(self, x, name):
        if _is_torch(x):
            t = _device_buffer(x, (self.n, 4), self._torch_dtype(), name)
            return C.c_void_p(t.data_ptr()), N.NB_DEVICE, t
        a = np.ascontiguousarray(x, dtype=self.dtype).reshape(self.n, 4)
        return a.ctypes.data_as(C.c_void_p), N.NB_HOST, a

    def set_state(self, pos, vel, stream=None):
        pp, wp, keep_p = self._buf(pos, "pos")
        vp, wv, keep_v = self._buf(vel, "vel")
        if wp != wv:
            raise ValueError("pos and vel must both be host or both be device buffers")
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_set_state(self.handle, pp, vp, wp, C.c_void_p(s)), "nb_set_state")
        if wp == N.NB_DEVICE and (keep_p is not pos or keep_v is not vel):
            _torch().cuda.synchronize()  # the copies read converted temporaries
        del keep_p, keep_v

    def get_state(self, stream=None):
        pos = np.empty((self.n, 4), self.dtype)
        vel = np.empty((self.n, 4), self.dtype)
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_get_state(self.handle, pos.ctypes.data_as(C.c_void_p),
                                      vel.ctypes.data_as(C.c_void_p), N.NB_HOST, C.c_void_p(s)),
                "nb_get_state")
        return pos, vel

    def get_state_device(self, pos_t, vel_t, stream=None):
        """Copy the state into the CUDA tensors pos_t, vel_t ((n, 4), the
        context's host dtype, contiguous: they are written in place)."""
        for t, name in ((pos_t, "pos_t"), (vel_t, "vel_t")):
            if not (_is_torch(t) and t.is_cuda and t.is_contiguous() and tuple(t.shape) == (self.n, 4)
                    and t.dtype == self._torch_dtype()):
                raise ValueError(f"{name}: needs a contiguous CUDA tensor of shape ({self.n}, 4) "
                                 f"and dtype {self._torch_dtype()}")
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_get_state(self.handle, C.c_void_p(pos_t.data_ptr()),
                                      C.c_void_p(vel_t.data_ptr()), N.NB_DEVICE, C.c_void_p(s)),
                "nb_get_state")

    def step(self, steps=1, stream=None):
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_step(self.handle, int(steps), C.c_void_p(s)), "nb_step")

    def set_params(self, eps2, damping, dt, G=1.0):
        """New eps2 (softening squared), damping, dt and G for the next steps
        (BodySystem<T>::setSoftening / setDamping / update(dt))."""
        N.check(self.lib.nb_set_params(self.handle, float(eps2), float(damping), float(dt), float(G)),
                "nb_set_params")

    def step_timed(self, steps=1, stream=None):
        """Step with per-kernel CUDA events; returns (force_ms, integrate_ms) summed."""
        f, g = C.c_float(0.0), C.c_float(0.0)
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_step_timed(self.handle, int(steps), C.byref(f), C.byref(g), C.c_void_p(s)),
                "nb_step_timed")
        return f.value, g.value

    def accel(self, stream=None):
        """Bare accelerations of the current state, (n, 3) numpy."""
        torch = _torch()
        tdt = torch.float64 if self.dtype == np.float64 else torch.float32
        out = torch.zeros((max(self.n, 1), 4), dtype=tdt, device="cuda")
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_accel(self.handle, C.c_void_p(out.data_ptr()), C.c_void_p(s)), "nb_accel")
        torch.cuda.current_stream().synchronize()
        return out[: self.n, :3].cpu().numpy()

    def energy(self, with_bodies=False, stream=None):
        """(kinetic, potential, px, py, pz) reduced in FP64 on the GPU; with
        with_bodies, also the per-body (acc xyz, potential over j != i) (n, 4)."""
        torch = _torch()
        out = (C.c_double * 5)()
        s = current_stream_handle() if stream is None else stream
        buf = None
        if with_bodies:
            tdt = torch.float64 if self.precision in ("f32comp", "f64") else torch.float32
            buf = torch.zeros((max(self.n, 1), 4), dtype=tdt, device="cuda")
        N.check(self.lib.nb_energy(self.handle, out, C.c_void_p(buf.data_ptr() if buf is not None else 0),
                                   C.c_void_p(s)), "nb_energy")
        e = np.array(list(out))
        if with_bodies:
            torch.cuda.current_stream().synchronize()
            return e, buf[: self.n].cpu().numpy()
        return e

    def adj_forward(self, steps, ckpt_every, stream=None):
        """Advance `steps` steps keeping a checkpoint every `ckpt_every` steps.
        Returns the generation number of this recorded forward pass (also kept
        as self.adj_generation, the default of adj_backward)."""
        s = current_stream_handle() if stream is None else stream
        gen = C.c_ulonglong(0)
        N.check(self.lib.nb_adj_forward(self.handle, int(steps), int(ckpt_every), C.c_void_p(s),
                                        C.byref(gen)), "nb_adj_forward")
        self.adj_generation = int(gen.value)
        return self.adj_generation

    def adj_backward(self, gx_T, gv_T=None, stream=None, generation=None):
        """Cotangents of the final (n,4) positions / velocities (torch CUDA
        float32; gv_T may be None) -> (dL/dx0 (n,4), dL/dv0 (n,4), dL/dm (n,)).
        `generation` names the forward pass (default: the last adj_forward
        of this object); a pass the context no longer holds raises."""
        torch = _torch()
        gx0 = torch.zeros((self.n, 4), dtype=torch.float32, device="cuda")
        gv0 = torch.zeros((self.n, 4), dtype=torch.float32, device="cuda")
        gm = torch.zeros((self.n,), dtype=torch.float32, device="cuda")
        s = current_stream_handle() if stream is None else stream
        gx = _device_buffer(gx_T, (self.n, 4), torch.float32, "gx_T")
        gv = _device_buffer(gv_T, (self.n, 4), torch.float32, "gv_T") if gv_T is not None else None
        gv_ptr = C.c_void_p(gv.data_ptr()) if gv is not None else C.c_void_p(0)
        gen = getattr(self, "adj_generation", 0) if generation is None else int(generation)
        N.check(self.lib.nb_adj_backward(self.handle, C.c_ulonglong(gen), C.c_void_p(gx.data_ptr()), gv_ptr,
                                         C.c_void_p(gx0.data_ptr()), C.c_void_p(gv0.data_ptr()),
                                         C.c_void_p(gm.data_ptr()), C.c_void_p(s)),
                "nb_adj_backward")
        if gx is not gx_T or (gv is not None and gv is not gv_T):
            torch.cuda.synchronize()  # the pass read converted temporaries
        return gx0, gv0, gm

    def run_host(self, pos, vel, loops, out_interval, stream=None):
        """Task-style run with host buffers; returns (frames (k, n, 4), timings[4])."""
        pos = np.ascontiguousarray(pos, dtype=self.dtype).reshape(self.n, 4)
        vel = np.ascontiguousarray(vel, dtype=self.dtype).reshape(self.n, 4)
        k = loops // out_interval if out_interval > 0 else 0
        out = np.zeros((max(k, 1), self.n, 4), self.dtype)
        t = (C.c_double * 4)()
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_run_host(self.handle, pos.ctypes.data_as(C.c_void_p),
                                     vel.ctypes.data_as(C.c_void_p), int(loops), int(out_interval),
                                     out.ctypes.data_as(C.c_void_p), t, C.c_void_p(s)),
                "nb_run_host")
        return out[:k], list(t)

    def state_ptrs(self):
        p, v = C.c_void_p(), C.c_void_p()
        N.check(self.lib.nb_state_ptrs(self.handle, C.byref(p), C.byref(v)), "nb_state_ptrs")
        return p.value, v.value

    def plan_info(self):
        info = (C.c_int * 5)()
        N.check(self.lib.nb_plan_info(self.handle, info), "nb_plan_info")
        return dict(zip(["block", "bpt", "grid", "tbsize", "slots"], list(info)))

    def source_info(self):
        """Symmetric contexts: {"side": "fixed" or "triangular", "bands": k,
        "mib": scratch of the source side in MiB}."""
        info = (C.c_int * 4)()
        N.check(self.lib.nb_source_info(self.handle, info), "nb_source_info")
        side = {N.NB_SOURCE_FIXED: "fixed", N.NB_SOURCE_TRIANGULAR: "triangular"}.get(info[0])
        return {"side": side, "bands": info[1], "mib": info[2]}

    def launches_per_step(self):
        return self.lib.nb_launches_per_step(self.handle)

    def autotune(self, reps=3, cache_path=None, stream=None):
        """Time every compiled shape of this context's force kernel on the
        current state (restored afterwards) and keep the fastest; returns
        (threads per CTA, bodies per lane)."""
        s = current_stream_handle() if stream is None else stream
        out = (C.c_int * 2)()
        N.check(self.lib.nb_autotune(self.handle, int(reps), cache_path.encode() if cache_path else None,
                                     C.c_void_p(s), out), "nb_autotune")
        return int(out[0]), int(out[1])


def probe_fma_peak(iters=20000, packed=True, stream=None):
    """Measured FMA peak in FLOP/s on the current device: FP32 (packed True or
    False) or FP64 (packed=2)."""
    flops, ms = C.c_double(), C.c_float()
    s = current_stream_handle() if stream is None else stream
    N.check(N.lib().nb_probe_fma_peak(int(iters), 2 if packed == 2 else int(bool(packed)), C.byref(flops), C.byref(ms),
                                      C.c_void_p(s)), "nb_probe_fma_peak")
    return flops.value / (ms.value * 1e-3), ms.value


class NBodyBatch:
    """Many independent systems (sizes[s] bodies each) in one context; state
    arrays are the systems' (n, 4) arrays concatenated: float32 for precision
    "f32" (algo "sym", each unordered pair once, or "fast", directed), float64
    for "f64" (algo "sym": float-float pair terms on the FP32 pipe, the
    reference multi-task app's default state type)."""

    def __init__(self, sizes, kick="physical", eps2=1e-3, damping=1.0, dt=1e-3, G=1.0,
                 warps_per_cta=0, bodies_per_lane=0, algo="sym", precision="f32"):
        self.lib = N.lib()
        p = N.NbParams()
        self.lib.nb_params_default(C.byref(p))
        p.precision = _PREC[precision]
        p.algo = _ALGO[algo]
        self.precision = precision
        self.dtype = np.float64 if precision == "f64" else np.float32
        p.kick = _KICK[kick]
        p.eps2, p.damping, p.dt, p.G = float(eps2), float(damping), float(dt), float(G)
        p.block = int(warps_per_cta) * 32
        p.bpt = int(bodies_per_lane)
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.nbody = int(self.sizes.sum())
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        h = C.c_void_p()
        N.check(self.lib.nb_batch_create(C.byref(p), len(self.sizes),
                                         self.sizes.ctypes.data_as(C.c_void_p), C.byref(h)),
                "nb_batch_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            N.check(self.lib.nb_batch_destroy(self.handle), "nb_batch_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, pos, vel, stream=None):
        s = current_stream_handle() if stream is None else stream
        if _is_torch(pos) or _is_torch(vel):
            torch = _torch()
            tdt = torch.float64 if self.dtype == np.float64 else torch.float32
            p = _device_buffer(pos, (self.nbody, 4), tdt, "pos")
            v = _device_buffer(vel, (self.nbody, 4), tdt, "vel")
            N.check(self.lib.nb_batch_set_state(self.handle, C.c_void_p(p.data_ptr()),
                                                C.c_void_p(v.data_ptr()), N.NB_DEVICE, C.c_void_p(s)),
                    "nb_batch_set_state")
            if p is not pos or v is not vel:
                torch.cuda.synchronize()  # the copies read converted temporaries
            return
        pos = np.ascontiguousarray(pos, dtype=self.dtype).reshape(self.nbody, 4)
        vel = np.ascontiguousarray(vel, dtype=self.dtype).reshape(self.nbody, 4)
        N.check(self.lib.nb_batch_set_state(self.handle, pos.ctypes.data_as(C.c_void_p),
                                            vel.ctypes.data_as(C.c_void_p), N.NB_HOST, C.c_void_p(s)),
                "nb_batch_set_state")

    def get_state(self, stream=None):
        pos = np.empty((self.nbody, 4), self.dtype)
        vel = np.empty((self.nbody, 4), self.dtype)
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_batch_get_state(self.handle, pos.ctypes.data_as(C.c_void_p),
                                            vel.ctypes.data_as(C.c_void_p), N.NB_HOST, C.c_void_p(s)),
                "nb_batch_get_state")
        return pos, vel

    def step(self, steps=1, stream=None):
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_batch_step(self.handle, int(steps), C.c_void_p(s)), "nb_batch_step")

    def set_params(self, eps2, damping, dt, G=1.0):
        N.check(self.lib.nb_batch_set_params(self.handle, float(eps2), float(damping), float(dt), float(G)),
                "nb_batch_set_params")

    def run(self, steps, stream):
        """`steps` steps as one CUDA graph on a non-default stream handle."""
        N.check(self.lib.nb_batch_run(self.handle, int(steps), C.c_void_p(stream)), "nb_batch_run")

    def step_per_system(self, steps=1, stream=None):
        s = current_stream_handle() if stream is None else stream
        N.check(self.lib.nb_batch_step_per_system(self.handle, int(steps), C.c_void_p(s)),
                "nb_batch_step_per_system")

    def step_tasks(self, steps, ntasks):
        """Reference-pattern baseline: ntasks threads/streams, sync every step."""
        N.check(self.lib.nb_batch_step_tasks(self.handle, int(steps), int(ntasks)), "nb_batch_step_tasks")

    def autotune(self, reps=2, cache_path=None, stream=None):
        s = current_stream_handle() if stream is None else stream
        out = (C.c_int * 2)()
        N.check(self.lib.nb_batch_autotune(self.handle, int(reps),
                                           cache_path.encode() if cache_path else None,
                                           C.c_void_p(s), out), "nb_batch_autotune")
        return int(out[0]), int(out[1])

    def adj_forward(self, steps, ckpt_every, stream=None):
        """As NBodySystem.adj_forward, for all systems; returns the generation."""
        s = current_stream_handle() if stream is None else stream
        gen = C.c_ulonglong(0)
        N.check(self.lib.nb_batch_adj_forward(self.handle, int(steps), int(ckpt_every), C.c_void_p(s),
                                              C.byref(gen)), "nb_batch_adj_forward")
        self.adj_generation = int(gen.value)
        return self.adj_generation

    def adj_backward(self, gx_T, gv_T=None, stream=None, generation=None):
        """Cotangents (nbody, 4) torch CUDA float32 -> (dL/dx0, dL/dv0, dL/dm);
        `generation` as in NBodySystem.adj_backward."""
        torch = _torch()
        gx0 = torch.zeros((self.nbody, 4), dtype=torch.float32, device="cuda")
        gv0 = torch.zeros((self.nbody, 4), dtype=torch.float32, device="cuda")
        gm = torch.zeros((self.nbody,), dtype=torch.float32, device="cuda")
        s = current_stream_handle() if stream is None else stream
        gx = _device_buffer(gx_T, (self.nbody, 4), torch.float32, "gx_T")
        gv = _device_buffer(gv_T, (self.nbody, 4), torch.float32, "gv_T") if gv_T is not None else None
        gen = getattr(self, "adj_generation", 0) if generation is None else int(generation)
        N.check(self.lib.nb_batch_adj_backward(
            self.handle, C.c_ulonglong(gen), C.c_void_p(gx.data_ptr()),
            C.c_void_p(gv.data_ptr() if gv is not None else 0),
            C.c_void_p(gx0.data_ptr()), C.c_void_p(gv0.data_ptr()), C.c_void_p(gm.data_ptr()),
            C.c_void_p(s)), "nb_batch_adj_backward")
        if gx is not gx_T or (gv is not None and gv is not gv_T):
            torch.cuda.synchronize()  # the pass read converted temporaries
        return gx0, gv0, gm

    def set_shape(self, warps_per_cta, bodies_per_lane):
        N.check(self.lib.nb_batch_set_shape(self.handle, int(warps_per_cta), int(bodies_per_lane)),
                "nb_batch_set_shape")

    def plan_info(self):
        info = (C.c_longlong * 6)()
        N.check(self.lib.nb_batch_plan_info(self.handle, info), "nb_batch_plan_info")
        return dict(zip(["warps_per_cta", "bodies_per_lane", "grid", "workers", "iterations", "slots"],
                        list(info)))


def gpu_initial_conditions(kind, n, seed=0, a=1.0, G=1.0, M=1.0, vmax=0.01, precision="f32", stream=None):
    """Seeded bodies drawn on the GPU: kind "cube", "plummer", or the
    reference app's "random", "shell", "expand" (a = clusterScale, vmax =
    velocityScale).  Returns (pos, vel) torch CUDA tensors (n, 4)."""
    torch = _torch()
    tdt = torch.float64 if precision == "f64" else torch.float32
    pos = torch.empty((max(n, 1), 4), dtype=tdt, device="cuda")
    vel = torch.empty((max(n, 1), 4), dtype=tdt, device="cuda")
    nbytes = N.lib().nb_ics_scratch_bytes(int(n))
    scratch = torch.empty((max(nbytes, 8) // 8,), dtype=torch.float64, device="cuda")
    s = current_stream_handle() if stream is None else stream
    kinds = {"cube": 0, "plummer": 1, "random": 2, "shell": 3, "expand": 4}
    N.check(N.lib().nb_ics_generate(kinds[kind], int(n), int(seed), float(a), float(G),
                                    float(M), float(vmax), _PREC[precision], C.c_void_p(pos.data_ptr()),
                                    C.c_void_p(vel.data_ptr()), C.c_void_p(scratch.data_ptr()), C.c_void_p(s)),
            "nb_ics_generate")
    return pos[:n], vel[:n]
