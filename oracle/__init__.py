"""CPU oracle for the nbody all-pairs step -- TEST INFRASTRUCTURE ONLY.

Only the test suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg import this package.  It wraps two shared libraries:

* ``liboracle.so`` -- the C restatement in ``nbody_oracle.c``, which follows
  the reference's sequential ``BodySystem<T>`` (benchapps/nbody/seq/
  bodysystem.cc:103-182, bodysystem.h:71-96) operation for operation, so that
  float and double runs are bit-identical to it;
* ``_ref/libnbref.so`` (optional) -- the reference's own
  ``benchapps/nbody/seq/bodysystem.cc`` compiled where it lies, present only
  where the reference checkout is available.  Used to pin the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_CUBIN = os.path.join(HERE, "_ref", "ref_kernel_sm103a.cubin")

KICK_REFERENCE = 0
KICK_PHYSICAL = 1

_lock = threading.Lock()
_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def ref_root() -> str | None:
    """The reference checkout's utc-0.1 directory, from $NB_REF_ROOT (None
    when unset or absent: the reference builds are then skipped)."""
    root = os.environ.get("NB_REF_ROOT")
    return root if root and os.path.isdir(root) else None


def build(ref: bool | None = None) -> None:
    """Compile liboracle.so, and the reference's own code into _ref/ when
    $NB_REF_ROOT names the reference checkout."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    root = ref_root()
    if ref is None:
        ref = root is not None
    if ref:
        if root is None:
            raise RuntimeError("oracle.build(ref=True) needs NB_REF_ROOT (the reference's utc-0.1 directory)")
        subprocess.run(["make", "-s", "-C", HERE, "ref", "ref-gpu", "NB_REF_ROOT=" + root], check=True)


def _declare(lib):
    I, F, D = C.c_int, C.c_float, C.c_double
    sig = {
        "orc_accel_f32": (I, [I, _f32p, F, _f32p, I]),
        "orc_accel_f64": (I, [I, _f64p, D, _f64p, I]),
        "orc_accel_subset_f64": (I, [I, _f64p, I, _i32p, D, _f64p, I]),
        "orc_accel_phi_subset_f64": (I, [I, _f64p, I, _i32p, D, _f64p, _f64p, I]),
        "orc_step_f32": (I, [I, _f32p, _f32p, F, F, F, I, I, F, I]),
        "orc_step_f64": (I, [I, _f64p, _f64p, D, D, D, I, I, D, I]),
        "orc_step_range_f32": (I, [I, _f32p, _f32p, _f32p, I, I, F, F, F, I, F, I]),
        "orc_energy_f64": (I, [I, _f64p, _f64p, D, D, _f64p, I]),
        "orc_adjoint_f64": (I, [I, _f64p, _f64p, D, D, D, I, I, D, _f64p,
                                C.POINTER(D), _f64p, _f64p, _f64p, I]),
        "orc_loss_f64": (I, [I, _f64p, _f64p, D, D, D, I, I, D, _f64p,
                             C.POINTER(D), I]),
        "orc_srand": (None, [C.c_uint]),
        "orc_randomize_f32": (I, [I, _f32p, _f32p, F, F, I]),
        "orc_randomize_f64": (I, [I, _f64p, _f64p, F, F, I]),
        "orc_demo_params": (None, [I, I] + [C.POINTER(F)] * 5),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    """The restatement library (built on first use if missing)."""
    global _lib
    with _lock:
        if _lib is None:
            path = os.path.join(HERE, "liboracle.so")
            if not os.path.exists(path):
                subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
            _lib = _declare(C.CDLL(path))
        return _lib


def ref_lib():
    """The reference's own seq code, or None where it was not built."""
    global _ref
    with _lock:
        if _ref is None:
            path = os.path.join(HERE, "_ref", "libnbref.so")
            if not os.path.exists(path):
                return None
            try:
                r = C.CDLL(path)
            except OSError:  # e.g. built for another architecture
                return None
            I, F, D = C.c_int, C.c_float, C.c_double
            r.ref_srand.argtypes = [C.c_uint]
            r.ref_srand.restype = None
            r.ref_randomize_f32.argtypes = [I, _f32p, _f32p, F, F, I]
            r.ref_randomize_f64.argtypes = [I, _f64p, _f64p, F, F, I]
            r.ref_run_f32.argtypes = [I, _f32p, _f32p, F, F, F, I]
            r.ref_run_f64.argtypes = [I, _f64p, _f64p, D, D, D, I]
            for f in (r.ref_randomize_f32, r.ref_randomize_f64, r.ref_run_f32, r.ref_run_f64):
                f.restype = I
            _ref = r
        return _ref


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


# --------------------------------------------------------------------------
# numpy conveniences
# --------------------------------------------------------------------------
def accel(pos, eps2, nthreads=None):
    """Bare acceleration sums (n,3) for pos (n,4), in pos's dtype."""
    pos = np.ascontiguousarray(pos)
    n = pos.shape[0]
    nt = nthreads or default_threads()
    if pos.dtype == np.float32:
        out = np.zeros((n, 3), np.float32)
        _check(lib().orc_accel_f32(n, pos.reshape(-1), np.float32(eps2), out.reshape(-1), nt), "accel_f32")
    else:
        pos = pos.astype(np.float64, copy=False)
        out = np.zeros((n, 3), np.float64)
        _check(lib().orc_accel_f64(n, pos.reshape(-1), float(eps2), out.reshape(-1), nt), "accel_f64")
    return out


def accel_subset_f64(pos, tidx, eps2, nthreads=None):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    tidx = np.ascontiguousarray(tidx, dtype=np.int32)
    out = np.zeros((tidx.shape[0], 3), np.float64)
    _check(lib().orc_accel_subset_f64(pos.shape[0], pos.reshape(-1), tidx.shape[0], tidx,
                                      float(eps2), out.reshape(-1), nthreads or default_threads()),
           "accel_subset_f64")
    return out


def accel_phi_subset_f64(pos, tidx, eps2, nthreads=None):
    """FP64 (acc (nt,3), phi over j != i (nt,)) for targets tidx against all bodies."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    tidx = np.ascontiguousarray(tidx, dtype=np.int32)
    acc = np.zeros((tidx.shape[0], 3), np.float64)
    phi = np.zeros(tidx.shape[0], np.float64)
    _check(lib().orc_accel_phi_subset_f64(pos.shape[0], pos.reshape(-1), tidx.shape[0], tidx,
                                          float(eps2), acc.reshape(-1), phi,
                                          nthreads or default_threads()), "accel_phi_subset_f64")
    return acc, phi


def step(pos, vel, eps2, damping, dt, steps, kick_mode=KICK_REFERENCE, G=1.0, nthreads=None):
    """Run `steps` reference steps; returns new (pos, vel) copies in the input dtype."""
    pos = np.array(pos, copy=True, order="C")
    vel = np.array(vel, copy=True, order="C")
    n = pos.shape[0]
    nt = nthreads or default_threads()
    if pos.dtype == np.float32:
        vel = vel.astype(np.float32, copy=False)
        _check(lib().orc_step_f32(n, pos.reshape(-1), vel.reshape(-1), np.float32(eps2),
                                  np.float32(damping), np.float32(dt), steps, kick_mode,
                                  np.float32(G), nt), "step_f32")
    else:
        pos = pos.astype(np.float64, copy=False)
        vel = vel.astype(np.float64, copy=False)
        _check(lib().orc_step_f64(n, pos.reshape(-1), vel.reshape(-1), float(eps2), float(damping),
                                  float(dt), steps, kick_mode, float(G), nt), "step_f64")
    return pos, vel


def step_range(pos_old, pos_new, vel, i0, i1, eps2, damping, dt, kick_mode=KICK_REFERENCE, G=1.0,
               nthreads=None):
    """One float step of targets [i0, i1) against every body of pos_old,
    written into pos_new[i0:i1] and vel[i0:i1] in place (float32 (n, 4)
    C-contiguous arrays): the share of one shard of a target partition."""
    n = pos_old.shape[0]
    _check(lib().orc_step_range_f32(n, pos_old.reshape(-1), pos_new.reshape(-1), vel.reshape(-1), int(i0),
                                    int(i1), np.float32(eps2), np.float32(damping), np.float32(dt),
                                    kick_mode, np.float32(G), nthreads or default_threads()), "step_range_f32")


def energy(pos, vel, eps2, G=1.0, nthreads=None):
    """(kinetic, potential, px, py, pz) in double."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    out = np.zeros(5, np.float64)
    _check(lib().orc_energy_f64(pos.shape[0], pos.reshape(-1), vel.reshape(-1), float(eps2),
                                float(G), out, nthreads or default_threads()), "energy")
    return out


def loss(pos, vel, y, eps2, damping, dt, steps, kick_mode=KICK_PHYSICAL, G=1.0, nthreads=None):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    L = C.c_double(0.0)
    _check(lib().orc_loss_f64(pos.shape[0], pos.reshape(-1), vel.reshape(-1), float(eps2),
                              float(damping), float(dt), steps, kick_mode, float(G),
                              y.reshape(-1), C.byref(L), nthreads or default_threads()), "loss")
    return L.value


def adjoint(pos, vel, y, eps2, damping, dt, steps, kick_mode=KICK_PHYSICAL, G=1.0, nthreads=None):
    """FP64 reference adjoint: (loss, dL/dx0 (n,3), dL/dv0 (n,3), dL/dm (n,))."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    n = pos.shape[0]
    gx = np.zeros((n, 3)); gv = np.zeros((n, 3)); gm = np.zeros(n)
    L = C.c_double(0.0)
    _check(lib().orc_adjoint_f64(n, pos.reshape(-1), vel.reshape(-1), float(eps2), float(damping),
                                 float(dt), steps, kick_mode, float(G), y.reshape(-1), C.byref(L),
                                 gx.reshape(-1), gv.reshape(-1), gm, nthreads or default_threads()),
           "adjoint")
    return L.value, gx, gv, gm


def demo_params(para_select, n):
    """(dt, clusterScale, velocityScale, softening, damping) of the app preset."""
    vals = [C.c_float() for _ in range(5)]
    lib().orc_demo_params(para_select, n, *[C.byref(v) for v in vals])
    return tuple(v.value for v in vals)


def randomize(config, n, dtype=np.float32, seed=1):
    """randomizeBodies(config) from a fresh rand() state (srand(seed))."""
    pos = np.zeros((n, 4), dtype)
    vel = np.zeros((n, 4), dtype)
    _, cs, vs, _, _ = demo_params(0, n)
    lib().orc_srand(seed)
    fn = lib().orc_randomize_f32 if dtype == np.float32 else lib().orc_randomize_f64
    _check(fn(config, pos.reshape(-1), vel.reshape(-1), cs, vs, n), "randomize")
    return pos, vel


def format_frames(frames, dt):
    """The app's text output (seq/nbody_main.cc:195-211): per frame a "%f"
    time line (frame index x dt) then one "%.5f %.5f %.5f %.5f" line per body."""
    out = []
    for i, fr in enumerate(frames):
        out.append("%f\n" % float(np.float32(i) * np.float32(dt)))
        for b in np.asarray(fr).reshape(-1, 4):
            out.append("%.5f %.5f %.5f %.5f\n" % (float(b[0]), float(b[1]), float(b[2]), float(b[3])))
    return "".join(out)
