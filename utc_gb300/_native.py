"""ctypes binding of the C ABI in include/nbody_gb300.h.

The library is the in-tree ``libnbody_gb300.so`` built by ``utc_gb300.build``.
There is no fallback: if it is missing, importing the binding raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libnbody_gb300.so")
TASK_LIB_PATH = os.path.join(PKG, "libnbody_task.so")
HEADER = os.path.join(REPO, "include", "nbody_gb300.h")

NB_OK, NB_ERR_INVALID, NB_ERR_CUDA, NB_ERR_OOM, NB_ERR_STATE, NB_ERR_UNSUPPORTED, NB_ERR_TIMEOUT = range(7)
NB_F32, NB_F64, NB_F32_COMP = 0, 1, 2
NB_ALGO_FAST, NB_ALGO_EXACT, NB_ALGO_SYM, NB_ALGO_SYM_FP64 = 0, 1, 2, 3
NB_KICK_REFERENCE, NB_KICK_PHYSICAL = 0, 1
NB_HOST, NB_DEVICE = 0, 1
NB_MEM_PAGEABLE, NB_MEM_PINNED, NB_MEM_UNIFIED = 0, 1, 2
NB_SOURCE_AUTO, NB_SOURCE_TRIANGULAR, NB_SOURCE_FIXED = 0, 1, 2


class NbParams(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("precision", C.c_int), ("algo", C.c_int), ("kick", C.c_int),
        ("eps2", C.c_double), ("damping", C.c_double), ("dt", C.c_double), ("G", C.c_double),
        ("block", C.c_int), ("bpt", C.c_int), ("ctas_per_sm", C.c_int), ("memtype", C.c_int),
        ("source_side", C.c_int), ("bands", C.c_int), ("reserved", C.c_int * 2),
    ]


class NbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"nbody_gb300 status {status}: {msg}")
        self.status = status


_lib = None
_task = None


def _declare(lib):
    vp, I, D = C.c_void_p, C.c_int, C.c_double
    P = C.POINTER
    sig = {
        "nb_params_default": (None, [P(NbParams)]),
        "nb_create": (I, [P(NbParams), P(vp)]),
        "nb_destroy": (I, [vp]),
        "nb_set_state": (I, [vp, vp, vp, I, vp]),
        "nb_get_state": (I, [vp, vp, vp, I, vp]),
        "nb_step": (I, [vp, I, vp]),
        "nb_set_params": (I, [vp, D, D, D, D]),
        "nb_accel": (I, [vp, vp, vp]),
        "nb_step_timed": (I, [vp, I, P(C.c_float), P(C.c_float), vp]),
        "nb_energy": (I, [vp, P(D), vp, vp]),
        "nb_adj_forward": (I, [vp, I, I, vp, P(C.c_ulonglong)]),
        "nb_adj_backward": (I, [vp, C.c_ulonglong, vp, vp, vp, vp, vp, vp]),
        "nb_autotune": (I, [vp, I, C.c_char_p, vp, P(I)]),
        "nb_step_f32_noalloc": (I, [vp, vp, vp, I, C.c_float, C.c_float, C.c_float, I, C.c_float, vp]),
        "nb_run_host": (I, [vp, vp, vp, I, I, vp, P(D), vp]),
        "nb_state_ptrs": (I, [vp, P(vp), P(vp)]),
        "nb_plan_info": (I, [vp, P(I)]),
        "nb_source_info": (I, [vp, P(I)]),
        "nb_launches_per_step": (I, [vp]),
        "nb_probe_fma_peak": (I, [I, I, P(D), P(C.c_float), vp]),
        "nb_create_shard": (I, [P(NbParams), I, I, P(vp)]),
        "nb_shard_info": (I, [vp, P(I)]),
        "nb_batch_create": (I, [P(NbParams), I, vp, P(vp)]),
        "nb_batch_destroy": (I, [vp]),
        "nb_batch_set_state": (I, [vp, vp, vp, I, vp]),
        "nb_batch_get_state": (I, [vp, vp, vp, I, vp]),
        "nb_batch_step": (I, [vp, I, vp]),
        "nb_batch_set_params": (I, [vp, D, D, D, D]),
        "nb_batch_run": (I, [vp, I, vp]),
        "nb_batch_autotune": (I, [vp, I, C.c_char_p, vp, P(I)]),
        "nb_batch_set_shape": (I, [vp, I, I]),
        "nb_batch_plan_info": (I, [vp, P(C.c_longlong)]),
        "nb_batch_launches_per_step": (I, [vp]),
        "nb_batch_step_per_system": (I, [vp, I, vp]),
        "nb_batch_adj_forward": (I, [vp, I, I, vp, P(C.c_ulonglong)]),
        "nb_batch_step_tasks": (I, [vp, I, I]),
        "nb_batch_adj_backward": (I, [vp, C.c_ulonglong, vp, vp, vp, vp, vp, vp]),
        "nb_ics_generate": (I, [I, I, C.c_ulonglong, D, D, D, D, I, vp, vp, vp, vp]),
        "nb_ics_scratch_bytes": (C.c_size_t, [I]),
        "nb_last_error": (C.c_char_p, []),
        "nb_abi_version": (I, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with utc_gb300.build.build() "
                              "(no CPU fallback exists)")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def task_lib():
    """The C++ drop-in task library (BodySystemGB300<T> behind nbt_run_*)."""
    global _task
    if _task is None:
        lib()  # load the kernel library first (the task library links it)
        if not os.path.exists(TASK_LIB_PATH):
            raise ImportError(f"{TASK_LIB_PATH} is missing: build with utc_gb300.build.build()")
        t = C.CDLL(TASK_LIB_PATH)
        U, I, F, D, vp = C.c_uint, C.c_int, C.c_float, C.c_double, C.c_void_p
        t.nbt_run_f32.argtypes = [U, F, F, vp, vp, vp, I, I, I, F, vp, I, I, I]
        t.nbt_run_f64.argtypes = [U, D, D, vp, vp, vp, I, I, I, D, vp, I, I, I]
        t.nbt_run_f32.restype = I
        t.nbt_run_f64.restype = I
        t.nbt_randomize_f32.argtypes = [I, vp, vp, F, F, I, U]
        t.nbt_randomize_f64.argtypes = [I, vp, vp, F, F, I, U]
        t.nbt_randomize_f32.restype = I
        t.nbt_randomize_f64.restype = I
        # nsys, sizes, pos[], vel[], out[], eps2[], damping, dt, loops, outInterval, members, timeout,
        # status[], runtime[4 nsys]
        t.nbt_group_run_f32.argtypes = [I, vp, vp, vp, vp, vp, F, F, I, I, I, D, vp, vp]
        t.nbt_group_run_f64.argtypes = [I, vp, vp, vp, vp, vp, D, D, I, I, I, D, vp, vp]
        t.nbt_group_run_f32.restype = I
        t.nbt_group_run_f64.restype = I
        _task = t
    return _task


def check(status, what=""):
    if status != NB_OK:
        msg = lib().nb_last_error()
        raise NbError(status, (what + ": " if what else "") + (msg.decode() if msg else ""))


def header_symbols():
    """Function names declared in include/nbody_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nb_[a-z0-9_]+)\s*\(", text)))
