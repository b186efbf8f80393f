"""C-ABI library checks that need no GPU: it loads, exports every symbol the
header declares, rejects bad arguments with status codes, and the stream-K
partition it uses covers every (target block, source group) exactly once."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from utc_gb300 import _native as N


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_library_exports_every_header_symbol(built):
    syms = N.header_symbols()
    assert len(syms) >= 14
    ex = exported(N.LIB_PATH)
    missing = [s for s in syms if s not in ex]
    assert not missing, missing
    lib = N.lib()
    for s in syms:
        assert hasattr(lib, s)
    assert lib.nb_abi_version() == 2


def test_task_library_exports(built):
    ex = exported(N.TASK_LIB_PATH)
    for s in ("nbt_run_f32", "nbt_run_f64", "nbt_randomize_f32", "nbt_randomize_f64", "nbt_mgpu_run_f32",
              "nbt_mgpu_run_f64"):
        assert s in ex
    N.task_lib()


def _params(**kw):
    p = N.NbParams()
    N.lib().nb_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("kw,status", [
    (dict(n=-1), N.NB_ERR_INVALID),
    (dict(n=(1 << 30) + 1), N.NB_ERR_INVALID),
    (dict(n=8, precision=7), N.NB_ERR_INVALID),
    (dict(n=8, algo=9), N.NB_ERR_INVALID),
    (dict(n=8, kick=3), N.NB_ERR_INVALID),
    (dict(n=8, memtype=5), N.NB_ERR_INVALID),
    (dict(n=8, dt=float("nan")), N.NB_ERR_INVALID),
    (dict(n=8, source_side=3), N.NB_ERR_INVALID),
    (dict(n=8, bands=1), N.NB_ERR_INVALID),
    (dict(n=8, bands=-1), N.NB_ERR_INVALID),
    (dict(n=8, bands=513), N.NB_ERR_INVALID),
    (dict(n=8, source_side=-1, precision=N.NB_F64, algo=N.NB_ALGO_EXACT), N.NB_ERR_INVALID),
    (dict(n=8, precision=N.NB_F64, algo=N.NB_ALGO_FAST), N.NB_ERR_UNSUPPORTED),
    (dict(n=8, precision=N.NB_F32, algo=N.NB_ALGO_SYM_FP64), N.NB_ERR_UNSUPPORTED),
])
def test_create_rejects_bad_params(built, kw, status):
    p = _params(**kw)
    h = C.c_void_p()
    rc = N.lib().nb_create(C.byref(p), C.byref(h))
    assert rc == status
    assert h.value is None
    assert N.lib().nb_last_error()


@pytest.mark.parametrize("kw,status", [
    (dict(eps2=float("inf")), N.NB_ERR_INVALID),
    (dict(dt=float("nan")), N.NB_ERR_INVALID),
    (dict(kick=3), N.NB_ERR_INVALID),
    (dict(source_side=7), N.NB_ERR_INVALID),
    (dict(precision=N.NB_F64), N.NB_ERR_UNSUPPORTED),
    (dict(algo=N.NB_ALGO_EXACT), N.NB_ERR_UNSUPPORTED),
])
def test_batch_create_rejects_bad_params(built, kw, status):
    """Checked before any CUDA call, so this runs without a GPU."""
    p = _params(**kw)
    sizes = (C.c_int * 2)(16, 40)
    h = C.c_void_p()
    rc = N.lib().nb_batch_create(C.byref(p), 2, sizes, C.byref(h))
    assert rc == status
    assert h.value is None
    assert N.lib().nb_last_error()


def test_null_handles_are_rejected(built):
    lib = N.lib()
    assert lib.nb_step(None, 1, None) == N.NB_ERR_INVALID
    assert lib.nb_set_state(None, None, None, 0, None) == N.NB_ERR_INVALID
    assert lib.nb_create(None, None) == N.NB_ERR_INVALID
    assert lib.nb_destroy(None) == N.NB_OK
    assert lib.nb_launches_per_step(None) == -1
    assert lib.nb_autotune(None, 1, None, None, None) == N.NB_ERR_INVALID


# ---------------------------------------------------------------------------
# stream-K partition (restates sk_start / sk_owner of nb_internal.cuh)
# ---------------------------------------------------------------------------
def sk_start(c, total, grid):
    return (c * total) // grid


def sk_owner(it, total, grid):
    return ((it + 1) * grid - 1) // total


@pytest.mark.parametrize("ntb,ngroups,grid", [(1, 1, 1), (1, 32, 32), (32, 2048, 304),
                                              (8, 512, 304), (512, 32768, 304), (3, 7, 20),
                                              (5, 3, 15), (2, 33, 456), (17, 129, 152)])
def test_stream_k_partition_and_slots(ntb, ngroups, grid):
    total = ntb * ngroups
    grid = min(grid, total)
    seen = np.zeros(total, np.int64)
    slots = {}
    for c in range(grid):
        a, b = sk_start(c, total, grid), sk_start(c + 1, total, grid)
        assert b > a  # grid <= total: no empty CTA
        seen[a:b] += 1
        it = a
        while it < b:
            tb = it // ngroups
            seg_end = min(b, (tb + 1) * ngroups)
            slot = c + tb
            assert slot not in slots, "two (cta, block) pairs share a slot"
            slots[slot] = (c, tb)
            it = seg_end
    assert (seen == 1).all()
    assert max(slots) < grid + ntb - 1 + 1
    # the integrator's owner range for each target block lists exactly the
    # CTAs that wrote a partial for it, in increasing order
    for tb in range(ntb):
        c0 = sk_owner(tb * ngroups, total, grid)
        c1 = sk_owner(tb * ngroups + ngroups - 1, total, grid)
        writers = sorted(c for (c, t) in slots.values() if t == tb)
        assert writers == list(range(c0, c1 + 1))
    # balance: every CTA gets floor or ceil of total / grid iterations
    sizes = [sk_start(c + 1, total, grid) - sk_start(c, total, grid) for c in range(grid)]
    assert max(sizes) - min(sizes) <= 1


@pytest.mark.parametrize("config,n,dtype", [(1, 1024, np.float32), (0, 333, np.float32),
                                            (2, 200, np.float64), (1, 4096, np.float64)])
def test_product_initialiser_matches_oracle(built, config, n, dtype):
    """NbodyInit<T> (the app's initialiser task) draws the reference's bodies."""
    import oracle

    t = N.task_lib()
    dt, cs, vs, _, _ = oracle.demo_params(0, n)
    pos = np.zeros((n, 4), dtype)
    vel = np.zeros((n, 4), dtype)
    fn = t.nbt_randomize_f32 if dtype == np.float32 else t.nbt_randomize_f64
    assert fn(config, pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p), cs, vs, n, 1) == 0
    op, ov = oracle.randomize(config, n, dtype)
    assert pos.tobytes() == op.tobytes() and vel.tobytes() == ov.tobytes()
