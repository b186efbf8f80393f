"""Generate the committed golden fixtures (tests/golden/*.json).

Run with $NB_REF_ROOT naming the reference checkout's utc-0.1 directory and
a built oracle/_ref/libnbref.so (``make -C oracle ref NB_REF_ROOT=...``):

    NB_REF_ROOT=<reference>/utc-0.1 python tests/golden/make_golden.py

What it records, all as SHA-256 digests plus summary numbers (no reference
data is copied):

* kat_shell_n1024.json -- the reference's two golden frame files,
  benchapps/nbody/seq/nbody_outpos.txt (the sequential run: SHELL bodies,
  N=1024, float, 100 steps of dt=0.016, softening 0.1, damping 1) and
  benchapps/nbody/cuda/nbody_outpos.txt (the same scenario on a GPU), their
  digests and the envelope of the GPU file around the sequential one.
* ref_runs.json -- digests of the float/double state produced by the
  reference's own BodySystem<T> (compiled from its sources into
  oracle/_ref/libnbref.so) on a grid of initialisers, sizes and step counts,
  so that the oracle restatement can be pinned where the reference tree is
  absent.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle  # noqa: E402

REF_ROOT = os.environ.get("NB_REF_ROOT", "")

# (config, n, steps, dtype, para_select) of the pinned reference runs
REF_RUN_CASES = [
    (1, 1024, 100, "f32", 0),
    (1, 1024, 10, "f64", 0),
    (0, 512, 20, "f32", 1),
    (0, 256, 20, "f64", 1),
    (2, 128, 50, "f32", 4),
    (2, 64, 50, "f64", 5),
    (1, 4, 30, "f32", 0),
    (0, 8, 30, "f32", 2),
    (1, 2048, 5, "f32", 0),
    (0, 4096, 2, "f32", 0),
]


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def parse_frames(text):
    lines = text.splitlines()
    frames, times, i = [], [], 0
    while i < len(lines):
        times.append(lines[i])
        i += 1
        body = []
        while i < len(lines) and len(lines[i].split()) == 4:
            body.append([float(t) for t in lines[i].split()])
            i += 1
        frames.append(np.array(body))
    return times, frames


def kat():
    seq_path = os.path.join(REF_ROOT, "benchapps/nbody/seq/nbody_outpos.txt")
    gpu_path = os.path.join(REF_ROOT, "benchapps/nbody/cuda/nbody_outpos.txt")
    seq = open(seq_path, "rb").read()
    gpu = open(gpu_path, "rb").read()
    _, fs = parse_frames(seq.decode())
    _, fg = parse_frames(gpu.decode())
    d = np.abs(fs[-1][:, :3] - fg[-1][:, :3])
    return {
        "scenario": {"init": "SHELL", "n": 1024, "dtype": "float32", "steps": 100,
                     "out_interval": 100, "para_select": 0, "dt": 0.016,
                     "softening": 0.1, "damping": 1.0, "rand_seed": 1},
        "seq_outpos_sha256": sha(seq),
        "seq_outpos_bytes": len(seq),
        "gpu_outpos_sha256": sha(gpu),
        "gpu_vs_seq_final_frame": {
            "median_abs": float(np.median(d)),
            "p99_abs": float(np.quantile(d, 0.99)),
            "max_abs": float(d.max()),
            "max_abs_pos": float(np.abs(fs[-1][:, :3]).max()),
        },
        "source": "benchapps/nbody/{seq,cuda}/nbody_outpos.txt",
    }


def ref_runs():
    r = oracle.ref_lib()
    if r is None:
        raise SystemExit("oracle/_ref/libnbref.so missing: run `make -C oracle ref`")
    out = []
    for config, n, steps, dt_name, para in REF_RUN_CASES:
        dtype = np.float32 if dt_name == "f32" else np.float64
        dt, cs, vs, soft, damp = oracle.demo_params(para, n)
        pos = np.zeros((n, 4), dtype)
        vel = np.zeros((n, 4), dtype)
        r.ref_srand(1)
        if dtype == np.float32:
            r.ref_randomize_f32(config, pos.reshape(-1), vel.reshape(-1), cs, vs, n)
        else:
            r.ref_randomize_f64(config, pos.reshape(-1), vel.reshape(-1), cs, vs, n)
        init_digest = sha(pos.tobytes() + vel.tobytes())
        if dtype == np.float32:
            rc = r.ref_run_f32(n, pos.reshape(-1), vel.reshape(-1), np.float32(soft),
                               np.float32(damp), np.float32(dt), steps)
        else:
            rc = r.ref_run_f64(n, pos.reshape(-1), vel.reshape(-1), float(np.float32(soft)),
                               float(np.float32(damp)), float(np.float32(dt)), steps)
        assert rc == 0
        out.append({"config": config, "n": n, "steps": steps, "dtype": dt_name,
                    "para_select": para, "init_sha256": init_digest,
                    "final_sha256": sha(pos.tobytes() + vel.tobytes()),
                    "final_pos_abs_max": float(np.abs(pos[:, :3]).max())})
    return {"cases": out,
            "note": "softening, damping and dt are the float presets widened to the run dtype; "
                    "eps2 = softening*softening in the run dtype (bodysystem.h:21-23)"}


def main():
    if not REF_ROOT or not os.path.isdir(REF_ROOT):
        sys.exit("set NB_REF_ROOT to the reference checkout's utc-0.1 directory")
    oracle.build(ref=True)
    with open(os.path.join(HERE, "kat_shell_n1024.json"), "w") as f:
        json.dump(kat(), f, indent=1)
    with open(os.path.join(HERE, "ref_runs.json"), "w") as f:
        json.dump(ref_runs(), f, indent=1)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
