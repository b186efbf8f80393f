"""Fixed small runs of the kernels for profilers.

    python -m utc_gb300.profile_case --n 65536 --steps 4 [--algo fast|exact]
        [--block B --bpt K] [--kick physical|reference]

Runs `steps` steps of a seeded Plummer sphere (eps2=1e-4, dt=1e-4) through
the C ABI and prints the launch plan; used as the command under ncu.
"""
import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--algo", default="fast")
    ap.add_argument("--kick", default="physical")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--bpt", type=int, default=0)
    a = ap.parse_args()
    import torch

    from . import ics
    from .nbody import NBodySystem

    p, v = ics.plummer(a.n, seed=0)
    with NBodySystem(a.n, "f32", a.algo, kick=a.kick, eps2=np.float32(1e-4), damping=1.0,
                     dt=np.float32(1e-4), block=a.block, bpt=a.bpt) as s:
        s.set_state(ics.f32(p), ics.f32(v))
        s.step(a.steps)
        torch.cuda.synchronize()
        print("ok", a.n, a.steps, s.plan_info() if a.algo == "fast" else a.algo)


if __name__ == "__main__":
    main()
