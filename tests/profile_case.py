"""Fixed small runs of the kernels for profilers.

    python tests/profile_case.py --n 65536 --steps 4 [--algo fast|sym|exact]
        [--precision f32|f32comp|f64] [--case step|adjoint|batch]
        [--block B --bpt K] [--kick physical|reference] [--systems S]
        [--source-side auto|triangular|fixed] [--bands K]

case step:    `steps` steps of a seeded Plummer sphere (eps2=1e-4, dt=1e-4)
              through the C ABI;
case adjoint: a checkpointed forward of `steps` steps (one segment) and the
              reverse pass (`steps` VJP launches) on a uniform cube
              (eps2=1e-2, dt=1e-3);
case batch:   `steps` batched steps of `systems` Plummer systems with sizes
              log-uniform in [128, n] (float state, or double with
              --precision f64).
Prints the launch plan; used as the command under ncu (the commands in
profiles/*.md).  Kept with the tests: it is a measurement harness, not part
of the package.
"""
import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--algo", default="fast")
    ap.add_argument("--precision", default="f32", choices=["f32", "f32comp", "f64"])
    ap.add_argument("--case", default="step", choices=["step", "adjoint", "batch"])
    ap.add_argument("--kick", default="physical")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--bpt", type=int, default=0)
    ap.add_argument("--systems", type=int, default=64)
    ap.add_argument("--source-side", default="auto", choices=["auto", "triangular", "fixed"],
                    help="source side of the symmetric FP32 kernel")
    ap.add_argument("--bands", type=int, default=0,
                    help="symmetric kernels: the triangular array in K bands (0 = automatic)")
    a = ap.parse_args()
    import torch

    from utc_gb300 import ics
    from utc_gb300.nbody import NBodyBatch, NBodySystem

    if a.case == "batch":
        sizes = ics.batch_sizes(a.systems, lo=128, hi=a.n, seed=0)
        f64 = a.precision == "f64"
        ps, vs = [], []
        for k, nn in enumerate(sizes):
            p, v = ics.plummer(int(nn), seed=1000 + k)
            ps.append(p if f64 else ics.f32(p))
            vs.append(v if f64 else ics.f32(v))
        with NBodyBatch(sizes, kick=a.kick, eps2=1e-3 if f64 else np.float32(1e-3),
                        dt=1e-3 if f64 else np.float32(1e-3), algo=a.algo, precision="f64" if f64 else "f32",
                        warps_per_cta=a.block // 32, bodies_per_lane=a.bpt) as b:
            b.set_state(np.concatenate(ps), np.concatenate(vs))
            b.step(a.steps)
            torch.cuda.synchronize()
            print("ok", "batch", int(sizes.sum()), a.steps, b.plan_info())
        return
    if a.case == "adjoint":
        p, v = ics.uniform_cube(a.n, seed=0)
        with NBodySystem(a.n, "f32", a.algo, kick=a.kick, eps2=np.float32(1e-2), damping=1.0,
                         dt=np.float32(1e-3)) as s:
            s.set_state(ics.f32(p), ics.f32(v))
            s.adj_forward(a.steps, a.steps)
            g = torch.randn((a.n, 4), device="cuda") * 1e-3
            s.adj_backward(g)
            torch.cuda.synchronize()
            print("ok", "adjoint", a.n, a.steps, s.plan_info())
        return
    p, v = ics.plummer(a.n, seed=0)
    eps2 = 1e-4 if a.precision in ("f32comp", "f64") else np.float32(1e-4)
    with NBodySystem(a.n, a.precision, a.algo, kick=a.kick, eps2=eps2, damping=1.0,
                     dt=np.float32(1e-4), block=a.block, bpt=a.bpt, source_side=a.source_side,
                     bands=a.bands) as s:
        if a.precision in ("f32comp", "f64"):
            s.set_state(p, v)
        else:
            s.set_state(ics.f32(p), ics.f32(v))
        s.step(a.steps)
        torch.cuda.synchronize()
        print("ok", a.n, a.steps, s.plan_info() if a.algo in ("fast", "sym") else a.algo,
              s.source_info() if a.algo == "sym" else "")


if __name__ == "__main__":
    main()
