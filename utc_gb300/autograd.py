"""torch.autograd.Function over the C-ABI adjoint (test harness).

NBodyTrajectory.apply(x0, v0, m, system, steps, ckpt_every) runs `steps`
steps of `system` (an NB_F32 fast NBodySystem) from positions x0 (n,3),
velocities v0 (n,3) and masses m (n,) -- float32 CUDA tensors -- and
returns the final positions and velocities (n,3).  Its backward is the
hand-written adjoint (nb_adj_forward / nb_adj_backward): checkpoints every
`ckpt_every` steps, recomputation in between, gradients to x0, v0 and m.

Each forward keeps the generation number nb_adj_forward gave its recorded
pass; backward hands it to nb_adj_backward, which raises (NB_ERR_STATE) if
another apply() on the same system has recorded a newer pass since, instead
of returning that other trajectory's gradients.
"""
import torch


class NBodyTrajectory(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, m, system, steps, ckpt_every):
        n = x0.shape[0]
        pos = torch.empty((n, 4), dtype=torch.float32, device=x0.device)
        vel = torch.empty((n, 4), dtype=torch.float32, device=x0.device)
        pos[:, :3] = x0
        pos[:, 3] = m
        vel[:, :3] = v0
        vel[:, 3] = 1.0
        system.set_state(pos, vel)
        generation = system.adj_forward(steps, ckpt_every)
        pT = torch.empty_like(pos)
        vT = torch.empty_like(vel)
        system.get_state_device(pT, vT)
        ctx.system = system
        ctx.generation = generation
        ctx.n = n
        return pT[:, :3].clone(), vT[:, :3].clone()

    @staticmethod
    def backward(ctx, gxT, gvT):
        n = ctx.n
        gx = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        if gxT is not None:
            gx[:, :3] = gxT
        gv = None
        if gvT is not None:
            gv = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
            gv[:, :3] = gvT
        gx0, gv0, gm = ctx.system.adj_backward(gx, gv, generation=ctx.generation)
        return gx0[:, :3], gv0[:, :3], gm, None, None, None


def trajectory(x0, v0, m, system, steps, ckpt_every):
    return NBodyTrajectory.apply(x0, v0, m, system, steps, ckpt_every)
