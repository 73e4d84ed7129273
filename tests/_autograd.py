"""torch.autograd.Function over the library's IF-RK4 steps (test harness only).

forward runs `nsteps` steps from v_0 through the C ABI; backward calls
sc_adjoint_rk4_vjp with the upstream gradient.  Complex gradients follow
PyTorch's convention for a real loss L, dL/dRe z + i dL/dIm z, which is the
convention of the library's adjoint, so no conversion is needed.
"""
import numpy as np
import torch


class RK4Steps(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h, nsteps, checkpoint_every, vx, vy, vz):
        v0 = [t.detach().cpu().numpy() for t in (vx, vy, vz)]
        h.set_state(*v0)
        h.rk4_steps(nsteps)
        vt = h.get_state()
        ctx.h, ctx.nsteps, ctx.k, ctx.v0 = h, nsteps, checkpoint_every, v0
        return tuple(torch.from_numpy(a) for a in vt)

    @staticmethod
    def backward(ctx, gx, gy, gz):
        lam = [np.zeros(ctx.v0[0].shape, ctx.v0[0].dtype) if gr is None else gr.detach().cpu().numpy()
               for gr in (gx, gy, gz)]
        ctx.h.set_state(*ctx.v0)
        g = ctx.h.adjoint_vjp(ctx.nsteps, lam, ctx.k)
        return (None, None, None) + tuple(torch.from_numpy(a) for a in g)


def rk4_steps(h, nsteps, checkpoint_every, v):
    return RK4Steps.apply(h, nsteps, checkpoint_every, *v)
