"""torch.autograd wrapper over the engine's adjoint (check harness only).

MeanSquareDisplacement(vx, vy) runs the GPU engine from a fixed initial state
with the given velocities for a number of collisions and returns the MSD at a
fixed observation time; backward() returns the adjoint gradient computed by
edmd_msd_gradient (checkpointed reverse pass), so torch can chain it.
"""
import numpy as np
import torch


class _MSD(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vx, vy, runner):
        msd, gvx, gvy = runner(vx.detach().cpu().numpy(), vy.detach().cpu().numpy())
        ctx.save_for_backward(torch.from_numpy(gvx), torch.from_numpy(gvy))
        return torch.tensor(msd, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        gvx, gvy = ctx.saved_tensors
        return grad * gvx, grad * gvy, None


class MeanSquareDisplacement:
    def __init__(self, edmd, init, Lx, Ly, n_coll, t_obs, ckpt_every=250):
        self.edmd, self.init, self.Lx, self.Ly = edmd, init, Lx, Ly
        self.n_coll, self.t_obs, self.ckpt_every = n_coll, t_obs, ckpt_every

    def _run(self, vx, vy):
        s = {k: np.asarray(self.init[k], np.float64) for k in ("x", "y", "rad", "m")}
        s["vx"], s["vy"] = np.ascontiguousarray(vx), np.ascontiguousarray(vy)
        desc = self.edmd.default_desc(len(vx), self.Lx, self.Ly)
        eng = self.edmd.Engine([dict(desc=desc, vr=None, **s)])
        msd, g = eng.msd_gradient(self.n_coll, self.ckpt_every, self.t_obs)
        eng.close()
        return msd, g["vx"], g["vy"]

    def __call__(self, vx, vy):
        return _MSD.apply(vx, vy, self._run)
