"""Test-harness wrapper of the CUDA adjoint (wave_adjoint_gradient) as a
torch.autograd.Function: the misfit J(vp, vs, rho) = 1/2 sum (d - d_obs)^2 of
one 2-D elastic shot, whose backward returns the adjoint gradients. Used only
by the tests, to check the gradients through torch.autograd against finite
differences and against the FP64 oracle gradient."""
import numpy as np
import torch


class ElasticMisfit(torch.autograd.Function):
    """J = ElasticMisfit.apply(vp, vs, rho, solver, dobs, checkpoint_every):
    vp, vs, rho are float32 tensors of the grid's N points (the solver's
    model); `solver` is a wave ForwardSolver with its acquisition set."""

    @staticmethod
    def forward(ctx, vp, vs, rho, solver, dobs, checkpoint_every):
        solver.prepareForModelling({k: t.detach().to(torch.float32).contiguous().cpu().numpy()
                                    for k, t in (("vp", vp), ("vs", vs), ("rho", rho))})
        J, gvp, gvs, grho = solver.adjoint_gradient(np.ascontiguousarray(dobs, np.float32), checkpoint_every=checkpoint_every)
        ctx.save_for_backward(*(torch.from_numpy(np.asarray(g, np.float32)).to(vp.device) for g in (gvp, gvs, grho)))
        return torch.tensor(J, dtype=torch.float64, device=vp.device)

    @staticmethod
    def backward(ctx, gJ):
        gvp, gvs, grho = ctx.saved_tensors
        s = gJ.to(torch.float32)
        return s * gvp, s * gvs, s * grho, None, None, None


def misfit(vp, vs, rho, solver, dobs, checkpoint_every=50):
    return ElasticMisfit.apply(vp, vs, rho, solver, dobs, checkpoint_every)
