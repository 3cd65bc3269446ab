"""torch.autograd.Function over the C-ABI adjoint (verification harness only).

forward() runs tpm_adjoint_run for the objective J(RU0, A, tau_p) and keeps
the gradients it returns; backward() scales them by the incoming gradient.
"""
import numpy as np
import torch

from tpm import inputs


class TpmObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, RU0, A, tau, capi, p, s, nsteps, w_tke, w_cvar):
        pp = p.replace(A1=float(A), A2=float(A))
        st = inputs.State(RU=RU0.detach().cpu().numpy(), Rho=s.Rho, P=s.P, part=s.part, P0=s.P0,
                          tau=np.full(s.npart, float(tau)))
        c = capi.Context(pp, s.npart)
        c.load(st)
        c.initialize()
        J, g, gA, gt = c.adjoint(nsteps, w_tke=w_tke, w_cvar=w_cvar)
        c.close()
        ctx.save_for_backward(torch.from_numpy(g), torch.tensor(gA, dtype=torch.float64),
                              torch.tensor(gt, dtype=torch.float64))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        g, gA, gt = ctx.saved_tensors
        return gJ * g, gJ * gA, gJ * gt, None, None, None, None, None, None
