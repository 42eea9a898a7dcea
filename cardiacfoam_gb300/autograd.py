"""torch.autograd interface of the adjoint step.

``ProbeMisfit.apply(problem, log_gna, log_gk1, sigma)`` runs the forward
monodomain simulation of an :class:`~cardiacfoam_gb300.api.AdjointProblem`
(checkpointed) and returns the probe-voltage misfit J as a 0-d float64
tensor; ``backward`` runs the adjoint kernels and returns dJ/dlog_gna,
dJ/dlog_gk1 (per cell) and dJ/dsigma = (dJ/dsigma_l, dJ/dsigma_t), scaled by
the incoming gradient.  The tensors may live on any device; the simulation
runs on the problem's GPU through the C ABI.
"""
from __future__ import annotations

import numpy as np
import torch


class ProbeMisfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, problem, log_gna, log_gk1, sigma):
        a = log_gna.detach().to("cpu", torch.float64).numpy()
        b = log_gk1.detach().to("cpu", torch.float64).numpy()
        s = sigma.detach().to("cpu", torch.float64).numpy()
        loss, _ = problem.forward(a, b, float(s[0]), float(s[1]))
        ctx.problem = problem
        ctx.devices = (log_gna.device, log_gk1.device, sigma.device)
        return torch.tensor(loss, dtype=torch.float64, device=log_gna.device)

    @staticmethod
    def backward(ctx, grad_out):
        ga, gb, gs = ctx.problem.backward()
        g = float(grad_out.detach().cpu())
        da, db, dsig = ctx.devices
        return (None,
                torch.from_numpy(np.ascontiguousarray(ga * g)).to(da),
                torch.from_numpy(np.ascontiguousarray(gb * g)).to(db),
                torch.from_numpy(np.ascontiguousarray(gs * g)).to(dsig))


def probe_misfit(problem, log_gna, log_gk1, sigma):
    return ProbeMisfit.apply(problem, log_gna, log_gk1, sigma)
