"""torch.autograd.Function over npbmz_adjoint: the Python counterpart of the
ChainRulesCore rrule in julia/NPBAppsGPUChainRules.jl.

    J = TerminalObjective.apply(forcing, u0, problem, u_target, nsteps)
    J.backward()            # forcing.grad = dJ/dforcing, u0.grad = dJ/du0

forcing, u0 and u_target are float64 tensors of the dense all-zone layout
(zone z: [5][nz][ny][nx], zones back to back, flattened); J is
1/2 sum (u_N - u_target)^2 after nsteps BT-MZ steps.  The forward call runs
the discrete adjoint on the GPU as well (one forward pass with checkpoints
plus one reverse pass), so backward only scales the stored gradients.
"""
import numpy as np
import torch

from . import FORCING, U


class TerminalObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, forcing, u0, problem, u_target, nsteps, checkpoint_every=10):
        f = forcing.detach().to("cpu", torch.float64).contiguous().numpy().reshape(-1)
        u = u0.detach().to("cpu", torch.float64).contiguous().numpy().reshape(-1)
        t = u_target.detach().to("cpu", torch.float64).contiguous().numpy().reshape(-1)
        problem.upload_all(FORCING, f)
        problem.upload_all(U, u)
        J, gf, gu = problem.adjoint(int(nsteps), t, checkpoint_every=int(checkpoint_every))
        ctx.save_for_backward(torch.from_numpy(problem.flatten(gf)).view_as(forcing).to(forcing.device),
                              torch.from_numpy(problem.flatten(gu)).view_as(u0).to(u0.device))
        return torch.tensor(J, dtype=torch.float64, device=forcing.device)

    @staticmethod
    def backward(ctx, gJ):
        gf, gu = ctx.saved_tensors
        return gJ * gf, gJ * gu, None, None, None, None


def terminal_objective(problem, forcing, u0, u_target, nsteps, checkpoint_every=10):
    return TerminalObjective.apply(forcing, u0, problem, u_target, nsteps, checkpoint_every)
