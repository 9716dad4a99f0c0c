"""torch.autograd.Functions around K steps of the solver and around one
residual evaluation, for verifying the hand-written discrete adjoint with
torch's tools (gradcheck-style directional tests).  The forward and the
backward both run in the CUDA library through the C ABI (fvgb_adjoint_forward
/ fvgb_adjoint_backward; fvgb_rhs / fvgb_rhs_vjp); tensors are float64 on the
host in the reference's numbering, shape (4, N)."""
import numpy as np
import torch

from . import adjoint_backward, adjoint_forward


class StepsFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U0, solver, nsteps, n_checkpoints):
        UK, _ = adjoint_forward(solver, U0.detach().cpu().numpy(), nsteps, n_checkpoints)
        ctx.solver = solver
        return torch.from_numpy(UK)

    @staticmethod
    def backward(ctx, grad_UK):
        g, _ = adjoint_backward(ctx.solver, np.ascontiguousarray(grad_UK.detach().cpu().numpy()))
        return torch.from_numpy(g), None, None, None


def steps(U0, solver, nsteps, n_checkpoints=None):
    """U_K = K steps of solver from U0, differentiable with respect to U0."""
    nck = n_checkpoints if n_checkpoints is not None else max(1, int(round(nsteps ** 0.5)))
    return StepsFunction.apply(U0, solver, int(nsteps), int(nck))


class RhsFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U, solver):
        Un = np.ascontiguousarray(U.detach().cpu().numpy())
        ctx.solver, ctx.U = solver, Un
        return torch.from_numpy(solver.rhs(Un))

    @staticmethod
    def backward(ctx, grad_R):
        g = ctx.solver.rhs_vjp(ctx.U, np.ascontiguousarray(grad_R.detach().cpu().numpy()))
        return torch.from_numpy(g), None


def rhs(U, solver):
    """R(U) = calculateFunctionF at U, differentiable with respect to U."""
    return RhsFunction.apply(U, solver)
