"""torch.autograd binding of the discrete adjoint: a differentiable SSP-RK trajectory.

    u_final = trajectory(solver, u0, mu, steps, dt, checkpoint_interval)

u0 is the state at the volume points ([points][d+2] conserved, float64), mu a 0-d float64 tensor (the
dynamic viscosity; Navier-Stokes handles only).  The forward runs sdg_forward_steps on the GPU (the
steps with their checkpoints kept); backward runs sdg_adjoint_recorded (the checkpointed reverse sweep of
that trajectory; if the solver's state changed in between, it replays the forward first) and returns dL/du0 and dL/dmu for any loss L computed in
torch from u_final, e.g. the kinetic energy sum(w * rho |u|^2 / 2) with w = solver.volume_weights().
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi


class _Trajectory(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, mu, solver, steps, dt, interval):
        ns = solver.config.equation == _abi.NAVIER_STOKES
        if ns:
            solver.set_viscosity(float(mu))
        u0_host = u0.detach().to("cpu", torch.float64).contiguous().numpy()
        solver.set_state_point(u0_host)
        solver.forward_steps(dt, steps, interval)  # keeps the checkpoints for the backward pass
        uN = solver.state_point()
        ctx.solver, ctx.steps, ctx.dt, ctx.interval, ctx.ns = solver, steps, dt, interval, ns
        ctx.u0 = u0_host.copy()
        ctx.mu = float(mu)
        ctx.device = u0.device
        return torch.from_numpy(uN).to(u0.device)

    @staticmethod
    def backward(ctx, grad_uN):
        s = ctx.solver
        g = grad_uN.detach().to("cpu", torch.float64).contiguous().numpy()
        try:
            lam0, mubar = s.adjoint_recorded(g)     # the forward's trajectory is still the solver's state
        except _abi.SdgError as e:
            if e.code != _abi.SDG_ERR_STATE:
                raise
            if ctx.ns:                              # the solver was used in between: replay the forward
                s.set_viscosity(ctx.mu)
            s.set_state_point(ctx.u0)
            lam0, mubar = s.adjoint_steps(ctx.dt, ctx.steps, g, ctx.interval)
        dmu = torch.tensor(mubar if ctx.ns else 0.0, dtype=torch.float64)
        return torch.from_numpy(np.ascontiguousarray(lam0)).to(ctx.device), dmu, None, None, None, None


def trajectory(solver, u0: torch.Tensor, mu: torch.Tensor, steps: int, dt: float, checkpoint_interval: int = 25):
    """U_N as a differentiable function of (u0, mu) through `steps` steps of size dt."""
    return _Trajectory.apply(u0, mu, solver, steps, dt, checkpoint_interval)


def kinetic_energy(solver, u: torch.Tensor) -> torch.Tensor:
    """Integral of rho |u|^2 / 2 over the domain from point values (volume-point quadrature)."""
    w = torch.from_numpy(solver.volume_weights()).to(u.device)
    d = u.shape[1] - 2
    rho, m = u[:, 0], u[:, 1:1 + d]
    return torch.sum(w * 0.5 * torch.sum(m * m, 1) / rho)
