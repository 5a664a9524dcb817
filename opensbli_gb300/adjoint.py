"""Gradients through the time loop: the hand-written discrete adjoint of the periodic central scheme
and of its RK3 step (osb_adjoint_step, FP64) behind a torch.autograd.Function, with checkpointing.

The reference has no adjoint; this is the differentiable counterpart of its Taylor-Green time loop
(apps/taylor_green_vortex/taylor_green_vortex.py: central skew-symmetric convective terms,
constant-viscosity viscous terms, RK3 of schemes/temporal/rk_sbli.py).

    q_T = Rollout.apply(q0, solver, nsteps, dt, every)

runs `nsteps` RK3 steps of `dt` from the FP64 state q0 ([5][n2][n1][n0], on the solver's device),
keeping the state every `every` steps; its backward re-runs each segment from its checkpoint,
keeps that segment's step states, and applies the adjoint step to them in reverse order.  Memory:
nsteps/every checkpoints plus `every` step states.  Everything around it (the map from an initial
velocity to the state, the objective) is ordinary differentiable torch code, e.g.
ke_gradient_tgv().
"""
import math

import torch

from .plan import tgv_plan
from .runtime import Solver


class Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q0, solver, nsteps, dt, every):
        every = max(1, int(every))
        solver.set_state64(q0.detach())
        ckpts = [q0.detach().clone()]
        done = 0
        while done < nsteps:
            k = min(every, nsteps - done)
            solver.step(k, dt)
            done += k
            if done < nsteps:
                ckpts.append(solver.state64())
        qT = solver.state64()
        ctx.solver, ctx.nsteps, ctx.dt, ctx.every, ctx.ckpts = solver, nsteps, dt, every, ckpts
        return qT

    @staticmethod
    def backward(ctx, grad_qT):
        s, dt, every, nsteps = ctx.solver, ctx.dt, ctx.every, ctx.nsteps
        lam = grad_qT.detach().to(torch.float64).contiguous()
        for seg in reversed(range(len(ctx.ckpts))):
            start = seg * every
            nseg = min(every, nsteps - start)
            states = [ctx.ckpts[seg]]
            s.set_state64(states[0])
            for _ in range(nseg - 1):
                s.step(1, dt)
                states.append(s.state64())
            for t in reversed(range(nseg)):
                s.set_state64(states[t])
                lam = s.adjoint_step(lam, dt)
        ctx.ckpts = None
        return lam, None, None, None, None


def tgv_base(plan, device):
    """Base pressure and density of the Taylor-Green initial condition on the grid
    (apps/taylor_green_vortex/taylor_green_vortex.py:87-101: rho = gama Minf^2 p)."""
    n0, n1, n2 = plan.n
    ax = [torch.arange(n, dtype=torch.float64, device=device) * d for n, d in zip(plan.n, plan.delta)]
    Z, Y, X = torch.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    p = 1.0 / (plan.gama * plan.Minf ** 2) + (torch.cos(2 * X) + torch.cos(2 * Y)) * (2 + torch.cos(2 * Z)) / 16.0
    rho = plan.gama * plan.Minf ** 2 * p
    vel = torch.stack([torch.sin(X) * torch.cos(Y) * torch.cos(Z), -torch.cos(X) * torch.sin(Y) * torch.cos(Z),
                       torch.zeros_like(X)])
    return p, rho, vel


def state_from_velocity(vel, p, rho, gama):
    """Conserved state [5][z][y][x] with velocity `vel` [3][z][y][x] and the given p, rho."""
    E = p / (gama - 1.0) + 0.5 * rho * (vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2)
    return torch.stack([rho, rho * vel[0], rho * vel[1], rho * vel[2], E])


def kinetic_energy(q, delta):
    """Volume-integrated kinetic energy: sum of |rho u|^2 / (2 rho) times the cell volume."""
    return 0.5 * ((q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]).sum() * (delta[0] * delta[1] * delta[2])


def ke_gradient_tgv(n, vel0=None, nsteps=400, dt=5e-3, every=20, Minf=0.1, Re=1600.0, solver=None):
    """Kinetic energy at t = nsteps*dt of the periodic central Taylor-Green run started from the
    velocity field vel0 ([3][n][n][n] FP64; default the Taylor-Green field), and its gradient with
    respect to vel0.  Returns (J, dJ/dvel0)."""
    plan = tgv_plan(n, conv="central_skew", precision="fp64", Minf=Minf, Re=Re)
    own = solver is None
    s = solver or Solver(plan)
    p, rho, base = tgv_base(plan, s.device)
    v = (base if vel0 is None else vel0.to(s.device, torch.float64)).clone().requires_grad_(True)
    q0 = state_from_velocity(v, p, rho, plan.gama)
    qT = Rollout.apply(q0, s, nsteps, dt, every)
    J = kinetic_energy(qT, plan.delta)
    J.backward()
    if own:
        s.close()
    return J.detach(), v.grad.detach()
