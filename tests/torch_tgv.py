"""A plain FP64 PyTorch statement of the periodic 3D central scheme (test infrastructure).

Same discretisation as the generated Taylor-Green solver (apps/taylor_green_vortex/taylor_green_vortex.py
with the 4th-order central skew-symmetric convective terms, constant-viscosity viscous and heat-flux
terms, 2-register RK3 of schemes/temporal/rk_sbli.py:117-124) on a periodic [0, 2pi)^3 box, written
with torch.roll stencils so that torch.autograd can differentiate whole trajectories.  It is the
autograd reference for the hand-written adjoint kernels; it is never used by the library.

Arrays are [var][z][y][x] (x fastest), conserved variables (rho, rhou0, rhou1, rhou2, rhoE).
"""
import math

import torch

C1 = (1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0)
C2 = (-1.0 / 12.0, 4.0 / 3.0, -2.5, 4.0 / 3.0, -1.0 / 12.0)
RKOLD = (1.0 / 4.0, 3.0 / 20.0, 3.0 / 5.0)
RKNEW = (2.0 / 3.0, 5.0 / 12.0, 3.0 / 5.0)
DIM = {0: -1, 1: -2, 2: -3}  # axis d -> tensor dim of a [z][y][x] field


def shift(f, d, o):
    """f at offset o along axis d (periodic)."""
    return torch.roll(f, shifts=-o, dims=DIM[d])


def d1(f, d, idl):
    return (C1[0] * shift(f, d, -2) + C1[1] * shift(f, d, -1) + C1[3] * shift(f, d, 1) + C1[4] * shift(f, d, 2)) * idl[d]


def d2(f, d, idl):
    acc = sum(C2[t] * shift(f, d, t - 2) for t in range(5))
    return acc * idl[d] * idl[d]


class Params:
    def __init__(self, n, gama=1.4, Minf=0.1, Re=1600.0, Pr=0.71, viscous=True):
        self.n = n
        self.delta = tuple(2 * math.pi / k for k in n)
        self.idl = tuple(1.0 / dd for dd in self.delta)
        self.gama, self.Minf, self.Re, self.Pr = gama, Minf, Re, Pr
        self.gm1 = gama - 1.0
        self.gM2 = gama * Minf * Minf
        self.invRe = 1.0 / Re
        self.kT = 1.0 / ((gama - 1.0) * Minf * Minf * Pr * Re)
        if not viscous:
            self.invRe = self.kT = 0.0


def rhs(q, P):
    """Residual R(q) of the central scheme (convective skew-symmetric + viscous)."""
    idl = P.idl
    rho, E = q[0], q[4]
    u = [q[1 + c] / rho for c in range(3)]
    p = P.gm1 * (E - 0.5 * rho * u[0] * u[0] - 0.5 * rho * u[1] * u[1] - 0.5 * rho * u[2] * u[2])
    T = P.gM2 * p / rho
    du = [[d1(u[c], d, idl) for d in range(3)] for c in range(3)]
    divu = du[0][0] + du[1][1] + du[2][2]
    phi = [rho, rho * u[0], rho * u[1], rho * u[2], E]
    R = [torch.zeros_like(rho) for _ in range(5)]
    for v in range(5):
        acc = sum(d1(phi[v] * u[d], d, idl) + u[d] * d1(phi[v], d, idl) for d in range(3))
        R[v] = R[v] - 0.5 * (acc + phi[v] * divu)
    for d in range(3):
        R[1 + d] = R[1 + d] - d1(p, d, idl)
    R[4] = R[4] - sum(d1(p * u[d], d, idl) for d in range(3))
    # viscous and heat-flux terms
    d2u = [[d2(u[c], d, idl) for d in range(3)] for c in range(3)]
    lapT = sum(d2(T, d, idl) for d in range(3))
    mom = []
    for c in range(3):
        ddiv = d2u[c][c] + sum(d1(d1(u[e], min(c, e), idl), max(c, e), idl) for e in range(3) if e != c)
        m = P.invRe * (d2u[c][0] + d2u[c][1] + d2u[c][2] + ddiv / 3.0)
        mom.append(m)
        R[1 + c] = R[1 + c] + m
    e = P.kT * lapT
    for a in range(3):
        for b in range(3):
            tau = du[a][b] + du[b][a]
            if a == b:
                tau = tau - 2.0 / 3.0 * divu
            e = e + P.invRe * tau * du[a][b]
    e = e + u[0] * mom[0] + u[1] * mom[1] + u[2] * mom[2]
    R[4] = R[4] + e
    return torch.stack(R)


def rk3_step(q, dt, P):
    o = q
    for s in range(3):
        r = rhs(q, P)
        qn = o + dt * RKNEW[s] * r
        o = o + dt * RKOLD[s] * r
        q = qn
    return q


def base_fields(P, device="cpu"):
    """TGV base pressure and density on the grid (rho = gama Minf^2 p, the script's choice)."""
    n0, n1, n2 = P.n
    x = torch.arange(n0, dtype=torch.float64, device=device) * P.delta[0]
    y = torch.arange(n1, dtype=torch.float64, device=device) * P.delta[1]
    z = torch.arange(n2, dtype=torch.float64, device=device) * P.delta[2]
    Z, Y, X = torch.meshgrid(z, y, x, indexing="ij")
    p = 1.0 / (P.gama * P.Minf ** 2) + (torch.cos(2 * X) + torch.cos(2 * Y)) * (2 + torch.cos(2 * Z)) / 16.0
    rho = P.gM2 * p
    u = torch.stack([torch.sin(X) * torch.cos(Y) * torch.cos(Z), -torch.cos(X) * torch.sin(Y) * torch.cos(Z),
                     torch.zeros_like(X)])
    return p, rho, u


def state_from_velocity(vel, p, rho, P):
    """Conserved state with the given velocity field and the base pressure and density."""
    E = p / P.gm1 + 0.5 * rho * (vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2)
    return torch.stack([rho, rho * vel[0], rho * vel[1], rho * vel[2], E])


def kinetic_energy(q, P):
    """Volume-integrated kinetic energy, sum of 1/2 |rho u|^2 / rho times the cell volume."""
    dv = P.delta[0] * P.delta[1] * P.delta[2]
    return 0.5 * ((q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]).sum() * dv
