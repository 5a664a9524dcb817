"""GPU: the hand-written discrete adjoint (osb_adjoint_residual / osb_adjoint_step and the
checkpointed Rollout autograd Function) against torch.autograd through a plain FP64 PyTorch
statement of the same discretisation (tests/torch_tgv.py) and against central finite differences.

Bars: adjoint residual and adjoint step <= 1e-12 (max-normalised) against autograd; whole-trajectory
gradients at 32^3 <= 1e-10 against autograd; directional derivatives within 1e-5 (relative) of
central finite differences with h = 1e-6.
"""
import numpy as np
import pytest
import torch

from opensbli_gb300.adjoint import Rollout, ke_gradient_tgv, kinetic_energy, state_from_velocity, tgv_base
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver
import torch_tgv as TT

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def perturbed_state(n, seed, Minf=0.1):
    P = TT.Params(n, Minf=Minf)
    p, rho, u = TT.base_fields(P, device=DEV)
    g = torch.Generator(device=DEV).manual_seed(seed)
    u = u * (1 + 0.1 * torch.rand(u.shape, generator=g, device=DEV, dtype=torch.float64))
    p = p * (1 + 0.01 * torch.rand(p.shape, generator=g, device=DEV, dtype=torch.float64))
    return TT.state_from_velocity(u, p, rho, P)


def maxrel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("n,viscous", [((16, 14, 12), True), ((20, 16, 18), False)])
def test_adjoint_residual_matches_autograd(n, viscous):
    q = perturbed_state(n, 1)
    lam = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(2), device=DEV, dtype=torch.float64)
    P = TT.Params(n, viscous=viscous)
    qq = q.clone().requires_grad_(True)
    ref, = torch.autograd.grad((TT.rhs(qq, P) * lam).sum(), qq)
    s = Solver(tgv_plan(n, visc="const" if viscous else "none"))
    s.set_state64(q)
    out = s.adjoint_residual(lam)
    s.close()
    assert maxrel(out, ref) <= 1e-12


def test_adjoint_step_matches_autograd():
    n, dt = (16, 18, 14), 5e-3
    q = perturbed_state(n, 3)
    lam = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(4), device=DEV, dtype=torch.float64)
    P = TT.Params(n)
    qq = q.clone().requires_grad_(True)
    ref, = torch.autograd.grad((TT.rk3_step(qq, dt, P) * lam).sum(), qq)
    s = Solver(tgv_plan(n))
    s.set_state64(q)
    out = s.adjoint_step(lam, dt)
    q_after = s.state64()
    s.close()
    assert maxrel(out, ref) <= 1e-12
    assert torch.equal(q_after, q)  # the bound state is left unchanged


def test_rollout_gradient_matches_autograd_32():
    """dJ/du0 of the kinetic energy after 22 steps (checkpoints every 5: ragged last segment)."""
    n, nsteps, dt = (32, 32, 32), 22, 5e-3
    plan = tgv_plan(n)
    P = TT.Params(n)
    p, rho, base = TT.base_fields(P, device=DEV)
    u = base.clone().requires_grad_(True)
    q = TT.state_from_velocity(u, p, rho, P)
    for _ in range(nsteps):
        q = TT.rk3_step(q, dt, P)
    J_ref = TT.kinetic_energy(q, P)
    g_ref, = torch.autograd.grad(J_ref, u)
    s = Solver(plan)
    v = base.clone().requires_grad_(True)
    qT = Rollout.apply(state_from_velocity(v, p, rho, plan.gama), s, nsteps, dt, 5)
    J = kinetic_energy(qT, plan.delta)
    J.backward()
    s.close()
    assert abs(float(J) - float(J_ref)) <= 1e-12 * abs(float(J_ref))
    assert maxrel(v.grad, g_ref) <= 1e-10


def test_gradient_matches_finite_differences():
    n, nsteps, dt, h = 24, 40, 5e-3, 1e-6
    J, grad = ke_gradient_tgv(n, nsteps=nsteps, dt=dt, every=8)
    plan = tgv_plan(n)
    s = Solver(plan)
    p, rho, base = tgv_base(plan, s.device)

    def J_of(vel):
        s.set_state64(state_from_velocity(vel, p, rho, plan.gama))
        s.step(nsteps, dt)
        return float(kinetic_energy(s.state64(), plan.delta))

    for seed in range(4):
        d = torch.randn(base.shape, generator=torch.Generator(device=DEV).manual_seed(seed), device=DEV,
                        dtype=torch.float64)
        fd = (J_of(base + h * d) - J_of(base - h * d)) / (2 * h)
        ad = float((grad * d).sum())
        assert abs(fd - ad) <= 1e-5 * abs(ad), (seed, fd, ad)
    s.close()


@pytest.mark.parametrize("plan", [tgv_plan(16, precision="mixed"), tgv_plan(16, conv="weno5js", Minf=1.25,
                                                                       precision="mixed"),
                                  tgv_plan(16).replace(bc=(("symmetry", "symmetry"),) * 3)])
def test_adjoint_rejects_other_plans(plan):
    s = Solver(plan)
    s.init_tgv() if plan.bc[0][0] == "periodic" else None
    with pytest.raises(NotImplementedError):
        s.adjoint_residual(torch.zeros((5,) + s.shape, dtype=torch.float64, device=DEV))
    s.close()


# ---- WENO5-JS: the transposed characteristic flux difference (reverse mode through the Roe average,
# the eigenvectors, the LLF splitting and the nonlinear weights) plus the viscous adjoint, against
# central finite differences of the GPU's own FP64 residual and step ----

def _weno_case(n, viscous=True, conv="weno5js"):
    """A Taylor-Green state with additive momentum noise.  The LLF wave speed max|u_D| over a window
    is not differentiable where u_D vanishes on the whole window, which the unperturbed Taylor-Green
    field does on its symmetry lines (u_1 = 0 wherever cos x = 0); there the adjoint takes a one-sided
    derivative and central differences straddle the kink, so the checks use states without such
    lines."""
    plan = tgv_plan(n, conv=conv, Minf=1.25, visc="const" if viscous else "none")
    q = perturbed_state(n, 5, Minf=1.25)
    g = torch.Generator(device=DEV).manual_seed(8)
    q[1:4] += 0.05 * q[0] * torch.randn(q[1:4].shape, generator=g, device=DEV, dtype=torch.float64)
    return plan, q


@pytest.mark.parametrize("n,viscous", [((16, 14, 12), True), ((12, 16, 14), False)])
def test_weno_adjoint_residual_matches_finite_differences(n, viscous):
    plan, q = _weno_case(n, viscous)
    lam = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(6), device=DEV, dtype=torch.float64)
    s = Solver(plan)
    s.set_state64(q)
    adj = s.adjoint_residual(lam)
    # a small step: the wave speeds are maxima over windows, and a step straddling two nearly equal
    # candidates sees a kink the adjoint does not
    h = 1e-7
    for seed in range(3):
        v = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(10 + seed), device=DEV,
                        dtype=torch.float64) * q.abs().mean(dim=(1, 2, 3), keepdim=True)
        s.set_state64(q + h * v)
        rp = s.residual().double()
        s.set_state64(q - h * v)
        rm = s.residual().double()
        fd = float((lam * (rp - rm)).sum() / (2 * h))
        ad = float((adj * v).sum())
        assert abs(fd - ad) <= 1e-5 * abs(ad), (seed, fd, ad)
    s.close()


def test_weno_adjoint_step_matches_finite_differences():
    n, dt = (14, 12, 16), 2e-3
    plan, q = _weno_case(n)
    lam = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(7), device=DEV, dtype=torch.float64)
    s = Solver(plan)
    s.set_state64(q)
    adj = s.adjoint_step(lam, dt)
    assert torch.equal(s.state64(), q)
    h = 1e-6
    for seed in range(3):
        v = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(20 + seed), device=DEV,
                        dtype=torch.float64) * q.abs().mean(dim=(1, 2, 3), keepdim=True)
        s.set_state64(q + h * v)
        s.step(1, dt)
        qp = s.state64()
        s.set_state64(q - h * v)
        s.step(1, dt)
        qm = s.state64()
        fd = float((lam * (qp - qm)).sum() / (2 * h))
        ad = float((adj * v).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (seed, fd, ad)
    s.close()


def test_weno_rollout_gradient_matches_finite_differences():
    """dJ/du0 of the kinetic energy after 12 WENO5-JS steps at Mach 1.25 through the checkpointed
    Rollout (every 4 steps), against central differences of the forward solver."""
    n, nsteps, dt, h = 16, 12, 2e-3, 1e-6
    plan = tgv_plan(n, conv="weno5js", Minf=1.25)
    s = Solver(plan)
    p, rho, base = tgv_base(plan, s.device)
    # additive noise: no window with u_D = 0 throughout (see _weno_case)
    base = base + 0.05 * torch.randn(base.shape, generator=torch.Generator(device=DEV).manual_seed(9), device=DEV,
                                     dtype=torch.float64)
    v = base.clone().requires_grad_(True)
    qT = Rollout.apply(state_from_velocity(v, p, rho, plan.gama), s, nsteps, dt, 4)
    J = kinetic_energy(qT, plan.delta)
    J.backward()
    grad = v.grad.detach()

    def J_of(vel):
        s.set_state64(state_from_velocity(vel, p, rho, plan.gama))
        s.step(nsteps, dt)
        return float(kinetic_energy(s.state64(), plan.delta))

    for seed in range(3):
        d = torch.randn(base.shape, generator=torch.Generator(device=DEV).manual_seed(30 + seed), device=DEV,
                        dtype=torch.float64)
        fd = (J_of(base + h * d) - J_of(base - h * d)) / (2 * h)
        ad = float((grad * d).sum())
        assert abs(fd - ad) <= 1e-5 * abs(ad), (seed, fd, ad)
    s.close()


@pytest.mark.parametrize("conv,tol", [("weno5z", 1e-4), ("teno5", 1e-5), ("teno6", 1e-5)])
def test_characteristic_adjoint_residual_matches_finite_differences(conv, tol):
    """WENO5-Z (its eps = 1e-14 makes the weights too ill-conditioned on smooth data for central
    differences to resolve them closely, hence the looser bar) and TENO5/TENO6 (weights constant between
    cut-off switches; the smaller of two steps' errors, since a step may straddle a switch)."""
    plan, q = _weno_case((14, 12, 16), True, conv)
    lam = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(11), device=DEV, dtype=torch.float64)
    s = Solver(plan)
    s.set_state64(q)
    adj = s.adjoint_residual(lam)
    for seed in range(3):
        v = torch.randn(q.shape, generator=torch.Generator(device=DEV).manual_seed(40 + seed), device=DEV,
                        dtype=torch.float64) * q.abs().mean(dim=(1, 2, 3), keepdim=True)
        ad = float((adj * v).sum())
        errs = []
        for h in (1e-6, 1e-7):
            s.set_state64(q + h * v)
            rp = s.residual().double()
            s.set_state64(q - h * v)
            rm = s.residual().double()
            errs.append(abs(float((lam * (rp - rm)).sum() / (2 * h)) - ad) / abs(ad))
        assert min(errs) <= tol, (conv, seed, errs)
    s.close()
