"""The adjoint formulas the CUDA kernels implement (opensbli_gb300/csrc/osb_adjoint.cu: pass 1
sensitivities, pass 2 transposed stencils and the chain rule to the conserved variables), stated
with torch.roll stencils and checked against torch.autograd through tests/torch_tgv.py on CPU."""
import pytest
import torch

import torch_tgv as TT


def hand_adjoint(q, lam, P):
    idl = P.idl
    D = lambda f, d: TT.d1(f, d, idl)
    D2 = lambda f, d: TT.d2(f, d, idl)
    M = lambda f, a, b: TT.d1(TT.d1(f, min(a, b), idl), max(a, b), idl)
    rho, E = q[0], q[4]
    u = [q[1 + c] / rho for c in range(3)]
    p = P.gm1 * (E - 0.5 * rho * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2))
    T = P.gM2 * p / rho
    phi = [q[v] for v in range(5)]
    du = [[D(u[c], d) for d in range(3)] for c in range(3)]
    divu = du[0][0] + du[1][1] + du[2][2]
    mom = [P.invRe * (sum(D2(u[c], d) for d in range(3))
                      + (D2(u[c], c) + sum(M(u[e], c, e) for e in range(3) if e != c)) / 3) for c in range(3)]
    # pass 1
    lamu = [[lam[v] * u[d] for d in range(3)] for v in range(5)]
    kap = [lam[1 + c] + lam[4] * u[c] for c in range(3)]
    sig = -0.5 * sum(lam[v] * phi[v] for v in range(5))
    tau = [[du[a][b] + du[b][a] - (2 / 3 * divu if a == b else 0) for b in range(3)] for a in range(3)]
    S = [[(sig if a == b else 0) + 2 * P.invRe * lam[4] * tau[a][b] for b in range(3)] for a in range(3)]
    loc_u = [-0.5 * sum(lam[v] * D(phi[v], c) for v in range(5)) + lam[4] * mom[c] for c in range(3)]
    loc_phi = [-0.5 * lam[v] * divu for v in range(5)]
    # pass 2
    Gphi = [0.5 * sum(D(lamu[v][d], d) for d in range(3)) + 0.5 * sum(u[d] * D(lam[v], d) for d in range(3))
            + loc_phi[v] for v in range(5)]
    Gu = []
    for c in range(3):
        g = -sum(D(S[c][b], b) for b in range(3))
        g = g + P.invRe * (sum(D2(kap[c], d) for d in range(3)) + D2(kap[c], c) / 3)
        g = g + P.invRe / 3 * sum(M(kap[e], c, e) for e in range(3) if e != c)
        g = g + loc_u[c] + 0.5 * sum(phi[v] * D(lam[v], c) for v in range(5)) + p * D(lam[4], c)
        Gu.append(g)
    Gp = sum(D(lam[1 + d], d) for d in range(3)) + sum(u[d] * D(lam[4], d) for d in range(3))
    GT = P.kT * sum(D2(lam[4], d) for d in range(3))
    Gpt = Gp + P.gM2 / rho * GT
    Grho = Gphi[0] + sum(u[c] * Gphi[1 + c] for c in range(3)) - T / rho * GT \
        - 0.5 * P.gm1 * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2) * Gpt
    Gut = [Gu[c] + rho * Gphi[1 + c] - P.gm1 * rho * u[c] * Gpt for c in range(3)]
    GE = Gphi[4] + P.gm1 * Gpt
    return torch.stack([Grho - sum(u[c] / rho * Gut[c] for c in range(3))] + [Gut[c] / rho for c in range(3)] + [GE])


@pytest.mark.parametrize("n,viscous", [((12, 10, 8), True), ((9, 11, 10), False)])
def test_hand_adjoint_formulas_match_autograd(n, viscous):
    torch.manual_seed(0)
    P = TT.Params(n, viscous=viscous)
    p, rho, u = TT.base_fields(P)
    q = TT.state_from_velocity(u * (1 + 0.1 * torch.rand_like(u)), p * (1 + 0.01 * torch.rand_like(p)), rho, P)
    lam = torch.randn_like(q)
    qq = q.clone().requires_grad_(True)
    ref, = torch.autograd.grad((TT.rhs(qq, P) * lam).sum(), qq)
    mine = hand_adjoint(q, lam, P)
    assert float((mine - ref).abs().max() / ref.abs().max()) <= 1e-13
