// osb_adjoint.cu -- discrete adjoint of the periodic central and WENO5-JS schemes and of their RK3
// step (FP64).
//
// The forward residual (osb_central.cu; the generated Taylor-Green solver's convective
// skew-symmetric and constant-viscosity viscous terms) is, at every point, a function of point
// values and of central-difference stencils applied to point "features" (rho u_c, p, T, the
// conserved vector and products of them).  Its transpose splits into
//   pass 1 (at every point i, forward stencils + the adjoint input lambda_i): the sensitivity of
//     lambda_i . R_i to every stencil value it uses, combined per (feature, stencil, axis) into
//     29 fields, and the pointwise part of the feature adjoints (8 fields);
//   periodic halos of those fields;
//   pass 2 (at every point j): the transposed stencils gathered at j (a periodic first-derivative
//     stencil transposes to minus itself, second and nested mixed derivatives to themselves) plus
//     the pointwise parts, then the chain rule from the features to the conserved variables.
// With s[X] = d(lambda.R)/d(stencil value X):
//   s[D_d(phi_v u_d)] = -1/2 lambda_v      s[D_d phi_v] = -1/2 lambda_v u_d
//   s[D_b u_a] = delta_ab sigma + 2/Re lambda_4 tau_ab, sigma = -1/2 sum_v lambda_v phi_v
//   s[D_d p] = -lambda_{1+d}   s[D_d (p u_d)] = -lambda_4   s[D2_d T] = kT lambda_4
//   s[D2_d u_c] = kappa_c (1 + delta_cd / 3) / Re,   s[D_{min(c,e)} D_{max(c,e)} u_e] = kappa_c / (3 Re),
//   kappa_c = lambda_{1+c} + lambda_4 u_c.
// The 2-register RK3 step (schemes/temporal/rk_sbli.py:117-124) is reversed stage by stage from the
// recomputed stage states.  With characteristic fluxes (WENO5-JS, WENO5-Z, TENO5, TENO6) the
// convective part is replaced by the transpose of the flux difference (k_adj_weno, the reverse mode
// of osb_adjoint_weno.cuh) and the passes above carry the viscous and heat-flux terms only.  Periodic
// FP64 plans are accepted.
#include <cstdio>
#include <type_traits>

#include "osb_adjoint_weno.cuh"
#include "osb_common.cuh"
#include "osb_internal.h"

namespace osb {

namespace {
constexpr int NA_HALO = 29;  // lambda_v u_d (15), kappa_c (3), S_ab (6), lambda (5)
constexpr int NA = NA_HALO + 8;  // + pointwise u-part (3) and phi-part (5)
enum { A_LU = 0, A_KAP = 15, A_S = 18, A_LAM = 24, A_LOCU = 29, A_LOCPHI = 32 };
// S_ab storage: (0,0) (1,1) (2,2) (0,1) (0,2) (1,2)
__host__ __device__ constexpr int s_idx(int a, int b) {
  return a == b ? a : (a + b == 1 ? 3 : (a + b == 2 ? 4 : 5));
}

struct FieldSet {
  double *f[NA];
};
struct Prim5 {
  double *u[3];
  double *p, *T;
};

__device__ __forceinline__ double c1w(int t) {
  return t == 0 ? 1.0 / 12.0 : t == 1 ? -2.0 / 3.0 : t == 2 ? 0.0 : t == 3 ? 2.0 / 3.0 : -1.0 / 12.0;
}
__device__ __forceinline__ double c2w(int t) {
  return t == 0 ? -1.0 / 12.0 : t == 1 ? 4.0 / 3.0 : t == 2 ? -2.5 : t == 3 ? 4.0 / 3.0 : -1.0 / 12.0;
}
}  // namespace

// point primitives over the whole padded array (the state's halos are filled)
__global__ void k_adj_prims(int64_t numel, Fields5<const double> q, Prim5 pr, double gm1, double gM2) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < numel; t += (int64_t)gridDim.x * blockDim.x) {
    const double rho = q.v[0][t];
    if (!(rho > 0.0)) {  // unused padding
      pr.u[0][t] = pr.u[1][t] = pr.u[2][t] = pr.p[t] = pr.T[t] = 0.0;
      continue;
    }
    const double ir = 1.0 / rho;
    const double u0 = q.v[1][t] * ir, u1 = q.v[2][t] * ir, u2 = q.v[3][t] * ir;
    const double p = gm1 * (q.v[4][t] - 0.5 * rho * u0 * u0 - 0.5 * rho * u1 * u1 - 0.5 * rho * u2 * u2);
    pr.u[0][t] = u0;
    pr.u[1][t] = u1;
    pr.u[2][t] = u2;
    pr.p[t] = p;
    pr.T[t] = gM2 * p * ir;
  }
}

// conv = 0 (characteristic-flux plans): the skew-symmetric convective sensitivities are zero and only
// the viscous and heat-flux ones are formed; the flux adjoint comes from k_adj_weno.
__global__ void k_adj_pass1(Grid g, Fields5<const double> q, Prim5 pr, FieldSet A, Phys ph, int conv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n0) return;
  const int64_t n = gidx(g, i, j, k);
  const int64_t st[3] = {1, g.sy, g.sz};
  const double idl[3] = {ph.inv_delta[0], ph.inv_delta[1], ph.inv_delta[2]};
  const double invRe = ph.invRe;
  // forward stencil values at n
  double du[3][3], dphi[5][3], d2u[3][3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double a1 = 0, a2 = 0;
#pragma unroll
      for (int t = 0; t < 5; ++t) {
        const double v = pr.u[c][n + (t - 2) * st[d]];
        a1 += c1w(t) * v;
        a2 += c2w(t) * v;
      }
      du[c][d] = a1 * idl[d];
      d2u[c][d] = a2 * idl[d] * idl[d];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double a1 = 0;
#pragma unroll
      for (int t = 0; t < 5; ++t) a1 += c1w(t) * q.v[v][n + (t - 2) * st[d]];
      dphi[v][d] = a1 * idl[d];
    }
  }
  auto mixed = [&](int e, int a, int b) -> double {  // D_b (D_a u_e), a < b
    double outer = 0;
#pragma unroll
    for (int tb = 0; tb < 5; ++tb) {
      if (tb == 2) continue;
      double inner = 0;
#pragma unroll
      for (int ta = 0; ta < 5; ++ta) {
        if (ta == 2) continue;
        inner += c1w(ta) * pr.u[e][n + (ta - 2) * st[a] + (tb - 2) * st[b]];
      }
      outer += c1w(tb) * (inner * idl[a]);
    }
    return outer * idl[b];
  };
  const double divu = du[0][0] + du[1][1] + du[2][2];
  double mom[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double ddiv = d2u[c][c];
#pragma unroll
    for (int e = 0; e < 3; ++e)
      if (e != c) ddiv += mixed(e, c < e ? c : e, c < e ? e : c);
    mom[c] = invRe * (d2u[c][0] + d2u[c][1] + d2u[c][2] + ddiv / 3.0);
  }
  double L[5], phi[5], u[3];
  const double cv = conv ? 1.0 : 0.0;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    L[v] = A.f[A_LAM + v][n];
    phi[v] = q.v[v][n];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = pr.u[c][n];
#pragma unroll
  for (int v = 0; v < 5; ++v)
#pragma unroll
    for (int d = 0; d < 3; ++d) A.f[A_LU + 3 * v + d][n] = cv * L[v] * u[d];
#pragma unroll
  for (int c = 0; c < 3; ++c) A.f[A_KAP + c][n] = L[1 + c] + L[4] * u[c];
  double sigma = 0;
#pragma unroll
  for (int v = 0; v < 5; ++v) sigma += L[v] * phi[v];
  sigma *= -0.5 * cv;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      double tau = du[a][b] + du[b][a];
      if (a == b) tau -= 2.0 / 3.0 * divu;
      A.f[A_S + s_idx(a, b)][n] = (a == b ? sigma : 0.0) + 2.0 * invRe * L[4] * tau;
    }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double s = 0;
#pragma unroll
    for (int v = 0; v < 5; ++v) s += L[v] * dphi[v][c];
    A.f[A_LOCU + c][n] = -0.5 * cv * s + L[4] * mom[c];
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) A.f[A_LOCPHI + v][n] = -0.5 * cv * L[v] * divu;
}

__global__ void k_adj_pass2(Grid g, Fields5<const double> q, Prim5 pr, FieldSet A, Phys ph, double *out, double scale,
                            int conv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n0) return;
  const int64_t n = gidx(g, i, j, k);
  const int64_t st[3] = {1, g.sy, g.sz};
  const double idl[3] = {ph.inv_delta[0], ph.inv_delta[1], ph.inv_delta[2]};
  const double invRe = ph.invRe, kT = ph.kT, gm1 = ph.gm1, gM2 = ph.gM2;
  auto D1 = [&](const double *f, int d) -> double {
    double a = 0;
#pragma unroll
    for (int t = 0; t < 5; ++t)
      if (t != 2) a += c1w(t) * f[n + (t - 2) * st[d]];
    return a * idl[d];
  };
  auto D2 = [&](const double *f, int d) -> double {
    double a = 0;
#pragma unroll
    for (int t = 0; t < 5; ++t) a += c2w(t) * f[n + (t - 2) * st[d]];
    return a * idl[d] * idl[d];
  };
  auto MX = [&](const double *f, int a, int b) -> double {  // D_b D_a f, a < b
    double outer = 0;
#pragma unroll
    for (int tb = 0; tb < 5; ++tb) {
      if (tb == 2) continue;
      double inner = 0;
#pragma unroll
      for (int ta = 0; ta < 5; ++ta) {
        if (ta == 2) continue;
        inner += c1w(ta) * f[n + (ta - 2) * st[a] + (tb - 2) * st[b]];
      }
      outer += c1w(tb) * (inner * idl[a]);
    }
    return outer * idl[b];
  };
  double u[3], phi[5];
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = pr.u[c][n];
#pragma unroll
  for (int v = 0; v < 5; ++v) phi[v] = q.v[v][n];
  const double p = pr.p[n], T = pr.T[n], rho = phi[0];
  double DL[5][3];
#pragma unroll
  for (int v = 0; v < 5; ++v)
#pragma unroll
    for (int d = 0; d < 3; ++d) DL[v][d] = D1(A.f[A_LAM + v], d);
  double Gphi[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double a = 0, b = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      a += D1(A.f[A_LU + 3 * v + d], d);
      b += u[d] * DL[v][d];
    }
    Gphi[v] = conv ? 0.5 * a + 0.5 * b + A.f[A_LOCPHI + v][n] : 0.0;
  }
  double Gu[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double g = 0;
#pragma unroll
    for (int b = 0; b < 3; ++b) g -= D1(A.f[A_S + s_idx(c, b)], b);
    const double *kap = A.f[A_KAP + c];
    g += invRe * (D2(kap, 0) + D2(kap, 1) + D2(kap, 2) + D2(kap, c) / 3.0);
#pragma unroll
    for (int e = 0; e < 3; ++e)
      if (e != c) g += invRe / 3.0 * MX(A.f[A_KAP + e], c < e ? c : e, c < e ? e : c);
    double s = 0;
#pragma unroll
    for (int v = 0; v < 5; ++v) s += phi[v] * DL[v][c];
    g += A.f[A_LOCU + c][n] + (conv ? 0.5 * s + p * DL[4][c] : 0.0);
    Gu[c] = g;
  }
  double Gp = 0, GT = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (conv) Gp += DL[1 + d][d] + u[d] * DL[4][d];
    GT += D2(A.f[A_LAM + 4], d);
  }
  GT *= kT;
  const double ir = 1.0 / rho;
  const double Gpt = Gp + gM2 * ir * GT;
  const double usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  double Grho = Gphi[0] - T * ir * GT - 0.5 * gm1 * usq * Gpt;
  double Gut[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Grho += u[c] * Gphi[1 + c];
    Gut[c] = Gu[c] + rho * Gphi[1 + c] - gm1 * rho * u[c] * Gpt;
  }
  const double GE = Gphi[4] + gm1 * Gpt;
  const int64_t m = (int64_t)i + (int64_t)g.n0 * (j + (int64_t)g.n1 * k);  // dense interior index
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  out[m] = scale * (Grho - ir * (u[0] * Gut[0] + u[1] * Gut[1] + u[2] * Gut[2]));
#pragma unroll
  for (int c = 0; c < 3; ++c) out[(1 + c) * N + m] = scale * Gut[c] * ir;
  out[4 * N + m] = scale * GE;
}

// The characteristic WENO5-JS flux along D, transposed.  The forward residual of cell c is
// -(F_{c+1/2} - F_{c-1/2}) / delta_D with the interface fluxes of left points L = -1 .. n-1 computed
// on the periodically filled state, so an interface's flux adjoint is
//   F_bar(L) = (lambda_{L+1} [L+1 < n] - lambda_L [L >= 0]) / delta_D,
// and its window's six points receive (dF/dQ)^T F_bar, folded back onto their periodic images.  One
// thread per interface; the contributions of the six interfaces sharing a point meet in FP64 atomics.
template <int D, int SCH>
__global__ void k_adj_weno(Grid g, Fields5<const double> q, FieldSet A, Phys ph, double *out, double scale) {
  const int nd = D == 0 ? g.n0 : D == 1 ? g.n1 : g.n2;
  const int na = D == 0 ? g.n1 : g.n0, nb = D == 2 ? g.n1 : g.n2;  // transverse extents
  const int64_t total = (int64_t)(nd + 1) * na * nb;
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  const int64_t sd = D == 0 ? 1 : D == 1 ? g.sy : g.sz;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int L = (int)(w % (nd + 1)) - 1;
    const int64_t rest = w / (nd + 1);
    const int ia = (int)(rest % na), ib = (int)(rest / na);
    int i = 0, j = 0, k = 0;  // coordinates of the left point
    if (D == 0) { i = L; j = ia; k = ib; }
    else if (D == 1) { i = ia; j = L; k = ib; }
    else { i = ia; j = ib; k = L; }
    const int64_t nL = gidx(g, i, j, k);
    double Fb[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double f = 0.0;
      if (L >= 0) f -= A.f[A_LAM + v][nL];
      if (L + 1 < nd) f += A.f[A_LAM + v][nL + sd];
      Fb[v] = f * ph.inv_delta[D];
    }
    double Q[6][5], Qb[6][5];
#pragma unroll
    for (int t = 0; t < 6; ++t)
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        Q[t][v] = q.v[v][nL + (int64_t)(t - 2) * sd];
        Qb[t][v] = 0.0;
      }
    adjw::interface_flux_adj<D, SCH>(Q, Fb, ph.gama, Qb, nullptr, ph.weno_eps, ph.teno_ct);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const int c = ((L - 2 + t) % nd + nd) % nd;
      const int64_t m = D == 0 ? (int64_t)c + (int64_t)g.n0 * (j + (int64_t)g.n1 * k)
                        : D == 1 ? (int64_t)i + (int64_t)g.n0 * (c + (int64_t)g.n1 * k)
                                 : (int64_t)i + (int64_t)g.n0 * (j + (int64_t)g.n1 * c);
#pragma unroll
      for (int v = 0; v < 5; ++v) atomicAdd(out + v * N + m, scale * Qb[t][v]);
    }
  }
}

}  // namespace osb

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
namespace osb {

namespace {
struct PtrList {
  double *f[NA];
  int nf;
};

// periodic halos of nf padded FP64 fields, one axis per launch (x, y, z: corners come out right)
__global__ void k_adj_halo(Grid g, PtrList L, int axis, int depth) {
  const int n[3] = {g.n0, g.n1, g.n2};
  const int ha[3] = {HX, HY, HZ};
  const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
  const int eb = n[b] + 2 * ha[b], ec = n[c] + 2 * ha[c];
  const int64_t total = (int64_t)2 * depth * eb * ec;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    const int ib = (int)(r % eb) - ha[b];
    r /= eb;
    const int ic = (int)(r % ec) - ha[c];
    r /= ec;
    const int dd = (int)(r % depth) + 1;
    const int side = (int)(r / depth);
    int to[3], fr[3];
    to[b] = fr[b] = ib;
    to[c] = fr[c] = ic;
    if (side == 0) { to[axis] = -dd; fr[axis] = n[axis] - dd; }
    else { to[axis] = n[axis] - 1 + dd; fr[axis] = dd - 1; }
    const int64_t it = gidx(g, to[0], to[1], to[2]), ifr = gidx(g, fr[0], fr[1], fr[2]);
    for (int f = 0; f < L.nf; ++f) L.f[f][it] = L.f[f][ifr];
  }
}

// lambda_r = a x + b y (dense interior inputs, y may be null) into the padded lambda fields
__global__ void k_adj_lam(Grid g, const double *x, const double *y, double a, double b, FieldSet A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n0) return;
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  const int64_t m = (int64_t)i + (int64_t)g.n0 * (j + (int64_t)g.n1 * k);
  const int64_t n = gidx(g, i, j, k);
#pragma unroll
  for (int v = 0; v < 5; ++v) A.f[A_LAM + v][n] = a * x[v * N + m] + (y ? b * y[v * N + m] : 0.0);
}

// out = x + y (+ z), dense; any of the inputs may alias out
__global__ void k_adj_sum(int64_t n, double *out, const double *x, const double *y, const double *z) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    out[t] = x[t] + y[t] + (z ? z[t] : 0.0);
}

__global__ void k_adj_copy5(int64_t n, Fields5<const double> a, Fields5<double> b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int v = 0; v < 5; ++v) b.v[v][t] = a.v[v][t];
}

int grid_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? b : 152 * 32);
}
}  // namespace

void adj_halos(const Ctx &c, double *const *f, int nf, cudaStream_t s, int64_t *launches) {
  PtrList L{};
  L.nf = nf;
  for (int i = 0; i < nf; ++i) L.f[i] = f[i];
  const int n[3] = {c.g.n0, c.g.n1, c.g.n2};
  const int ha[3] = {HX, HY, HZ};
  for (int axis = 0; axis < 3; ++axis) {
    const int b = axis == 0 ? 1 : 0, cc = axis == 2 ? 1 : 2;
    const int64_t total = (int64_t)2 * 2 * (n[b] + 2 * ha[b]) * (n[cc] + 2 * ha[cc]);
    k_adj_halo<<<grid_blocks(total), 256, 0, s>>>(c.g, L, axis, 2);
    ++*launches;
  }
}
}  // namespace osb

namespace osb {

namespace {
struct AdjView {
  Fields5<double> Q1, Q2, O;
  Prim5 pr;
  FieldSet A;
  double *lq, *lo, *mu;  // dense [5][n2][n1][n0]
};

AdjView adj_view(const Ctx &c) {
  AdjView v{};
  double *p = c.adj;
  const int64_t m = c.g.numel, N = (int64_t)c.g.n0 * c.g.n1 * c.g.n2;
  for (int f = 0; f < 5; ++f) v.Q1.v[f] = p + (0 + f) * m;
  for (int f = 0; f < 5; ++f) v.Q2.v[f] = p + (5 + f) * m;
  for (int f = 0; f < 5; ++f) v.O.v[f] = p + (10 + f) * m;
  for (int f = 0; f < 3; ++f) v.pr.u[f] = p + (15 + f) * m;
  v.pr.p = p + 18 * m;
  v.pr.T = p + 19 * m;
  for (int f = 0; f < NA; ++f) v.A.f[f] = p + (20 + f) * m;
  double *d = p + (20 + NA) * m;
  v.lq = d;
  v.lo = d + 5 * N;
  v.mu = d + 10 * N;
  return v;
}

Fields5<const double> cq(Fields5<double> a) {
  Fields5<const double> b;
  for (int v = 0; v < 5; ++v) b.v[v] = a.v[v];
  return b;
}

// physical constants of the adjoint: viscous terms switched off for inviscid plans
Phys adj_phys(const Ctx &c) {
  Phys ph = c.ph;
  if (c.plan.visc != OSB_VISC_CONST) ph.invRe = ph.kT = 0.0;
  return ph;
}

// out (dense) = scale * (dR/dq)^T(qs) lambda, lambda already in the A_LAM fields' interior;
// qs padded with filled halos
void adj_rhs(Ctx &c, const AdjView &v, Fields5<double> qs, double *out, double scale, cudaStream_t s) {
  const Phys ph = adj_phys(c);
  adj_halos(c, v.A.f + A_LAM, 5, s, &c.launches);
  k_adj_prims<<<grid_blocks(c.g.numel), 256, 0, s>>>(c.g.numel, cq(qs), v.pr, ph.gm1, ph.gM2);
  const dim3 grid((c.g.n0 + 127) / 128, c.g.n1, c.g.n2);
  const int conv = c.plan.conv == OSB_CONV_CENTRAL_SKEW ? 1 : 0;
  k_adj_pass1<<<grid, 128, 0, s>>>(c.g, cq(qs), v.pr, v.A, ph, conv);
  adj_halos(c, v.A.f, NA_HALO, s, &c.launches);
  k_adj_pass2<<<grid, 128, 0, s>>>(c.g, cq(qs), v.pr, v.A, ph, out, scale, conv);
  c.launches += 3;
  if (!conv) {  // characteristic fluxes: their transposes, added into out
    const int64_t per = (int64_t)c.g.n0 * c.g.n1 * c.g.n2;
    const int nb = grid_blocks(per + per / 8 + 1);
    auto launch = [&](auto sch) {
      constexpr int S = decltype(sch)::value;
      k_adj_weno<0, S><<<nb, 128, 0, s>>>(c.g, cq(qs), v.A, ph, out, scale);
      k_adj_weno<1, S><<<nb, 128, 0, s>>>(c.g, cq(qs), v.A, ph, out, scale);
      k_adj_weno<2, S><<<nb, 128, 0, s>>>(c.g, cq(qs), v.A, ph, out, scale);
    };
    switch (c.plan.conv) {
      case OSB_CONV_WENO5Z: launch(std::integral_constant<int, adjw::ADJ_Z>{}); break;
      case OSB_CONV_TENO5: launch(std::integral_constant<int, adjw::ADJ_TENO5>{}); break;
      case OSB_CONV_TENO6: launch(std::integral_constant<int, adjw::ADJ_TENO6>{}); break;
      default: launch(std::integral_constant<int, adjw::ADJ_JS>{}); break;
    }
    c.launches += 3;
  }
}

// one forward RK3 stage of the plan from qs into qn (the FP64 register o updated): the same kernels as
// the solver's step
void fwd_stage(Ctx &c, Fields5<double> qs, Fields5<double> qn, Fields5<double> o, Fields5<double> res, double dtn,
               double dto, cudaStream_t s) {
  const int visc = c.plan.visc == OSB_VISC_CONST ? CRK_VISC : 0;
  if (c.plan.conv == OSB_CONV_CENTRAL_SKEW) {
    launch_central_rk<double>(c, cq(qs), qn, o, res, res, dtn, dto, CRK_SKEW | visc | CRK_UPDATE, s, &c.launches);
    return;
  }
  for (int d = 0; d < 3; ++d) launch_weno_dir<double>(c, cq(qs), res, d, s, &c.launches);
  launch_central_rk<double>(c, cq(qs), qn, o, res, res, dtn, dto, CRK_RIN | visc | CRK_UPDATE, s, &c.launches);
}
}  // namespace

cudaError_t adj_ensure(Ctx &c) {
  if (c.adj) return cudaSuccess;
  const int64_t N = (int64_t)c.g.n0 * c.g.n1 * c.g.n2;
  const size_t bytes = sizeof(double) * ((size_t)(20 + NA) * c.g.numel + 15 * (size_t)N);
  cudaError_t e = cudaMalloc(&c.adj, bytes);
  if (e != cudaSuccess) {
    c.adj = nullptr;
    return e;
  }
  // zero once so that the padding outside the halos holds finite values
  return cudaMemsetAsync(c.adj, 0, bytes, c.stream);
}

cudaError_t adj_residual(Ctx &c, Fields5<double> q, const double *lam, double *out) {
  cudaStream_t s = c.stream;
  const AdjView v = adj_view(c);
  launch_halos<double>(c, q, s, &c.launches);
  const dim3 grid((c.g.n0 + 127) / 128, c.g.n1, c.g.n2);
  k_adj_lam<<<grid, 128, 0, s>>>(c.g, lam, nullptr, 1.0, 0.0, v.A);
  ++c.launches;
  adj_rhs(c, v, q, out, 1.0, s);
  return cudaGetLastError();
}

// lam_out = (d Phi / d q^n)^T lam_in for one 2-register RK3 step Phi of size dt from the state q
// (the bound state, left unchanged):
//   stage s: q_{s+1} = o_s + dt b_s R(q_s),  o_{s+1} = o_s + dt a_s R(q_s),  q_0 = o_0 = q^n;
//   reverse: lo = lam_in, lq = dt b_2 R^T(q_2) lam_in;
//            r1 = dt (b_1 lq + a_1 lo),  lo <- lq + lo,  lq <- R^T(q_1) r1;
//            r0 = dt (b_0 lq + a_0 lo),  lam_out = lq + lo + R^T(q^n) r0.
cudaError_t adj_step(Ctx &c, Fields5<double> q, double dt, const double *lam_in, double *lam_out) {
  cudaStream_t s = c.stream;
  const AdjView v = adj_view(c);
  const int64_t N5 = 5 * (int64_t)c.g.n0 * c.g.n1 * c.g.n2;
  const double *a = c.plan.rk_a, *b = c.plan.rk_b;
  Fields5<double> res;
  for (int f = 0; f < 5; ++f) res.v[f] = static_cast<double *>(c.res[f]);
  // forward stage states q_1, q_2
  launch_halos<double>(c, q, s, &c.launches);
  k_adj_copy5<<<grid_blocks(c.g.numel), 256, 0, s>>>(c.g.numel, cq(q), v.O);
  ++c.launches;
  fwd_stage(c, q, v.Q1, v.O, res, dt * b[0], dt * a[0], s);
  launch_halos<double>(c, v.Q1, s, &c.launches);
  fwd_stage(c, v.Q1, v.Q2, v.O, res, dt * b[1], dt * a[1], s);
  launch_halos<double>(c, v.Q2, s, &c.launches);
  // reverse
  const dim3 grid((c.g.n0 + 127) / 128, c.g.n1, c.g.n2);
  const int nb = grid_blocks(N5);
  k_adj_lam<<<grid, 128, 0, s>>>(c.g, lam_in, nullptr, dt * b[2], 0.0, v.A);
  adj_rhs(c, v, v.Q2, v.lq, 1.0, s);
  cudaMemcpyAsync(v.lo, lam_in, sizeof(double) * N5, cudaMemcpyDeviceToDevice, s);
  k_adj_lam<<<grid, 128, 0, s>>>(c.g, v.lq, v.lo, dt * b[1], dt * a[1], v.A);
  k_adj_sum<<<nb, 256, 0, s>>>(N5, v.lo, v.lq, v.lo, nullptr);
  adj_rhs(c, v, v.Q1, v.lq, 1.0, s);
  k_adj_lam<<<grid, 128, 0, s>>>(c.g, v.lq, v.lo, dt * b[0], dt * a[0], v.A);
  adj_rhs(c, v, q, v.mu, 1.0, s);
  k_adj_sum<<<nb, 256, 0, s>>>(N5, lam_out, v.lq, v.lo, v.mu);
  c.launches += 6;
  return cudaGetLastError();
}

}  // namespace osb
