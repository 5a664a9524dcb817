// osb_api.cu -- the C ABI (include/osb_gb300.h): contexts, binding, the time loop, reductions.
//
// The time loop restates TraditionalAlgorithmRK.generate_solution (algorithm.py:384-477) for one
// block: every RK stage fills the boundary halos of the current state, evaluates the residual and
// applies the RK update into the other state buffer; the FP64 RK register is the master copy, so
// the reference's per-iteration "Save equations" copy (rk_sbli.py:126-133) is needed only before
// the first step after the caller wrote the state itself.  One step (three stages) can be
// captured as a CUDA graph and replayed.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "osb_common.cuh"
#include "osb_internal.h"

using namespace osb;

struct osb_ctx : public Ctx {};

namespace {

int set_err(osb_ctx *c, int code, const char *msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_err(osb_ctx *c, cudaError_t e, const char *where) {
  if (e == cudaSuccess) return OSB_OK;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", where, cudaGetErrorString(e));
  return set_err(c, OSB_ECUDA, buf);
}

// a span-periodic 3D wall-bounded block (the 2D shock/boundary-layer faces in x0 and x1)
bool wall3(const osb_plan_desc &p) { return p.ndim == 3 && p.bc[1][0] == OSB_BC_ISOTHERMAL_WALL; }
// the channel form of a 3D wall-bounded block: periodic x0, isothermal walls on both x1 faces
bool channel3(const osb_plan_desc &p) { return wall3(p) && p.bc[0][0] == OSB_BC_PERIODIC; }

// the characteristic-flux schemes of the 3D kernels (WENO5-JS, WENO5-Z, TENO5)
bool char_fluxes(const osb_plan_desc &p) {
  return p.conv == OSB_CONV_WENO5JS || p.conv == OSB_CONV_WENO5Z || p.conv == OSB_CONV_TENO5 ||
         p.conv == OSB_CONV_TENO6;
}

int validate(const osb_plan_desc *p, char *why, size_t n) {
  if (!p) { snprintf(why, n, "null plan"); return OSB_EINVAL; }
  if (p->abi_version != OSB_ABI_VERSION) { snprintf(why, n, "abi_version %d != %d", p->abi_version, OSB_ABI_VERSION); return OSB_EINVAL; }
  if (!(p->shock_fp64 == 0.0 || (p->shock_fp64 >= 1.0 && std::isfinite(p->shock_fp64)))) {
    snprintf(why, n, "shock_fp64 = %g: 0 (off) or a pressure ratio >= 1", p->shock_fp64);
    return OSB_EINVAL;
  }
  if (p->ndim == 3 && (p->averaging != OSB_AVG_ROE || p->cartesian != 0)) {
    snprintf(why, n, "3D blocks: Roe averaging, cartesian = 0");
    return OSB_EUNSUPPORTED;
  }
  const bool chan2 = p->ndim == 2 && p->conv == OSB_CONV_CENTRAL_SKEW;  // laminar_channel.py
  if (!wall3(*p) && !chan2 && (p->forcing[0] != 0 || p->forcing[1] != 0 || p->forcing[2] != 0)) {
    snprintf(why, n, "forcing: 3D wall-bounded blocks only");
    return OSB_EUNSUPPORTED;
  }
  if (p->ndim == 1) {
    // 1D Euler block (Sod_shock_tube.py, shu_osher.py): Dirichlet faces (side 1 may extrapolate), FP64
    if (p->n[0] < 8 || p->n[0] > (1 << 24)) { snprintf(why, n, "n[0] = %d out of range [8, 2^24]", p->n[0]); return OSB_EINVAL; }
    if (!(p->delta[0] > 0)) { snprintf(why, n, "delta[0] must be > 0"); return OSB_EINVAL; }
    if (p->bc[0][0] != OSB_BC_DIRICHLET || (p->bc[0][1] != OSB_BC_DIRICHLET && p->bc[0][1] != OSB_BC_EXTRAPOLATION)) {
      snprintf(why, n, "1D blocks: a Dirichlet face at x0 = 0, a Dirichlet or extrapolation face at the end");
      return OSB_EUNSUPPORTED;
    }
    if (p->conv != OSB_CONV_TENO5 && p->conv != OSB_CONV_WENO5JS && p->conv != OSB_CONV_WENO5Z &&
        p->conv != OSB_CONV_TENO6) {
      snprintf(why, n, "1D blocks: TENO5, TENO6, WENO5-JS or WENO5-Z fluxes");
      return OSB_EUNSUPPORTED;
    }
    if (p->teno_adaptive || p->filter != OSB_FILTER_NONE || p->shock_fp64 != 0.0) {
      snprintf(why, n, "1D blocks: fixed TENO cut-off, no filter");
      return OSB_EUNSUPPORTED;
    }
    if (p->visc != OSB_VISC_NONE) { snprintf(why, n, "1D blocks: Euler equations (no viscosity)"); return OSB_EUNSUPPORTED; }
    if (p->rk != OSB_RK3_LS) { snprintf(why, n, "1D blocks: low-storage RK3"); return OSB_EUNSUPPORTED; }
    if (p->precision != OSB_PREC_FP64) { snprintf(why, n, "1D blocks: FP64"); return OSB_EUNSUPPORTED; }
    if (p->averaging != OSB_AVG_ROE && p->averaging != OSB_AVG_SIMPLE) {
      snprintf(why, n, "averaging %d: OSB_AVG_ROE or OSB_AVG_SIMPLE", p->averaging);
      return OSB_EINVAL;
    }
    for (int side = 0; side < 2; ++side)
      for (int v = 0; v < 3; ++v)
        if (!std::isfinite(p->dirichlet_x0[side][v])) { snprintf(why, n, "dirichlet_x0 must be finite"); return OSB_EINVAL; }
    if (!(p->gama > 1.0)) { snprintf(why, n, "bad physical constants"); return OSB_EINVAL; }
    return OSB_OK;
  }
  if (p->ndim == 2) {
    for (int d = 0; d < 2; ++d) {
      if (p->n[d] < 8 || p->n[d] > 16384) { snprintf(why, n, "n[%d] = %d out of range [8, 16384]", d, p->n[d]); return OSB_EINVAL; }
      if (!(p->delta[d] > 0)) { snprintf(why, n, "delta[%d] must be > 0", d); return OSB_EINVAL; }
    }
    if (p->averaging != OSB_AVG_ROE && p->averaging != OSB_AVG_SIMPLE) {
      snprintf(why, n, "averaging %d: OSB_AVG_ROE or OSB_AVG_SIMPLE", p->averaging);
      return OSB_EINVAL;
    }
    if (p->visc == OSB_VISC_NONE) {
      // Euler block (inviscid_shock_reflection.py): Cartesian, Dirichlet/inlet and Dirichlet/extrapolation
      // x0 faces, a symmetry face at x1 = 0, a Dirichlet or symmetry face at the top
      const int *b0 = p->bc[0], *b1 = p->bc[1];
      const bool periodic = b0[0] == OSB_BC_PERIODIC && b0[1] == OSB_BC_PERIODIC && b1[0] == OSB_BC_PERIODIC &&
                            b1[1] == OSB_BC_PERIODIC;  // euler_wave.py
      const bool ok = periodic ||
                      ((b0[0] == OSB_BC_INLET_PRESSURE_EXTRAPOLATE || b0[0] == OSB_BC_DIRICHLET) &&
                       (b0[1] == OSB_BC_EXTRAPOLATION || b0[1] == OSB_BC_DIRICHLET) && b1[0] == OSB_BC_SYMMETRY &&
                       (b1[1] == OSB_BC_DIRICHLET || b1[1] == OSB_BC_SYMMETRY));
      if (!ok) {
        snprintf(why, n, "2D Euler blocks: periodic on both axes, or inlet or Dirichlet / extrapolation or Dirichlet "
                         "(x0), symmetry / Dirichlet or symmetry (x1)");
        return OSB_EUNSUPPORTED;
      }
      if (p->cartesian != 1) { snprintf(why, n, "2D Euler blocks: Cartesian (cartesian = 1)"); return OSB_EUNSUPPORTED; }
      for (int side = 0; side < 2; ++side)
        for (int v = 0; v < 4; ++v)
          if (!std::isfinite(p->dirichlet_x0[side][v])) {
            snprintf(why, n, "dirichlet_x0 must be finite");
            return OSB_EINVAL;
          }
    } else if (p->visc == OSB_VISC_CONST) {
      // Cartesian viscous block (viscous_shock_tube.py): adiabatic walls, a symmetry top face, mu = 1
      if (p->bc[0][0] != OSB_BC_ADIABATIC_WALL || p->bc[0][1] != OSB_BC_ADIABATIC_WALL ||
          p->bc[1][0] != OSB_BC_ADIABATIC_WALL || p->bc[1][1] != OSB_BC_SYMMETRY || p->cartesian != 1) {
        snprintf(why, n, "2D constant-viscosity blocks: Cartesian, adiabatic walls (x0, x1 side 0), symmetry top");
        return OSB_EUNSUPPORTED;
      }
    } else if (!chan2 && (p->bc[0][0] != OSB_BC_INLET_PRESSURE_EXTRAPOLATE || p->bc[0][1] != OSB_BC_EXTRAPOLATION ||
                          p->bc[1][0] != OSB_BC_ISOTHERMAL_WALL || p->bc[1][1] != OSB_BC_DIRICHLET)) {
      snprintf(why, n, "2D blocks: boundary conditions must be inlet/extrapolation (x0) and isothermal wall/Dirichlet (x1)");
      return OSB_EUNSUPPORTED;
    } else if (!chan2 && p->cartesian != 0) {
      snprintf(why, n, "2D viscous blocks: metrics stretched in x1 (cartesian = 0)");
      return OSB_EUNSUPPORTED;
    }
    if (p->conv != OSB_CONV_TENO5 && p->conv != OSB_CONV_WENO5JS && p->conv != OSB_CONV_WENO5Z &&
        p->conv != OSB_CONV_TENO6 && !chan2) {
      snprintf(why, n, "2D blocks: TENO5, TENO6, WENO5-JS or WENO5-Z fluxes (central skew on channel blocks)");
      return OSB_EUNSUPPORTED;
    }
    if (chan2) {  // Cartesian, periodic x0, isothermal walls on both x1 faces, Sutherland, forcing
      if (p->bc[0][0] != OSB_BC_PERIODIC || p->bc[0][1] != OSB_BC_PERIODIC || p->bc[1][0] != OSB_BC_ISOTHERMAL_WALL ||
          p->bc[1][1] != OSB_BC_ISOTHERMAL_WALL || p->cartesian != 1 || p->visc != OSB_VISC_SUTHERLAND ||
          p->rk != OSB_RK3_LS || p->forcing[2] != 0 || !std::isfinite(p->forcing[0]) || !std::isfinite(p->forcing[1])) {
        snprintf(why, n, "2D central-skew blocks: the laminar channel (Cartesian, periodic x0, isothermal walls on both "
                         "x1 faces, Sutherland, LS-RK3, finite forcing c0, c1)");
        return OSB_EUNSUPPORTED;
      }
      for (int side = 0; side < 2; ++side)
        if (p->closure[1][side] != OSB_CLOSURE_REDUCED_ACCESS && p->closure[1][side] != OSB_CLOSURE_CARPENTER) {
          snprintf(why, n, "closure[1][%d]: OSB_CLOSURE_REDUCED_ACCESS or OSB_CLOSURE_CARPENTER", side);
          return OSB_EINVAL;
        }
      if (!(p->gama > 1.0) || !(p->Minf > 0) || !(p->Re > 0) || !(p->Pr > 0) || !(p->Twall > 0) || !(p->RefT > 0)) {
        snprintf(why, n, "bad physical constants");
        return OSB_EINVAL;
      }
      if (p->precision != OSB_PREC_FP64 && p->precision != OSB_PREC_MIXED) { snprintf(why, n, "precision"); return OSB_EINVAL; }
      return OSB_OK;
    }
    if (p->teno_adaptive) {
      if (p->conv != OSB_CONV_TENO5) { snprintf(why, n, "teno_adaptive needs TENO5 fluxes"); return OSB_EINVAL; }
      if (!(p->sensor_eps >= 0) || !std::isfinite(p->teno_a1) || !std::isfinite(p->teno_a2)) {
        snprintf(why, n, "adaptive TENO: sensor_eps >= 0 and finite teno_a1, teno_a2");
        return OSB_EINVAL;
      }
    }
    for (int d = 0; d < 2; ++d)
      for (int side = 0; side < 2; ++side) {
        const int cl = p->closure[d][side];
        const bool none_ok = cl == OSB_CLOSURE_NONE && p->bc[d][side] == OSB_BC_SYMMETRY && p->visc == OSB_VISC_CONST;
        if (cl != OSB_CLOSURE_REDUCED_ACCESS && cl != OSB_CLOSURE_CARPENTER && !none_ok) {
          snprintf(why, n, "closure[%d][%d] = %d: OSB_CLOSURE_REDUCED_ACCESS or OSB_CLOSURE_CARPENTER (NONE on the "
                           "symmetry face of a constant-viscosity block)", d, side, cl);
          return OSB_EINVAL;
        }
      }
    if (p->visc != OSB_VISC_SUTHERLAND && p->visc != OSB_VISC_NONE && p->visc != OSB_VISC_CONST) {
      snprintf(why, n, "2D blocks: Sutherland or constant viscosity, or none");
      return OSB_EUNSUPPORTED;
    }
    if (p->rk != OSB_RK3_LS && !(p->rk == OSB_RK3_2REG && p->visc == OSB_VISC_NONE)) {
      snprintf(why, n, "2D blocks: low-storage RK3 (2D Euler blocks also the two-register RK3)");
      return OSB_EUNSUPPORTED;
    }
    if (p->precision != OSB_PREC_FP64 && p->precision != OSB_PREC_MIXED) { snprintf(why, n, "precision %d", p->precision); return OSB_EINVAL; }
    if (!(p->gama > 1.0) || !(p->Minf > 0) || !(p->Re > 0) || !(p->Pr > 0) || !(p->Twall > 0) || !(p->RefT > 0)) {
      snprintf(why, n, "bad physical constants");
      return OSB_EINVAL;
    }
    return OSB_OK;
  }
  if (p->ndim != 3) { snprintf(why, n, "ndim %d: this library implements 1D, 2D and 3D blocks", p->ndim); return OSB_EUNSUPPORTED; }
  if (wall3(*p)) {
    // span-periodic wall-bounded block: the 2D configuration's faces in x0 and x1, or the channel's
    // periodic x0 and isothermal walls on both x1 faces; periodic x2
    const bool sbli = p->bc[0][0] == OSB_BC_INLET_PRESSURE_EXTRAPOLATE && p->bc[0][1] == OSB_BC_EXTRAPOLATION &&
                      p->bc[1][1] == OSB_BC_DIRICHLET;
    const bool chan = p->bc[0][0] == OSB_BC_PERIODIC && p->bc[0][1] == OSB_BC_PERIODIC &&
                      p->bc[1][1] == OSB_BC_ISOTHERMAL_WALL;
    if (!(sbli || chan) || p->bc[2][0] != OSB_BC_PERIODIC || p->bc[2][1] != OSB_BC_PERIODIC) {
      snprintf(why, n, "3D wall-bounded blocks: inlet/extrapolation (x0) with isothermal wall/Dirichlet (x1), or "
                       "periodic x0 with isothermal walls on both x1 faces; periodic x2");
      return OSB_EUNSUPPORTED;
    }
    for (int d = 0; d < 3; ++d) {
      if (p->n[d] < 8 || p->n[d] > 4096) { snprintf(why, n, "n[%d] = %d out of range [8, 4096]", d, p->n[d]); return OSB_EINVAL; }
      if (!(p->delta[d] > 0)) { snprintf(why, n, "delta[%d] must be > 0", d); return OSB_EINVAL; }
    }
    if (p->conv != OSB_CONV_TENO5 && p->conv != OSB_CONV_WENO5JS && p->conv != OSB_CONV_WENO5Z &&
        p->conv != OSB_CONV_TENO6) {
      snprintf(why, n, "3D wall-bounded blocks: TENO5, TENO6, WENO5-JS or WENO5-Z fluxes");
      return OSB_EUNSUPPORTED;
    }
    if (p->teno_adaptive && ((p->conv != OSB_CONV_TENO5 && p->conv != OSB_CONV_TENO6) || !(p->sensor_eps >= 0) ||
                             !std::isfinite(p->teno_a1) || !std::isfinite(p->teno_a2))) {
      snprintf(why, n, "adaptive TENO: TENO5 or TENO6, sensor_eps >= 0 and finite teno_a1, teno_a2");
      return OSB_EINVAL;
    }
    for (int k = 0; k < 5; ++k)
      if (!std::isfinite(p->body_force[k])) { snprintf(why, n, "body_force[%d] must be finite", k); return OSB_EINVAL; }
    if (p->dirichlet_ke != 0 && p->dirichlet_ke != 1) { snprintf(why, n, "dirichlet_ke: 0 or 1"); return OSB_EINVAL; }
    if (p->filter != OSB_FILTER_NONE) { snprintf(why, n, "3D wall-bounded blocks: no WENO filter"); return OSB_EUNSUPPORTED; }
    for (int d = 0; d < 2; ++d)
      for (int side = 0; side < 2; ++side)
        if (p->closure[d][side] != OSB_CLOSURE_REDUCED_ACCESS && p->closure[d][side] != OSB_CLOSURE_CARPENTER) {
          snprintf(why, n, "closure[%d][%d] = %d: OSB_CLOSURE_REDUCED_ACCESS or OSB_CLOSURE_CARPENTER", d, side,
                   p->closure[d][side]);
          return OSB_EINVAL;
        }
    if (p->visc != OSB_VISC_SUTHERLAND && p->visc != OSB_VISC_POWER) {
      snprintf(why, n, "3D wall-bounded blocks: Sutherland or power-law viscosity");
      return OSB_EUNSUPPORTED;
    }
    if (p->visc == OSB_VISC_POWER && !(p->visc_exp > 0 && p->visc_exp < 8)) {
      snprintf(why, n, "visc_exp must lie in (0, 8)");
      return OSB_EINVAL;
    }
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(p->forcing[k])) { snprintf(why, n, "forcing[%d] must be finite", k); return OSB_EINVAL; }
    if (p->rk != OSB_RK3_LS) { snprintf(why, n, "3D wall-bounded blocks: low-storage RK3"); return OSB_EUNSUPPORTED; }
    if (p->precision != OSB_PREC_FP64 && p->precision != OSB_PREC_MIXED) { snprintf(why, n, "precision %d", p->precision); return OSB_EINVAL; }
    if (!(p->gama > 1.0) || !(p->Minf > 0) || !(p->Re > 0) || !(p->Pr > 0) || !(p->Twall > 0) || !(p->RefT > 0)) {
      snprintf(why, n, "bad physical constants");
      return OSB_EINVAL;
    }
    return OSB_OK;
  }
  if (p->teno_adaptive) {
    if (p->conv != OSB_CONV_TENO5 && p->conv != OSB_CONV_TENO6) {
      snprintf(why, n, "teno_adaptive needs TENO5 or TENO6 fluxes");
      return OSB_EINVAL;
    }
    if (!(p->sensor_eps >= 0) || !std::isfinite(p->teno_a1) || !std::isfinite(p->teno_a2)) {
      snprintf(why, n, "adaptive TENO: sensor_eps >= 0 and finite teno_a1, teno_a2");
      return OSB_EINVAL;
    }
  }
  if (p->filter != OSB_FILTER_NONE && p->filter != OSB_FILTER_WENO5_CONSTANT) {
    snprintf(why, n, "filter %d: OSB_FILTER_NONE or OSB_FILTER_WENO5_CONSTANT", p->filter);
    return OSB_EUNSUPPORTED;
  }
  if (p->filter != OSB_FILTER_NONE && !std::isfinite(p->filter_control)) {
    snprintf(why, n, "filter_control must be finite");
    return OSB_EINVAL;
  }
  for (int d = 0; d < 3; ++d) {
    if (p->n[d] < 8 || p->n[d] > 4096) { snprintf(why, n, "n[%d] = %d out of range [8, 4096]", d, p->n[d]); return OSB_EINVAL; }
    if (!(p->delta[d] > 0)) { snprintf(why, n, "delta[%d] must be > 0", d); return OSB_EINVAL; }
    for (int s = 0; s < 2; ++s)
      if (p->bc[d][s] != OSB_BC_PERIODIC && p->bc[d][s] != OSB_BC_SYMMETRY) {
        snprintf(why, n, "bc[%d][%d] = %d not supported on 3D blocks", d, s, p->bc[d][s]);
        return OSB_EUNSUPPORTED;
      }
    if ((p->bc[d][0] == OSB_BC_PERIODIC) != (p->bc[d][1] == OSB_BC_PERIODIC)) {
      snprintf(why, n, "axis %d: periodic must be set on both sides", d);
      return OSB_EINVAL;
    }
  }
  if (p->conv != OSB_CONV_CENTRAL_SKEW && p->conv != OSB_CONV_WENO5JS && p->conv != OSB_CONV_WENO5Z &&
      p->conv != OSB_CONV_TENO5 && p->conv != OSB_CONV_TENO6) {
    snprintf(why, n, "convective scheme %d not supported on 3D blocks", p->conv);
    return OSB_EUNSUPPORTED;
  }
  if (p->visc != OSB_VISC_NONE && p->visc != OSB_VISC_CONST) {
    snprintf(why, n, "viscosity model %d not supported on 3D blocks", p->visc);
    return OSB_EUNSUPPORTED;
  }
  if (p->rk != OSB_RK3_2REG) { snprintf(why, n, "time scheme %d not supported on 3D blocks", p->rk); return OSB_EUNSUPPORTED; }
  if (p->precision != OSB_PREC_FP64 && p->precision != OSB_PREC_MIXED) { snprintf(why, n, "precision %d", p->precision); return OSB_EINVAL; }
  if (!(p->gama > 1.0) || !(p->Minf > 0) || !(p->Re > 0) || !(p->Pr > 0)) { snprintf(why, n, "bad physical constants"); return OSB_EINVAL; }
  return OSB_OK;
}

Grid make_grid(const osb_plan_desc *p) {
  Grid g;
  if (p->ndim == 1) {  // one row with a 4-point x halo
    g.n0 = p->n[0];
    g.n1 = 1;
    g.n2 = 1;
    int64_t px = p->n[0] + 8;
    px = (px + 7) / 8 * 8;
    g.sy = px;
    g.sz = px;
    g.off0 = 4;
    g.numel = px;
    return g;
  }
  if (p->ndim == 2) {  // x fastest, 4-point halo on every side, one plane
    g.n0 = p->n[0];
    g.n1 = p->n[1];
    g.n2 = 1;
    int64_t px = p->n[0] + 8;
    px = (px + 7) / 8 * 8;
    g.sy = px;
    g.sz = px * (p->n[1] + 8);
    g.off0 = 4 + 4 * g.sy;
    g.numel = g.sz;
    return g;
  }
  g.n0 = p->n[0];
  g.n1 = p->n[1];
  g.n2 = p->n[2];
  int64_t px = p->n[0] + 2 * HX;
  px = (px + 7) / 8 * 8;  // rows start on 32-byte boundaries for both element sizes
  const int64_t py = p->n[1] + 2 * HY, pz = p->n[2] + 2 * HZ;
  g.sy = px;
  g.sz = px * py;
  g.off0 = HX + HY * g.sy + HZ * g.sz;
  g.numel = px * py * pz;
  return g;
}

template <typename T> Fields5<T> fields(void *const *a) {
  Fields5<T> f;
  for (int v = 0; v < 5; ++v) f.v[v] = static_cast<T *>(a[v]);
  return f;
}
Fields5<double> fields_d(double *const *a) {
  Fields5<double> f;
  for (int v = 0; v < 5; ++v) f.v[v] = a[v];
  return f;
}

// ---------------------------------------------------------------------------------------------
// small kernels: initial condition, state copies, packing, reductions
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_init_tgv(Grid g, Fields5<T> q, Fields5<double> qold, double d0, double d1, double d2, double gama,
                           double Minf) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const double x0 = d0 * i, x1 = d1 * j, x2 = d2 * k;
    const double u0 = sin(x0) * cos(x1) * cos(x2), u1 = -sin(x1) * cos(x0) * cos(x2), u2 = 0.0;
    const double p = (0.0625 * cos(2.0 * x0) + 0.0625 * cos(2.0 * x1)) * (cos(2.0 * x2) + 2.0) + 1.0 / (Minf * Minf * gama);
    const double r = Minf * Minf * gama * p;
    const double vals[5] = {r, r * u0, r * u1, r * u2, p / (gama - 1) + 0.5 * r * (u0 * u0 + u1 * u1 + u2 * u2)};
    const int64_t n = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      qold.v[v][n] = vals[v];
      q.v[v][n] = (T)vals[v];
    }
  }
}

template <typename T> __global__ void k_save(Grid g, Fields5<const T> q, Fields5<double> qold) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) qold.v[v][n] = (double)q.v[v][n];
  }
}

template <typename T> __global__ void k_set64(Grid g, const double *src, T *q, double *qold) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
    qold[n] = src[t];
    q[n] = (T)src[t];
  }
}

__global__ void k_get64(Grid g, const double *qold, double *dst) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    dst[t] = qold[gidx(g, i, j, k)];
  }
}

template <typename T> __global__ void k_pack(Grid g, Fields5<const T> r, T *dst) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v * N + t] = r.v[v][n];
  }
}

// Block-partial FP64 sums, then one block adds the partials in a fixed order (deterministic).
constexpr int RED_THREADS = 256;
__device__ __forceinline__ double block_sum(double x) {
  __shared__ double sh[RED_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
  __syncthreads();
  x = threadIdx.x < RED_THREADS / 32 ? sh[threadIdx.x] : 0.0;
  if (threadIdx.x < 32)
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_reduce(Grid g, Fields5<const double> qold, Fields5<const T> q, int what,
                                                        double i0, double i1, double i2, double *partial) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
    if (what == OSB_RED_KE) {
      const double r = qold.v[0][n];
      acc += 0.5 * (qold.v[1][n] * qold.v[1][n] + qold.v[2][n] * qold.v[2][n] + qold.v[3][n] * qold.v[3][n]) / r;
    } else if (what == OSB_RED_NANCHECK) {
      for (int v = 0; v < 5; ++v)
        if (!isfinite((double)q.v[v][n])) acc = 1.0;
    } else {  // enstrophy: 0.5 rho |curl u|^2 with 4th-order central first derivatives
      const double c1[5] = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0};
      const int64_t st[3] = {1, g.sy, g.sz};
      const double id[3] = {i0, i1, i2};
      double du[3][3];
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) {
          double s = 0.0;
          for (int o = -2; o <= 2; ++o) {
            if (!o) continue;
            const int64_t m = n + o * st[d];
            s += c1[o + 2] * ((double)q.v[1 + c][m] / (double)q.v[0][m]);
          }
          du[c][d] = s * id[d];
        }
      const double w0 = du[2][1] - du[1][2], w1 = du[0][2] - du[2][0], w2 = du[1][0] - du[0][1];
      acc += 0.5 * qold.v[0][n] * (w0 * w0 + w1 * w1 + w2 * w2);
    }
  }
  const double s = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = (what == OSB_RED_NANCHECK) ? (s > 0 ? 1.0 : 0.0) : s;
}

__global__ void k_reduce_final(const double *partial, int nb, int what, double scale, double *out) {
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += partial[b];
  const double s = block_sum(acc);
  if (threadIdx.x == 0) out[0] = what == OSB_RED_NANCHECK ? (s > 0 ? 1.0 : 0.0) : s * scale;
}

int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return (int)(b < 1 ? 1 : b);
}

// ---------------------------------------------------------------------------------------------
// per-family event timing (eager path only)
// ---------------------------------------------------------------------------------------------
struct ProfScope {
  osb_ctx *c;
  int family;
  cudaStream_t s;
  cudaEvent_t a = nullptr;
  ProfScope(osb_ctx *c_, int f, cudaStream_t s_) : c(c_), family(f), s(s_) {
    if (c->prof_on) {
      cudaEventCreate(&a);
      cudaEventRecord(a, s);
    }
  }
  ~ProfScope() {
    if (c->prof_on) {
      cudaEvent_t b;
      cudaEventCreate(&b);
      cudaEventRecord(b, s);
      c->prof_pending.push_back({family, a, b});
    }
  }
};

void prof_collect(osb_ctx *c) {
  for (auto &r : c->prof_pending) {
    float ms = 0;
    cudaEventSynchronize(r.b);
    cudaEventElapsedTime(&ms, r.a, r.b);
    c->prof_ms[r.family] += ms;
    c->prof_n[r.family] += 1;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  c->prof_pending.clear();
}

// ---------------------------------------------------------------------------------------------
// time loop
// ---------------------------------------------------------------------------------------------
template <typename T> void weno_all(osb_ctx *c, Fields5<const T> qc, Fields5<T> r, cudaStream_t s) {
  if (c->plan.teno_adaptive) {
    ProfScope ps(c, PF_OTHER, s);
    launch_sensor_ct3<T>(*c, qc, s, &c->launches);
  }
  for (int d = 0; d < 3; ++d) {
    ProfScope ps(c, PF_WENO_X + d, s);
    launch_weno_dir<T>(*c, qc, r, d, s, &c->launches);
  }
}

template <typename T> void residual_into(osb_ctx *c, int cur, cudaStream_t s) {
  void **qs = cur == 0 ? c->qa : c->qb;
  Fields5<T> q = fields<T>(qs);
  Fields5<const T> qc = fields<const T>(qs);
  Fields5<T> r = fields<T>(c->res);
  launch_halos<T>(*c, q, s, &c->launches);
  if (char_fluxes(c->plan)) {
    weno_all<T>(c, qc, r, s);
    const int mode = CRK_RIN | (c->plan.visc == OSB_VISC_CONST ? CRK_VISC : 0);
    launch_central_rk<T>(*c, qc, r, fields_d(c->qold), r, r, 0.0, 0.0, mode, s, &c->launches);
  } else {
    const int mode = CRK_SKEW | (c->plan.visc == OSB_VISC_CONST ? CRK_VISC : 0);
    launch_central_rk<T>(*c, qc, r, fields_d(c->qold), r, r, 0.0, 0.0, mode, s, &c->launches);
  }
}

template <typename T> void one_step(osb_ctx *c, int start, double dt, cudaStream_t s) {
  int cur = start;
  for (int st = 0; st < 3; ++st) {
    void **qs = cur == 0 ? c->qa : c->qb;
    void **qn = cur == 0 ? c->qb : c->qa;
    Fields5<T> q = fields<T>(qs);
    Fields5<const T> qc = fields<const T>(qs);
    Fields5<T> r = fields<T>(c->res);
    {
      ProfScope ps(c, PF_HALO, s);
      launch_halos<T>(*c, q, s, &c->launches);
    }
    const double dtn = dt * c->plan.rk_b[st], dto = dt * c->plan.rk_a[st];
    const int visc = c->plan.visc == OSB_VISC_CONST ? CRK_VISC : 0;
    if (char_fluxes(c->plan)) {
      weno_all<T>(c, qc, r, s);
      ProfScope ps(c, PF_CENTRAL_RK, s);
      launch_central_rk<T>(*c, qc, fields<T>(qn), fields_d(c->qold), r, r, dtn, dto, CRK_RIN | visc | CRK_UPDATE, s,
                           &c->launches);
    } else {
      ProfScope ps(c, PF_CENTRAL_RK, s);
      launch_central_rk<T>(*c, qc, fields<T>(qn), fields_d(c->qold), r, r, dtn, dto, CRK_SKEW | visc | CRK_UPDATE, s,
                           &c->launches);
    }
    cur ^= 1;
  }
  if (c->plan.filter != OSB_FILTER_NONE) {
    // the WENO5 filter after the full step (the generated loop runs its kernels after the stage
    // loop, algorithm.py:418-428 with filters/WENO_filter.py): halos of the new state, the filter's
    // flux differences into the residual scratch, then q += dt * shock_filter_control * R
    void **qs = cur == 0 ? c->qa : c->qb;
    Fields5<T> r = fields<T>(c->res);
    {
      ProfScope ps(c, PF_HALO, s);
      launch_halos<T>(*c, fields<T>(qs), s, &c->launches);
    }
    ProfScope ps(c, PF_OTHER, s);
    for (int dir = 0; dir < 3; ++dir) launch_filter_dir<T>(*c, fields<const T>(qs), r, dir, s, &c->launches);
    launch_filter_apply<T>(*c, fields<T>(qs), fields_d(c->qold), fields<const T>(c->res), dt * c->plan.filter_control,
                           s, &c->launches);
  }
}

template <typename T> int step_impl(osb_ctx *c, int nsteps, double dt) {
  cudaStream_t s = c->stream;
  c->launches = 0;
  if (!c->qold_valid) {
    k_save<T><<<blocks_for((int64_t)c->g.n0 * c->g.n1 * c->g.n2), 256, 0, s>>>(c->g, fields<const T>(c->qa),
                                                                               fields_d(c->qold));
    ++c->launches;
    c->qold_valid = 1;
  }
  for (int it = 0; it < nsteps; ++it) {
    const int start = c->cur;
    // graphs need a capturable stream: not the legacy default stream
    if (c->plan.use_graphs && !c->prof_on && c->stream != nullptr) {
      if (c->graph[start] && c->graph_dt[start] != dt) {
        cudaGraphExecDestroy(c->graph[start]);
        c->graph[start] = nullptr;
      }
      if (!c->graph[start]) {
        cudaGraph_t gr;
        int64_t l0 = c->launches;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaStreamBeginCapture");
        one_step<T>(c, start, dt, s);
        e = cudaStreamEndCapture(s, &gr);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&c->graph[start], gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphInstantiate");
        c->graph_dt[start] = dt;
        c->graph_launches = c->launches - l0;
        c->launches = l0;
      }
      cudaError_t e = cudaGraphLaunch(c->graph[start], s);
      if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphLaunch");
      c->launches += c->graph_launches;
    } else {
      one_step<T>(c, start, dt, s);
    }
    c->cur ^= 1;  // three stages flip the buffer
  }
  if (c->cur == 1) {
    for (int v = 0; v < 5; ++v) {
      cudaError_t e = cudaMemcpyAsync(c->qa[v], c->qb[v], (size_t)c->g.numel * c->elem, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_err(c, e, "copy back");
    }
    c->cur = 0;
  }
  launch_halos<T>(*c, fields<T>(c->qa), s, &c->launches);
  if (c->prof_on) prof_collect(c);
  return cuda_err(c, cudaGetLastError(), "osb_step launch");
}

// One LS-RK3 step on a span-periodic 3D wall-bounded block: face conditions (and the working state),
// then per stage the right-hand side with the update du = A du + dt R, q += B du on the FP64 master
// and the face conditions again (algorithm.py:384-477).
template <typename T> void one_step3w(osb_ctx *c, double dt, cudaStream_t s) {
  launch3w_tick(*c, 0, dt, s, &c->launches);  // body force: sin(omega dt iter) of this step
  {
    ProfScope ps(c, PF_HALO, s);
    launch3w_bcs<T>(*c, s, &c->launches);
  }
  for (int st = 0; st < 3; ++st) {
    {
      ProfScope ps(c, PF_CENTRAL_RK, s);
      launch3w_rhs<T>(*c, 1, c->plan.rk_a[st], c->plan.rk_b[st], dt, s, &c->launches);
    }
    ProfScope ps(c, PF_HALO, s);
    launch3w_bcs<T>(*c, s, &c->launches);
  }
  launch3w_tick(*c, 1, dt, s, &c->launches);
}

template <typename T> int step3w_impl(osb_ctx *c, int nsteps, double dt) {
  cudaStream_t s = c->stream;
  c->launches = 0;
  for (int it = 0; it < nsteps; ++it) {
    if (c->plan.use_graphs && !c->prof_on && c->stream != nullptr) {
      if (c->graph[0] && c->graph_dt[0] != dt) {
        cudaGraphExecDestroy(c->graph[0]);
        c->graph[0] = nullptr;
      }
      if (!c->graph[0]) {
        cudaGraph_t gr;
        int64_t l0 = c->launches;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaStreamBeginCapture");
        one_step3w<T>(c, dt, s);
        e = cudaStreamEndCapture(s, &gr);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&c->graph[0], gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphInstantiate");
        c->graph_dt[0] = dt;
        c->graph_launches = c->launches - l0;
        c->launches = l0;
      }
      cudaError_t e = cudaGraphLaunch(c->graph[0], s);
      if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphLaunch");
      c->launches += c->graph_launches;
    } else {
      one_step3w<T>(c, dt, s);
    }
  }
  if (c->prof_on) prof_collect(c);
  return cuda_err(c, cudaGetLastError(), "osb_step launch");
}

// One LS-RK3 step on a 2D block: boundary conditions, then per stage the right-hand side with the
// update du = A du + dt R, q += B du, and the boundary conditions again (algorithm.py:384-477).
template <typename T> void one_step2(osb_ctx *c, double dt, cudaStream_t s) {
  if (c->plan.ndim == 1) {  // 1D Euler block (FP64): faces, then per stage fluxes + update and faces
    launch1_bcs(*c, s, &c->launches);
    for (int st = 0; st < 3; ++st) {
      launch1_rhs(*c, 1, c->plan.rk_a[st], c->plan.rk_b[st], dt, s, &c->launches);
      launch1_bcs(*c, s, &c->launches);
    }
    return;
  }
  {
    ProfScope ps(c, PF_HALO, s);
    launch2_bcs(*c, s, &c->launches);
  }
  if (c->plan.rk == OSB_RK3_2REG) launch2_save(*c, s, &c->launches);  // qold = q
  for (int st = 0; st < 3; ++st) {
    {
      ProfScope ps(c, PF_CENTRAL_RK, s);
      launch2_rhs<T>(*c, 1, c->plan.rk_a[st], c->plan.rk_b[st], dt, s, &c->launches);
    }
    ProfScope ps(c, PF_HALO, s);
    launch2_bcs(*c, s, &c->launches);
  }
  // mixed: each stage's right-hand side rounds the master into the FP32 state itself; this leaves
  // the bound FP32 arrays holding the step's final state
  launch2_to_state(*c, s, &c->launches);
}

template <typename T> int step2_impl(osb_ctx *c, int nsteps, double dt) {
  cudaStream_t s = c->stream;
  c->launches = 0;
  for (int it = 0; it < nsteps; ++it) {
    if (c->plan.use_graphs && !c->prof_on && s != nullptr) {
      if (c->graph[0] && c->graph_dt[0] != dt) {
        cudaGraphExecDestroy(c->graph[0]);
        c->graph[0] = nullptr;
      }
      if (!c->graph[0]) {
        cudaGraph_t gr;
        const int64_t l0 = c->launches;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaStreamBeginCapture");
        one_step2<T>(c, dt, s);
        e = cudaStreamEndCapture(s, &gr);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&c->graph[0], gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphInstantiate");
        c->graph_dt[0] = dt;
        c->graph_launches = c->launches - l0;
        c->launches = l0;
      }
      cudaError_t e = cudaGraphLaunch(c->graph[0], s);
      if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphLaunch");
      c->launches += c->graph_launches;
    } else {
      one_step2<T>(c, dt, s);
    }
  }
  if (c->prof_on) prof_collect(c);
  return cuda_err(c, cudaGetLastError(), "osb_step launch");
}

template <typename T> __global__ void k_set64_padded(Grid g, const double *src, int h, T *q, double *q64) {
  // a 1D block (n1 = 1) has no x1 halo, a 2D block (n2 = 1) no x2 halo
  const int w = g.n0 + 2 * h, hgt = g.n1 == 1 ? 1 : g.n1 + 2 * h, dep = g.n2 == 1 ? 1 : g.n2 + 2 * h;
  const int64_t N = (int64_t)w * hgt * dep;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % w) - h, j = g.n1 == 1 ? 0 : (int)((t / w) % hgt) - h;
    const int k = g.n2 == 1 ? 0 : (int)(t / ((int64_t)w * hgt)) - h;
    const int64_t n = gidx(g, i, j, k);
    q64[n] = src[t];
    q[n] = (T)src[t];
  }
}

__global__ void k_copy_padded(Grid g, const double *src, int h, double *dst) {
  const int w = g.n0 + 2 * h, hgt = g.n1 + 2 * h;
  const int64_t N = (int64_t)w * hgt;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % w) - h, j = (int)(t / w) - h;
    dst[gidx(g, i, j, 0)] = src[t];
  }
}

struct P4 {
  const double *v[5];
};
template <typename T> __global__ void k_pack_d(Grid g, P4 src4, T *dst, int nvar) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    for (int v = 0; v < nvar; ++v) dst[v * N + t] = (T)src4.v[v][gidx(g, i, j, k)];
  }
}

struct D4 {
  const double *v[4];
};
__global__ void k_reduce2(Grid g, D4 q, int what, double *partial, int nvar) {
  // 2D blocks (rho, rhou0, rhou1, rhoE) and 1D blocks (rho, rhou0, rhoE)
  const int64_t N = (int64_t)g.n0 * g.n1;
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)(t / g.n0);
    const int64_t n = gidx(g, i, j, 0);
    if (what == OSB_RED_KE) {
      const double m1 = nvar == 4 ? q.v[2][n] : 0.0;
      acc += 0.5 * (q.v[1][n] * q.v[1][n] + m1 * m1) / q.v[0][n];
    } else {
      for (int v = 0; v < nvar; ++v)
        if (!isfinite(q.v[v][n])) acc = 1.0;
    }
  }
  const double s = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = (what == OSB_RED_NANCHECK) ? (s > 0 ? 1.0 : 0.0) : s;
}

}  // namespace

namespace osb {
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// Boxes of 40 x (TY+4) x 1 elements of one padded conserved array: x from interior i0-4 (a multiple
// of 32 in padded coordinates, so every copy starts on a 16-byte boundary), all rows of the plane's
// tile and its 2-point halo.  Out-of-range parts of a box read as zeros (never used).
int encode_state_maps(Ctx &c, int buf) {
  c.tma_ok[buf] = 0;
  EncodeTiledFn fn = encode_tiled();
  if (!fn || c.plan.ndim != 3 || !c.mixed) return OSB_OK;  // the TMA path serves FP32 3D states
  void *const *arrays = buf == 0 ? c.qa : c.qb;
  for (int v = 0; v < 5; ++v)
    if (!arrays[v] || (reinterpret_cast<uintptr_t>(arrays[v]) & 15)) return OSB_OK;
  const size_t e = (size_t)c.elem;
  const cuuint64_t dims[3] = {(cuuint64_t)c.g.sy, (cuuint64_t)(c.g.n1 + 2 * HY), (cuuint64_t)(c.g.n2 + 2 * HZ)};
  const cuuint64_t strides[2] = {(cuuint64_t)(c.g.sy * e), (cuuint64_t)(c.g.sz * e)};
  const cuuint32_t estr[3] = {1, 1, 1};
  for (int t = 0; t < 2; ++t) {
    const cuuint32_t box[3] = {40, (cuuint32_t)((t == 0 ? 8 : 16) + 4), 1};
    for (int v = 0; v < 5; ++v) {
      CUresult r = fn(&c.tma[buf][t].m[v], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, arrays[v], dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return OSB_OK;  // keep the register path
    }
  }
  c.tma_ok[buf] = 1;
  return OSB_OK;
}

int plan_validate(const osb_plan_desc *p, char *why, size_t n) { return validate(p, why, n); }
Grid plan_grid(const osb_plan_desc *p) { return make_grid(p); }
Phys plan_phys(const osb_plan_desc *plan) {
  Phys ph{};
  ph.gama = plan->gama;
  ph.Minf = plan->Minf;
  ph.Re = plan->Re;
  ph.Pr = plan->Pr;
  for (int d = 0; d < 3; ++d) ph.inv_delta[d] = 1.0 / plan->delta[d];
  ph.weno_eps = (plan->conv == OSB_CONV_TENO5 || plan->conv == OSB_CONV_TENO6) ? plan->teno_eps
                : plan->weno_eps > 0 ? plan->weno_eps : 1e-6;
  ph.teno_ct = plan->teno_ct;
  ph.f_teno_ct = (float)plan->teno_ct;
  ph.gm1 = plan->gama - 1.0;
  ph.igm1 = 1.0 / ph.gm1;
  ph.gM2 = plan->Minf * plan->Minf * plan->gama;
  ph.invRe = 1.0 / plan->Re;
  ph.kT = 1.0 / ((plan->gama - 1.0) * plan->Minf * plan->Minf * plan->Pr * plan->Re);
  ph.f_gama = (float)ph.gama;
  ph.f_gm1 = (float)ph.gm1;
  ph.f_igm1 = (float)ph.igm1;
  ph.f_gM2 = (float)ph.gM2;
  ph.f_invRe = (float)ph.invRe;
  ph.f_kT = (float)ph.kT;
  ph.f_eps = (float)ph.weno_eps;
  for (int d = 0; d < 3; ++d) ph.f_inv_delta[d] = (float)ph.inv_delta[d];
  ph.f_gm1_lo = (float)(ph.gm1 - (double)ph.f_gm1);
  for (int d = 0; d < 3; ++d) ph.f_inv_delta_lo[d] = (float)(ph.inv_delta[d] - (double)ph.f_inv_delta[d]);
  return ph;
}
}  // namespace osb

extern "C" {

static int check_bound(osb_ctx *c);

int osb_set_state64_padded(osb_ctx *c, int var, const double *src, int h) {
  if (!c) return OSB_EINVAL;
  if (int rc = check_bound(c)) return rc;
  const int hmax = c->plan.ndim <= 2 ? 4 : HY;
  if (var < 0 || var >= c->nvar || !src || h < 1 || h > hmax) return set_err(c, OSB_EINVAL, "bad var, pointer or halo");
  double *m = c->plan.ndim <= 2 ? c->q64_2d[var] : c->qold[var];
  const int64_t N = (int64_t)(c->g.n0 + 2 * h) * (c->plan.ndim == 1 ? 1 : c->g.n1 + 2 * h) *
                    (c->plan.ndim <= 2 ? 1 : c->g.n2 + 2 * h);
  const int nb = blocks_for(N);
  if (c->mixed) k_set64_padded<float><<<nb, 256, 0, c->stream>>>(c->g, src, h, (float *)c->qa[var], m);
  else k_set64_padded<double><<<nb, 256, 0, c->stream>>>(c->g, src, h, (double *)c->qa[var], m);
  c->qold_valid = 1;
  c->cur = 0;
  return cuda_err(c, cudaGetLastError(), "osb_set_state64_padded");
}

int osb_set_coordinate(osb_ctx *c, int axis, const double *src, int h) {
  if (!c) return OSB_EINVAL;
  if (wall3(c->plan)) {
    // the x1 coordinate is a function of j alone: a line of n1 + 2h values
    if (axis != 1) return set_err(c, OSB_EUNSUPPORTED, "coordinates: blocks stretched in x1 only");
    if (!src || h < 0 || h > 4) return set_err(c, OSB_EINVAL, "coordinate line needs a halo of 0..4 points");
    cudaError_t e = cudaMemcpyAsync(c->x1, src + h, (size_t)c->g.n1 * sizeof(double), cudaMemcpyDefault, c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "osb_set_coordinate");
    int64_t l = 0;
    launch3w_metrics(*c, c->x1, c->stream, &l);
    launch3w_bf_tables(*c, c->stream, &l);
    c->metrics_valid = 1;
    return cuda_err(c, cudaGetLastError(), "osb_set_coordinate");
  }
  if (c->plan.ndim != 2 || axis != 1) return set_err(c, OSB_EUNSUPPORTED, "coordinates: 2D blocks stretched in x1 only");
  if (c->plan.cartesian) return set_err(c, OSB_EINVAL, "Cartesian 2D block: no coordinate to set");
  if (!src || h < 4 || h > 4) return set_err(c, OSB_EINVAL, "coordinate array needs a 4-point halo");
  const int nb = blocks_for((int64_t)(c->g.n0 + 2 * h) * (c->g.n1 + 2 * h));
  k_copy_padded<<<nb, 256, 0, c->stream>>>(c->g, src, h, c->x1);
  int64_t l = 0;
  launch2_metrics(*c, c->x1, c->stream, &l);
  c->metrics_valid = 1;
  return cuda_err(c, cudaGetLastError(), "osb_set_coordinate");
}

int osb_query_layout(const osb_plan_desc *plan, osb_layout *out) {
  char why[256];
  int rc = validate(plan, why, sizeof why);
  if (rc) return rc;
  if (!out) return OSB_EINVAL;
  Grid g = make_grid(plan);
  out->numel = g.numel;
  out->offset = g.off0;
  out->stride_y = g.sy;
  out->stride_z = g.sz;
  out->halo[0] = HX;
  out->halo[1] = plan->ndim == 1 ? 0 : plan->ndim == 2 ? 4 : HY;
  out->halo[2] = plan->ndim <= 2 ? 0 : HZ;
  out->nvar = plan->ndim + 2;
  out->state_bytes = plan->precision == OSB_PREC_MIXED ? 4 : 8;
  return OSB_OK;
}

int osb_create(const osb_plan_desc *plan, osb_ctx **out) {
  if (!out) return OSB_EINVAL;
  *out = nullptr;
  char why[256];
  int rc = validate(plan, why, sizeof why);
  if (rc) {
    fprintf(stderr, "osb_create: %s\n", why);
    return rc;
  }
  osb_ctx *c = new (std::nothrow) osb_ctx();
  if (!c) return OSB_EINVAL;
  c->plan = *plan;
  c->g = make_grid(plan);
  c->mixed = plan->precision == OSB_PREC_MIXED;
  c->elem = c->mixed ? 4 : 8;
  c->ph = plan_phys(plan);
  const size_t bytes = (size_t)c->g.numel * c->elem;
  cudaError_t e = cudaSuccess;
  if (plan->ndim <= 2) {  // 2D blocks, and 1D blocks on the same storage
    c->nvar = plan->ndim + 2;
    const size_t b64 = (size_t)c->g.numel * sizeof(double);
    for (int v = 0; v < c->nvar && e == cudaSuccess; ++v) {
      if (c->mixed) {
        e = cudaMalloc(&c->q64_2d[v], b64);
        if (e == cudaSuccess) e = cudaMemset(c->q64_2d[v], 0, b64);
      }
      if (e == cudaSuccess) e = cudaMalloc(&c->du2[v], b64);
      if (e == cudaSuccess) e = cudaMemset(c->du2[v], 0, b64);
      if (e == cudaSuccess) e = cudaMalloc(&c->res[v], bytes);
      if (e == cudaSuccess) e = cudaMemset(c->res[v], 0, bytes);
    }
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) {
      e = cudaMalloc(&c->prim2[k], bytes);
      if (e == cudaSuccess) e = cudaMemset(c->prim2[k], 0, bytes);
    }
    if (e == cudaSuccess && plan->teno_adaptive) {
      e = cudaMalloc(&c->ct2, bytes);
      if (e == cudaSuccess) e = cudaMemset(c->ct2, 0, bytes);
    }
    for (int v = 0; v < 4 && e == cudaSuccess; ++v) {
      e = cudaMalloc(&c->resy[v], bytes);
      if (e == cudaSuccess) e = cudaMemset(c->resy[v], 0, bytes);
    }
    for (int v = 0; v < 3 && e == cudaSuccess; ++v) {
      e = cudaMalloc(&c->resv[v], bytes);
      if (e == cudaSuccess) e = cudaMemset(c->resv[v], 0, bytes);
    }
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      e = cudaStreamCreateWithFlags(&c->side2[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join2[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&c->x1, b64);
    if (e == cudaSuccess) e = cudaMalloc(&c->d11, b64);
    if (e == cudaSuccess) e = cudaMalloc(&c->sd111, b64);
    if (e == cudaSuccess) e = cudaMemset(c->d11, 0, b64);
    if (e == cudaSuccess) e = cudaMemset(c->sd111, 0, b64);
    if (e == cudaSuccess && (plan->cartesian || plan->ndim == 1)) {  // no metric terms: D11 = 1, SD111 = 0
      std::vector<double> ones((size_t)c->g.numel, 1.0);
      e = cudaMemcpy(c->d11, ones.data(), b64, cudaMemcpyHostToDevice);
      c->metrics_valid = 1;
    }
    c->red_blocks = 152 * 8;
    if (e == cudaSuccess) e = cudaMalloc(&c->red, (c->red_blocks + 1) * sizeof(double));
    if (e == cudaSuccess) e = upload2_closure_weights();
    if (e != cudaSuccess) {
      fprintf(stderr, "osb_create: %s\n", cudaGetErrorString(e));
      osb_destroy(c);
      return OSB_ECUDA;
    }
    *out = c;
    return OSB_OK;
  }
  {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && nsm > 0)
      c->num_sms = nsm;
  }
  if (c->mixed) { setup_central<float>(); setup_weno<float>(); }
  else { setup_central<double>(); setup_weno<double>(); }
  e = cudaGetLastError();
  for (int v = 0; v < 5 && e == cudaSuccess; ++v) {
    e = cudaMalloc(&c->qb[v], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->qold[v], (size_t)c->g.numel * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->res[v], bytes);
    if (e == cudaSuccess) e = cudaMemset(c->qb[v], 0, bytes);
    if (e == cudaSuccess) e = cudaMemset(c->qold[v], 0, (size_t)c->g.numel * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(c->res[v], 0, bytes);
  }
  if (e == cudaSuccess && plan->teno_adaptive) {
    e = cudaMalloc(&c->ct2, bytes);
    if (e == cudaSuccess) e = cudaMemset(c->ct2, 0, bytes);
    c->ph.ctp = c->ct2;
  }
  if (e == cudaSuccess && wall3(*plan)) {
    // LS-RK register, viscous terms, the x1 metric lines, a side stream for the viscous terms
    const size_t b64 = (size_t)c->g.numel * sizeof(double), nl = (size_t)c->g.n1;
    for (int v = 0; v < 5 && e == cudaSuccess; ++v) {
      e = cudaMalloc(&c->du2[v], b64);
      if (e == cudaSuccess) e = cudaMemset(c->du2[v], 0, b64);
    }
    for (int v = 0; v < 4 && e == cudaSuccess; ++v) {
      e = cudaMalloc(&c->resv[v], bytes);
      if (e == cudaSuccess) e = cudaMemset(c->resv[v], 0, bytes);
    }
    if (e == cudaSuccess) e = cudaMalloc(&c->x1, nl * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->d11, nl * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->sd111, nl * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->ysc_d, nl * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->ysc_f, nl * sizeof(float2));
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      e = cudaStreamCreateWithFlags(&c->side2[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join2[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork2, cudaEventDisableTiming);
    c->ph.ysc_d = c->ysc_d;
    c->ph.ysc_f = c->ysc_f;
    if (e == cudaSuccess && plan->body_force[0] != 0.0) {
      e = cudaMalloc(&c->bf_xy, (size_t)c->g.n0 * c->g.n1 * sizeof(double));
      if (e == cudaSuccess) e = cudaMalloc(&c->bf_z, (size_t)c->g.n2 * sizeof(double));
      if (e == cudaSuccess) e = cudaMalloc(&c->bf_t, sizeof(double));
      if (e == cudaSuccess) e = cudaMalloc(&c->d_iter, sizeof(long long));
      if (e == cudaSuccess) e = cudaMemset(c->bf_xy, 0, (size_t)c->g.n0 * c->g.n1 * sizeof(double));
      if (e == cudaSuccess) e = cudaMemset(c->bf_z, 0, (size_t)c->g.n2 * sizeof(double));
      if (e == cudaSuccess) e = cudaMemset(c->bf_t, 0, sizeof(double));
      if (e == cudaSuccess) e = cudaMemset(c->d_iter, 0, sizeof(long long));
    }
    if (e == cudaSuccess) {
      if (c->mixed) setup3w<float>();
      else setup3w<double>();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = upload2_closure_weights();  // Carpenter closure tables of the derivatives
  }
  c->red_blocks = 152 * 8;
  if (e == cudaSuccess) e = cudaMalloc(&c->red, (c->red_blocks + 1) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(int));
  if (e != cudaSuccess) {
    fprintf(stderr, "osb_create: %s\n", cudaGetErrorString(e));
    osb_destroy(c);
    return OSB_ECUDA;
  }
  if (plan->ndim == 3) encode_state_maps(*c, 1);
  *out = c;
  return OSB_OK;
}

int osb_bind_field(osb_ctx *c, int var, void *dev_ptr) {
  if (!c) return OSB_EINVAL;
  if (var < 0 || var >= c->nvar) return set_err(c, OSB_EINVAL, "var out of range");
  if (!dev_ptr || ((uintptr_t)dev_ptr % 32) != 0) return set_err(c, OSB_EINVAL, "device pointer null or not 32-byte aligned");
  c->qa[var] = dev_ptr;
  if (c->plan.ndim <= 2 && !c->mixed) c->q64_2d[var] = static_cast<double *>(dev_ptr);
  c->qold_valid = 0;
  c->cur = 0;
  if (c->plan.ndim == 3) encode_state_maps(*c, 0);
  for (int s = 0; s < 2; ++s)
    if (c->graph[s]) { cudaGraphExecDestroy(c->graph[s]); c->graph[s] = nullptr; }
  return OSB_OK;
}

int osb_set_stream(osb_ctx *c, void *stream) {
  if (!c) return OSB_EINVAL;
  c->stream = (cudaStream_t)stream;
  for (int s = 0; s < 2; ++s)
    if (c->graph[s]) { cudaGraphExecDestroy(c->graph[s]); c->graph[s] = nullptr; }
  return OSB_OK;
}

static int check_bound(osb_ctx *c) {
  for (int v = 0; v < c->nvar; ++v)
    if (!c->qa[v]) return set_err(c, OSB_ENOTBOUND, "a conserved variable is not bound");
  return OSB_OK;
}

int osb_init_tgv(osb_ctx *c) {
  if (!c) return OSB_EINVAL;
  if (int rc = check_bound(c)) return rc;
  if (c->plan.ndim != 3 || wall3(c->plan))
    return set_err(c, OSB_EUNSUPPORTED, "the Taylor-Green initial condition is for periodic or symmetric 3D blocks");
  const int nb = blocks_for((int64_t)c->g.n0 * c->g.n1 * c->g.n2);
  const osb_plan_desc &p = c->plan;
  if (c->mixed)
    k_init_tgv<float><<<nb, 256, 0, c->stream>>>(c->g, fields<float>(c->qa), fields_d(c->qold), p.delta[0], p.delta[1], p.delta[2], p.gama, p.Minf);
  else
    k_init_tgv<double><<<nb, 256, 0, c->stream>>>(c->g, fields<double>(c->qa), fields_d(c->qold), p.delta[0], p.delta[1], p.delta[2], p.gama, p.Minf);
  c->qold_valid = 1;
  c->cur = 0;
  int64_t l = 0;
  if (c->mixed) launch_halos<float>(*c, fields<float>(c->qa), c->stream, &l);
  else launch_halos<double>(*c, fields<double>(c->qa), c->stream, &l);
  return cuda_err(c, cudaGetLastError(), "osb_init_tgv");
}

// The address a kernel may use for p: device and managed memory as they are, page-locked host
// memory (cudaHostAlloc / cudaHostRegister, which unified addressing maps into the device's address
// space) through its device pointer, so that the kernels read or write it over the host link without
// a staging copy; nullptr for memory the device cannot reach (pageable host memory).
static const void *device_access(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

int osb_set_state64(osb_ctx *c, int var, const double *src) {
  if (!c) return OSB_EINVAL;
  if (int rc = check_bound(c)) return rc;
  if (var < 0 || var >= c->nvar || !src) return set_err(c, OSB_EINVAL, "bad var or pointer");
  src = static_cast<const double *>(device_access(src));
  if (!src) return set_err(c, OSB_EINVAL, "osb_set_state64: source is neither device nor page-locked host memory");
  const int nb = blocks_for((int64_t)c->g.n0 * c->g.n1 * c->g.n2);
  if (c->plan.ndim <= 2) {
    if (c->mixed) k_set64<float><<<nb, 256, 0, c->stream>>>(c->g, src, (float *)c->qa[var], c->q64_2d[var]);
    else k_set64<double><<<nb, 256, 0, c->stream>>>(c->g, src, (double *)c->qa[var], c->q64_2d[var]);
    c->qold_valid = 1;
    return cuda_err(c, cudaGetLastError(), "osb_set_state64");
  }
  if (c->mixed) k_set64<float><<<nb, 256, 0, c->stream>>>(c->g, src, (float *)c->qa[var], c->qold[var]);
  else k_set64<double><<<nb, 256, 0, c->stream>>>(c->g, src, (double *)c->qa[var], c->qold[var]);
  c->qold_valid = 1;
  c->cur = 0;
  if (var == 4 && !wall3(c->plan)) {  // wall-bounded blocks fill their halos at the start of a step
    int64_t l = 0;
    if (c->mixed) launch_halos<float>(*c, fields<float>(c->qa), c->stream, &l);
    else launch_halos<double>(*c, fields<double>(c->qa), c->stream, &l);
  }
  return cuda_err(c, cudaGetLastError(), "osb_set_state64");
}

}  // extern "C"

// point probes: what = 0..nvar-1 conserved variable, OSB_PROBE_U0.. derived (FP64 master state)
__global__ void k_probe(Grid g, Fields5<double> m, int nvar, int n, const int *req, double *out, double gm1, double gM2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int what = req[4 * t], i = req[4 * t + 1], j = req[4 * t + 2], k = req[4 * t + 3];
  const int64_t idx = gidx(g, i, j, k);
  if (what < nvar) {
    out[t] = m.v[what][idx];
    return;
  }
  const double rho = m.v[0][idx], E = m.v[nvar - 1][idx];
  const int ndim = nvar - 2;
  double ke = 0.0, u[3] = {0.0, 0.0, 0.0};
  for (int c = 0; c < ndim; ++c) {
    u[c] = m.v[1 + c][idx] / rho;
    ke += 0.5 * rho * u[c] * u[c];
  }
  const double p = gm1 * (E - ke);
  double v = 0.0;
  if (what <= OSB_PROBE_U2) v = u[what - OSB_PROBE_U0];
  else if (what == OSB_PROBE_P) v = p;
  else v = gM2 * p / rho;
  out[t] = v;
}

extern "C" {

int osb_probe(osb_ctx *c, int n, const int *what_ijk, double *host_out) {
  if (!c || n < 0 || (n > 0 && (!what_ijk || !host_out))) return OSB_EINVAL;
  if (n == 0) return OSB_OK;
  if (n > OSB_PROBE_MAX) return set_err(c, OSB_ETOOLARGE, "osb_probe: too many probes");
  if (!c->qold_valid) return set_err(c, OSB_EINVAL, "no state yet: call osb_init_tgv, osb_set_state64 or osb_step");
  const int n2 = c->plan.ndim <= 2 ? 1 : c->g.n2;
  for (int t = 0; t < n; ++t) {
    const int w = what_ijk[4 * t], i = what_ijk[4 * t + 1], j = what_ijk[4 * t + 2], k = what_ijk[4 * t + 3];
    const bool ok_w = (w >= 0 && w < c->nvar) || (w >= OSB_PROBE_U0 && w <= OSB_PROBE_T &&
                                                   (w != OSB_PROBE_U2 || c->plan.ndim == 3) &&
                                                   (w != OSB_PROBE_U1 || c->plan.ndim >= 2));
    if (!ok_w || i < 0 || i >= c->g.n0 || j < 0 || j >= c->g.n1 || k < 0 || k >= n2)
      return set_err(c, OSB_EINVAL, "osb_probe: quantity or index out of range");
  }
  cudaError_t e = cudaSuccess;
  if (!c->probe_buf) e = cudaMalloc(&c->probe_buf, OSB_PROBE_MAX * (4 * sizeof(int) + sizeof(double)));
  if (e != cudaSuccess) return cuda_err(c, e, "osb_probe allocation");
  int *req = reinterpret_cast<int *>(c->probe_buf);
  double *out = reinterpret_cast<double *>(req + 4 * OSB_PROBE_MAX);
  e = cudaMemcpyAsync(req, what_ijk, sizeof(int) * 4 * n, cudaMemcpyHostToDevice, c->stream);
  Fields5<double> m;
  for (int v = 0; v < 5; ++v) m.v[v] = v < c->nvar ? (c->plan.ndim <= 2 ? c->q64_2d[v] : c->qold[v]) : nullptr;
  if (e == cudaSuccess) {
    k_probe<<<(n + 127) / 128, 128, 0, c->stream>>>(c->g, m, c->nvar, n, req, out, c->ph.gm1, c->ph.gM2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(host_out, out, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "osb_probe");
}

int osb_get_state64(osb_ctx *c, int var, double *dst) {
  if (!c) return OSB_EINVAL;
  if (var < 0 || var >= c->nvar || !dst) return set_err(c, OSB_EINVAL, "bad var or pointer");
  dst = const_cast<double *>(static_cast<const double *>(device_access(dst)));
  if (!dst) return set_err(c, OSB_EINVAL, "osb_get_state64: destination is neither device nor page-locked host memory");
  if (!c->qold_valid) return set_err(c, OSB_EINVAL, "no state yet: call osb_init_tgv, osb_set_state64 or osb_step");
  const int nb = blocks_for((int64_t)c->g.n0 * c->g.n1 * c->g.n2);
  k_get64<<<nb, 256, 0, c->stream>>>(c->g, c->plan.ndim <= 2 ? c->q64_2d[var] : c->qold[var], dst);
  return cuda_err(c, cudaGetLastError(), "osb_get_state64");
}

int osb_teno_cutoff(osb_ctx *c, double *dev_out) {
  if (!c) return OSB_EINVAL;
  if (!dev_out) return set_err(c, OSB_EINVAL, "null output");
  if (!c->plan.teno_adaptive) return set_err(c, OSB_EINVAL, "plan has no adaptive TENO");
  if (int rc = check_bound(c)) return rc;
  if (c->plan.ndim == 1) return set_err(c, OSB_EUNSUPPORTED, "osb_teno_cutoff: 1D blocks have a fixed cut-off");
  if (wall3(c->plan)) {
    if (!c->metrics_valid) return set_err(c, OSB_EINVAL, "3D wall-bounded block: call osb_set_coordinate first");
    if (!c->qold_valid) return set_err(c, OSB_EINVAL, "set the state first");
    int64_t l = 0;
    if (c->mixed) launch3w_cutoff<float>(*c, dev_out, c->stream, &l);
    else launch3w_cutoff<double>(*c, dev_out, c->stream, &l);
    return cuda_err(c, cudaGetLastError(), "osb_teno_cutoff");
  }
  if (c->plan.ndim == 3) {
    if (!c->qold_valid) return set_err(c, OSB_EINVAL, "set the state first");
    int64_t l = 0;
    if (c->mixed) {
      launch_halos<float>(*c, fields<float>(c->qa), c->stream, &l);
      launch_cutoff3<float>(*c, fields<const float>(c->qa), dev_out, c->stream, &l);
    } else {
      launch_halos<double>(*c, fields<double>(c->qa), c->stream, &l);
      launch_cutoff3<double>(*c, fields<const double>(c->qa), dev_out, c->stream, &l);
    }
    return cuda_err(c, cudaGetLastError(), "osb_teno_cutoff");
  }
  if (!c->metrics_valid) return set_err(c, OSB_EINVAL, "2D block: call osb_set_coordinate first");
  if (!c->qold_valid) return set_err(c, OSB_EINVAL, "2D block: set the state first");
  int64_t l = 0;
  launch2_bcs(*c, c->stream, &l);
  if (c->mixed) launch2_cutoff<float>(*c, dev_out, c->stream, &l);
  else launch2_cutoff<double>(*c, dev_out, c->stream, &l);
  return cuda_err(c, cudaGetLastError(), "osb_teno_cutoff");
}

int osb_step(osb_ctx *c, int nsteps, double dt) {
  if (!c) return OSB_EINVAL;
  if (int rc = check_bound(c)) return rc;
  if (nsteps < 0 || !(dt > 0)) return set_err(c, OSB_EINVAL, "nsteps >= 0 and dt > 0 required");
  if (c->plan.ndim <= 2) {  // one_step2 steps 1D blocks too
    if (!c->metrics_valid) return set_err(c, OSB_EINVAL, "2D block: call osb_set_coordinate first");
    if (!c->qold_valid) return set_err(c, OSB_EINVAL, "set the state first");
    return c->mixed ? step2_impl<float>(c, nsteps, dt) : step2_impl<double>(c, nsteps, dt);
  }
  if (wall3(c->plan)) {
    if (!c->metrics_valid) return set_err(c, OSB_EINVAL, "3D wall-bounded block: call osb_set_coordinate first");
    if (!c->qold_valid) return set_err(c, OSB_EINVAL, "3D wall-bounded block: set the state first");
    return c->mixed ? step3w_impl<float>(c, nsteps, dt) : step3w_impl<double>(c, nsteps, dt);
  }
  return c->mixed ? step_impl<float>(c, nsteps, dt) : step_impl<double>(c, nsteps, dt);
}

int osb_residual(osb_ctx *c, void *dev_out) {
  if (!c) return OSB_EINVAL;
  if (int rc = check_bound(c)) return rc;
  if (!dev_out) return set_err(c, OSB_EINVAL, "null output");
  const int nb = blocks_for((int64_t)c->g.n0 * c->g.n1 * c->g.n2);
  if (c->plan.ndim == 1) {
    int64_t l = 0;
    launch1_bcs(*c, c->stream, &l);
    launch1_rhs(*c, 0, 0.0, 0.0, 0.0, c->stream, &l);
    P4 d;
    for (int v = 0; v < 3; ++v) d.v[v] = c->du2[v];
    k_pack_d<double><<<nb, 256, 0, c->stream>>>(c->g, d, (double *)dev_out, 3);
    return cuda_err(c, cudaGetLastError(), "osb_residual");
  }
  if (c->plan.ndim == 2) {
    if (!c->metrics_valid) return set_err(c, OSB_EINVAL, "2D block: call osb_set_coordinate first");
    int64_t l = 0;
    launch2_bcs(*c, c->stream, &l);
    P4 d;
    for (int v = 0; v < 4; ++v) d.v[v] = c->du2[v];
    if (c->mixed) {
      launch2_rhs<float>(*c, 0, 0.0, 0.0, 0.0, c->stream, &l);
      k_pack_d<float><<<nb, 256, 0, c->stream>>>(c->g, d, (float *)dev_out, 4);
    } else {
      launch2_rhs<double>(*c, 0, 0.0, 0.0, 0.0, c->stream, &l);
      k_pack_d<double><<<nb, 256, 0, c->stream>>>(c->g, d, (double *)dev_out, 4);
    }
    return cuda_err(c, cudaGetLastError(), "osb_residual");
  }
  if (wall3(c->plan)) {
    if (!c->metrics_valid) return set_err(c, OSB_EINVAL, "3D wall-bounded block: call osb_set_coordinate first");
    int64_t l = 0;
    P4 d;
    for (int v = 0; v < 5; ++v) d.v[v] = c->du2[v];
    if (c->mixed) {
      launch3w_bcs<float>(*c, c->stream, &l);
      launch3w_rhs<float>(*c, 0, 0.0, 0.0, 0.0, c->stream, &l);
      k_pack_d<float><<<nb, 256, 0, c->stream>>>(c->g, d, (float *)dev_out, 5);
    } else {
      launch3w_bcs<double>(*c, c->stream, &l);
      launch3w_rhs<double>(*c, 0, 0.0, 0.0, 0.0, c->stream, &l);
      k_pack_d<double><<<nb, 256, 0, c->stream>>>(c->g, d, (double *)dev_out, 5);
    }
    return cuda_err(c, cudaGetLastError(), "osb_residual");
  }
  if (c->mixed) {
    residual_into<float>(c, c->cur, c->stream);
    k_pack<float><<<nb, 256, 0, c->stream>>>(c->g, fields<const float>(c->res), (float *)dev_out);
  } else {
    residual_into<double>(c, c->cur, c->stream);
    k_pack<double><<<nb, 256, 0, c->stream>>>(c->g, fields<const double>(c->res), (double *)dev_out);
  }
  return cuda_err(c, cudaGetLastError(), "osb_residual");
}

int osb_reduce(osb_ctx *c, int what, double *out) {
  if (!c || !out) return OSB_EINVAL;
  if (int rc = check_bound(c)) return rc;
  if (what < OSB_RED_KE || what > OSB_RED_NANCHECK) return set_err(c, OSB_EINVAL, "unknown reduction");
  if (!c->qold_valid) return set_err(c, OSB_EINVAL, "no state yet");
  void **qs = c->cur == 0 ? c->qa : c->qb;
  const int64_t N = (int64_t)c->g.n0 * c->g.n1 * c->g.n2;
  int nb = blocks_for(N);
  if (nb > c->red_blocks) nb = c->red_blocks;
  if (c->plan.ndim <= 2) {
    if (what == OSB_RED_ENSTROPHY) return set_err(c, OSB_EUNSUPPORTED, "enstrophy: 3D blocks");
    D4 q2;
    for (int v = 0; v < 4; ++v) q2.v[v] = c->q64_2d[v];
    k_reduce2<<<nb, RED_THREADS, 0, c->stream>>>(c->g, q2, what, c->red, c->nvar);
    k_reduce_final<<<1, RED_THREADS, 0, c->stream>>>(c->red, nb, what, 1.0 / (double)N, c->red + c->red_blocks);
    double h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->red + c->red_blocks, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "osb_reduce");
    *out = h;
    if (what == OSB_RED_NANCHECK && h != 0.0) return set_err(c, OSB_ENONFINITE, "non-finite value in the state");
    return OSB_OK;
  }
  Fields5<const double> qo;
  for (int v = 0; v < 5; ++v) qo.v[v] = c->qold[v];
  const double *id = c->ph.inv_delta;
  if (c->mixed) k_reduce<float><<<nb, RED_THREADS, 0, c->stream>>>(c->g, qo, fields<const float>(qs), what, id[0], id[1], id[2], c->red);
  else k_reduce<double><<<nb, RED_THREADS, 0, c->stream>>>(c->g, qo, fields<const double>(qs), what, id[0], id[1], id[2], c->red);
  k_reduce_final<<<1, RED_THREADS, 0, c->stream>>>(c->red, nb, what, 1.0 / (double)N, c->red + c->red_blocks);
  double h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, c->red + c->red_blocks, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  int status = 0;
  if (e == cudaSuccess && c->d_status)
    e = cudaMemcpyAsync(&status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "osb_reduce");
  *out = h;
  if (status) return set_err(c, OSB_ETIMEOUT, "a bounded device wait gave up in an earlier step (status word set)");
  if (what == OSB_RED_NANCHECK && h != 0.0) return set_err(c, OSB_ENONFINITE, "non-finite value in the state");
  return OSB_OK;
}

int64_t osb_launch_count(osb_ctx *c) { return c ? c->launches : -1; }

int osb_profile(osb_ctx *c, int enable) {
  if (!c) return OSB_EINVAL;
  c->prof_on = enable ? 1 : 0;
  for (int f = 0; f < PF_COUNT; ++f) {
    c->prof_ms[f] = 0;
    c->prof_n[f] = 0;
  }
  return OSB_OK;
}

int osb_profile_read(osb_ctx *c, double *total_ms, int64_t *counts, int n) {
  if (!c || !total_ms || !counts) return OSB_EINVAL;
  for (int f = 0; f < n && f < PF_COUNT; ++f) {
    total_ms[f] = c->prof_ms[f];
    counts[f] = c->prof_n[f];
  }
  return PF_COUNT;
}

static void drop_graphs(osb_ctx *c) {
  for (int s = 0; s < 2; ++s)
    if (c->graph[s]) {
      cudaGraphExecDestroy(c->graph[s]);
      c->graph[s] = nullptr;
    }
}

int osb_set_weno_shape(osb_ctx *c, int dir, int kind, int seg) {
  if (!c) return OSB_EINVAL;
  if (dir < 0 || dir > 2) return set_err(c, OSB_EINVAL, "osb_set_weno_shape: dir must be 0, 1 or 2");
  if (kind != OSB_WENO_TILE && kind != OSB_WENO_MARCH4 && kind != OSB_WENO_MARCH8)
    return set_err(c, OSB_EINVAL, "osb_set_weno_shape: unknown kind");
  if (seg < 4 || seg > 4096) return set_err(c, OSB_EINVAL, "osb_set_weno_shape: seg must lie in [4, 4096]");
  c->wcfg[dir] = WenoCfg{kind, seg};
  drop_graphs(c);
  return OSB_OK;
}

int osb_get_weno_shape(osb_ctx *c, int dir, int *kind, int *seg) {
  if (!c || dir < 0 || dir > 2 || !kind || !seg) return OSB_EINVAL;
  *kind = c->wcfg[dir].kind;
  *seg = c->wcfg[dir].seg;
  return OSB_OK;
}

}  // extern "C"

template <typename T> static int autotune_impl(osb_ctx *c, int reps, double *best_ms) {
  cudaStream_t s = c->stream;
  void **qs = c->cur == 0 ? c->qa : c->qb;
  Fields5<const T> qc = fields<const T>(qs);
  Fields5<T> r = fields<T>(c->res);
  launch_halos<T>(*c, fields<T>(qs), s, &c->launches);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t err = cudaSuccess;
  // time `launch` (one warm-up, then reps launches); returns ms per launch, or -1 on error
  auto timeit = [&](auto &&launch) -> float {
    launch();
    cudaEventRecord(e0, s);
    for (int k = 0; k < reps; ++k) launch();
    cudaEventRecord(e1, s);
    err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err != cudaSuccess) return -1.0f;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / reps;
  };
  for (int t = 0; t < OSB_TUNE_SLOTS && best_ms; ++t) best_ms[t] = 0.0;
  const int n[3] = {c->g.n0, c->g.n1, c->g.n2};
  const bool weno = char_fluxes(c->plan);
  for (int d = 0; d < 3 && weno && err == cudaSuccess; ++d) {
    std::vector<WenoCfg> cand{{WENO_TILE, 32}};
    for (int kind : {WENO_MARCH4, WENO_MARCH8}) {
      for (int seg : {16, 24, 32, 48, 64, 96, 128, 192, 256})
        if (seg < n[d]) cand.push_back({kind, seg});
      cand.push_back({kind, n[d]});
    }
    float best = 1e30f;
    WenoCfg choice = c->wcfg[d];
    for (const WenoCfg &w : cand) {
      const float ms = timeit([&] { launch_weno_cfg<T>(*c, qc, r, d, w, s); });
      if (ms < 0) break;
      if (ms < best) {
        best = ms;
        choice = w;
      }
    }
    c->wcfg[d] = choice;
    if (best_ms) best_ms[d] = best;
  }
  if (err == cudaSuccess) {
    // residual-only form of the step's central kernel: same stencils and loads, writes R into the
    // residual scratch instead of touching the state and the RK register
    const int visc = c->plan.visc == OSB_VISC_CONST ? CRK_VISC : 0;
    const int mode = (weno ? CRK_RIN : CRK_SKEW) | visc;
    float best = 1e30f;
    int choice = c->crk_ty;
    for (int ty : {8, 16}) {
      c->crk_ty = ty;
      int64_t dummy = 0;
      const float ms = timeit([&] {
        launch_central_rk<T>(*c, qc, r, fields_d(c->qold), r, r, 0.0, 0.0, mode, s, &dummy);
      });
      if (ms < 0) break;
      if (ms < best) {
        best = ms;
        choice = ty;
      }
    }
    c->crk_ty = choice;
    if (best_ms) best_ms[3] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  drop_graphs(c);
  return cuda_err(c, err, "osb_autotune");
}

extern "C" {

static int adjoint_check(osb_ctx *c) {
  if (!c) return OSB_EINVAL;
  const osb_plan_desc &p = c->plan;
  if (p.ndim != 3 || c->mixed || (p.conv != OSB_CONV_CENTRAL_SKEW && !char_fluxes(p)))
    return set_err(c, OSB_EUNSUPPORTED, "adjoint: FP64 3D plans with central or characteristic fluxes only");
  for (int d = 0; d < 3; ++d)
    if (p.bc[d][0] != OSB_BC_PERIODIC || p.bc[d][1] != OSB_BC_PERIODIC)
      return set_err(c, OSB_EUNSUPPORTED, "adjoint: periodic boundaries only");
  if (p.teno_adaptive || p.filter != OSB_FILTER_NONE)
    return set_err(c, OSB_EUNSUPPORTED, "adjoint: fixed TENO cut-off and no WENO filter");
  int rc = check_bound(c);
  if (rc) return rc;
  return cuda_err(c, adj_ensure(*c), "adjoint scratch allocation");
}

int osb_adjoint_residual(osb_ctx *c, const double *lam, double *out) {
  int rc = adjoint_check(c);
  if (rc) return rc;
  if (!lam || !out) return set_err(c, OSB_EINVAL, "osb_adjoint_residual: null array");
  return cuda_err(c, adj_residual(*c, fields<double>(c->cur == 0 ? c->qa : c->qb), lam, out), "osb_adjoint_residual");
}

int osb_adjoint_step(osb_ctx *c, double dt, const double *lam_in, double *lam_out) {
  int rc = adjoint_check(c);
  if (rc) return rc;
  if (!lam_in || !lam_out) return set_err(c, OSB_EINVAL, "osb_adjoint_step: null array");
  return cuda_err(c, adj_step(*c, fields<double>(c->cur == 0 ? c->qa : c->qb), dt, lam_in, lam_out),
                  "osb_adjoint_step");
}

int osb_set_central_shape(osb_ctx *c, int ty) {
  if (!c) return OSB_EINVAL;
  if (ty != 8 && ty != 16) return set_err(c, OSB_EINVAL, "osb_set_central_shape: ty must be 8 or 16");
  c->crk_ty = ty;
  drop_graphs(c);
  return OSB_OK;
}

int osb_set_tma(osb_ctx *c, int enable) {
  if (!c) return OSB_EINVAL;
  c->tma_enabled = enable ? 1 : 0;
  drop_graphs(c);
  return OSB_OK;
}

int osb_tma_active(osb_ctx *c) {
  if (!c) return OSB_EINVAL;
  const int buf_ok = c->cur == 0 ? c->tma_ok[0] : c->tma_ok[1];
  return (c->tma_enabled && buf_ok && c->plan.ndim == 3 && c->mixed &&
          (char_fluxes(c->plan))) ? 1 : 0;
}

int osb_get_central_shape(osb_ctx *c, int *ty) {
  if (!c || !ty) return OSB_EINVAL;
  *ty = c->crk_ty;
  return OSB_OK;
}

int osb_autotune(osb_ctx *c, int reps, double *best_ms) {
  if (!c) return OSB_EINVAL;
  if (reps < 1) return set_err(c, OSB_EINVAL, "osb_autotune: reps must be >= 1");
  if (c->plan.ndim != 3 || wall3(c->plan)) {  // the tuner times the periodic blocks' kernels
    for (int t = 0; t < OSB_TUNE_SLOTS && best_ms; ++t) best_ms[t] = 0.0;
    return OSB_OK;
  }
  int rc = check_bound(c);
  if (rc) return rc;
  return c->mixed ? autotune_impl<float>(c, reps, best_ms) : autotune_impl<double>(c, reps, best_ms);
}

int osb_get_error(osb_ctx *c, char *buf, int n) {
  if (!c || !buf || n <= 0) return OSB_EINVAL;
  snprintf(buf, (size_t)n, "%s", c->err.c_str());
  return OSB_OK;
}

void osb_destroy(osb_ctx *c) {
  if (!c) return;
  for (int s = 0; s < 2; ++s)
    if (c->graph[s]) cudaGraphExecDestroy(c->graph[s]);
  for (int v = 0; v < 5; ++v) {
    cudaFree(c->qb[v]);
    cudaFree(c->qold[v]);
    cudaFree(c->res[v]);
  }
  cudaFree(c->red);
  cudaFree(c->d_status);
  cudaFree(c->adj);
  cudaFree(c->probe_buf);
  for (int v = 0; v < 4; ++v)
    if (c->mixed) cudaFree(c->q64_2d[v]);
  for (int v = 0; v < 5; ++v) cudaFree(c->du2[v]);
  for (int k = 0; k < 6; ++k) cudaFree(c->prim2[k]);
  for (int v = 0; v < 4; ++v) cudaFree(c->resy[v]);
  for (int v = 0; v < 4; ++v) cudaFree(c->resv[v]);
  cudaFree(c->ysc_d);
  cudaFree(c->ysc_f);
  cudaFree(c->bf_xy);
  cudaFree(c->bf_z);
  cudaFree(c->bf_t);
  cudaFree(c->d_iter);
  for (int k = 0; k < 2; ++k) {
    if (c->side2[k]) cudaStreamDestroy(c->side2[k]);
    if (c->ev_join2[k]) cudaEventDestroy(c->ev_join2[k]);
  }
  if (c->ev_fork2) cudaEventDestroy(c->ev_fork2);
  cudaFree(c->ct2);
  cudaFree(c->x1);
  cudaFree(c->d11);
  cudaFree(c->sd111);
  delete c;
}

}  // extern "C"
