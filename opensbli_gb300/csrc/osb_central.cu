// osb_central.cu -- fused central-difference RHS and Runge-Kutta update.
//
// One kernel evaluates, per interior point, everything the generated solver spreads over its
// "CR*", "Convective terms group d", "Convective CD ...", "Convective residual", "Viscous CD ...",
// "Viscous residual", "Sub stage advancement" and "Temporal solution advancement" kernels
// (algorithm.py:384-477; probe census: ~75 ops_par_loops and ~45 full-grid work arrays per stage),
// without any intermediate array in HBM:
//   * constituent relations u_i = rhou_i/rho, p = (gama-1)(rhoE - 1/2 rho |u|^2),
//     T = gama Minf^2 p/rho (apps/taylor_green_vortex/taylor_green_vortex.py:30-32);
//   * skew-symmetric convective terms (core/parsing.py:75-111, schemes/spatial/scheme.py:187-271)
//       mass    -1/2 [ d_j(rho u_j) + u_j d_j rho + rho d_j u_j ]
//       mom_i   -1/2 [ d_j(rhou_i u_j) + u_j d_j rhou_i + rhou_i d_j u_j ] - d_i p
//       energy  -1/2 [ d_j(rhoE u_j) + u_j d_j rhoE + rhoE d_j u_j ] - d_j(p u_j);
//   * viscous and heat-flux terms, constant viscosity (taylor_green_vortex.py:18-19), expanded as
//     the generated "Viscous residual" kernel: mom_i += (lap u_i + 1/3 d_i div u)/Re,
//     energy += kT lap T + tau_ij d_j u_i + u_i d_j tau_ij, mixed second derivatives as nested
//     first derivatives, inner axis the lower one (scheme.py:360-387);
//   * 4th-order central weights (opensblifunctions.py:485-521, scheme.py:81-85);
//   * the 2-register RK3 update (schemes/temporal/rk_sbli.py:117-124):
//       q = qold + dt*rknew[s]*R,  qold = qold + dt*rkold[s]*R   (qold kept in FP64).
//
// Tiling: a 32 x TY (x,y) tile per block marches through a chunk of z.  A ring of 5 shared-memory
// planes holds the primitive fields of planes k-2..k+2 with a 2-point x/y halo, so every first,
// second and mixed derivative of the stencil is read from shared memory; each global point is
// loaded once per plane visit (coalesced along x).  The ring holds u0, u1, u2, T and, when the
// skew-symmetric convective terms are evaluated, rho, p and rhoE as well (with WENO fluxes the
// kernel needs only the viscous stencils: 4 fields, so more blocks fit on an SM).
#include <cstdio>

#include "osb_common.cuh"
#include "osb_cvt.cuh"
#include "osb_internal.h"

namespace osb {

namespace {
constexpr int TX = 32, PX = TX + 4, NP = 5;
enum { F_U0 = 0, F_U1, F_U2, F_T, F_RHO, F_P, F_E };
template <int MODE> __host__ __device__ constexpr int ring_fields() { return (MODE & CRK_SKEW) ? 7 : 4; }
// FP32: the 4-field ring allows 1024 resident threads per SM (64 registers); the 7-field ring is
// limited by shared memory to 3 blocks of 32x8 or 1 of 32x16.  FP64 runs on the FP64 pipe's rate.
template <typename T, int MODE, int TY> __host__ __device__ constexpr int central_min_blocks() {
  return sizeof(T) != 4 ? 1 : (MODE & CRK_SKEW) ? (TY == 8 ? 3 : 1) : 1024 / (TX * TY);
}
template <typename T, int MODE, int TY> __host__ __device__ constexpr size_t ring_bytes() {
  return sizeof(T) * (size_t)NP * ring_fields<MODE>() * (TY + 4) * PX;
}
}  // namespace

// One tile: output points (bx*32 .. +31, by*TY .. +TY-1) for the z-planes of chunk bz.  Called by
// the per-block kernel below and by the batched persistent kernel (osb_batch.cu).
template <typename T, int MODE, int TY, bool TMA = false>
__device__ __forceinline__ void central_tile(const Grid &g, Fields5<const T> q, Fields5<T> qnew, Fields5<double> qold,
                                             Fields5<T> rin, Fields5<T> rout, const Phys &ph, double dt_new,
                                             double dt_old, T ddt, int zchunk, int bx, int by, int bz,
                                             unsigned char *smem_raw, const TmaPlanes *tp = nullptr,
                                             int *status = nullptr) {
  constexpr int NF = ring_fields<MODE>(), PY = TY + 4;
  T *ring = reinterpret_cast<T *>(smem_raw);  // [NP][NF][PY][PX]
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = bx * TX, j0 = by * TY, k0 = bz * zchunk;
  const int k1 = min(k0 + zchunk, g.n2);
  const T gm1 = pick<T>(ph.gm1, ph.f_gm1), gm1_lo = pick<T>(0.0, ph.f_gm1_lo);
  const T gM2 = pick<T>(ph.gM2, ph.f_gM2);

  auto slot = [](int k) { return ((k % NP) + NP) % NP; };
  auto at = [&](int sl, int f, int py, int px) -> T & { return ring[((sl * NF + f) * PY + py) * PX + px]; };
  // Plane loads are software-pipelined: the global loads of plane k+3 are issued into registers
  // before the stencil work on plane k and written (as primitives) into the ring after it.
  constexpr int PPT = (PX * PY + TX * TY - 1) / (TX * TY);  // points per thread per plane
  T pre[PPT][5];
  auto fetch = [&](int k) {
#pragma unroll
    for (int r = 0; r < PPT; ++r) {
      const int e = tid + r * TX * TY;
      const int px = e % PX, py = e / PX;
      const int i = i0 - 2 + px, j = j0 - 2 + py;
      if (e < PX * PY && i < g.n0 + 2 && j < g.n1 + 2 && k < g.n2 + 2) {
        const int64_t n = gidx(g, i, j, k);
#pragma unroll
        for (int v = 0; v < 5; ++v) pre[r][v] = q.v[v][n];
      }
    }
  };
  // primitives of one point into ring slot sl at (py, px)
  // (FP32: u, p and T rounded once from their exact values, prims_f32, so the first- and second-
  // derivative stencils see no extra rounding noise in them)
  auto put = [&](int sl, int py, int px, T rho, T r0, T r1, T r2, T E) {
    T u0, u1, u2, p, Tt;
    if constexpr (sizeof(T) == 4) {
      float irho, u[3], p_lo;
      prims_f32(rho, r0, r1, r2, E, gm1, gm1_lo, irho, u, p, p_lo);
      u0 = u[0];
      u1 = u[1];
      u2 = u[2];
      Tt = scaled_ratio_f32(gM2, p, p_lo, rho, irho);
    } else {
      const T irho = T(1) / rho;  // correctly rounded: u and T feed the viscous terms
      u0 = r0 * irho;
      u1 = r1 * irho;
      u2 = r2 * irho;
      const T half = T(0.5);
      p = gm1 * (E - half * rho * u0 * u0 - half * rho * u1 * u1 - half * rho * u2 * u2);
      Tt = gM2 * p * irho;
    }
    at(sl, F_U0, py, px) = u0;
    at(sl, F_U1, py, px) = u1;
    at(sl, F_U2, py, px) = u2;
    at(sl, F_T, py, px) = Tt;
    if (NF == 7) {
      at(sl, F_RHO, py, px) = rho;
      at(sl, F_P, py, px) = p;
      at(sl, F_E, py, px) = E;
    }
  };
  auto store = [&](int k) {
    const int sl = slot(k);
#pragma unroll
    for (int r = 0; r < PPT; ++r) {
      const int e = tid + r * TX * TY;
      const int px = e % PX, py = e / PX;
      const int i = i0 - 2 + px, j = j0 - 2 + py;
      if (e < PX * PY && i < g.n0 + 2 && j < g.n1 + 2 && k < g.n2 + 2)
        put(sl, py, px, pre[r][0], pre[r][1], pre[r][2], pre[r][3], pre[r][4]);
    }
  };

  // TMA path: the conserved planes arrive as boxes of RX x PY points per field (x from i0-4, so the
  // copy starts on a 16-byte boundary), NS planes ahead, each completing on its own mbarrier
  constexpr int NS = 2, RX = 40;
  constexpr uint32_t PLANE_BYTES = 5u * RX * PY * sizeof(T);
  __shared__ __align__(8) uint64_t bars[NS];
  __shared__ int failed;
  T *raw = reinterpret_cast<T *>(smem_raw + ((ring_bytes<T, MODE, TY>() + 127) / 128) * 128);  // [NS][5][PY][RX]
  const int zfirst = k0 - 2, zlast = min(k1 + 1, g.n2 + 1);
  auto issue = [&](int z) {  // one thread
    const int st = (z - zfirst) % NS;
    mbar_expect_tx(&bars[st], PLANE_BYTES);
#pragma unroll
    for (int v = 0; v < 5; ++v)
      tma_load_3d(raw + (st * 5 + v) * PY * RX, &tp->m[v], i0, j0 - 2 + HY, z + HZ, &bars[st]);
  };
  auto wait_plane = [&](int z) {
    const int st = (z - zfirst) % NS;
    const uint32_t par = ((z - zfirst) / NS) & 1u;
    if (failed) return;
    for (uint32_t it = 0;; ++it) {
      if (mbar_try_wait(&bars[st], par)) return;
      if (it > (1u << 22)) {  // bounded: report through the status word and carry on
        failed = 1;
        if (status) atomicExch(status, 1);
        return;
      }
    }
  };
  auto convert = [&](int z) {  // raw plane z -> ring
    const int st = (z - zfirst) % NS, sl = slot(z);
    const T *b = raw + st * 5 * PY * RX;
#pragma unroll
    for (int r = 0; r < PPT; ++r) {
      const int e = tid + r * TX * TY;
      const int px = e % PX, py = e / PX;
      const int i = i0 - 2 + px, j = j0 - 2 + py;
      if (e < PX * PY && i < g.n0 + 2 && j < g.n1 + 2) {
        const int o = py * RX + px + 2;
        put(sl, py, px, b[o], b[PY * RX + o], b[2 * PY * RX + o], b[3 * PY * RX + o], b[4 * PY * RX + o]);
      }
    }
  };

  const T c2[5] = {T(-1.0 / 12.0), T(4.0 / 3.0), T(-2.5), T(4.0 / 3.0), T(-1.0 / 12.0)};
  // 4th-order first derivative (times delta) from the values at offsets -2, -1, +1, +2, written on the
  // differences of opposite points: rounding then scales with those differences, not with |f|
  auto d1 = [](T fm2, T fm1, T fp1, T fp2) -> T { return T(2.0 / 3.0) * (fp1 - fm1) - T(1.0 / 12.0) * (fp2 - fm2); };
  // 4th-order second derivative (times delta^2): FP32 on the differences from the centre value, FP64
  // as the weighted sum
  auto d2 = [&](T fm2, T fm1, T f0, T fp1, T fp2) -> T {
    if constexpr (sizeof(T) == 4)
      return T(4.0 / 3.0) * ((fp1 - f0) + (fm1 - f0)) - T(1.0 / 12.0) * ((fp2 - f0) + (fm2 - f0));
    return c2[0] * fm2 + c2[1] * fm1 + c2[2] * f0 + c2[3] * fp1 + c2[4] * fp2;
  };
  const T idl[3] = {pick<T>(ph.inv_delta[0], ph.f_inv_delta[0]), pick<T>(ph.inv_delta[1], ph.f_inv_delta[1]),
                    pick<T>(ph.inv_delta[2], ph.f_inv_delta[2])};
  const T idl_lo[3] = {pick<T>(0.0, ph.f_inv_delta_lo[0]), pick<T>(0.0, ph.f_inv_delta_lo[1]),
                       pick<T>(0.0, ph.f_inv_delta_lo[2])};

  if constexpr (TMA) {
    // every TMA destination must sit on a 128-byte boundary: refuse (status 2) rather than copy
    if ((smem_u32(raw) & 127u) != 0u) {
      if (tid == 0 && status) atomicExch(status, 2);
      return;
    }
    if (tid == 0) {
      for (int s = 0; s < NS; ++s) mbar_init(&bars[s], 1);
      failed = 0;
      fence_async_smem();
    }
    __syncthreads();
    if (tid == 0)
      for (int z = zfirst; z < zfirst + NS && z <= zlast; ++z) issue(z);
    for (int z = k0 - 2; z < k0 + 3; ++z) {
      wait_plane(z);
      convert(z);
      __syncthreads();  // ring visible; the raw stage of z may be refilled
      if (tid == 0 && z + NS <= zlast) issue(z + NS);
    }
  } else {
    for (int k = k0 - 2; k < k0 + 3; ++k) {
      fetch(k);
      store(k);
    }
  }
  for (int k = k0; k < k1; ++k) {
    __syncthreads();
    if constexpr (TMA) {
      // the raw stage of plane k+2 (converted at the end of the previous iteration) is free now
      if (k > k0 && tid == 0 && k + 2 + NS <= zlast) issue(k + 2 + NS);
    } else {
      if (k + 3 < k1 + 2) fetch(k + 3);
    }
    const int i = i0 + tx, j = j0 + ty;
    const bool active = i < g.n0 && j < g.n1;
    // the residual already in rin and the FP64 register at the output point, loaded early
    T rpre[5];
    double opre[5];
    int64_t nout = 0;
    if (active) {
      nout = gidx(g, i, j, k);
      if (k + 2 < k1) {
        // L2 prefetch of the output-point arrays two planes ahead (no registers held)
        const int64_t np = nout + 2 * g.sz;
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          if (MODE & CRK_RIN) prefetch_l2(rin.v[v] + np);
          if (MODE & CRK_UPDATE) prefetch_l2(qold.v[v] + np);
        }
      }
      if (MODE & CRK_RIN) {
#pragma unroll
        for (int v = 0; v < 5; ++v) rpre[v] = rin.v[v][nout];
      }
      if (MODE & CRK_UPDATE) {
#pragma unroll
        for (int v = 0; v < 5; ++v) opre[v] = qold.v[v][nout];
      }
    }
    if (active) {
      // field f at offset (dz, dy, dx) from the output point
      auto S = [&](int f, int dz, int dy, int dx) -> T { return at(slot(k + dz), f, ty + 2 + dy, tx + 2 + dx); };
      auto SA = [&](int f, int axis, int o) -> T {
        return axis == 0 ? S(f, 0, 0, o) : axis == 1 ? S(f, 0, o, 0) : S(f, o, 0, 0);
      };
      T R[5] = {T(0), T(0), T(0), T(0), T(0)};
      // first derivatives of the velocity, shared by both parts: du[c][d] = d_d u_c
      T du[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          du[c][d] = mul_hl(d1(SA(F_U0 + c, d, -2), SA(F_U0 + c, d, -1), SA(F_U0 + c, d, 1), SA(F_U0 + c, d, 2)),
                            idl[d], idl_lo[d]);
        }
      const T divu = du[0][0] + du[1][1] + du[2][2];
      const T uu[3] = {S(F_U0, 0, 0, 0), S(F_U1, 0, 0, 0), S(F_U2, 0, 0, 0)};

      if constexpr ((MODE & CRK_SKEW) != 0) {
        const T rho0 = S(F_RHO, 0, 0, 0);
        const T phi0[5] = {rho0, rho0 * uu[0], rho0 * uu[1], rho0 * uu[2], S(F_E, 0, 0, 0)};
        T acc[5] = {T(0), T(0), T(0), T(0), T(0)};
        T dpu = T(0);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          // the five conserved quantities phi, phi u_d, p and p u_d at offsets -2, -1, +1, +2 along d
          T phi[4][5], phu[4][5], pp[4], ppu[4];
#pragma unroll
          for (int s4 = 0; s4 < 4; ++s4) {
            const int o = s4 < 2 ? s4 - 2 : s4 - 1;
            const T r = SA(F_RHO, d, o), ud = SA(F_U0 + d, d, o);
            phi[s4][0] = r;
            phi[s4][1] = r * SA(F_U0, d, o);
            phi[s4][2] = r * SA(F_U1, d, o);
            phi[s4][3] = r * SA(F_U2, d, o);
            phi[s4][4] = SA(F_E, d, o);
#pragma unroll
            for (int v = 0; v < 5; ++v) phu[s4][v] = phi[s4][v] * ud;
            pp[s4] = SA(F_P, d, o);
            ppu[s4] = pp[s4] * ud;
          }
          T dphi[5], dphiu[5];
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            dphi[v] = d1(phi[0][v], phi[1][v], phi[2][v], phi[3][v]);
            dphiu[v] = d1(phu[0][v], phu[1][v], phu[2][v], phu[3][v]);
          }
          const T dp = d1(pp[0], pp[1], pp[2], pp[3]), dpud = d1(ppu[0], ppu[1], ppu[2], ppu[3]);
#pragma unroll
          for (int v = 0; v < 5; ++v) acc[v] += mul_hl(dphiu[v] + uu[d] * dphi[v], idl[d], idl_lo[d]);
          R[1 + d] -= mul_hl(dp, idl[d], idl_lo[d]);
          dpu += mul_hl(dpud, idl[d], idl_lo[d]);
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) R[v] -= T(0.5) * (acc[v] + phi0[v] * divu);
        R[4] -= dpu;
      }

      if (MODE & CRK_VISC) {
        const T invRe = pick<T>(ph.invRe, ph.f_invRe);
        const T kT = pick<T>(ph.kT, ph.f_kT);
        // own-axis second derivatives of u_c and T
        T d2u[3][3], lapT = T(0);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const T id2 = idl[d] * idl[d];
#pragma unroll
          for (int c = 0; c < 3; ++c)
            d2u[c][d] = d2(SA(F_U0 + c, d, -2), SA(F_U0 + c, d, -1), SA(F_U0 + c, d, 0), SA(F_U0 + c, d, 1),
                           SA(F_U0 + c, d, 2)) * id2;
          lapT += d2(SA(F_T, d, -2), SA(F_T, d, -1), SA(F_T, d, 0), SA(F_T, d, 1), SA(F_T, d, 2)) * id2;
        }
        // mixed derivative d_b(d_a u_c), a < b
        auto mixed = [&](int c, int a, int b) -> T {
          T inner[4];
#pragma unroll
          for (int sb = 0; sb < 4; ++sb) {
            const int ob = sb < 2 ? sb - 2 : sb - 1;
            T f[4];
#pragma unroll
            for (int sa = 0; sa < 4; ++sa) {
              int o[3] = {0, 0, 0};
              o[a] = sa < 2 ? sa - 2 : sa - 1;
              o[b] = ob;
              f[sa] = S(F_U0 + c, o[2], o[1], o[0]);
            }
            inner[sb] = d1(f[0], f[1], f[2], f[3]) * idl[a];
          }
          return d1(inner[0], inner[1], inner[2], inner[3]) * idl[b];
        };
        // d_i(div u) = d_ii u_i + sum_{c != i} d_i d_c u_c
        const T m01_1 = mixed(1, 0, 1), m02_2 = mixed(2, 0, 2);  // for i = 0
        const T m01_0 = mixed(0, 0, 1), m12_2 = mixed(2, 1, 2);  // for i = 1
        const T m02_0 = mixed(0, 0, 2), m12_1 = mixed(1, 1, 2);  // for i = 2
        const T ddiv[3] = {d2u[0][0] + m01_1 + m02_2, d2u[1][1] + m01_0 + m12_2, d2u[2][2] + m02_0 + m12_1};
        T mom[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          mom[c] = invRe * (d2u[c][0] + d2u[c][1] + d2u[c][2] + T(1.0 / 3.0) * ddiv[c]);
          R[1 + c] += mom[c];
        }
        T e = kT * lapT;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            T tau = du[a][b] + du[b][a];
            if (a == b) tau -= T(2.0 / 3.0) * divu;
            e += invRe * tau * du[a][b];
          }
        e += uu[0] * mom[0] + uu[1] * mom[1] + uu[2] * mom[2];
        R[4] += e;
      }

      const int64_t n = nout;
      if (MODE & CRK_RIN) {
#pragma unroll
        for (int v = 0; v < 5; ++v) R[v] += rpre[v];
      }
      if (MODE & CRK_UPDATE) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const double o = opre[v];
          if constexpr (sizeof(T) == 8) {
            const double r = (double)R[v];
            qold.v[v][n] = dt_old * r + o;
            qnew.v[v][n] = (T)(dt_new * r + o);
          } else {
            // FP32 state: the stage value q = qold + dt_new R equals qold' + (dt_new - dt_old) R;
            // rounding qold' and adding the small FP32 correction leaves one FP64 FMA per variable
            // on the FP64 pipe, the conversions run on the integer pipes (osb_cvt.cuh)
            const double o2 = fma(dt_old, cvt_f32_f64(R[v]), o);
            qold.v[v][n] = o2;
            qnew.v[v][n] = cvt_f64_f32(o2) + ddt * R[v];
          }
        }
      } else {
#pragma unroll
        for (int v = 0; v < 5; ++v) rout.v[v][n] = R[v];
      }
    }
    __syncthreads();
    if (k + 3 < k1 + 2) {
      if constexpr (TMA) {
        wait_plane(k + 3);
        convert(k + 3);
      } else {
        store(k + 3);
      }
    }
  }
  if constexpr (TMA) {
    // after a timed-out wait, give copies still in flight a bounded chance to land before the
    // block's shared memory is released
    if (failed && tid == 0)
      for (int s = 0; s < NS; ++s)
        for (uint32_t it = 0; it < (1u << 20); ++it)
          if (mbar_try_wait(&bars[s], 0u) || mbar_try_wait(&bars[s], 1u)) break;
  }
}

template <typename T, int MODE, int TY>
__global__ void __launch_bounds__(TX * TY, central_min_blocks<T, MODE, TY>())
    k_central_rk(Grid g, Fields5<const T> q, Fields5<T> qnew, Fields5<double> qold, Fields5<T> rin, Fields5<T> rout,
                 Phys ph, double dt_new, double dt_old, T ddt, int zchunk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  central_tile<T, MODE, TY>(g, q, qnew, qold, rin, rout, ph, dt_new, dt_old, ddt, zchunk, blockIdx.x, blockIdx.y,
                            blockIdx.z,
                            smem_raw);
}

// the same kernel with the conserved planes brought in by TMA (FP32 state, residual-input modes)
template <typename T, int MODE, int TY>
__global__ void __launch_bounds__(TX * TY, central_min_blocks<T, MODE, TY>())
    k_central_rk_tma(const __grid_constant__ TmaPlanes maps, Grid g, Fields5<T> qnew, Fields5<double> qold,
                     Fields5<T> rin, Fields5<T> rout, Phys ph, double dt_new, double dt_old, T ddt, int zchunk,
                     int *status) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // TMA destinations must start on 128-byte boundaries of the shared window; the dynamic region
  // follows the static shared variables, so align its base explicitly (128 bytes are reserved)
  unsigned char *base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  Fields5<const T> qnull{};
  central_tile<T, MODE, TY, true>(g, qnull, qnew, qold, rin, rout, ph, dt_new, dt_old, ddt, zchunk, blockIdx.x,
                                  blockIdx.y, blockIdx.z, base, &maps, status);
}

template <typename T, int MODE, int TY> constexpr size_t tma_smem_bytes() {
  // 128 bytes of slack for aligning the region's base, the ring rounded to 128, two raw planes
  return 128 + ((ring_bytes<T, MODE, TY>() + 127) / 128) * 128 + 2 * 5 * 40 * (TY + 4) * sizeof(T);
}

// resident blocks per SM of one kernel instance (occupancy calculator, cached per instance)
template <typename T, int MODE, int TY> static int resident_per_sm() {
  static int nb = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_central_rk<T, MODE, TY>, TX * TY,
                                                      ring_bytes<T, MODE, TY>()) != cudaSuccess || b < 1)
      b = 1;
    return b;
  }();
  return nb;
}

template <typename T, int MODE, int TY> static int resident_per_sm_tma() {
  static int nb = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_central_rk_tma<T, MODE, TY>, TX * TY,
                                                      tma_smem_bytes<T, MODE, TY>()) != cudaSuccess || b < 1)
      b = 1;
    return b;
  }();
  return nb;
}

template <typename T, int MODE, int TY>
static void launch_mode(const Ctx &c, Fields5<const T> q, Fields5<T> qnew, Fields5<double> qold, Fields5<T> rin,
                        Fields5<T> rout, double dt_new, double dt_old, cudaStream_t s) {
  // TMA plane loads: FP32 state with the residual-input modes (the skew modes' 7-field ring leaves no
  // shared memory for the staging buffers without losing resident blocks)
  constexpr bool tma_mode = sizeof(T) == 4 && (MODE & CRK_RIN) && !(MODE & CRK_SKEW);
  if constexpr (tma_mode) {
    const int buf = q.v[0] == static_cast<const T *>(c.qa[0]) ? 0 : q.v[0] == static_cast<const T *>(c.qb[0]) ? 1 : -1;
    if (buf >= 0 && c.tma_enabled && c.tma_ok[buf] && c.d_status) {
      const TmaPlanes &maps = c.tma[buf][TY == 16 ? 1 : 0];
      const int bx = (c.g.n0 + TX - 1) / TX, by = (c.g.n1 + TY - 1) / TY;
      const int resident = c.num_sms * resident_per_sm_tma<T, MODE, TY>();
      int nzc = (4 * resident + bx * by - 1) / (bx * by);
      nzc = max(1, min(nzc, (c.g.n2 + 7) / 8));
      const int zchunk = (c.g.n2 + nzc - 1) / nzc;
      nzc = (c.g.n2 + zchunk - 1) / zchunk;
      const T ddt = (T)(dt_new - dt_old);
      k_central_rk_tma<T, MODE, TY><<<dim3(bx, by, nzc), dim3(TX, TY), tma_smem_bytes<T, MODE, TY>(), s>>>(
          maps, c.g, qnew, qold, rin, rout, c.ph, dt_new, dt_old, ddt, zchunk, c.d_status);
      return;
    }
  }
  const int bx = (c.g.n0 + TX - 1) / TX, by = (c.g.n1 + TY - 1) / TY;
  // z-chunks: about four waves of resident blocks so the last wave's tail is short; at least 8
  // planes per chunk so the 4 halo planes of each chunk cost at most half a chunk's loads
  const int resident = c.num_sms * resident_per_sm<T, MODE, TY>();
  int nzc = (4 * resident + bx * by - 1) / (bx * by);
  nzc = max(1, min(nzc, (c.g.n2 + 7) / 8));
  const int zchunk = (c.g.n2 + nzc - 1) / nzc;
  nzc = (c.g.n2 + zchunk - 1) / zchunk;
  dim3 grid(bx, by, nzc), block(TX, TY);
  // (dt_new - dt_old) in the state precision, formed once here: the FP32 stage update adds it times R
  const T ddt = (T)(dt_new - dt_old);
  k_central_rk<T, MODE, TY><<<grid, block, ring_bytes<T, MODE, TY>(), s>>>(c.g, q, qnew, qold, rin, rout, c.ph, dt_new,
                                                                          dt_old, ddt, zchunk);
}

template <typename T, int MODE>
static void launch_ty(const Ctx &c, Fields5<const T> q, Fields5<T> qnew, Fields5<double> qold, Fields5<T> rin,
                      Fields5<T> rout, double dt_new, double dt_old, cudaStream_t s) {
  if (c.crk_ty == 16) launch_mode<T, MODE, 16>(c, q, qnew, qold, rin, rout, dt_new, dt_old, s);
  else launch_mode<T, MODE, 8>(c, q, qnew, qold, rin, rout, dt_new, dt_old, s);
}

template <typename T>
void launch_central_rk(const Ctx &c, Fields5<const T> q, Fields5<T> qnew, Fields5<double> qold, Fields5<T> rin,
                       Fields5<T> rout, double dt_new, double dt_old, int mode, cudaStream_t s, int64_t *launches) {
  ++*launches;
  switch (mode) {
#define OSB_CASE(M) \
  case M: launch_ty<T, M>(c, q, qnew, qold, rin, rout, dt_new, dt_old, s); break;
    OSB_CASE(CRK_SKEW | CRK_VISC | CRK_UPDATE)
    OSB_CASE(CRK_SKEW | CRK_VISC)
    OSB_CASE(CRK_SKEW | CRK_UPDATE)
    OSB_CASE(CRK_SKEW)
    OSB_CASE(CRK_VISC | CRK_RIN | CRK_UPDATE)
    OSB_CASE(CRK_VISC | CRK_RIN)
    OSB_CASE(CRK_RIN | CRK_UPDATE)
    OSB_CASE(CRK_RIN)
#undef OSB_CASE
    default:
      --*launches;
      break;
  }
}

template <typename T, int MODE> static void attr_tma() {
  cudaFuncSetAttribute(k_central_rk_tma<T, MODE, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tma_smem_bytes<T, MODE, 8>());
  cudaFuncSetAttribute(k_central_rk_tma<T, MODE, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tma_smem_bytes<T, MODE, 16>());
}

template <typename T, int MODE> static void attr_mode() {
  cudaFuncSetAttribute(k_central_rk<T, MODE, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)ring_bytes<T, MODE, 8>());
  cudaFuncSetAttribute(k_central_rk<T, MODE, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)ring_bytes<T, MODE, 16>());
}
template <typename T> static void attr_batch();
template <typename T> void setup_central() {
  attr_mode<T, CRK_SKEW | CRK_VISC | CRK_UPDATE>();
  attr_mode<T, CRK_SKEW | CRK_VISC>();
  attr_mode<T, CRK_SKEW | CRK_UPDATE>();
  attr_mode<T, CRK_SKEW>();
  attr_mode<T, CRK_VISC | CRK_RIN | CRK_UPDATE>();
  attr_mode<T, CRK_VISC | CRK_RIN>();
  attr_mode<T, CRK_RIN | CRK_UPDATE>();
  attr_mode<T, CRK_RIN>();
  attr_batch<T>();
  if constexpr (sizeof(T) == 4) {
    attr_tma<T, CRK_VISC | CRK_RIN | CRK_UPDATE>();
    attr_tma<T, CRK_VISC | CRK_RIN>();
    attr_tma<T, CRK_RIN | CRK_UPDATE>();
    attr_tma<T, CRK_RIN>();
  }
}
// Descriptor table of the batch being stepped, in this module's constant memory: the persistent
// kernels read an instance's grid, constants and pointers through the constant cache (uniform per
// block), so they cost no registers.  batch_table_upload_central copies a device-resident table here,
// stream-ordered (capturable); batches stepping at the same time must share one stream.
static __constant__ __align__(16) unsigned char c_batch_table[BATCH_TABLE_BYTES];

cudaError_t batch_table_upload_central(const void *src_dev, size_t bytes, cudaStream_t s) {
  if (bytes > BATCH_TABLE_BYTES) return cudaErrorInvalidValue;
  return cudaMemcpyToSymbolAsync(c_batch_table, src_dev, bytes, 0, cudaMemcpyDeviceToDevice, s);
}

// ---------------------------------------------------------------------------------------------
// batched ensemble: one persistent launch per kernel mode over the tiles of every instance that
// uses that mode (items {instance, bx, by, bz} taken from a tile queue)
// ---------------------------------------------------------------------------------------------
template <typename T, int MODE, int TY>
__global__ void __launch_bounds__(TX * TY, central_min_blocks<T, MODE, TY>())
    k_batch_central(const int4 *items, int nitems, int *counter, int parity, int stage) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int slot;
  for (;;) {
    const int it = next_item(counter, &slot);
    if (it >= nitems) return;
    const int4 w = items[it];
    const BatchInst<T> &d = reinterpret_cast<const BatchInst<T> *>(c_batch_table)[w.x];
    Fields5<const T> q;
    Fields5<T> qn, r;
    Fields5<double> qo;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      q.v[v] = d.q[parity][v];
      qn.v[v] = d.q[parity ^ 1][v];
      r.v[v] = d.res[v];
      qo.v[v] = d.qold[v];
    }
    central_tile<T, MODE, TY>(d.g, q, qn, qo, r, r, d.ph, d.dtn[stage], d.dto[stage], (T)d.ddt[stage], d.zchunk, w.y,
                              w.z, w.w, smem_raw);
  }
}

template <typename T, int MODE, int TY> static int occ_batch() {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_central<T, MODE, TY>, TX * TY,
                                                    ring_bytes<T, MODE, TY>()) != cudaSuccess || b < 1)
    b = 1;
  return b;
}

// mode: CRK_SKEW or CRK_RIN, with CRK_VISC as the plan says; CRK_UPDATE is implied
template <typename T> int batch_central_blocks_per_sm(int mode, int ty) {
  const int m = mode | CRK_UPDATE;
#define OSB_OCC(M) \
  if (m == (M)) return ty == 16 ? occ_batch<T, M, 16>() : occ_batch<T, M, 8>();
  OSB_OCC(CRK_SKEW | CRK_VISC | CRK_UPDATE)
  OSB_OCC(CRK_SKEW | CRK_UPDATE)
  OSB_OCC(CRK_RIN | CRK_VISC | CRK_UPDATE)
  OSB_OCC(CRK_RIN | CRK_UPDATE)
#undef OSB_OCC
  return 1;
}

template <typename T, int MODE>
static void batch_mode(const int4 *items, int nitems, int *counter, int parity, int stage, int ty,
                       int nblocks, cudaStream_t s) {
  if (ty == 16)
    k_batch_central<T, MODE, 16><<<nblocks, dim3(TX, 16), ring_bytes<T, MODE, 16>(), s>>>(items, nitems, counter,
                                                                                          parity, stage);
  else
    k_batch_central<T, MODE, 8><<<nblocks, dim3(TX, 8), ring_bytes<T, MODE, 8>(), s>>>(items, nitems, counter,
                                                                                        parity, stage);
}

template <typename T>
void launch_batch_central(const int4 *items, int nitems, int *counter, int parity, int stage, int mode, int ty,
                          int nblocks, cudaStream_t s) {
  switch (mode | CRK_UPDATE) {
    case CRK_SKEW | CRK_VISC | CRK_UPDATE:
      batch_mode<T, CRK_SKEW | CRK_VISC | CRK_UPDATE>(items, nitems, counter, parity, stage, ty, nblocks, s);
      break;
    case CRK_SKEW | CRK_UPDATE:
      batch_mode<T, CRK_SKEW | CRK_UPDATE>(items, nitems, counter, parity, stage, ty, nblocks, s);
      break;
    case CRK_RIN | CRK_VISC | CRK_UPDATE:
      batch_mode<T, CRK_RIN | CRK_VISC | CRK_UPDATE>(items, nitems, counter, parity, stage, ty, nblocks, s);
      break;
    case CRK_RIN | CRK_UPDATE:
      batch_mode<T, CRK_RIN | CRK_UPDATE>(items, nitems, counter, parity, stage, ty, nblocks, s);
      break;
    default:
      break;
  }
}

template <typename T, int MODE> static void attr_batch_mode() {
  cudaFuncSetAttribute(k_batch_central<T, MODE, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)ring_bytes<T, MODE, 8>());
  cudaFuncSetAttribute(k_batch_central<T, MODE, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)ring_bytes<T, MODE, 16>());
}
template <typename T> static void attr_batch() {
  attr_batch_mode<T, CRK_SKEW | CRK_VISC | CRK_UPDATE>();
  attr_batch_mode<T, CRK_SKEW | CRK_UPDATE>();
  attr_batch_mode<T, CRK_RIN | CRK_VISC | CRK_UPDATE>();
  attr_batch_mode<T, CRK_RIN | CRK_UPDATE>();
}

template void setup_central<float>();
template void setup_central<double>();
template int batch_central_blocks_per_sm<float>(int, int);
template int batch_central_blocks_per_sm<double>(int, int);
template void launch_batch_central<float>(const int4 *, int, int *, int, int, int, int, int, cudaStream_t);
template void launch_batch_central<double>(const int4 *, int, int *, int, int, int, int, int, cudaStream_t);

template void launch_central_rk<float>(const Ctx &, Fields5<const float>, Fields5<float>, Fields5<double>,
                                       Fields5<float>, Fields5<float>, double, double, int, cudaStream_t, int64_t *);
template void launch_central_rk<double>(const Ctx &, Fields5<const double>, Fields5<double>, Fields5<double>,
                                        Fields5<double>, Fields5<double>, double, double, int, cudaStream_t,
                                        int64_t *);

}  // namespace osb
