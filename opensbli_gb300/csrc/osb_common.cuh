// osb_common.cuh -- shared device-side types for the GB300 kernels.
//
// Every per-variable array uses one padded layout: x fastest, interior point (i,j,k) at
// off0 + i + j*sy + k*sz.  Halos: 4 in x (keeps interior rows 16-byte aligned for both element
// sizes), 3 in y and z (the WENO5/TENO5 stencil reaches 3 points; central 4th order reaches 2).
#pragma once
#include <cstdint>
#include <cuda.h>  // CUtensorMap (the type only; maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

namespace osb {

constexpr int HX = 4;
constexpr int HY = 3;
constexpr int HZ = 3;

struct Grid {
  int n0, n1, n2;
  int64_t sy, sz, off0, numel;
};

__host__ __device__ inline int64_t gidx(const Grid &g, int i, int j, int k) {
  return g.off0 + (int64_t)i + (int64_t)j * g.sy + (int64_t)k * g.sz;
}

template <typename T> struct Fields5 {
  T *v[5];
};

// Physical and numerical constants of a plan, passed by value to every kernel.
struct Phys {
  double gama, Minf, Re, Pr;
  double inv_delta[3];
  double weno_eps;
  // derived constants, filled on the host in both precisions so kernels do no FP64 set-up work:
  // gama-1, 1/(gama-1), gama*Minf^2, 1/Re, kT = 1/((gama-1) Minf^2 Pr Re)
  double gm1, igm1, gM2, invRe, kT;
  float f_gama, f_gm1, f_igm1, f_gM2, f_invRe, f_kT, f_eps, f_inv_delta[3];
  // FP32 remainders: gama-1 = f_gm1 + f_gm1_lo, 1/delta_d = f_inv_delta[d] + f_inv_delta_lo[d].  A
  // constant rounded to FP32 alone would scale every pressure or every flux difference by the same
  // factor (1/delta: up to 6e-8), a bias that grows linearly in time instead of averaging out.
  float f_gm1_lo, f_inv_delta_lo[3];
  // TENO cut-off C_T (weno_eps holds TENO's eps for TENO plans)
  double teno_ct;
  float f_teno_ct;
  // adaptive TENO on 3D blocks: C_T per point (state precision, padded layout); the interface
  // between cells c-1 and c takes the value at c-1.  Null for a fixed cut-off.
  const void *ctp;
  // blocks stretched in x1: the x1 flux difference of cell j is scaled by inv_delta1 D11(j), given
  // per j in FP64 and as an FP32 pair (in place of inv_delta[1]).  Null on Cartesian blocks.
  const double *ysc_d;
  const float2 *ysc_f;
};

// the FP64 or FP32 copy of a plan constant
template <typename T> __host__ __device__ __forceinline__ T pick(double d, float f);
template <> __host__ __device__ __forceinline__ double pick<double>(double d, float) { return d; }
template <> __host__ __device__ __forceinline__ float pick<float>(double, float f) { return f; }

template <typename T> __device__ __forceinline__ T sqrt_t(T x);
template <> __device__ __forceinline__ float sqrt_t<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double sqrt_t<double>(double x) { return sqrt(x); }

// tensor maps of the five conserved arrays of one state buffer (for one box shape)
struct TmaPlanes {
  CUtensorMap m[5];
};

// ---- TMA (cp.async.bulk.tensor) and mbarrier helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// make the initialised barriers visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 3D tiled bulk copy global -> shared of the box at (x, y, z) described by *map, completing on *bar
__device__ __forceinline__ void tma_load_3d(void *dst, const void *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// bring the line holding *p into L2 (a hint: no register is written, nothing waits for it)
__device__ __forceinline__ void prefetch_l2(const void *p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// 1/x: the fast hardware reciprocal in FP32 (2 ulp), the exact quotient in FP64
template <typename T> __device__ __forceinline__ T rcp_t(T x);
template <> __device__ __forceinline__ float rcp_t<float>(float x) { return __fdividef(1.0f, x); }
template <> __device__ __forceinline__ double rcp_t<double>(double x) { return 1.0 / x; }

// ---- FP32 primitives rounded once.  The FP32 state is exact input; what the mixed path must avoid is
// extra rounding noise in u, p and T, which the derivative stencils and flux differences amplify by
// 1/delta or 1/delta^2 (p = (g-1)(E - |m|^2/(2 rho)) also loses bits to cancellation).  Error-free
// transformations (the exact division residual from one FMA, Dekker/Knuth two-product and two-sum)
// carry the discarded parts: u_c comes out correctly rounded in almost every case, p within about one
// ulp of (g-1)_f32 (E - |m|^2/(2 rho)) evaluated exactly.  p_lo is the part of p below p_hi.
__device__ __forceinline__ void prims_f32(float rho, float m0, float m1, float m2, float E, float gm1, float gm1_lo,
                                          float &irho, float (&u)[3], float &p_hi, float &p_lo) {
  // __fmul_rn/__fadd_rn are never contracted into FMAs: the two-sum identities need the rounded
  // sums and products they are written with
  irho = 1.0f / rho;
  const float m[3] = {m0, m1, m2};
  float k_hi = 0.0f, k_lo = 0.0f;  // |m|^2 / rho as an unevaluated sum
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float q = __fmul_rn(m[c], irho);
    const float e = fmaf(-q, rho, m[c]);  // m - q rho, exact
    u[c] = fmaf(e, irho, q);
    // m (m / rho) = m q + m e / rho
    const float ph = __fmul_rn(m[c], q);
    const float pl = fmaf(m[c], q, -ph) + m[c] * (e * irho);
    const float s = __fadd_rn(k_hi, ph), bv = __fsub_rn(s, k_hi);
    k_lo += __fadd_rn(__fsub_rn(k_hi, __fsub_rn(s, bv)), __fsub_rn(ph, bv)) + pl;
    k_hi = s;
  }
  const float h = -0.5f * k_hi;  // exact
  const float d = __fadd_rn(E, h), bv = __fsub_rn(d, E);
  const float d_lo = __fadd_rn(__fsub_rn(E, __fsub_rn(d, bv)), __fsub_rn(h, bv)) - 0.5f * k_lo;
  const float ph = __fmul_rn(gm1, d);
  const float pl = fmaf(gm1, d, -ph) + fmaf(gm1, d_lo, gm1_lo * d);
  p_hi = __fadd_rn(ph, pl);  // renormalise
  p_lo = __fsub_rn(pl, __fsub_rn(p_hi, ph));
}

// c (p_hi + p_lo) / rho rounded once (T = gama Minf^2 p / rho)
__device__ __forceinline__ float scaled_ratio_f32(float c, float p_hi, float p_lo, float rho, float irho) {
  const float n_hi = __fmul_rn(c, p_hi);
  const float n_lo = fmaf(c, p_hi, -n_hi) + c * p_lo;
  const float q = __fmul_rn(n_hi, irho);
  const float e = fmaf(-q, rho, n_hi) + n_lo;
  return fmaf(e, irho, q);
}

// x * (hi + lo) for a constant carried as an FP32 pair; FP64 ignores lo
__device__ __forceinline__ float mul_hl(float x, float hi, float lo) { return fmaf(x, hi, x * lo); }
__device__ __forceinline__ double mul_hl(double x, double hi, double) { return x * hi; }

template <typename T> __device__ __forceinline__ T abs_t(T x) { return x < T(0) ? -x : x; }
template <typename T> __device__ __forceinline__ T max_t(T a, T b) { return a > b ? a : b; }

// Tile queue of the persistent batched kernels: one thread of the block takes the next item index
// from a global counter (atomicAdd, never waits); all threads then read it.
__device__ __forceinline__ int next_item(int *counter, int *slot) {
  __syncthreads();  // every thread is done with the previous item index
  if (threadIdx.x == 0 && threadIdx.y == 0) *slot = atomicAdd(counter, 1);
  __syncthreads();
  return *slot;
}

// bytes of the constant-memory descriptor table of a batch (BatchInst entries)
constexpr size_t BATCH_TABLE_BYTES = 56 * 1024;

// One instance of a batched ensemble: its grid, constants, ping-pong state buffers, residual and
// FP64 RK register (all padded, as for a single plan), time step and scheme.
template <typename T> struct BatchInst {
  Grid g;
  Phys ph;
  T *q[2][5];
  T *res[5];
  double *qold[5];
  double dt;
  double dtn[3], dto[3];  // dt * rknew[s], dt * rkold[s] of the three stages
  float ddt[3];           // dt * (rknew[s] - rkold[s]), the FP32 stage increment factor
  int conv;    // OSB_CONV_CENTRAL_SKEW or OSB_CONV_WENO5JS
  int visc;    // 1: constant-viscosity viscous terms
  int zchunk;  // z-planes per central-kernel tile
  int pad;
};

}  // namespace osb
