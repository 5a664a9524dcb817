// osb_weno.cu -- characteristic WENO5-JS flux kernels, one per direction, and their launch
// variants.
//
// The per-interface arithmetic (Roe average, LLF splitting, WENO5-JS, back-projection) lives in
// osb_weno.cuh; this file restates how the generated code applies it along each direction and
// forms the "LLFWeno Residual" (shock_capturing.py:21-34, opensblifunctions.py:575-593),
// R -= (flux_{i+1/2} - flux_{i-1/2}) / delta_d, fused so that interface fluxes never reach HBM.
//
// Two kernel shapes:
//  * tiled (all directions): a block covers TA lines along d and TI consecutive interfaces per
//    line, giving the flux difference of TI-1 cells.  The conserved and primitive values of the
//    TI+5 points of every line are staged in shared memory with loads coalesced along x; each
//    thread owns IPT consecutive interfaces of one line and slides a six-point register window
//    along it, so a point's values are read from shared memory once per thread.  Interface
//    fluxes go back through shared memory for the difference.
//  * line-marching (y and z): a thread owns one (x, transverse) line segment of L cells and walks
//    along it; the warp's 32 lanes are 32 consecutive x points, so every global load is one
//    coalesced 128-byte (FP32) row.  The next point's conserved vector and the residual of the
//    cell being finished are loaded one interface ahead, the previous interface flux stays in
//    registers, and no shared memory or barrier is used.  Each segment re-reads the 5 points of
//    its stencil halo and recomputes one interface flux.
//  * line-marching (x): a warp owns 32 y-lines and walks along x; conserved vectors and residuals
//    pass through a per-warp shared-memory transpose so global accesses stay row-contiguous.
// Which shape runs, and the segment length, is chosen per direction by osb_autotune.
#include "osb_common.cuh"
#include "osb_internal.h"
#include "osb_weno.cuh"

namespace osb {

namespace {
enum { W_RHO = 0, W_RU0, W_RU1, W_RU2, W_E, W_P, W_A, W_UD, W_UDLO, W_PLO };
// staged fields per point: FP32 also keeps u_D's and p's remainders for the double-float point flux
template <typename T> __host__ __device__ constexpr int wnf() { return sizeof(T) == 4 ? 10 : 8; }

// Tiles: 32 lines x 32 interfaces, four consecutive interfaces per thread, in every direction.
// For x the shared arrays are [field][line][position] (lines are y rows of the block), otherwise
// [field][position][line] (lines are the 32 consecutive x points).
template <int DIR> struct WTile {
  static constexpr int TI = 32, TA = 32, IPT = 4;
  static constexpr int FS = DIR == 0 ? TI + 1 : TA;  // row pitch of the flux array (x: padded)
};

// 1/delta of the x1 flux difference at row j of a block stretched in x1 (inv_delta1 D11(j)) as the
// pair the flux difference is multiplied by
__device__ __forceinline__ void ysc_pair(const Phys &ph, int j, float &hi, float &lo) {
  const float2 p = ph.ysc_f[j];
  hi = p.x;
  lo = p.y;
}
__device__ __forceinline__ void ysc_pair(const Phys &ph, int j, double &hi, double &lo) {
  hi = ph.ysc_d[j];
  lo = 0.0;
}

template <typename T, int D, typename Pt>
__device__ __forceinline__ void load_point(const Pt &P, int t, WPt<T> &w, PtFlux &pf) {
  w.Q[0] = P(W_RHO, t);
  w.Q[1] = P(W_RU0, t);
  w.Q[2] = P(W_RU1, t);
  w.Q[3] = P(W_RU2, t);
  w.Q[4] = P(W_E, t);
  w.ud = P(W_UD, t);
  w.p = P(W_P, t);
  w.a = P(W_A, t);
  if constexpr (sizeof(T) == 4) point_flux_ff<D>(w.Q, w.ud, P(W_UDLO, t), w.p, P(W_PLO, t), pf);
}
}  // namespace

template <typename T, int DIR, bool ACCUM, int SCH>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1) k_weno(Grid g, Fields5<const T> q, Fields5<T> res, Phys ph) {
  using Tl = WTile<DIR>;
  constexpr int TI = Tl::TI, TA = Tl::TA, NPT = TI + 5, FS = Tl::FS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NF = wnf<T>();
  T *sf = reinterpret_cast<T *>(smem_raw);   // [NF][TA][NPT] (DIR==0) or [NF][NPT][TA]
  T *sflux = sf + NF * NPT * TA;             // [5][TA][FS] (DIR==0) or [5][TI][TA]
  T *sdf = sflux + 5 * (DIR == 0 ? TA * FS : TI * TA);  // FP32: F(left point) - F(point before), same layout
  const int tid = threadIdx.x;
  const int n[3] = {g.n0, g.n1, g.n2};
  const T gm1 = pick<T>(ph.gm1, ph.f_gm1), gama = pick<T>(ph.gama, ph.f_gama);
  const T igm1 = pick<T>(ph.igm1, ph.f_igm1), eps = pick<T>(ph.weno_eps, ph.f_eps);
  const T ct = pick<T>(ph.teno_ct, ph.f_teno_ct);
  const T gm1_lo = pick<T>(0.0, ph.f_gm1_lo);

  // tile origin: first cell whose flux difference this block writes (d0), across-line origin
  int d0, a0, o1, o2;
  if (DIR == 0) { d0 = blockIdx.x * (TI - 1); a0 = blockIdx.y * TA; o2 = blockIdx.z; o1 = 0; }
  else if (DIR == 1) { a0 = blockIdx.x * TA; d0 = blockIdx.y * (TI - 1); o2 = blockIdx.z; o1 = 0; }
  else { a0 = blockIdx.x * TA; o1 = blockIdx.y; d0 = blockIdx.z * (TI - 1); o2 = 0; }

  auto sidx = [&](int f, int pos, int a) -> int {
    return DIR == 0 ? (f * TA + a) * NPT + pos : (f * NPT + pos) * TA + a;
  };
  auto fidx = [&](int v, int m, int a) -> int { return DIR == 0 ? (v * TA + a) * FS + m : (v * TI + m) * TA + a; };
  auto coords = [&](int pos, int a, int &i, int &j, int &k) {
    const int c = d0 - 3 + pos;
    if (DIR == 0) { i = c; j = a0 + a; k = o2; }
    else if (DIR == 1) { i = a0 + a; j = c; k = o2; }
    else { i = a0 + a; j = o1; k = c; }
  };
  const int nd = n[DIR];
  const int na = DIR == 0 ? n[1] : n[0];

  // ---- stage the tile's points: all loads of a thread are issued before any of them is used
  constexpr int NLD = (NPT * TA + 255) / 256;
  {
    T r[NLD][5];
    bool ok[NLD];
#pragma unroll
    for (int l = 0; l < NLD; ++l) {
      const int t = tid + 256 * l;
      int pos, a;
      if (DIR == 0) { a = t / NPT; pos = t % NPT; }
      else { pos = t / TA; a = t % TA; }
      ok[l] = t < NPT * TA && d0 - 3 + pos <= nd + 2 && a0 + a < na;
      if (ok[l]) {
        int i, j, k;
        coords(pos, a, i, j, k);
        const int64_t m = gidx(g, i, j, k);
#pragma unroll
        for (int v = 0; v < 5; ++v) r[l][v] = __ldg(q.v[v] + m);
      }
    }
#pragma unroll
    for (int l = 0; l < NLD; ++l) {
      if (!ok[l]) continue;
      const int t = tid + 256 * l;
      int pos, a;
      if (DIR == 0) { a = t / NPT; pos = t % NPT; }
      else { pos = t / TA; a = t % TA; }
      WPt<T> w;
      float lo2[2];
      point_prims<T, DIR>(r[l], gm1, gm1_lo, gama, w, nullptr, lo2);
      if constexpr (sizeof(T) == 4) {
        sf[sidx(W_UDLO, pos, a)] = lo2[0];
        sf[sidx(W_PLO, pos, a)] = lo2[1];
      }
      sf[sidx(W_RHO, pos, a)] = w.Q[0];
      sf[sidx(W_RU0, pos, a)] = w.Q[1];
      sf[sidx(W_RU1, pos, a)] = w.Q[2];
      sf[sidx(W_RU2, pos, a)] = w.Q[3];
      sf[sidx(W_E, pos, a)] = w.Q[4];
      sf[sidx(W_P, pos, a)] = w.p;
      sf[sidx(W_A, pos, a)] = w.a;
      sf[sidx(W_UD, pos, a)] = w.ud;
    }
  }
  __syncthreads();

  // ---- interface fluxes: interface m of a line sits between cells d0-1+m and d0+m and uses the
  //      points at positions m..m+5; each thread slides a window over IPT interfaces
  {
    const int a = tid % TA, m0 = (tid / TA) * Tl::IPT;
    auto P = [&](int f, int t) -> T { return sf[sidx(f, m0 + t, a)]; };
    if (a0 + a < na && d0 - 1 + m0 <= nd - 1) {
      WPt<T> W[6];
      PtFlux fl_last, fl_new;
#pragma unroll
      for (int t = 0; t < 5; ++t) {
        load_point<T, DIR>(P, t, W[t], fl_new);
        if (t > 0) link_flux(W[t - 1], fl_last, fl_new);
        fl_last = fl_new;
      }
#pragma unroll 1
      for (int w = 0; w < Tl::IPT; ++w) {
        if (d0 - 1 + m0 + w <= nd - 1) {
          load_point<T, DIR>(P, w + 5, W[5], fl_new);
          link_flux(W[4], fl_last, fl_new);
          fl_last = fl_new;
          T fl[5];
          T cti = ct;
          if constexpr (SCH == SCH_TENO || SCH == SCH_TENO6) {
            if (ph.ctp) {  // cut-off at the interface's left point, cell d0-1+m0+w
              int i, j, k;
              coords(m0 + w + 2, a, i, j, k);
              cti = static_cast<const T *>(ph.ctp)[gidx(g, i, j, k)];
            }
          }
          interface_flux<T, DIR, SCH>(W, gm1, igm1, eps, cti, fl);
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            sflux[fidx(v, m0 + w, a)] = fl[v];
            if constexpr (sizeof(T) == 4 && SCH != SCH_FILTER) sdf[fidx(v, m0 + w, a)] = W[1].dF[v];
          }
        }
#pragma unroll
        for (int t = 0; t < 5; ++t) W[t] = W[t + 1];
      }
    }
  }
  __syncthreads();

  // ---- flux difference for cells d0 .. d0+TI-2 (residual loads issued before the stores)
  const T idd = pick<T>(ph.inv_delta[DIR], ph.f_inv_delta[DIR]);
  const T idd_lo = pick<T>(0.0, ph.f_inv_delta_lo[DIR]);
  constexpr int NST = ((TI - 1) * TA + 255) / 256;
  T rv[NST][5];
  int64_t gi[NST];
#pragma unroll
  for (int l = 0; l < NST; ++l) {
    const int t = tid + 256 * l;
    int m, a;
    if (DIR == 0) { a = t / (TI - 1); m = t % (TI - 1); }
    else { m = t / TA; a = t % TA; }
    gi[l] = -1;
    if (t < (TI - 1) * TA && d0 + m < nd && a0 + a < na) {
      int i, j, k;
      coords(m + 3, a, i, j, k);
      gi[l] = gidx(g, i, j, k);
      if (ACCUM) {
#pragma unroll
        for (int v = 0; v < 5; ++v) rv[l][v] = res.v[v][gi[l]];
      }
    }
  }
#pragma unroll
  for (int l = 0; l < NST; ++l) {
    if (gi[l] < 0) continue;
    const int t = tid + 256 * l;
    int m, a;
    if (DIR == 0) { a = t / (TI - 1); m = t % (TI - 1); }
    else { m = t / TA; a = t % TA; }
    T sh = idd, sl = idd_lo;
    if (DIR == 1 && ph.ysc_d) ysc_pair(ph, d0 + m, sh, sl);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      T diff = sflux[fidx(v, m + 1, a)] - sflux[fidx(v, m, a)];
      if constexpr (sizeof(T) == 4 && SCH != SCH_FILTER)
        diff = sdf[fidx(v, m + 1, a)] + diff;  // (F_i - F_{i-1}) + (G_i - G_{i-1})
      const T d = -mul_hl(diff, sh, sl);
      res.v[v][gi[l]] = ACCUM ? rv[l][v] + d : d;
    }
  }
}

// Line-marching flux kernel for DIR 1 (y) and 2 (z); block = 32 x-lanes by BY transverse lines,
// blockIdx.z = segment of L cells along DIR.
template <typename T, int DIR, bool ACCUM, int BY, int SCH>
__device__ __forceinline__ void weno_march_tile(const Grid &g, Fields5<const T> q, Fields5<T> res, const Phys &ph,
                                                int L, int bx, int by, int bz) {
  static_assert(DIR == 1 || DIR == 2, "marching runs along y or z");
  const int i = bx * 32 + threadIdx.x;
  const int o = by * BY + threadIdx.y;  // k for DIR 1, j for DIR 2
  const int nd = DIR == 1 ? g.n1 : g.n2, no = DIR == 1 ? g.n2 : g.n1;
  if (i >= g.n0 || o >= no) return;
  const int c0 = bz * L;
  const int c1 = min(c0 + L, nd);  // this thread finishes cells c0 .. c1-1
  const int64_t sd = DIR == 1 ? g.sy : g.sz;
  const int64_t mline = DIR == 1 ? gidx(g, i, 0, o) : gidx(g, i, o, 0);  // cell 0 of the line
  const T gm1 = pick<T>(ph.gm1, ph.f_gm1), gama = pick<T>(ph.gama, ph.f_gama);
  const T igm1 = pick<T>(ph.igm1, ph.f_igm1), eps = pick<T>(ph.weno_eps, ph.f_eps);
  const T ct = pick<T>(ph.teno_ct, ph.f_teno_ct);
  const T idd = pick<T>(ph.inv_delta[DIR], ph.f_inv_delta[DIR]);
  const T idd_lo = pick<T>(0.0, ph.f_inv_delta_lo[DIR]), gm1_lo = pick<T>(0.0, ph.f_gm1_lo);

  // points c0-3 .. c0+1 fill the window; point c0+2 is the first one streamed in
  WPt<T> W[6];
  PtFlux fl_last, fl_new;  // FP32: double-float fluxes of the newest window point and of the one added now
  PtFlux *const pfl = sizeof(T) == 4 ? &fl_new : nullptr;
  {
    T r[5][5];
#pragma unroll
    for (int t = 0; t < 5; ++t)
#pragma unroll
      for (int v = 0; v < 5; ++v) r[t][v] = __ldg(q.v[v] + mline + (int64_t)(c0 - 3 + t) * sd);
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      point_prims<T, DIR>(r[t], gm1, gm1_lo, gama, W[t], pfl);
      if (t > 0) link_flux(W[t - 1], fl_last, fl_new);
      fl_last = fl_new;
    }
  }
  T nq[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) nq[v] = __ldg(q.v[v] + mline + (int64_t)(c0 + 2) * sd);
  T Fp[5];
  // interface c lies between cells c-1 and c and uses points c-3 .. c+2
#pragma unroll 1
  for (int c = c0; c <= c1; ++c) {
    point_prims<T, DIR>(nq, gm1, gm1_lo, gama, W[5], pfl);
    link_flux(W[4], fl_last, fl_new);
    fl_last = fl_new;
    if (c < c1) {  // point c+3 <= nd+2 lies inside the halo
#pragma unroll
      for (int v = 0; v < 5; ++v) nq[v] = __ldg(q.v[v] + mline + (int64_t)(c + 3) * sd);
    }
    const int64_t mc = mline + (int64_t)(c - 1) * sd;  // cell finished by this interface
    T rv[5];
    if (ACCUM && c > c0) {
#pragma unroll
      for (int v = 0; v < 5; ++v) rv[v] = res.v[v][mc];
    }
    T F[5];
    T cti = ct;
    if constexpr (SCH == SCH_TENO || SCH == SCH_TENO6)
      if (ph.ctp) cti = static_cast<const T *>(ph.ctp)[mline + (int64_t)(c - 1) * sd];
    interface_flux<T, DIR, SCH>(W, gm1, igm1, eps, cti, F);
    if (c > c0) {
      T sh = idd, sl = idd_lo;
      if (DIR == 1 && ph.ysc_d) ysc_pair(ph, c - 1, sh, sl);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const T d = -mul_hl(flux_difference<SCH>(W, v, F[v], Fp[v]), sh, sl);
        res.v[v][mc] = ACCUM ? rv[v] + d : d;
      }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) Fp[v] = F[v];
#pragma unroll
    for (int t = 0; t < 5; ++t) W[t] = W[t + 1];
  }
}

// FP32: 384 threads per SM (168 registers with 4 lines per block): the two-lane side arithmetic
// keeps both sides live at once and spilled at 128 registers; measured 4 % faster per step at 256^3
// than the scalar sides at 512 threads.
template <typename T, int DIR, bool ACCUM, int BY, int SCH>
__global__ void __launch_bounds__(32 * BY, (sizeof(T) == 4 ? 384 : 256) / (32 * BY))
    k_weno_march(Grid g, Fields5<const T> q, Fields5<T> res, Phys ph, int L) {
  weno_march_tile<T, DIR, ACCUM, BY, SCH>(g, q, res, ph, L, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Line-marching flux kernel for x.  A warp owns 32 consecutive y-lines of one z-plane and walks a
// segment of L cells along x; lane l computes line j0+l.  The conserved vectors arrive in chunks of
// XC points of all 32 lines, loaded with the lanes spread along x (each row's XC values are
// contiguous) and transposed through a per-warp shared-memory tile; the next chunk's loads are in
// flight while the current one is consumed.  Residuals are staged the same way and written back in
// row pieces aligned with the 32-byte sectors of the padded layout (interior x = 0 sits 4 elements
// into a row).  Only __syncwarp orders the per-warp tiles; the x sweep writes R (no accumulation).
template <typename T> struct MX {
  static constexpr int XC = 4;            // points per load chunk
  static constexpr int RG = 8;            // cells per residual group
  static constexpr int QP = XC + 1;       // row pitch of the staged conserved tile
  static constexpr int RP = RG + 1;       // row pitch of the staged residual tile
  static constexpr int WARP_ELEMS = 5 * 32 * QP + 5 * 32 * RP;
};

template <typename T, int BY, int SCH>
__device__ __forceinline__ void weno_march_x_tile(const Grid &g, Fields5<const T> q, Fields5<T> res, const Phys &ph,
                                                  int L, int bx, int by, int bz, unsigned char *smem_raw) {
  using M = MX<T>;
  constexpr int XC = M::XC, RG = M::RG, QP = M::QP, RP = M::RP;
  constexpr int RPI = 32 / XC;  // rows covered by one load instruction
  const int lane = threadIdx.x, w = threadIdx.y;
  T *qs = reinterpret_cast<T *>(smem_raw) + (size_t)w * M::WARP_ELEMS;  // [5][32][QP]
  T *rs = qs + 5 * 32 * QP;                                              // [5][32][RP]
  const int j0 = by * 32, k = bz * BY + w;
  if (k >= g.n2) return;  // uniform per warp
  const int n0 = g.n0, n1 = g.n1;
  const int c0 = bx * L, c1 = min(c0 + L, n0);  // cells c0 .. c1-1
  const int pfirst = c0 - 3, plast = c1 + 2;            // points of the segment's stencils
  const T gm1 = pick<T>(ph.gm1, ph.f_gm1), gama = pick<T>(ph.gama, ph.f_gama);
  const T igm1 = pick<T>(ph.igm1, ph.f_igm1), eps = pick<T>(ph.weno_eps, ph.f_eps);
  const T ct = pick<T>(ph.teno_ct, ph.f_teno_ct);
  const T idd = pick<T>(ph.inv_delta[0], ph.f_inv_delta[0]);
  const T idd_lo = pick<T>(0.0, ph.f_inv_delta_lo[0]), gm1_lo = pick<T>(0.0, ph.f_gm1_lo);
  const int lrow = lane / XC, lcol = lane % XC;  // loader position inside a chunk
  const bool row_ok = j0 + lane < n1;

  T buf[5][XC];  // this lane's share of a chunk: XC rows (lrow + RPI*it), one point each
  auto load_chunk = [&](int xs) {
#pragma unroll
    for (int it = 0; it < XC; ++it) {
      const int row = lrow + RPI * it, x = xs + lcol;
      if (j0 + row < n1 && x <= n0 + 3) {
        const int64_t m = gidx(g, x, j0 + row, k);
#pragma unroll
        for (int v = 0; v < 5; ++v) buf[v][it] = __ldg(q.v[v] + m);
      }
    }
  };
  auto stage_chunk = [&]() {
#pragma unroll
    for (int it = 0; it < XC; ++it) {
      const int row = lrow + RPI * it;
#pragma unroll
      for (int v = 0; v < 5; ++v) qs[(v * 32 + row) * QP + lcol] = buf[v][it];
    }
  };
  // residual groups: cells [gs, gs+RG) with gs = 8m - 4, i.e. whole 32-byte sectors of a row
  auto flush = [&](int gs, int lo, int hi) {
    __syncwarp();
    constexpr int RR = 32 / RG;  // rows per store instruction
#pragma unroll
    for (int it = 0; it < RG; ++it) {
      const int row = lane / RG + RR * it, col = lane % RG, x = gs + col;
      if (j0 + row < n1 && x >= lo && x <= hi) {
        const int64_t m = gidx(g, x, j0 + row, k);
#pragma unroll
        for (int v = 0; v < 5; ++v) res.v[v][m] = rs[(v * 32 + row) * RP + col];
      }
    }
    __syncwarp();
  };

  WPt<T> W[6];
  T Fp[5];
  PtFlux fl_last, fl_new;  // FP32: double-float fluxes of the previous and the new window point
  PtFlux *const pfl = sizeof(T) == 4 ? &fl_new : nullptr;
  int xc = ((pfirst + 4) / XC) * XC - 4;  // chunk containing pfirst (pfirst + 4 >= 1)
  load_chunk(xc);
#pragma unroll 1
  for (; xc <= plast; xc += XC) {
    __syncwarp();
    stage_chunk();
    __syncwarp();
    if (xc + XC <= plast) load_chunk(xc + XC);
    const int pa = max(xc, pfirst), pb = min(xc + XC - 1, plast);
#pragma unroll 1
    for (int p = pa; p <= pb; ++p) {
#pragma unroll
      for (int t = 0; t < 5; ++t) W[t] = W[t + 1];
      T r[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) r[v] = qs[(v * 32 + lane) * QP + (p - xc)];
      point_prims<T, 0>(r, gm1, gm1_lo, gama, W[5], pfl);
      if (p > pfirst) link_flux(W[4], fl_last, fl_new);
      fl_last = fl_new;
      if (p >= c0 + 2) {  // window holds points c-3 .. c+2 of interface c = p - 2
        const int c = p - 2;
        T F[5] = {T(0), T(0), T(0), T(0), T(0)};  // rows past n1: defined, never stored
        if (row_ok) {
          T cti = ct;
          if constexpr (SCH == SCH_TENO || SCH == SCH_TENO6)
            if (ph.ctp) cti = static_cast<const T *>(ph.ctp)[gidx(g, c - 1, j0 + lane, k)];
          interface_flux<T, 0, SCH>(W, gm1, igm1, eps, cti, F);
        }
        if (c > c0) {
          const int cc = c - 1;  // cell finished by this interface
          const int gs = ((cc + 4) / RG) * RG - 4, col = cc - gs;
#pragma unroll
          for (int v = 0; v < 5; ++v)
            rs[(v * 32 + lane) * RP + col] = -mul_hl(flux_difference<SCH>(W, v, F[v], Fp[v]), idd, idd_lo);
          if (col == RG - 1 || cc == c1 - 1) flush(gs, c0, c1 - 1);
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) Fp[v] = F[v];
      }
    }
  }
}

// FP32: 384 resident threads per SM, so the difference-form flux fits in registers without spills
template <typename T, int BY, int SCH>
__global__ void __launch_bounds__(32 * BY, (sizeof(T) == 4 ? 384 : 256) / (32 * BY))
    k_weno_march_x(Grid g, Fields5<const T> q, Fields5<T> res, Phys ph, int L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  weno_march_x_tile<T, BY, SCH>(g, q, res, ph, L, blockIdx.x, blockIdx.y, blockIdx.z, smem_raw);
}

template <typename T, int DIR> constexpr size_t tile_smem() {
  using Tl = WTile<DIR>;
  // staged points, interface fluxes (FP32: their deviations G and the point-flux differences)
  return sizeof(T) * ((size_t)wnf<T>() * (Tl::TI + 5) * Tl::TA +
                      (sizeof(T) == 4 ? 2 : 1) * 5 * (DIR == 0 ? Tl::TA * Tl::FS : Tl::TI * Tl::TA));
}

template <typename T, int DIR, bool ACCUM, int SCH>
static void launch_tile(const Ctx &c, Fields5<const T> q, Fields5<T> r, cudaStream_t s) {
  using Tl = WTile<DIR>;
  const int n[3] = {c.g.n0, c.g.n1, c.g.n2};
  const int nt = (n[DIR] + Tl::TI - 2) / (Tl::TI - 1);
  dim3 grid;
  if (DIR == 0) grid = dim3(nt, (n[1] + Tl::TA - 1) / Tl::TA, n[2]);
  else if (DIR == 1) grid = dim3((n[0] + Tl::TA - 1) / Tl::TA, nt, n[2]);
  else grid = dim3((n[0] + Tl::TA - 1) / Tl::TA, n[1], nt);
  k_weno<T, DIR, ACCUM, SCH><<<grid, 256, tile_smem<T, DIR>(), s>>>(c.g, q, r, c.ph);
}

template <typename T, int DIR, bool ACCUM, int BY, int SCH>
static void launch_march(const Ctx &c, Fields5<const T> q, Fields5<T> r, int L, cudaStream_t s) {
  const int nd = DIR == 1 ? c.g.n1 : c.g.n2, no = DIR == 1 ? c.g.n2 : c.g.n1;
  dim3 grid((c.g.n0 + 31) / 32, (no + BY - 1) / BY, (nd + L - 1) / L);
  k_weno_march<T, DIR, ACCUM, BY, SCH><<<grid, dim3(32, BY), 0, s>>>(c.g, q, r, c.ph, L);
}

template <typename T, int BY> constexpr size_t march_x_smem() { return sizeof(T) * (size_t)BY * MX<T>::WARP_ELEMS; }

template <typename T, int BY, int SCH>
static void launch_march_x(const Ctx &c, Fields5<const T> q, Fields5<T> r, int L, cudaStream_t s) {
  dim3 grid((c.g.n0 + L - 1) / L, (c.g.n1 + 31) / 32, (c.g.n2 + BY - 1) / BY);
  k_weno_march_x<T, BY, SCH><<<grid, dim3(32, BY), march_x_smem<T, BY>(), s>>>(c.g, q, r, c.ph, L);
}

template <typename T, int DIR, bool ACCUM, int SCH>
static void launch_shape(const Ctx &c, Fields5<const T> q, Fields5<T> r, WenoCfg w, cudaStream_t s) {
  if constexpr (DIR == 0) {
    static_assert(!ACCUM, "the x sweep writes the residual");
    if (w.kind == WENO_TILE) launch_tile<T, DIR, ACCUM, SCH>(c, q, r, s);
    else if (w.kind == WENO_MARCH4) launch_march_x<T, 4, SCH>(c, q, r, w.seg, s);
    else launch_march_x<T, 8, SCH>(c, q, r, w.seg, s);
  } else {
    if (w.kind == WENO_TILE) launch_tile<T, DIR, ACCUM, SCH>(c, q, r, s);
    else if (w.kind == WENO_MARCH4) launch_march<T, DIR, ACCUM, 4, SCH>(c, q, r, w.seg, s);
    else launch_march<T, DIR, ACCUM, 8, SCH>(c, q, r, w.seg, s);
  }
}

template <typename T, int DIR, bool ACCUM>
static void launch_variant(const Ctx &c, Fields5<const T> q, Fields5<T> r, WenoCfg w, cudaStream_t s) {
  if (c.plan.conv == OSB_CONV_WENO5Z) launch_shape<T, DIR, ACCUM, SCH_Z>(c, q, r, w, s);
  else if (c.plan.conv == OSB_CONV_TENO5) launch_shape<T, DIR, ACCUM, SCH_TENO>(c, q, r, w, s);
  else if (c.plan.conv == OSB_CONV_TENO6) launch_shape<T, DIR, ACCUM, SCH_TENO6>(c, q, r, w, s);
  else launch_shape<T, DIR, ACCUM, SCH_JS>(c, q, r, w, s);
}

template <typename T>
void launch_weno_dir(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, cudaStream_t s, int64_t *launches) {
  launch_weno_cfg<T>(c, q, r, dir, c.wcfg[dir], s);
  ++*launches;
}

template <typename T>
void launch_weno_cfg(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, WenoCfg w, cudaStream_t s) {
  if (dir == 0) launch_variant<T, 0, false>(c, q, r, w, s);
  else if (dir == 1) launch_variant<T, 1, true>(c, q, r, w, s);
  else launch_variant<T, 2, true>(c, q, r, w, s);
}

// Descriptor table of the batch being stepped, in this module's constant memory: the persistent
// kernels read an instance's grid, constants and pointers through the constant cache (uniform per
// block), so they cost no registers.  batch_table_upload_weno copies a device-resident table here,
// stream-ordered (capturable); batches stepping at the same time must share one stream.
static __constant__ __align__(16) unsigned char c_batch_table[BATCH_TABLE_BYTES];

cudaError_t batch_table_upload_weno(const void *src_dev, size_t bytes, cudaStream_t s) {
  if (bytes > BATCH_TABLE_BYTES) return cudaErrorInvalidValue;
  return cudaMemcpyToSymbolAsync(c_batch_table, src_dev, bytes, 0, cudaMemcpyDeviceToDevice, s);
}

// ---------------------------------------------------------------------------------------------
// batched ensemble: persistent launches over the line-marching tiles of every WENO instance
// (items {instance, bx, by, bz} from a tile queue; segment length common to the batch)
// ---------------------------------------------------------------------------------------------
// The tile loop and the descriptor reads add live values to the line-marching bodies: these
// kernels allow 3/4 of the single-plan kernels' resident threads (more registers, no spills).
template <typename T, int BY>
__global__ void __launch_bounds__(32 * BY, (sizeof(T) == 4 ? 384 : 192) / (32 * BY))
    k_batch_weno_x(const int4 *items, int nitems, int *counter, int parity, int L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int slot;
  for (;;) {
    const int it = next_item(counter, &slot);
    if (it >= nitems) return;
    const int4 w = items[it];
    const BatchInst<T> &d = reinterpret_cast<const BatchInst<T> *>(c_batch_table)[w.x];
    Fields5<const T> q;
    Fields5<T> r;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      q.v[v] = d.q[parity][v];
      r.v[v] = d.res[v];
    }
    weno_march_x_tile<T, BY, SCH_JS>(d.g, q, r, d.ph, L, w.y, w.z, w.w, smem_raw);
  }
}

template <typename T, int DIR, int BY>
__global__ void __launch_bounds__(32 * BY, (sizeof(T) == 4 ? 384 : 192) / (32 * BY))
    k_batch_weno_yz(const int4 *items, int nitems, int *counter, int parity, int L) {
  __shared__ int slot;
  for (;;) {
    const int it = next_item(counter, &slot);
    if (it >= nitems) return;
    const int4 w = items[it];
    const BatchInst<T> &d = reinterpret_cast<const BatchInst<T> *>(c_batch_table)[w.x];
    Fields5<const T> q;
    Fields5<T> r;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      q.v[v] = d.q[parity][v];
      r.v[v] = d.res[v];
    }
    weno_march_tile<T, DIR, true, BY, SCH_JS>(d.g, q, r, d.ph, L, w.y, w.z, w.w);
  }
}

template <typename T> int batch_weno_blocks_per_sm(int dir, int kind) {
  int b = 0;
  cudaError_t e;
  if (dir == 0)
    e = kind == WENO_MARCH8
            ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_weno_x<T, 8>, 256, march_x_smem<T, 8>())
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_weno_x<T, 4>, 128, march_x_smem<T, 4>());
  else if (dir == 1)
    e = kind == WENO_MARCH8 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_weno_yz<T, 1, 8>, 256, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_weno_yz<T, 1, 4>, 128, 0);
  else
    e = kind == WENO_MARCH8 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_weno_yz<T, 2, 8>, 256, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_weno_yz<T, 2, 4>, 128, 0);
  return (e != cudaSuccess || b < 1) ? 1 : b;
}

template <typename T>
void launch_batch_weno(const int4 *items, int nitems, int *counter, int parity, int dir,
                       int kind, int seg, int nblocks, cudaStream_t s) {
  const bool by8 = kind == WENO_MARCH8;
  if (dir == 0) {
    if (by8) k_batch_weno_x<T, 8><<<nblocks, dim3(32, 8), march_x_smem<T, 8>(), s>>>(items, nitems, counter, parity, seg);
    else k_batch_weno_x<T, 4><<<nblocks, dim3(32, 4), march_x_smem<T, 4>(), s>>>(items, nitems, counter, parity, seg);
  } else if (dir == 1) {
    if (by8) k_batch_weno_yz<T, 1, 8><<<nblocks, dim3(32, 8), 0, s>>>(items, nitems, counter, parity, seg);
    else k_batch_weno_yz<T, 1, 4><<<nblocks, dim3(32, 4), 0, s>>>(items, nitems, counter, parity, seg);
  } else {
    if (by8) k_batch_weno_yz<T, 2, 8><<<nblocks, dim3(32, 8), 0, s>>>(items, nitems, counter, parity, seg);
    else k_batch_weno_yz<T, 2, 4><<<nblocks, dim3(32, 4), 0, s>>>(items, nitems, counter, parity, seg);
  }
}

// ---------------------------------------------------------------------------------------------
// adaptive TENO cut-off (schemes/spatial/teno.py:430-443) from the modified Ducros sensor
// (schemes/spatial/shock_sensors.py:12-49)
// ---------------------------------------------------------------------------------------------
static __constant__ double c_p10n3[23] = {1e0,   1e-1,  1e-2,  1e-3,  1e-4,  1e-5,  1e-6,  1e-7,
                                          1e-8,  1e-9,  1e-10, 1e-11, 1e-12, 1e-13, 1e-14, 1e-15,
                                          1e-16, 1e-17, 1e-18, 1e-19, 1e-20, 1e-21, 1e-22};
// the same values rounded to FP32 (the FP32 state's cut-off)
static __constant__ float c_p10n3f[23] = {
    (float)1e0,   (float)1e-1,  (float)1e-2,  (float)1e-3,  (float)1e-4,  (float)1e-5,  (float)1e-6,  (float)1e-7,
    (float)1e-8,  (float)1e-9,  (float)1e-10, (float)1e-11, (float)1e-12, (float)1e-13, (float)1e-14, (float)1e-15,
    (float)1e-16, (float)1e-17, (float)1e-18, (float)1e-19, (float)1e-20, (float)1e-21, (float)1e-22};

__device__ __forceinline__ float tanh_s(float x) { return tanhf(x); }
__device__ __forceinline__ double tanh_s(double x) { return tanh(x); }

// Over the points [-1, n_d] of every axis (the left points of all interfaces the flux kernels
// form).  On the interior, with 4th-order central first derivatives of u_i = rhou_i / rho:
//   theta = (1/2 - 1/2 tanh(250 div + 2.5)) div^2 / (eps + |curl u|^2 + div^2);
// theta = 0 elsewhere (the sensor is evaluated on the interior only and the generated code never
// fills its halos).  C_T = 10^-floor(a1 - a2 (1 - (1 - theta)^4 (1 + 4 theta))), the exponent formed
// in the state precision (FP64 arithmetic costs as much as the rest of this kernel on this GPU, and an
// FP32 theta carries no more than FP32 accuracy into it) and the power taken from a table of
// correctly rounded 10^-k.
//
// A block covers an x-y tile of SX x SY points and marches along z over SK planes.  u_i is formed once
// per point (one division) into a ring of five planes of the tile and its two-point x-y margin in
// shared memory; every derivative reads the ring.  Margin points outside [-2, n_d + 2) are never
// read by an interior stencil and are not loaded.
template <typename T> struct SensorTile {
  static constexpr int SX = 32, SY = sizeof(T) == 4 ? 8 : 4, SK = 16;
  static constexpr int PX = SX + 4, PY = SY + 4;  // plane of the ring: tile and margin
};

template <typename T>
__global__ void __launch_bounds__(SensorTile<T>::SX * SensorTile<T>::SY)
    k_sensor_ct3(Grid g, Fields5<const T> q, T *ct, double i0, double i1, double i2, double a1, double a2,
                 double seps) {
  using St = SensorTile<T>;
  constexpr int SX = St::SX, SY = St::SY, SK = St::SK, PX = St::PX, PY = St::PY;
  __shared__ T ring[5][3][PY][PX];
  const int ti = threadIdx.x, tj = threadIdx.y, tid = tj * SX + ti;
  const int ib = (int)blockIdx.x * SX - 1, jb = (int)blockIdx.y * SY - 1, kb = (int)blockIdx.z * SK - 1;
  const int ke = min(kb + SK, g.n2 + 1);  // planes kb .. ke-1 of [-1, n2]
  const T id[3] = {T(i0), T(i1), T(i2)};
  // u of plane kk into ring slot (kk + 8) % 5 (kk >= -3)
  auto load_plane = [&](int kk) {
    const int slot = (kk + 8) % 5;
    for (int t = tid; t < PX * PY; t += SX * SY) {
      const int pi = t % PX, pj = t / PX;
      const int ii = ib - 2 + pi, jj = jb - 2 + pj;
      T u0 = T(0), u1 = T(0), u2 = T(0);
      if (ii >= -2 && ii < g.n0 + 2 && jj >= -2 && jj < g.n1 + 2 && kk >= -2 && kk < g.n2 + 2) {
        const int64_t m = gidx(g, ii, jj, kk);
        const T ir = T(1) / q.v[0][m];
        u0 = q.v[1][m] * ir;
        u1 = q.v[2][m] * ir;
        u2 = q.v[3][m] * ir;
      }
      ring[slot][0][pj][pi] = u0;
      ring[slot][1][pj][pi] = u1;
      ring[slot][2][pj][pi] = u2;
    }
  };
  for (int kk = kb - 2; kk < kb + 2; ++kk) load_plane(kk);
  const int i = ib + ti, j = jb + tj;
  for (int k = kb; k < ke; ++k) {
    load_plane(k + 2);
    __syncthreads();
    if (i <= g.n0 && j <= g.n1) {
      T th = T(0);
      if (i >= 0 && i < g.n0 && j >= 0 && j < g.n1 && k >= 0 && k < g.n2) {
        const int pi = ti + 2, pj = tj + 2, sc = (k + 8) % 5;
        T du[3][3];  // du[c][d] = d u_c / d x_d
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          // values at offsets -2, -1, +1, +2 along each axis
          const T x[4] = {ring[sc][c][pj][pi - 2], ring[sc][c][pj][pi - 1], ring[sc][c][pj][pi + 1],
                          ring[sc][c][pj][pi + 2]};
          const T y[4] = {ring[sc][c][pj - 2][pi], ring[sc][c][pj - 1][pi], ring[sc][c][pj + 1][pi],
                          ring[sc][c][pj + 2][pi]};
          const T z[4] = {ring[(k + 6) % 5][c][pj][pi], ring[(k + 7) % 5][c][pj][pi], ring[(k + 9) % 5][c][pj][pi],
                          ring[(k + 10) % 5][c][pj][pi]};
          du[c][0] = id[0] * ((x[0] - x[3]) * T(1.0 / 12.0) + (x[2] - x[1]) * T(2.0 / 3.0));
          du[c][1] = id[1] * ((y[0] - y[3]) * T(1.0 / 12.0) + (y[2] - y[1]) * T(2.0 / 3.0));
          du[c][2] = id[2] * ((z[0] - z[3]) * T(1.0 / 12.0) + (z[2] - z[1]) * T(2.0 / 3.0));
        }
        const T div = du[0][0] + du[1][1] + du[2][2];
        const T w0 = du[2][1] - du[1][2], w1 = du[0][2] - du[2][0], w2 = du[1][0] - du[0][1];
        const T sw = T(0.5) - T(0.5) * tanh_s(T(250) * div + T(2.5));
        th = sw * (div * div) / (T(seps) + w0 * w0 + w1 * w1 + w2 * w2 + div * div);
      }
      const T w = T(1) - th;
      const T e = floor(T(a1) - T(a2) * (T(1) - (w * w) * (w * w) * (T(4) * th + T(1))));
      const int64_t n = gidx(g, i, j, k);
      if (e >= T(0) && e <= T(22)) ct[n] = sizeof(T) == 4 ? T(c_p10n3f[(int)e]) : T(c_p10n3[(int)e]);
      else ct[n] = T(pow(10.0, -(double)e));
    }
    __syncthreads();  // the next plane's load overwrites the slot of plane k - 2
  }
}

template <typename T>
void launch_sensor_ct3(const Ctx &c, Fields5<const T> q, cudaStream_t s, int64_t *launches) {
  using St = SensorTile<T>;
  const osb_plan_desc &p = c.plan;
  dim3 b(St::SX, St::SY);
  dim3 gs((c.g.n0 + 2 + St::SX - 1) / St::SX, (c.g.n1 + 2 + St::SY - 1) / St::SY, (c.g.n2 + 2 + St::SK - 1) / St::SK);
  k_sensor_ct3<T><<<gs, b, 0, s>>>(c.g, q, static_cast<T *>(c.ct2), 1.0 / p.delta[0], 1.0 / p.delta[1],
                                   1.0 / p.delta[2], p.teno_a1, p.teno_a2, p.sensor_eps);
  ++*launches;
}

// The cut-off of the current state over the interior, FP64 [z][y][x] (the reference's TENO_B0).
template <typename T> __global__ void k_pack_ct3(Grid g, const T *ct, double *out) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    out[t] = (double)ct[gidx(g, i, j, k)];
  }
}

template <typename T>
void launch_cutoff3(const Ctx &c, Fields5<const T> q, double *out, cudaStream_t s, int64_t *launches) {
  launch_sensor_ct3<T>(c, q, s, launches);
  const int64_t N = (int64_t)c.g.n0 * c.g.n1 * c.g.n2;
  int blocks = (int)((N + 255) / 256);
  if (blocks > c.num_sms * 8) blocks = c.num_sms * 8;
  k_pack_ct3<T><<<blocks, 256, 0, s>>>(c.g, static_cast<const T *>(c.ct2), out);
  ++*launches;
}

// The filter's update of the interior (filters/WENO_filter.py:258-282, kappa = Wall = 1): the FP64
// master copy takes q + dt * shock_filter_control * R, the bound state its value (FP32: rounded once)
template <typename T>
__global__ void k_filter_apply(Grid g, Fields5<T> q, Fields5<double> qold, Fields5<const T> r, double dt_fc) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double x = dt_fc * (double)r.v[v][n] + qold.v[v][n];
      qold.v[v][n] = x;
      q.v[v][n] = (T)x;
    }
  }
}

template <typename T>
void launch_filter_apply(const Ctx &c, Fields5<T> q, Fields5<double> qold, Fields5<const T> r, double dt_fc,
                         cudaStream_t s, int64_t *launches) {
  const int64_t N = (int64_t)c.g.n0 * c.g.n1 * c.g.n2;
  int blocks = (int)((N + 255) / 256);
  const int cap = c.num_sms * 8;
  if (blocks > cap) blocks = cap;
  k_filter_apply<T><<<blocks, 256, 0, s>>>(c.g, q, qold, r, dt_fc);
  ++*launches;
}

// The WENO5 filter's flux passes: the same kernel shapes with the filter's interface flux
template <typename T>
void launch_filter_dir(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, cudaStream_t s, int64_t *launches) {
  if (dir == 0) launch_shape<T, 0, false, SCH_FILTER>(c, q, r, c.wcfg[0], s);
  else if (dir == 1) launch_shape<T, 1, true, SCH_FILTER>(c, q, r, c.wcfg[1], s);
  else launch_shape<T, 2, true, SCH_FILTER>(c, q, r, c.wcfg[2], s);
  ++*launches;
}

template <typename T, int DIR, bool ACCUM> static void attr_dir() {
  cudaFuncSetAttribute(k_weno<T, DIR, ACCUM, SCH_JS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tile_smem<T, DIR>());
  cudaFuncSetAttribute(k_weno<T, DIR, ACCUM, SCH_Z>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tile_smem<T, DIR>());
  cudaFuncSetAttribute(k_weno<T, DIR, ACCUM, SCH_TENO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tile_smem<T, DIR>());
  cudaFuncSetAttribute(k_weno<T, DIR, ACCUM, SCH_TENO6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tile_smem<T, DIR>());
  cudaFuncSetAttribute(k_weno<T, DIR, ACCUM, SCH_FILTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tile_smem<T, DIR>());
}
template <typename T> void setup_weno() {
  cudaFuncSetAttribute(k_batch_weno_x<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_x_smem<T, 4>());
  cudaFuncSetAttribute(k_batch_weno_x<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)march_x_smem<T, 8>());
  cudaFuncSetAttribute(k_weno_march_x<T, 4, SCH_JS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 4>());
  cudaFuncSetAttribute(k_weno_march_x<T, 8, SCH_JS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 8>());
  cudaFuncSetAttribute(k_weno_march_x<T, 4, SCH_Z>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 4>());
  cudaFuncSetAttribute(k_weno_march_x<T, 8, SCH_Z>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 8>());
  cudaFuncSetAttribute(k_weno_march_x<T, 4, SCH_TENO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 4>());
  cudaFuncSetAttribute(k_weno_march_x<T, 8, SCH_TENO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 8>());
  cudaFuncSetAttribute(k_weno_march_x<T, 4, SCH_TENO6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 4>());
  cudaFuncSetAttribute(k_weno_march_x<T, 8, SCH_TENO6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 8>());
  cudaFuncSetAttribute(k_weno_march_x<T, 4, SCH_FILTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 4>());
  cudaFuncSetAttribute(k_weno_march_x<T, 8, SCH_FILTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)march_x_smem<T, 8>());
  attr_dir<T, 0, false>();
  attr_dir<T, 1, true>();
  attr_dir<T, 2, true>();
}
template void setup_weno<float>();
template void setup_weno<double>();

template void launch_filter_apply<float>(const Ctx &, Fields5<float>, Fields5<double>, Fields5<const float>, double,
                                         cudaStream_t, int64_t *);
template void launch_filter_apply<double>(const Ctx &, Fields5<double>, Fields5<double>, Fields5<const double>,
                                          double, cudaStream_t, int64_t *);
template void launch_filter_dir<float>(const Ctx &, Fields5<const float>, Fields5<float>, int, cudaStream_t,
                                       int64_t *);
template void launch_filter_dir<double>(const Ctx &, Fields5<const double>, Fields5<double>, int, cudaStream_t,
                                        int64_t *);
template void launch_sensor_ct3<float>(const Ctx &, Fields5<const float>, cudaStream_t, int64_t *);
template void launch_sensor_ct3<double>(const Ctx &, Fields5<const double>, cudaStream_t, int64_t *);
template void launch_cutoff3<float>(const Ctx &, Fields5<const float>, double *, cudaStream_t, int64_t *);
template void launch_cutoff3<double>(const Ctx &, Fields5<const double>, double *, cudaStream_t, int64_t *);
template void launch_weno_dir<float>(const Ctx &, Fields5<const float>, Fields5<float>, int, cudaStream_t, int64_t *);
template void launch_weno_dir<double>(const Ctx &, Fields5<const double>, Fields5<double>, int, cudaStream_t,
                                      int64_t *);
template int batch_weno_blocks_per_sm<float>(int, int);
template int batch_weno_blocks_per_sm<double>(int, int);
template void launch_batch_weno<float>(const int4 *, int, int *, int, int, int, int, int,
                                       cudaStream_t);
template void launch_batch_weno<double>(const int4 *, int, int *, int, int, int, int, int,
                                        cudaStream_t);
template void launch_weno_cfg<float>(const Ctx &, Fields5<const float>, Fields5<float>, int, WenoCfg, cudaStream_t);
template void launch_weno_cfg<double>(const Ctx &, Fields5<const double>, Fields5<double>, int, WenoCfg,
                                      cudaStream_t);

}  // namespace osb
