// osb_internal.h -- host-side context shared by the translation units of libosbli_gb300.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/osb_gb300.h"
#include "osb_common.cuh"

namespace osb {

// launch shape of one direction's WENO flux kernel
enum { WENO_TILE = 0, WENO_MARCH4 = 1, WENO_MARCH8 = 2 };
struct WenoCfg {
  int kind;  // WENO_TILE, or line-marching with 4 or 8 transverse lines per block (y and z only)
  int seg;   // line-marching: cells per segment
};

struct Ctx {
  osb_plan_desc plan;
  Grid g;
  Phys ph;
  int mixed;                 // 1: FP32 state, FP64 accumulator
  int elem;                  // bytes per state element
  void *qa[5] = {};          // bound state (caller-owned)
  void *qb[5] = {};          // second state buffer (ping-pong partner), library-owned
  double *qold[5] = {};      // FP64 RK register (master copy), library-owned
  void *res[5] = {};         // residual, state precision, library-owned
  double *red = nullptr;     // reduction scratch (partial sums), library-owned
  int red_blocks = 0;
  int cur = 0;               // 0: state in qa, 1: state in qb
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  double graph_dt[2] = {0, 0};
  int64_t launches = 0;
  // WENO launch shapes: the autotuner's choice at 256^3 as the default (osb_autotune refines it)
  WenoCfg wcfg[3] = {{WENO_MARCH4, 32}, {WENO_MARCH4, 48}, {WENO_MARCH4, 48}};
  int crk_ty = 8;             // tile height of the fused central/RK kernel (8 or 16)
  double *adj = nullptr;      // adjoint scratch (stage states, primitives, sensitivity fields)
  // TMA tensor maps of the two state buffers (qa, qb) for the central kernel's plane boxes, tile
  // heights 8 and 16; a device status word that bounded device waits set when they give up
  TmaPlanes tma[2][2];
  int tma_ok[2] = {0, 0};
  int tma_enabled = 1;
  int *d_status = nullptr;
  void *probe_buf = nullptr;  // point-probe requests and results (osb_probe)
  int num_sms = 152;          // multiprocessors of the device (set at creation)
  int64_t graph_launches = 0;  // kernel launches recorded in one captured step
  int qold_valid = 0;          // the FP64 register holds the current state
  // 2D wall-bounded path
  int nvar = 5;
  int hx2 = 4, hy2 = 4;           // halos of the 2D layout
  double *q64_2d[4] = {};         // FP64 master state, padded (the bound arrays in FP64 mode)
  double *du2[5] = {};            // LS-RK register (2D and span-periodic 3D wall-bounded blocks)
  void *prim2[6] = {};            // u0, u1, p, a, T, mu (state precision, padded)
  void *ct2 = nullptr;            // adaptive TENO (2D and 3D): cut-off C_T per point (state precision, padded)
  // the stage's right-hand-side parts, formed concurrently: 2D: x fluxes into res, x1 fluxes into
  // resy, viscous terms (momentum 0, 1, energy) into resv; 3D wall-bounded: fluxes into res, viscous
  // terms (momentum 0..2, energy) into resv; two side streams and fork/join events
  void *resy[4] = {};
  void *resv[4] = {};
  cudaStream_t side2[2] = {nullptr, nullptr};
  cudaEvent_t ev_fork2 = nullptr, ev_join2[2] = {nullptr, nullptr};
  double *x1 = nullptr, *d11 = nullptr, *sd111 = nullptr;  // 2D: padded arrays; 3D wall-bounded: lines in j
  double *ysc_d = nullptr;        // 3D wall-bounded: inv_delta1 D11(j), FP64 and FP32 pair
  float2 *ysc_f = nullptr;
  // 3D wall-bounded body force: A exp(..) per (x0, x1) point, cos(bta x2) per plane, the step count
  // and the current step's sin(omega dt iter) (device words, advanced inside the step's graph)
  double *bf_xy = nullptr, *bf_z = nullptr, *bf_t = nullptr;
  long long *d_iter = nullptr;
  int metrics_valid = 0;
  std::string err;
  // per-kernel-family event timing (osb_profile); only used on the eager (non-graph) path
  int prof_on = 0;
  struct ProfRec {
    int family;
    cudaEvent_t a, b;
  };
  std::vector<ProfRec> prof_pending;
  double prof_ms[8] = {};
  int64_t prof_n[8] = {};
};

// encode the central kernel's tensor maps for state buffer `buf` (0: bound arrays, 1: partner)
int encode_state_maps(Ctx &c, int buf);

// plan checks and derived layout/constants (osb_api.cu)
int plan_validate(const osb_plan_desc *p, char *why, size_t n);
Grid plan_grid(const osb_plan_desc *p);
Phys plan_phys(const osb_plan_desc *p);

// kernel families reported by osb_profile_read
enum { PF_HALO = 0, PF_WENO_X, PF_WENO_Y, PF_WENO_Z, PF_CENTRAL_RK, PF_OTHER, PF_COUNT };

template <typename T> void setup_central();
template <typename T> void setup_weno();
template <typename T> void launch_halos(const Ctx &c, Fields5<T> q, cudaStream_t s, int64_t *launches);

template <typename T>
void launch_weno_dir(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, cudaStream_t s, int64_t *launches);
template <typename T>
void launch_weno_cfg(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, WenoCfg w, cudaStream_t s);
// adaptive TENO on 3D blocks: the cut-off C_T per point of the halo-filled state q into ct2
// (read by the flux kernels through Phys::ctp), and its interior packed as FP64 [z][y][x]
template <typename T>
void launch_sensor_ct3(const Ctx &c, Fields5<const T> q, cudaStream_t s, int64_t *launches);
template <typename T>
void launch_cutoff3(const Ctx &c, Fields5<const T> q, double *out, cudaStream_t s, int64_t *launches);
// the WENO5 non-linear filter: flux pass of one direction (x writes r, y and z accumulate), and the
// update qold += dt_fc * r, q = qold (FP32 state rounded once)
template <typename T>
void launch_filter_dir(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, cudaStream_t s, int64_t *launches);
template <typename T>
void launch_filter_apply(const Ctx &c, Fields5<T> q, Fields5<double> qold, Fields5<const T> r, double dt_fc,
                         cudaStream_t s, int64_t *launches);

template <typename T>
void launch_central_rk(const Ctx &c, Fields5<const T> q, Fields5<T> qnew, Fields5<double> qold, Fields5<T> rin,
                       Fields5<T> rout, double dt_new, double dt_old, int mode, cudaStream_t s, int64_t *launches);

cudaError_t upload2_closure_weights();
void launch2_metrics(const Ctx &c, const double *x1, cudaStream_t s, int64_t *launches);
void launch1_bcs(const Ctx &c, cudaStream_t s, int64_t *launches);
void launch1_rhs(const Ctx &c, int update, double A, double B, double dt, cudaStream_t s, int64_t *launches);
void launch2_bcs(const Ctx &c, cudaStream_t s, int64_t *launches);
void launch2_save(const Ctx &c, cudaStream_t s, int64_t *launches);
void launch2_to_state(const Ctx &c, cudaStream_t s, int64_t *launches);
template <typename T> void launch2_cutoff(const Ctx &c, double *out, cudaStream_t s, int64_t *launches);
template <typename T>
void launch2_rhs(const Ctx &c, int update, double A, double B, double dt, cudaStream_t s, int64_t *launches);
// span-periodic 3D wall-bounded blocks (osb_2d.cu): metrics from the x1 coordinate line, the face
// conditions + x2 wrap on the FP64 master followed by the working state, one stage's right-hand side
// with the LS-RK3 update (update = 1) or R into du2 (update = 0)
void launch3w_metrics(const Ctx &c, const double *x1_line, cudaStream_t s, int64_t *launches);
template <typename T> void launch3w_bcs(const Ctx &c, cudaStream_t s, int64_t *launches);
template <typename T>
void launch3w_rhs(const Ctx &c, int update, double A, double B, double dt, cudaStream_t s, int64_t *launches);
template <typename T> void setup3w();
void launch3w_bf_tables(const Ctx &c, cudaStream_t s, int64_t *launches);
void launch3w_tick(const Ctx &c, int advance, double dt, cudaStream_t s, int64_t *launches);
template <typename T> void launch3w_cutoff(const Ctx &c, double *out, cudaStream_t s, int64_t *launches);

// batched ensemble kernels (persistent, tile queue): items are int4 {instance, bx, by, bz}
cudaError_t batch_table_upload_central(const void *src_dev, size_t bytes, cudaStream_t s);
cudaError_t batch_table_upload_weno(const void *src_dev, size_t bytes, cudaStream_t s);
template <typename T>
void launch_batch_central(const int4 *items, int nitems, int *counter, int parity, int stage, int mode, int ty,
                          int nblocks, cudaStream_t s);
template <typename T> int batch_central_blocks_per_sm(int mode, int ty);
template <typename T>
void launch_batch_weno(const int4 *items, int nitems, int *counter, int parity, int dir,
                       int kind, int seg, int nblocks, cudaStream_t s);
template <typename T> int batch_weno_blocks_per_sm(int dir, int kind);

// discrete adjoint of the periodic central scheme (FP64 plans)
cudaError_t adj_ensure(Ctx &c);
cudaError_t adj_residual(Ctx &c, Fields5<double> q, const double *lam, double *out);
cudaError_t adj_step(Ctx &c, Fields5<double> q, double dt, const double *lam_in, double *lam_out);
void adj_halos(const Ctx &c, double *const *f, int nf, cudaStream_t s, int64_t *launches);

// mode bits for launch_central_rk
constexpr int CRK_SKEW = 1;      // add skew-symmetric central convective terms
constexpr int CRK_VISC = 2;      // add viscous / heat-flux terms
constexpr int CRK_RIN = 4;       // add the residual already in rin (WENO/TENO fluxes)
constexpr int CRK_UPDATE = 8;    // apply the RK update into qnew/qold (else write R into rout)

}  // namespace osb
