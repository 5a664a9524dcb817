// osb_batch.cu -- batched ensembles: many independent periodic 3D blocks of uneven size stepped
// together.
//
// The reference runs one block per process and one OPS kernel launch per loop; an ensemble of small
// blocks leaves a GB300 mostly idle.  Here every instance keeps its own padded arrays (as a single
// plan would), and each RK3 stage is a handful of launches over ALL instances:
//   * halos: one launch per axis, one block per (instance, chunk of the halo index space);
//   * WENO5-JS fluxes (instances that use them): one persistent line-marching launch per direction;
//   * fused central/RK update: one persistent launch per kernel mode (skew-symmetric or residual
//     input, with or without viscous terms).
// Persistent launches size their grid to the resident blocks of the device and pull tiles
// {instance, bx, by, bz} from a queue (an atomic counter per launch, reset by a memset node at the
// start of each stage; a block never waits on another).  Tiles are ordered largest instance first.
// A whole step is captured as one CUDA graph.  The instance descriptors (grid, constants, pointers,
// time step) live in a device table that every step copies into the kernels' constant-memory table.
// Tile shapes (WENO segment length and lines per block, central tile height) are chosen by
// osb_batch_autotune.
#include <algorithm>
#include <cstdio>
#include <numeric>
#include <string>
#include <vector>

#include "osb_common.cuh"
#include "osb_internal.h"

using namespace osb;

namespace {
constexpr int HALO_CHUNK = 2048;  // halo points per block
enum { Q_WX = 0, Q_WY, Q_WZ, Q_C0, Q_C1, Q_C2, Q_C3, Q_COUNT };  // tile queues (counters) of a stage
const int CENTRAL_MODES[4] = {CRK_SKEW | CRK_VISC, CRK_SKEW, CRK_RIN | CRK_VISC, CRK_RIN};

template <typename T>
__global__ void k_batch_halo(const BatchInst<T> *tab, const int2 *items, int parity, int axis) {
  const int2 it = items[blockIdx.x];
  const BatchInst<T> &d = tab[it.x];
  const Grid g = d.g;
  const int n[3] = {g.n0, g.n1, g.n2};
  const int ha[3] = {HX, HY, HZ};
  const int depth = 3;
  const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
  const int eb = n[b] + 2 * ha[b], ec = n[c] + 2 * ha[c];
  const int64_t total = (int64_t)2 * depth * eb * ec;
  const int64_t t1 = min(total, (int64_t)(it.y + 1) * HALO_CHUNK);
  T *const *q = d.q[parity];
  for (int64_t t = (int64_t)it.y * HALO_CHUNK + threadIdx.x; t < t1; t += blockDim.x) {
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
    const int64_t a = gidx(g, to[0], to[1], to[2]), s = gidx(g, fr[0], fr[1], fr[2]);
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v][a] = q[v][s];
  }
}

template <typename T> __global__ void k_batch_set(Grid g, const double *src, Fields5<T> q, Fields5<double> qold) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double x = src[v * N + t];
      qold.v[v][n] = x;
      q.v[v][n] = (T)x;
    }
  }
}

__global__ void k_batch_get(Grid g, Fields5<const double> qold, double *dst) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t n = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v * N + t] = qold.v[v][n];
  }
}

int blocks_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 16);
}
}  // namespace

struct osb_batch {
  int nb = 0, mixed = 0, elem = 8;
  std::vector<osb_plan_desc> plans;
  std::vector<Grid> grids;
  std::vector<unsigned char> table;  // host copy of BatchInst<T>[nb]
  size_t inst_bytes = 0;
  void *d_table = nullptr;
  void *pool = nullptr;
  double *qold_base = nullptr;  // every instance's FP64 register, contiguous
  size_t qold_bytes = 0;
  std::vector<int> order;  // instances, largest first
  // tile queues
  int4 *d_items = nullptr;
  int item_cap = 0;
  int item_off[Q_COUNT] = {}, item_cnt[Q_COUNT] = {};
  int nblocks[Q_COUNT] = {};
  int2 *d_halo = nullptr;
  int halo_off[3] = {}, halo_cnt[3] = {};
  int *d_counters = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int cur = 0;
  WenoCfg wcfg[3] = {{WENO_MARCH4, 48}, {WENO_MARCH4, 48}, {WENO_MARCH4, 48}};
  int crk_ty = 8;
  int zchunk = 16;
  int num_sms = 152;
  bool any_weno = false;
  int64_t launches = 0, graph_launches = 0;
  double rk_a[3] = {}, rk_b[3] = {};
  std::string err;
};

namespace {
int berr(osb_batch *b, int code, const char *msg) {
  if (b) b->err = msg;
  return code;
}
int bcuda(osb_batch *b, cudaError_t e, const char *where) {
  if (e == cudaSuccess) return OSB_OK;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", where, cudaGetErrorString(e));
  return berr(b, OSB_ECUDA, buf);
}
void drop_graphs(osb_batch *b) {
  for (int s = 0; s < 2; ++s)
    if (b->graph[s]) {
      cudaGraphExecDestroy(b->graph[s]);
      b->graph[s] = nullptr;
    }
}

template <typename T> BatchInst<T> &inst(osb_batch *b, int i) {
  return reinterpret_cast<BatchInst<T> *>(b->table.data())[i];
}

template <typename T> int central_mode(const BatchInst<T> &d) {
  return (d.conv == OSB_CONV_WENO5JS ? CRK_RIN : CRK_SKEW) | (d.visc ? CRK_VISC : 0);
}

// (re)build the tile queues for the current shapes and size the persistent grids
template <typename T> cudaError_t build_items(osb_batch *b) {
  std::vector<int4> items;
  std::vector<int2> halo;
  for (int q = 0; q < Q_COUNT; ++q) {
    b->item_off[q] = (int)items.size();
    for (int i : b->order) {
      BatchInst<T> &d = inst<T>(b, i);
      const Grid &g = d.g;
      if (q <= Q_WZ) {
        if (d.conv != OSB_CONV_WENO5JS) continue;
        const int L = b->wcfg[q].seg, by = b->wcfg[q].kind == WENO_MARCH8 ? 8 : 4;
        int nx, ny, nz;
        if (q == Q_WX) { nx = (g.n0 + L - 1) / L; ny = (g.n1 + 31) / 32; nz = (g.n2 + by - 1) / by; }
        else if (q == Q_WY) { nx = (g.n0 + 31) / 32; ny = (g.n2 + by - 1) / by; nz = (g.n1 + L - 1) / L; }
        else { nx = (g.n0 + 31) / 32; ny = (g.n1 + by - 1) / by; nz = (g.n2 + L - 1) / L; }
        for (int z = 0; z < nz; ++z)
          for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) items.push_back(make_int4(i, x, y, z));
      } else {
        if (central_mode(d) != CENTRAL_MODES[q - Q_C0]) continue;
        d.zchunk = std::min(b->zchunk, g.n2);
        const int nx = (g.n0 + 31) / 32, ny = (g.n1 + b->crk_ty - 1) / b->crk_ty, nz = (g.n2 + d.zchunk - 1) / d.zchunk;
        for (int z = 0; z < nz; ++z)
          for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) items.push_back(make_int4(i, x, y, z));
      }
    }
    b->item_cnt[q] = (int)items.size() - b->item_off[q];
    int per_sm = 1;
    if (b->item_cnt[q] > 0)
      per_sm = q <= Q_WZ ? batch_weno_blocks_per_sm<T>(q, b->wcfg[q].kind)
                         : batch_central_blocks_per_sm<T>(CENTRAL_MODES[q - Q_C0], b->crk_ty);
    b->nblocks[q] = std::max(1, std::min(b->item_cnt[q], b->num_sms * per_sm));
  }
  for (int axis = 0; axis < 3; ++axis) {
    b->halo_off[axis] = (int)halo.size();
    for (int i : b->order) {
      const Grid &g = inst<T>(b, i).g;
      const int n[3] = {g.n0, g.n1, g.n2}, ha[3] = {HX, HY, HZ};
      const int bb = axis == 0 ? 1 : 0, cc = axis == 2 ? 1 : 2;
      const int64_t total = (int64_t)2 * 3 * (n[bb] + 2 * ha[bb]) * (n[cc] + 2 * ha[cc]);
      for (int64_t c = 0; c * HALO_CHUNK < total; ++c) halo.push_back(make_int2(i, (int)c));
    }
    b->halo_cnt[axis] = (int)halo.size() - b->halo_off[axis];
  }
  // earlier launches may still read the old queues and table: wait for them, then copy in order
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e == cudaSuccess && (int)items.size() > b->item_cap) {
    cudaFree(b->d_items);
    b->item_cap = (int)items.size();
    e = cudaMalloc(&b->d_items, sizeof(int4) * std::max(1, b->item_cap));
  }
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpyAsync(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess && !b->d_halo) e = cudaMalloc(&b->d_halo, sizeof(int2) * halo.size());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_halo, halo.data(), sizeof(int2) * halo.size(), cudaMemcpyHostToDevice, b->stream);
  // descriptors changed (zchunk): refresh the device table
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_table, b->table.data(), b->table.size(), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  return e;
}

template <typename T> void launch_halos_b(osb_batch *b, int parity, cudaStream_t s) {
  for (int axis = 0; axis < 3; ++axis) {
    k_batch_halo<T><<<b->halo_cnt[axis], 256, 0, s>>>(static_cast<const BatchInst<T> *>(b->d_table),
                                                      b->d_halo + b->halo_off[axis], parity, axis);
    ++b->launches;
  }
}

template <typename T> void launch_weno_b(osb_batch *b, int q, int parity, cudaStream_t s) {
  if (!b->item_cnt[q]) return;
  launch_batch_weno<T>(b->d_items + b->item_off[q], b->item_cnt[q], b->d_counters + q, parity, q, b->wcfg[q].kind,
                       b->wcfg[q].seg, b->nblocks[q], s);
  ++b->launches;
}

template <typename T> void launch_central_b(osb_batch *b, int q, int parity, int stage, cudaStream_t s) {
  if (!b->item_cnt[q]) return;
  launch_batch_central<T>(b->d_items + b->item_off[q], b->item_cnt[q], b->d_counters + q, parity, stage,
                          CENTRAL_MODES[q - Q_C0], b->crk_ty, b->nblocks[q], s);
  ++b->launches;
}

template <typename T> void one_step_b(osb_batch *b, int start, cudaStream_t s) {
  batch_table_upload_central(b->d_table, b->table.size(), s);
  batch_table_upload_weno(b->d_table, b->table.size(), s);
  for (int st = 0; st < 3; ++st) {
    const int par = start ^ (st & 1);
    cudaMemsetAsync(b->d_counters, 0, sizeof(int) * Q_COUNT, s);
    launch_halos_b<T>(b, par, s);
    for (int q = Q_WX; q <= Q_WZ; ++q) launch_weno_b<T>(b, q, par, s);
    for (int q = Q_C0; q < Q_COUNT; ++q) launch_central_b<T>(b, q, par, st, s);
  }
}

template <typename T> int step_b(osb_batch *b, int nsteps) {
  cudaStream_t s = b->stream;
  b->launches = 0;
  for (int it = 0; it < nsteps; ++it) {
    const int start = b->cur;
    if (s != nullptr) {
      if (!b->graph[start]) {
        cudaGraph_t gr;
        const int64_t l0 = b->launches;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return bcuda(b, e, "cudaStreamBeginCapture");
        one_step_b<T>(b, start, s);
        e = cudaStreamEndCapture(s, &gr);
        if (e != cudaSuccess) return bcuda(b, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->graph[start], gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return bcuda(b, e, "cudaGraphInstantiate");
        b->graph_launches = b->launches - l0;
        b->launches = l0;
      }
      cudaError_t e = cudaGraphLaunch(b->graph[start], s);
      if (e != cudaSuccess) return bcuda(b, e, "cudaGraphLaunch");
      b->launches += b->graph_launches;
    } else {
      one_step_b<T>(b, start, s);
    }
    b->cur ^= 1;
  }
  return bcuda(b, cudaGetLastError(), "osb_batch_step");
}

template <typename T> int autotune_b(osb_batch *b, int reps, double *best_ms) {
  cudaStream_t s = b->stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t err = cudaSuccess;
  // the central kernels update the RK register: keep a copy and restore it afterwards
  double *save = nullptr;
  err = cudaMalloc(&save, b->qold_bytes);
  if (err == cudaSuccess) err = cudaMemcpyAsync(save, b->qold_base, b->qold_bytes, cudaMemcpyDeviceToDevice, s);
  const int par = b->cur;
  auto timeit = [&](auto &&launch) -> float {
    cudaMemsetAsync(b->d_counters, 0, sizeof(int) * Q_COUNT, s);
    launch();
    cudaEventRecord(e0, s);
    for (int k = 0; k < reps; ++k) {
      cudaMemsetAsync(b->d_counters, 0, sizeof(int) * Q_COUNT, s);
      launch();
    }
    cudaEventRecord(e1, s);
    err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err != cudaSuccess) return -1.0f;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / reps;
  };
  if (err == cudaSuccess) {
    batch_table_upload_central(b->d_table, b->table.size(), s);
    batch_table_upload_weno(b->d_table, b->table.size(), s);
    launch_halos_b<T>(b, par, s);
  }
  for (int t = 0; t < 4 && best_ms; ++t) best_ms[t] = 0.0;
  for (int q = Q_WX; q <= Q_WZ && err == cudaSuccess && b->any_weno; ++q) {
    float best = 1e30f;
    WenoCfg choice = b->wcfg[q];
    for (int kind : {WENO_MARCH4, WENO_MARCH8})
      for (int seg : {16, 24, 32, 48, 64, 96}) {
        b->wcfg[q] = WenoCfg{kind, seg};
        if ((err = build_items<T>(b)) != cudaSuccess) break;
        const float ms = timeit([&] { launch_weno_b<T>(b, q, par, s); });
        if (ms < 0) break;
        if (ms < best) {
          best = ms;
          choice = b->wcfg[q];
        }
      }
    b->wcfg[q] = choice;
    if (best_ms) best_ms[q] = best;
  }
  if (err == cudaSuccess) {
    float best = 1e30f;
    int cty = b->crk_ty, czc = b->zchunk;
    for (int ty : {8, 16})
      for (int zc : {8, 16, 32}) {
        b->crk_ty = ty;
        b->zchunk = zc;
        if ((err = build_items<T>(b)) != cudaSuccess) break;
        const float ms = timeit([&] {
          for (int q = Q_C0; q < Q_COUNT; ++q) launch_central_b<T>(b, q, par, 0, s);
        });
        if (ms < 0) break;
        if (ms < best) {
          best = ms;
          cty = ty;
          czc = zc;
        }
      }
    b->crk_ty = cty;
    b->zchunk = czc;
    if (best_ms) best_ms[3] = best;
  }
  if (save) {
    cudaError_t e2 = cudaMemcpyAsync(b->qold_base, save, b->qold_bytes, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess) err = e2;
    cudaStreamSynchronize(s);
    cudaFree(save);
  }
  if (err == cudaSuccess) err = build_items<T>(b);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return bcuda(b, err, "osb_batch_autotune");
}

template <typename T> void set_inst_dt(BatchInst<T> &d, double dt, const double *a, const double *b) {
  d.dt = dt;
  for (int s = 0; s < 3; ++s) {
    d.dtn[s] = dt * b[s];
    d.dto[s] = dt * a[s];
    d.ddt[s] = (float)(dt * b[s] - dt * a[s]);
  }
}

// the state arrays of stage-start parity `par` hold FP32 copies: re-derive them from the register
template <typename T> Fields5<T> state_fields(osb_batch *b, int i, int par) {
  Fields5<T> f;
  for (int v = 0; v < 5; ++v) f.v[v] = inst<T>(b, i).q[par][v];
  return f;
}
template <typename T> Fields5<double> qold_fields(osb_batch *b, int i) {
  Fields5<double> f;
  for (int v = 0; v < 5; ++v) f.v[v] = inst<T>(b, i).qold[v];
  return f;
}

template <typename T> int create_b(osb_batch *b) {
  b->inst_bytes = sizeof(BatchInst<T>);
  if ((size_t)b->nb * b->inst_bytes > BATCH_TABLE_BYTES) {
    char buf[160];
    snprintf(buf, sizeof buf, "osb_batch_create: at most %d instances", (int)(BATCH_TABLE_BYTES / b->inst_bytes));
    return berr(b, OSB_ETOOLARGE, buf);
  }
  b->table.assign((size_t)b->nb * b->inst_bytes, 0);
  size_t per_t = 0, per_d = 0;
  for (int i = 0; i < b->nb; ++i) {
    const Grid g = plan_grid(&b->plans[i]);
    per_t += (size_t)g.numel * 15;  // q[2][5], res[5]
    per_d += (size_t)g.numel * 5;   // qold[5]
  }
  b->qold_bytes = per_d * sizeof(double);
  const size_t bytes = per_d * sizeof(double) + per_t * sizeof(T);
  cudaError_t e = cudaMalloc(&b->pool, bytes);
  if (e == cudaSuccess) e = cudaMemset(b->pool, 0, bytes);
  if (e != cudaSuccess) return bcuda(b, e, "osb_batch_create: allocation");
  double *pd = static_cast<double *>(b->pool);
  b->qold_base = pd;
  T *pt = reinterpret_cast<T *>(pd + per_d);
  for (int i = 0; i < b->nb; ++i) {
    BatchInst<T> &d = inst<T>(b, i);
    const osb_plan_desc &p = b->plans[i];
    d.g = plan_grid(&p);
    d.ph = plan_phys(&p);
    for (int v = 0; v < 5; ++v) {
      d.qold[v] = pd;
      pd += d.g.numel;
    }
    for (int k = 0; k < 2; ++k)
      for (int v = 0; v < 5; ++v) {
        d.q[k][v] = pt;
        pt += d.g.numel;
      }
    for (int v = 0; v < 5; ++v) {
      d.res[v] = pt;
      pt += d.g.numel;
    }
    d.dt = 0.0;
    d.conv = p.conv;
    d.visc = p.visc == OSB_VISC_CONST ? 1 : 0;
    if (d.conv == OSB_CONV_WENO5JS) b->any_weno = true;
    b->grids.push_back(d.g);
  }
  b->order.resize(b->nb);
  std::iota(b->order.begin(), b->order.end(), 0);
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
    return b->grids[x].n0 * (int64_t)b->grids[x].n1 * b->grids[x].n2 >
           b->grids[y].n0 * (int64_t)b->grids[y].n1 * b->grids[y].n2;
  });
  e = cudaMalloc(&b->d_table, b->table.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, sizeof(int) * Q_COUNT);
  if (e == cudaSuccess) e = cudaMemset(b->d_counters, 0, sizeof(int) * Q_COUNT);
  if (e == cudaSuccess) e = build_items<T>(b);
  return bcuda(b, e, "osb_batch_create");
}
}  // namespace

extern "C" {

int osb_batch_create(const osb_plan_desc *plans, int n, osb_batch **out) {
  if (!plans || !out || n < 1) return OSB_EINVAL;
  *out = nullptr;
  char why[256];
  for (int i = 0; i < n; ++i) {
    const osb_plan_desc &p = plans[i];
    const int rc = plan_validate(&p, why, sizeof why);
    if (rc) return rc;
    if (p.ndim != 3 || (p.conv != OSB_CONV_CENTRAL_SKEW && p.conv != OSB_CONV_WENO5JS) || p.rk != OSB_RK3_2REG)
      return OSB_EUNSUPPORTED;
    for (int d = 0; d < 3; ++d)
      if (p.bc[d][0] != OSB_BC_PERIODIC || p.bc[d][1] != OSB_BC_PERIODIC) return OSB_EUNSUPPORTED;
    if (p.precision != plans[0].precision) return OSB_EINVAL;
    for (int s = 0; s < 3; ++s)
      if (p.rk_a[s] != plans[0].rk_a[s] || p.rk_b[s] != plans[0].rk_b[s]) return OSB_EINVAL;
  }
  osb_batch *b = new osb_batch();
  b->nb = n;
  b->plans.assign(plans, plans + n);
  b->mixed = plans[0].precision == OSB_PREC_MIXED;
  b->elem = b->mixed ? 4 : 8;
  for (int s = 0; s < 3; ++s) {
    b->rk_a[s] = plans[0].rk_a[s];
    b->rk_b[s] = plans[0].rk_b[s];
  }
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      nsm > 0)
    b->num_sms = nsm;
  if (b->mixed) { setup_central<float>(); setup_weno<float>(); }
  else { setup_central<double>(); setup_weno<double>(); }
  const int rc = b->mixed ? create_b<float>(b) : create_b<double>(b);
  if (rc) {
    osb_batch_destroy(b);
    return rc;
  }
  *out = b;
  return OSB_OK;
}

int osb_batch_set_stream(osb_batch *b, void *stream) {
  if (!b) return OSB_EINVAL;
  b->stream = static_cast<cudaStream_t>(stream);
  drop_graphs(b);
  return OSB_OK;
}

int osb_batch_set_dt(osb_batch *b, const double *dt) {
  if (!b || !dt) return OSB_EINVAL;
  for (int i = 0; i < b->nb; ++i) {
    if (!(dt[i] > 0)) return berr(b, OSB_EINVAL, "osb_batch_set_dt: every dt must be > 0");
    if (b->mixed) set_inst_dt(inst<float>(b, i), dt[i], b->rk_a, b->rk_b);
    else set_inst_dt(inst<double>(b, i), dt[i], b->rk_a, b->rk_b);
  }
  // stream-ordered, so steps already queued keep their time steps; the graphs copy the device table
  return bcuda(b, cudaMemcpyAsync(b->d_table, b->table.data(), b->table.size(), cudaMemcpyHostToDevice, b->stream),
               "osb_batch_set_dt");
}

int osb_batch_set_state64(osb_batch *b, int i, const double *src) {
  if (!b || !src || i < 0 || i >= b->nb) return OSB_EINVAL;
  const Grid g = b->grids[i];
  const int nbk = blocks_for((int64_t)g.n0 * g.n1 * g.n2);
  if (b->mixed)
    k_batch_set<float><<<nbk, 256, 0, b->stream>>>(g, src, state_fields<float>(b, i, b->cur), qold_fields<float>(b, i));
  else
    k_batch_set<double><<<nbk, 256, 0, b->stream>>>(g, src, state_fields<double>(b, i, b->cur),
                                                    qold_fields<double>(b, i));
  return bcuda(b, cudaGetLastError(), "osb_batch_set_state64");
}

int osb_batch_get_state64(osb_batch *b, int i, double *dst) {
  if (!b || !dst || i < 0 || i >= b->nb) return OSB_EINVAL;
  const Grid g = b->grids[i];
  Fields5<const double> qo;
  for (int v = 0; v < 5; ++v)
    qo.v[v] = b->mixed ? inst<float>(b, i).qold[v] : inst<double>(b, i).qold[v];
  k_batch_get<<<blocks_for((int64_t)g.n0 * g.n1 * g.n2), 256, 0, b->stream>>>(g, qo, dst);
  return bcuda(b, cudaGetLastError(), "osb_batch_get_state64");
}

int osb_batch_step(osb_batch *b, int nsteps) {
  if (!b || nsteps < 0) return OSB_EINVAL;
  for (int i = 0; i < b->nb; ++i) {
    const double dt = b->mixed ? inst<float>(b, i).dt : inst<double>(b, i).dt;
    if (!(dt > 0)) return berr(b, OSB_EINVAL, "osb_batch_step: time steps not set (osb_batch_set_dt)");
  }
  return b->mixed ? step_b<float>(b, nsteps) : step_b<double>(b, nsteps);
}

int osb_batch_autotune(osb_batch *b, int reps, double *best_ms) {
  if (!b || reps < 1) return OSB_EINVAL;
  return b->mixed ? autotune_b<float>(b, reps, best_ms) : autotune_b<double>(b, reps, best_ms);
}

int osb_batch_get_shape(osb_batch *b, int *out, int n) {
  if (!b || !out || n < 8) return OSB_EINVAL;
  for (int d = 0; d < 3; ++d) {
    out[2 * d] = b->wcfg[d].kind;
    out[2 * d + 1] = b->wcfg[d].seg;
  }
  out[6] = b->crk_ty;
  out[7] = b->zchunk;
  return OSB_OK;
}

int64_t osb_batch_launch_count(osb_batch *b) { return b ? b->launches : -1; }

int osb_batch_get_error(osb_batch *b, char *buf, int n) {
  if (!b || !buf || n <= 0) return OSB_EINVAL;
  snprintf(buf, (size_t)n, "%s", b->err.c_str());
  return OSB_OK;
}

void osb_batch_destroy(osb_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  else cudaDeviceSynchronize();
  drop_graphs(b);
  cudaFree(b->pool);
  cudaFree(b->d_table);
  cudaFree(b->d_items);
  cudaFree(b->d_halo);
  cudaFree(b->d_counters);
  delete b;
}

}  // extern "C"
