// osb_noalloc.cu -- osb_reduce_noalloc: the FP64 state reductions without any device allocation.
//
// osb_reduce works on a context, whose work arrays (including the reduction's partial sums) are
// allocated by osb_create.  Some callers cannot allocate device memory at the point where they want a
// diagnostic: host frameworks whose device memory belongs to a pool or caching allocator that must see
// every allocation, and monitoring hooks called between time steps of a running solver, where a
// cudaMalloc/cudaFree would synchronise the device or fragment the pool.  This entry point serves
// them: the caller passes the state arrays and a device output word, and the only scratch, one FP64
// partial sum per z-plane, is a file-scope __device__ array of fixed size.
//
// Scratch rules:
//  * OSB_NOALLOC_MAX_PLANES partial sums (16 KB) exist once per device that loads the library and
//    stay allocated until the process exits;
//  * host code cannot use the array's name as a device address, so the first call on each device
//    (with that device current) looks the address up with cudaGetSymbolAddress and keeps it; make
//    that first call before any stream capture on that device;
//  * every slot the final sum reads is written earlier in the same call, so nothing needs clearing
//    between calls, and the array keeps the last call's partial sums afterwards;
//  * all calls share the one array: calls whose work overlaps on the GPU (different streams, or
//    several host threads) race on it and give wrong results.  Serialise them.
#include <cstdio>
#include <mutex>

#include "osb_common.cuh"
#include "../../include/osb_gb300.h"

namespace osb {
namespace {

static __device__ __align__(256) double g_noalloc_partials[OSB_NOALLOC_MAX_PLANES];

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_DEVICES = 64;
double *g_partials_addr[NA_MAX_DEVICES] = {};
std::mutex g_setup_mutex;

__device__ __forceinline__ double na_block_sum(double x) {
  __shared__ double sh[NA_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
  __syncthreads();
  x = threadIdx.x < NA_THREADS / 32 ? sh[threadIdx.x] : 0.0;
  if (threadIdx.x < 32)
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// Block k reduces interior plane z = k in a fixed order and writes partial[k].
template <typename T>
__global__ void __launch_bounds__(NA_THREADS) k_reduce_planes(Grid g, Fields5<const T> q, int what, double i0, double i1,
                                                              double i2, double *partial) {
  const int k = blockIdx.x;
  const int nxy = g.n0 * g.n1;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nxy; t += NA_THREADS) {
    const int i = t % g.n0, j = t / g.n0;
    const int64_t n = gidx(g, i, j, k);
    if (what == OSB_RED_KE) {
      const double r = (double)q.v[0][n];
      const double m0 = (double)q.v[1][n], m1 = (double)q.v[2][n], m2 = (double)q.v[3][n];
      acc += 0.5 * (m0 * m0 + m1 * m1 + m2 * m2) / r;
    } else if (what == OSB_RED_NANCHECK) {
      for (int v = 0; v < 5; ++v)
        if (!isfinite((double)q.v[v][n])) acc = 1.0;
    } else {  // enstrophy, 4th-order central curl from the halo-filled state
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
      acc += 0.5 * (double)q.v[0][n] * (w0 * w0 + w1 * w1 + w2 * w2);
    }
  }
  const double s = na_block_sum(acc);
  if (threadIdx.x == 0) partial[k] = (what == OSB_RED_NANCHECK) ? (s > 0 ? 1.0 : 0.0) : s;
}

__global__ void k_sum_planes(const double *partial, int nplanes, int what, double scale, double *out) {
  double acc = 0.0;
  for (int b = threadIdx.x; b < nplanes; b += NA_THREADS) acc += partial[b];
  const double s = na_block_sum(acc);
  if (threadIdx.x == 0) out[0] = what == OSB_RED_NANCHECK ? (s > 0 ? 1.0 : 0.0) : s * scale;
}

// Device address of the scratch array on the current device, looked up once per device.
int partials_address(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    fprintf(stderr, "osb_reduce_noalloc: cudaGetDevice failed: %s\n", cudaGetErrorString(e));
    return OSB_ECUDA;
  }
  if (dev < 0 || dev >= NA_MAX_DEVICES) {
    fprintf(stderr, "osb_reduce_noalloc: device ordinal %d beyond the %d supported\n", dev, NA_MAX_DEVICES);
    return OSB_EINVAL;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_partials_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "osb_reduce_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
              cudaGetErrorString(e));
      return OSB_ECUDA;
    }
    g_partials_addr[dev] = static_cast<double *>(p);
  }
  *out = g_partials_addr[dev];
  return OSB_OK;
}

}  // namespace
}  // namespace osb

using namespace osb;

extern "C" int osb_reduce_noalloc(const osb_plan_desc *plan, void *const fields[5], int what, double *dev_out,
                                  void *stream) {
  osb_layout lay;
  int rc = osb_query_layout(plan, &lay);
  if (rc != OSB_OK) return rc;
  // The kernels read five conserved arrays and, for the enstrophy, +-2 planes in z: 2D blocks have
  // four arrays and no z-halo, so they are refused before any pointer is looked at (as osb_reduce does).
  if (plan->ndim != 3) {
    fprintf(stderr, "osb_reduce_noalloc: only 3D plans are supported (ndim = %d)\n", plan->ndim);
    return OSB_EUNSUPPORTED;
  }
  if (plan->n[2] > OSB_NOALLOC_MAX_PLANES) {
    fprintf(stderr, "osb_reduce_noalloc: %d z-planes exceed OSB_NOALLOC_MAX_PLANES (%d); use osb_reduce\n",
            plan->n[2], OSB_NOALLOC_MAX_PLANES);
    return OSB_ETOOLARGE;
  }
  if (what < OSB_RED_KE || what > OSB_RED_NANCHECK || !fields || !dev_out) return OSB_EINVAL;
  for (int v = 0; v < 5; ++v)
    if (!fields[v]) return OSB_EINVAL;
  double *partials = nullptr;
  rc = partials_address(&partials);
  if (rc != OSB_OK) return rc;
  // The scratch address belongs to the current device, so the stream and the output word must too.
  {
    int dev = -1, sdev = -1;
    cudaGetDevice(&dev);
    if (stream) {
      cudaError_t e = cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev);
      if (e != cudaSuccess || sdev != dev) {
        cudaGetLastError();
        fprintf(stderr, "osb_reduce_noalloc: the stream is not on the current device %d\n", dev);
        return OSB_EINVAL;
      }
    }
    cudaPointerAttributes pa;
    cudaError_t e = cudaPointerGetAttributes(&pa, dev_out);
    if (e != cudaSuccess || pa.type != cudaMemoryTypeDevice || pa.device != dev) {
      cudaGetLastError();
      fprintf(stderr, "osb_reduce_noalloc: dev_out is not device memory of the current device %d\n", dev);
      return OSB_EINVAL;
    }
  }

  Grid g;
  g.n0 = plan->n[0];
  g.n1 = plan->n[1];
  g.n2 = plan->n[2];
  g.sy = lay.stride_y;
  g.sz = lay.stride_z;
  g.off0 = lay.offset;
  g.numel = lay.numel;
  const double i0 = 1.0 / plan->delta[0], i1 = 1.0 / plan->delta[1], i2 = 1.0 / plan->delta[2];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (lay.state_bytes == 4) {
    Fields5<const float> q;
    for (int v = 0; v < 5; ++v) q.v[v] = static_cast<const float *>(fields[v]);
    k_reduce_planes<float><<<g.n2, NA_THREADS, 0, s>>>(g, q, what, i0, i1, i2, partials);
  } else {
    Fields5<const double> q;
    for (int v = 0; v < 5; ++v) q.v[v] = static_cast<const double *>(fields[v]);
    k_reduce_planes<double><<<g.n2, NA_THREADS, 0, s>>>(g, q, what, i0, i1, i2, partials);
  }
  const double N = (double)g.n0 * g.n1 * g.n2;
  k_sum_planes<<<1, NA_THREADS, 0, s>>>(partials, g.n2, what, 1.0 / N, dev_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "osb_reduce_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return OSB_ECUDA;
  }
  return OSB_OK;
}
