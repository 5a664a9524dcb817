// osb_bc.cu -- boundary halo fills for the conserved variables.
//
// One launch per axis fills both sides of that axis over the other axes' full haloed range, in
// the order x, y, z.  This is the order in which the generated code applies its boundary kernels
// and exchanges (bc_exchanges.h, algorithm.py:384-477), so corner halos get the same values:
//  * periodic: halo point (..., n+t, ...) <- (..., t, ...), (..., -1-t, ...) <- (..., n-1-t, ...)
//    (core/boundary_conditions/periodic.py:27-56 with exchange.py:9-57);
//  * symmetry: halo point -t mirrors +t about the boundary node, the momentum component normal to
//    the face changes sign (core/boundary_conditions/symmetry.py:23-50, Cartesian normals).
#include "osb_common.cuh"
#include "osb_internal.h"

namespace osb {

template <typename T>
__global__ void k_halo_axis(Grid g, Fields5<T> q, int axis, int depth, int bc_lo, int bc_hi) {
  // index space: side (2) x depth x extent(b) x extent(c), where b, c are the other two axes
  const int n[3] = {g.n0, g.n1, g.n2};
  const int ha[3] = {HX, HY, HZ};
  const int b = axis == 0 ? 1 : 0;
  const int c = axis == 2 ? 1 : 2;
  const int eb = n[b] + 2 * ha[b], ec = n[c] + 2 * ha[c];
  const int64_t total = (int64_t)2 * depth * eb * ec;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    const int ib = (int)(r % eb) - ha[b];
    r /= eb;
    const int ic = (int)(r % ec) - ha[c];
    r /= ec;
    const int dd = (int)(r % depth) + 1;  // 1..depth
    const int side = (int)(r / depth);
    const int kind = side == 0 ? bc_lo : bc_hi;
    int to[3], fr[3];
    to[b] = fr[b] = ib;
    to[c] = fr[c] = ic;
    if (kind == 0) {  // periodic
      if (side == 0) { to[axis] = -dd; fr[axis] = n[axis] - dd; }
      else { to[axis] = n[axis] - 1 + dd; fr[axis] = dd - 1; }
    } else {  // symmetry about the boundary node 0 or n-1
      if (side == 0) { to[axis] = -dd; fr[axis] = dd; }
      else { to[axis] = n[axis] - 1 + dd; fr[axis] = n[axis] - 1 - dd; }
    }
    const int64_t it = gidx(g, to[0], to[1], to[2]), ifr = gidx(g, fr[0], fr[1], fr[2]);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      T val = q.v[v][ifr];
      if (kind == 1 && v == 1 + axis) val = -val;
      q.v[v][it] = val;
    }
  }
}

template <typename T>
void launch_halos(const Ctx &c, Fields5<T> q, cudaStream_t s, int64_t *launches) {
  const int depth = 3;
  const int n[3] = {c.g.n0, c.g.n1, c.g.n2};
  const int ha[3] = {HX, HY, HZ};
  for (int axis = 0; axis < 3; ++axis) {
    const int b = axis == 0 ? 1 : 0, cc = axis == 2 ? 1 : 2;
    const int64_t total = (int64_t)2 * depth * (n[b] + 2 * ha[b]) * (n[cc] + 2 * ha[cc]);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_halo_axis<T><<<blocks, 256, 0, s>>>(c.g, q, axis, depth, c.plan.bc[axis][0], c.plan.bc[axis][1]);
    ++*launches;
  }
}

template void launch_halos<float>(const Ctx &, Fields5<float>, cudaStream_t, int64_t *);
template void launch_halos<double>(const Ctx &, Fields5<double>, cudaStream_t, int64_t *);

}  // namespace osb
