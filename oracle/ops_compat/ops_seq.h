/* ops_seq.h -- a sequential/OpenMP stand-in for the subset of the OPS C API that OpenSBLI's OPSC
 * writer emits (code_generation/opsc.py:537-722, core/kernel.py:233-274).
 *
 * Test infrastructure: this header lets the reference generator's own C output (opensbli.cpp,
 * opensbliblock00_kernels.h, defdec_data_set.h, bc_exchanges.h) compile and run on the host, so
 * that the CPU oracle and the timed CPU baseline are the reference's own arithmetic.  OPS itself
 * (github OP-DSL/OPS) is not vendored by the reference and is not available here; only its
 * documented sequential semantics are restated:
 *   - ops_decl_dat: a dat of `size` interior points with halos d_m (negative) and d_p per axis;
 *   - ops_par_loop: call the kernel once per point of the iteration range, handing each dat
 *     argument a pointer to that point; OPS_ACCn(x,y,z) indexes relative to it;
 *   - ops_halo_transfer: copy each halo's iteration box from its source to its destination dat;
 *   - ops_fetch_dat_hdf5_file: here a raw binary dump (header + padded array) instead of HDF5.
 * The outer loop of every par_loop runs under OpenMP, as OPS's OpenMP backend does.
 * Run-time parameters: osb_param_i/osb_param_d read OSB_<name> from the environment.
 */
#ifndef OSB_OPS_SEQ_H
#define OSB_OPS_SEQ_H

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <utility>
#ifdef _OPENMP
#include <omp.h>
#endif

#if !defined(OPS_2D) && !defined(OPS_3D) && !defined(OPS_1D)
#define OPS_3D
#endif

/* ---------- run-time parameters ---------- */
static inline int osb_param_i(const char *name, int def) {
  char key[128];
  snprintf(key, sizeof key, "OSB_%s", name);
  const char *v = getenv(key);
  return v ? atoi(v) : def;
}
static inline double osb_param_d(const char *name, double def) {
  char key[128];
  snprintf(key, sizeof key, "OSB_%s", name);
  const char *v = getenv(key);
  return v ? strtod(v, NULL) : def;
}

/* ---------- objects ---------- */
typedef struct ops_block_core { int dims; const char *name; } *ops_block;

typedef struct ops_dat_core {
  char *data;         /* start of the padded allocation */
  int elem;           /* bytes per element */
  int size[3];        /* interior points per axis */
  int d_m[3], d_p[3]; /* halo depths: d_m <= 0, d_p >= 0 */
  int pad[3];         /* padded extent per axis */
  const char *name;
  const char *type;
} *ops_dat;

typedef struct { int n; } *ops_stencil;

enum { OPS_READ = 0, OPS_WRITE = 1, OPS_RW = 2, OPS_INC = 3, OPS_MIN = 4, OPS_MAX = 5 };
typedef int ops_access;

typedef struct {
  int kind; /* 0 dat, 1 gbl, 2 idx */
  ops_dat dat;
  void *gbl;
} ops_arg;

typedef struct ops_halo_core {
  ops_dat from, to;
  int iter[3], from_base[3], to_base[3], from_dir[3], to_dir[3];
} *ops_halo;

typedef struct ops_halo_group_core { int n; ops_halo *h; } *ops_halo_group;

/* ---------- OPS_ACC macros: per-argument padded extents ---------- */
static int osb_xdim[128], osb_ydim[128];
#if defined(OPS_3D)
#define OSB_ACC(n, x, y, z) ((x) + osb_xdim[n] * (y) + osb_xdim[n] * osb_ydim[n] * (z))
#elif defined(OPS_1D)
#define OSB_ACC(n, x) (x)
#else
#define OSB_ACC(n, x, y) ((x) + osb_xdim[n] * (y))
#endif
/* OPS_ACC0 .. OPS_ACC99 */
#include "ops_acc_macros.h"

/* ---------- init / misc ---------- */
static inline void ops_init(int argc, char **argv, int level) { (void)argc; (void)argv; (void)level; }
static inline void ops_exit(void) {}
static inline void ops_partition(const char *s) { (void)s; }
template <typename T>
static inline void ops_decl_const(const char *name, int dim, const char *type, T *v) { (void)name; (void)dim; (void)type; (void)v; }
#define ops_printf printf

static inline void ops_timers(double *cpu, double *et) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  *et = ts.tv_sec + 1e-9 * ts.tv_nsec;
  *cpu = (double)clock() / CLOCKS_PER_SEC;
}

static inline ops_block ops_decl_block(int dims, const char *name) {
  ops_block b = (ops_block)calloc(1, sizeof(*b));
  b->dims = dims;
  b->name = name;
  return b;
}

static inline ops_stencil ops_decl_stencil(int dims, int npts, int *pts, const char *name) {
  (void)dims; (void)pts; (void)name;
  ops_stencil s = (ops_stencil)calloc(1, sizeof(*s));
  s->n = npts;
  return s;
}
#define ops_decl_strided_stencil(d, n, p, st, name) ops_decl_stencil(d, n, p, name)

template <typename T>
static inline ops_dat ops_decl_dat(ops_block block, int dim, int *size, int *base, int *d_m, int *d_p, T *value,
                                   const char *type, const char *name) {
  (void)dim; (void)base; (void)value;
  ops_dat d = (ops_dat)calloc(1, sizeof(*d));
  size_t n = 1;
  for (int a = 0; a < 3; ++a) {
    if (a < block->dims) {
      d->size[a] = size[a];
      d->d_m[a] = d_m[a];
      d->d_p[a] = d_p[a];
    } else {
      d->size[a] = 1;
      d->d_m[a] = 0;
      d->d_p[a] = 0;
    }
    d->pad[a] = d->size[a] - d->d_m[a] + d->d_p[a];
    n *= (size_t)d->pad[a];
  }
  d->elem = (int)sizeof(T);
  d->data = (char *)calloc(n, sizeof(T));
  d->name = name;
  d->type = type;
  return d;
}

static inline size_t osb_offset(ops_dat d, int x, int y, int z) {
  return (size_t)(x - d->d_m[0]) +
         (size_t)d->pad[0] * ((size_t)(y - d->d_m[1]) + (size_t)d->pad[1] * (size_t)(z - d->d_m[2]));
}

static inline ops_arg ops_arg_dat(ops_dat dat, int dim, ops_stencil s, const char *type, ops_access acc) {
  (void)dim; (void)s; (void)type; (void)acc;
  ops_arg a;
  a.kind = 0;
  a.dat = dat;
  a.gbl = NULL;
  return a;
}
template <typename T>
static inline ops_arg ops_arg_gbl(T *data, int dim, const char *type, ops_access acc) {
  (void)dim; (void)type; (void)acc;
  ops_arg a;
  a.kind = 1;
  a.dat = NULL;
  a.gbl = (void *)data;
  return a;
}
static inline ops_arg ops_arg_idx(void) {
  ops_arg a;
  a.kind = 2;
  a.dat = NULL;
  a.gbl = NULL;
  return a;
}

/* ---------- par_loop ---------- */
template <typename... P, size_t... I>
static inline void osb_invoke(void (*k)(P...), void **p, std::index_sequence<I...>) {
  k(static_cast<P>(p[I])...);
}

template <typename... P, typename... A>
static void ops_par_loop(void (*kernel)(P...), const char *name, ops_block block, int dim, int *range, A... argv) {
  (void)name;
  constexpr int nargs = (int)sizeof...(A);
  static_assert(sizeof...(P) == sizeof...(A), "kernel arity does not match the argument list");
  ops_arg args[nargs] = {argv...};
  for (int n = 0; n < nargs; ++n) {
    if (args[n].kind == 0) {
      osb_xdim[n] = args[n].dat->pad[0];
      osb_ydim[n] = args[n].dat->pad[1];
    }
  }
  int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  for (int a = 0; a < dim && a < 3; ++a) {
    lo[a] = range[2 * a];
    hi[a] = range[2 * a + 1];
  }
  (void)block;
  const int outer = dim == 3 ? 2 : 1;
  const int olo = lo[outer], ohi = hi[outer];
#pragma omp parallel for schedule(static)
  for (int o = olo; o < ohi; ++o) {
    void *p[nargs > 0 ? nargs : 1];
    int idx[3];
    int zlo = dim == 3 ? o : 0, zhi = dim == 3 ? o + 1 : 1;
    int ylo = dim == 3 ? lo[1] : o, yhi = dim == 3 ? hi[1] : o + 1;
    for (int z = zlo; z < zhi; ++z)
      for (int y = ylo; y < yhi; ++y)
        for (int x = lo[0]; x < hi[0]; ++x) {
          idx[0] = x;
          idx[1] = y;
          idx[2] = z;
          for (int n = 0; n < nargs; ++n) {
            if (args[n].kind == 0)
              p[n] = args[n].dat->data + (size_t)args[n].dat->elem * osb_offset(args[n].dat, x, y, z);
            else if (args[n].kind == 1)
              p[n] = args[n].gbl;
            else
              p[n] = (void *)idx;
          }
          osb_invoke(kernel, p, std::index_sequence_for<P...>{});
        }
  }
}

/* ops_NaNcheck: stop the run when a double dat holds a NaN anywhere (the generated code calls it every
 * few iterations when the script asks for print_iteration_ops(NaN_check=...)) */
static inline void ops_NaNcheck(ops_dat d) {
  const size_t n = (size_t)d->pad[0] * d->pad[1] * d->pad[2];
  const double *v = (const double *)d->data;
  for (size_t k = 0; k < n; ++k)
    if (v[k] != v[k]) {
      fprintf(stderr, "ops_NaNcheck: NaN in a dat\n");
      exit(1);
    }
}

/* ---------- halos ---------- */
static inline ops_halo ops_decl_halo(ops_dat from, ops_dat to, int *iter, int *from_base, int *to_base, int *from_dir,
                                     int *to_dir) {
  ops_halo h = (ops_halo)calloc(1, sizeof(*h));
  h->from = from;
  h->to = to;
  int nd = 3;
  for (int a = 0; a < 3; ++a) {
    h->iter[a] = 1;
    h->from_base[a] = h->to_base[a] = 0;
    h->from_dir[a] = h->to_dir[a] = a + 1;
  }
#if defined(OPS_2D)
  nd = 2;
#endif
  for (int a = 0; a < nd; ++a) {
    h->iter[a] = iter[a];
    h->from_base[a] = from_base[a];
    h->to_base[a] = to_base[a];
    h->from_dir[a] = from_dir[a];
    h->to_dir[a] = to_dir[a];
  }
  return h;
}

static inline ops_halo_group ops_decl_halo_group(int n, ops_halo *h) {
  ops_halo_group g = (ops_halo_group)calloc(1, sizeof(*g));
  g->n = n;
  g->h = (ops_halo *)calloc(n, sizeof(ops_halo));
  memcpy(g->h, h, n * sizeof(ops_halo));
  return g;
}

static inline void osb_halo_coord(const int *base, const int *dir, const int *iter, const int *it, int *c) {
  /* dir[d] = +-(axis+1): iteration axis d walks along data axis |dir[d]|-1, reversed if negative */
  for (int a = 0; a < 3; ++a) c[a] = base[a];
  for (int d = 0; d < 3; ++d) {
    int ax = abs(dir[d]) - 1;
    c[ax] = base[ax] + (dir[d] > 0 ? it[d] : iter[d] - 1 - it[d]);
  }
}

static inline void ops_halo_transfer(ops_halo_group g) {
  for (int n = 0; n < g->n; ++n) {
    ops_halo h = g->h[n];
    int it[3], fc[3], tc[3];
    for (it[2] = 0; it[2] < h->iter[2]; ++it[2])
      for (it[1] = 0; it[1] < h->iter[1]; ++it[1])
        for (it[0] = 0; it[0] < h->iter[0]; ++it[0]) {
          osb_halo_coord(h->from_base, h->from_dir, h->iter, it, fc);
          osb_halo_coord(h->to_base, h->to_dir, h->iter, it, tc);
          memcpy(h->to->data + (size_t)h->to->elem * osb_offset(h->to, tc[0], tc[1], tc[2]),
                 h->from->data + (size_t)h->from->elem * osb_offset(h->from, fc[0], fc[1], fc[2]), h->from->elem);
        }
  }
}

/* ---------- output: raw dumps in place of HDF5 ---------- */
static inline void ops_fetch_block_hdf5_file(ops_block b, const char *f) { (void)b; (void)f; }
static inline void ops_fetch_dat_hdf5_file(ops_dat d, const char *fname) {
  const char *dir = getenv("OSB_DUMP_DIR");
  if (!dir) return;
  char stem[256];
  snprintf(stem, sizeof stem, "%s", fname);
  char *dot = strstr(stem, ".h5");
  if (dot) *dot = 0;
  char path[1024];
  snprintf(path, sizeof path, "%s/%s.%s.bin", dir, stem, d->name);
  FILE *f = fopen(path, "wb");
  if (!f) return;
  int hdr[12] = {d->elem, d->size[0], d->size[1], d->size[2], d->d_m[0], d->d_m[1],
                 d->d_m[2], d->d_p[0], d->d_p[1], d->d_p[2], 0, 0};
  fwrite(hdr, sizeof(int), 12, f);
  fwrite(d->data, (size_t)d->elem, (size_t)d->pad[0] * d->pad[1] * d->pad[2], f);
  fclose(f);
}

#endif
