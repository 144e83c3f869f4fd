// Point sources shared by the evaluator kernels: a tile is 32 points, taken
// from a grid (4 j x 8 k points on one i plane), a point list, a list of
// indices into a point array, or a list of linear grid indices.  Every
// source wraps points into the molecular cell as field%grd does for
// molecules (src/fieldmod@proc.f90:921-943, flooreps = 1e-4).
#pragma once

#include "c2g_internal.h"

namespace c2g {

constexpr int kTilePoints = 32;

__device__ __forceinline__ void wrap_cell(const DevWfn &w, double (&x)[3]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    // within [-5e-5, 1 + 5e-5] cell lengths of the cell the quotient below
    // is inside its bounds by far, and the point stays: no division
    const double d = x[j] - w.cell_lo[j];
    if (d >= -5e-5 * w.cell_aa[j] && d <= (1.0 + 5e-5) * w.cell_aa[j]) continue;
    double f = d / w.cell_aa[j];
    if (f < -1e-4 || f > 1.0 + 1e-4) {
      f -= floor(f);
      x[j] = w.cell_lo[j] + f * w.cell_aa[j];
    }
  }
}

// ------------------------------------------------------------ point sources
// Each source also reports how many of the launched tiles can hold points
// (tiles(n)); list sources whose length lives on the device read it there.
struct ListSrc {
  const double *xyz;
  int n;
  bool wrap = true;  // false: the points as given (grd with periodic = .false.)
  __device__ int tiles(int nt) const { return nt; }
  __device__ bool point(const DevWfn &w, int tile, int p, double (&x)[3], long &idx) const {
    const long i = (long)tile * kTilePoints + p;
    idx = i;
    if (i >= n) return false;
    x[0] = xyz[3 * i];
    x[1] = xyz[3 * i + 1];
    x[2] = xyz[3 * i + 2];
    if (wrap) wrap_cell(w, x);
    return true;
  }
};

__device__ __forceinline__ void grid_xyz(const GridSpec &g, int i, int j, int k, double (&x)[3]) {
#pragma unroll
  for (int c = 0; c < 3; c++) x[c] = g.x0[c] + i * g.xmat[c] + j * g.xmat[3 + c] + k * g.xmat[6 + c];
}

// tiles of 4 (j) x 8 (k) points on one i plane
struct GridSrc {
  GridSpec g;
  int ntj, ntk;
  __device__ int tiles(int nt) const { return nt; }
  __device__ bool point(const DevWfn &w, int tile, int p, double (&x)[3], long &idx) const {
    const int i = tile / (ntj * ntk);
    const int r = tile - i * ntj * ntk;
    const int j = (r / ntk) * 4 + (p >> 3);
    const int k = (r % ntk) * 8 + (p & 7);
    idx = -1;
    if (j >= g.nstep[1] || k >= g.nstep[2]) return false;
    idx = ((long)i * g.nstep[1] + j) * g.nstep[2] + k;
    grid_xyz(g, i, j, k, x);
    wrap_cell(w, x);
    return true;
  }
};

// a device list of linear grid indices (k fastest); count read on device
struct GridListSrc {
  GridSpec g;
  const int *list;
  const int *count;
  __device__ int tiles(int nt) const { return min(nt, (*count + kTilePoints - 1) / kTilePoints); }
  __device__ bool point(const DevWfn &w, int tile, int p, double (&x)[3], long &idx) const {
    const long t = (long)tile * kTilePoints + p;
    idx = -1;
    if (t >= *count) return false;
    const long li = list[t];
    const int k = (int)(li % g.nstep[2]);
    const int j = (int)((li / g.nstep[2]) % g.nstep[1]);
    const int i = (int)(li / ((long)g.nstep[2] * g.nstep[1]));
    idx = li;
    grid_xyz(g, i, j, k, x);
    wrap_cell(w, x);
    return true;
  }
};

// points x(3, idx[t]) for t < *count (the live seeds of a Newton batch)
struct IndexSrc {
  const double *x;
  const int *idx;
  const int *count;
  __device__ int tiles(int nt) const { return min(nt, (*count + kTilePoints - 1) / kTilePoints); }
  __device__ bool point(const DevWfn &w, int tile, int p, double (&xx)[3], long &out) const {
    const long t = (long)tile * kTilePoints + p;
    out = t;
    if (t >= *count) return false;
    const long i = idx[t];
    xx[0] = x[3 * i];
    xx[1] = x[3 * i + 1];
    xx[2] = x[3 * i + 2];
    wrap_cell(w, xx);
    return true;
  }
};


}  // namespace c2g
