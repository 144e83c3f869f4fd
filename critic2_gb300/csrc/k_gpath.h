// Device-resident gradient paths (k_gpath.cu): the basin-integral surface
// search and makegraph's single paths.
#pragma once

#include <cuda_runtime.h>

#include "c2g_internal.h"
#include "gpath.h"

namespace c2g {

// One search: the CP list, the attractors and the rays (all device arrays),
// and the per-ray outputs.  Ray r = attractor r / nray, node r % nray.
struct BasinDev {
  int ncp;
  const double *cpx;  // 3 * ncp
  const int *cptyp;
  double prec, amin, amax;  // IAS precision; smallest and largest cell lengths
  int natt, nray;
  const double *att_x;  // 3 * natt
  const int *att_typ;
  const double *att_rmin, *att_rminsame;
  const double *ray_u;      // 3 * nray unit directions
  double *rbeta_scratch;    // grid * ncp: the beta radii of a block's current ray
  double *rsurf;            // natt * nray
  int *ray_npath, *ray_nwarn, *ray_nrestart, *ray_err;  // err: 1 no bracket, 2 restarts, 3 evaluations
  long *ray_nevals;
  unsigned long long *ray_next;  // the next ray to hand out (zero at launch)
};

// n single paths from x0 (3 * n) going iup (+1 up, -1 down), path length
// counted from pathini, with the default beta spheres; end point, ier,
// step count, length and evaluations per path.
struct PathsDev {
  int n;
  const double *x0, *pathini;
  const int *iup;
  int ncp;
  const double *cpx;
  const int *cptyp;
  double *xend, *plen;
  int *ier, *nstep;
  long *nevals;
};

void launch_trace_paths(const DevWfn &w, const gpath::PathGeom &g, const PathsDev &d, int grid, cudaStream_t st);

// Every ray of the search, one block of 256 threads per ray at a time.
void launch_basin_rays(const DevWfn &w, const gpath::PathGeom &g, const BasinDev &b, int grid, cudaStream_t st);

}  // namespace c2g
