// Gradient paths resident on the GPU: the zero-flux surface search of
// critic2's INTEGRALS, bisect_msurface (src/bisect@proc.f90:1208-1446) and
// lim_surf (:1039-1126) for one (attractor, angular node) per block at a
// time, and makegraph's single paths (src/autocp@proc.f90:2116-2268), one
// per block, both over field%gradient's paths (gpath.h).
//
// Thread 0 of a block runs the ray's state machine (bracket tries, the
// bisection, beta-sphere restarts, and the path's Bogacki-Shampine steps);
// whenever the machine needs the field at a point, the whole block evaluates
// it: the FP64 per-point evaluator's arithmetic (k_eval_fp64_pt: primitives
// within critic2's cutoffs compacted in primitive order by ballots, one MO
// per thread, a fixed-order block reduction), restricted to the density and
// its gradient, at the point wrapped into the molecular cell, with the EDF
// core and the nucleus rule (|grad| := 0 within 1e-5 bohr of a nucleus).
// The values are the ones the batched host-driven tracer gets from the
// per-point kernel, so the decisions are the same; no host round trip is
// left between the steps.  Every loop is bounded: a path by its step
// limit, a ray by its evaluation limit (kMaxRayEvals) and its restarts.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include <math_constants.h>

#include "c2g_internal.h"
#include "gpath.h"
#include "gto.cuh"
#include "k_gpath.h"
#include "points.cuh"

namespace c2g {
namespace {

using namespace gpath;

constexpr double kBsRNearNuc = 3.1622776601683794e-3;  // bs_rnearnuc = sqrt(1e-5)
constexpr int kNTries = 7;
constexpr int kMaxRestart = 16;           // beta-sphere restarts per ray
constexpr long kMaxRayEvals = 1L << 22;   // field evaluations per ray

// One ray's state (thread 0 of its block).
struct RayState {
  double xa[3], u[3];
  int typ;
  int phase, k;  // 0 inner tries, 1 outer tries, 2 bisection, 3 done
  double rin[kNTries], rout[kNTries];
  double riaprox, raprox, rother;
  double xin[3], xfin[3], xi[3], xf[3], xmed[3];
  double rlim;
  int npath, nwarn, nrestart, err;
  long nevals;
  bool tracing, own_rb;
  Path path;
};

struct Search {
  PathGeom g;
  BasinDev b;
  double *rb;  // this block's beta radii (valid once own_rb)
};

__device__ void sort7(double (&v)[kNTries]) {
  for (int i = 1; i < kNTries; i++) {
    const double t = v[i];
    int j = i - 1;
    while (j >= 0 && v[j] > t) v[j + 1] = v[j], j--;
    v[j + 1] = t;
  }
}

__device__ double dist3(const double *a, const double *b) {
  const double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
  return sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

__device__ void trace_from(RayState &y, const double x[3]) {
  start_path(y.path, x, 1);
  y.tracing = true;
  y.npath++;
}

__device__ void point_at(const RayState &y, double r, double x[3]) {
  for (int j = 0; j < 3; j++) x[j] = y.xa[j] + r * y.u[j];
}

__device__ void begin_bisection(RayState &y, const Search &s);

__device__ void begin_outer(RayState &y, const Search &s);

// inner tries, largest radius first (:1309-1330)
__device__ void next_inner(RayState &y, const Search &s) {
  if (y.k < 0) {
    begin_outer(y, s);
    return;
  }
  y.riaprox = y.rin[y.k];
  double x[3];
  point_at(y, y.riaprox, x);
  trace_from(y, x);
}

// outer tries, smallest first, each better than a bisection step (:1352-1394)
__device__ void next_outer(RayState &y, const Search &s) {
  while (y.k < kNTries) {
    y.raprox = y.rout[y.k];
    if (y.raprox > (y.rother + y.riaprox) / 2.0 || y.raprox < y.riaprox) {
      y.raprox = y.rother;
      y.k++;
      continue;
    }
    double x[3];
    point_at(y, y.raprox, x);
    trace_from(y, x);
    return;
  }
  begin_bisection(y, s);
}

__device__ void begin_outer(RayState &y, const Search &s) {
  y.phase = 1;
  y.k = 0;
  y.raprox = y.rother;
  next_outer(y, s);
}

__device__ void next_bisection(RayState &y, const Search &s);

__device__ void begin_bisection(RayState &y, const Search &s) {
  if (y.raprox == DBL_MAX || y.riaprox == 0.0) {
    y.err = 1;  // "Can not find ray limits"
    y.phase = 3;
    return;
  }
  point_at(y, y.riaprox, y.xin);
  point_at(y, y.raprox, y.xfin);
  y.phase = 2;
  // lim_surf from its label 1
  for (int j = 0; j < 3; j++) y.xi[j] = y.xin[j], y.xf[j] = y.xfin[j];
  next_bisection(y, s);
}

__device__ void next_bisection(RayState &y, const Search &s) {
  for (;;) {
    for (int j = 0; j < 3; j++) y.xmed[j] = 0.5 * (y.xi[j] + y.xf[j]);
    if (dist3(y.xi, y.xf) > s.b.prec) {
      trace_from(y, y.xmed);
      return;
    }
    // a surface point in the beta sphere of a CP of the attractor's type
    // shrinks that sphere (the ray's own copy) and restarts from the
    // bracket (:1110-1124)
    bool again = false;
    for (int i = 0; i < s.b.ncp && !again; i++) {
      if (s.b.cptyp[i] != y.typ) continue;
      const double rbi = y.own_rb ? s.rb[i] : kRBeta;
      if (dist3(s.b.cpx + 3 * i, y.xmed) > rbi) continue;
      if (y.nrestart >= kMaxRestart) {
        y.err = 2;
        y.phase = 3;
        return;
      }
      if (!y.own_rb) {
        for (int c = 0; c < s.b.ncp; c++) s.rb[c] = kRBeta;
        y.own_rb = true;
      }
      s.rb[i] *= 0.75;
      y.nrestart++;
      again = true;
    }
    if (!again) break;
    for (int j = 0; j < 3; j++) y.xi[j] = y.xin[j], y.xf[j] = y.xfin[j];
  }
  y.rlim = dist3(y.xmed, y.xa);
  y.phase = 3;
}

__device__ double nearest_attractor(const Search &s, const double *x) {
  double best = DBL_MAX;
  for (int i = 0; i < s.b.ncp; i++)
    if (s.b.cptyp[i] == -3) best = fmin(best, dist3(s.b.cpx + 3 * i, x));
  return best;
}

__device__ void path_done(RayState &y, const Search &s) {
  const Path &p = y.path;
  if (p.ier > 0) y.nwarn++;
  const double d = dist3(p.x, y.xa);
  if (y.phase == 0) {
    if (p.ier != 3 && d <= kBsRNearNuc) {
      begin_outer(y, s);
      return;
    }
    y.rother = fmin(y.rother, y.rin[y.k]);
    y.k--;
    next_inner(y, s);
  } else if (y.phase == 1) {
    if (p.ier != 3 && d > kBsRNearNuc) {
      begin_bisection(y, s);
      return;
    }
    if (y.raprox > y.riaprox) y.riaprox = y.raprox;
    y.raprox = y.rother;
    y.k++;
    next_outer(y, s);
  } else {
    bool inside;
    if (p.ier <= 0) inside = d <= kBsRNearNuc;
    else if (p.ier == 3) inside = false;
    else inside = nearest_attractor(s, p.x) <= kBsRNearNuc;
    for (int j = 0; j < 3; j++) (inside ? y.xi[j] : y.xf[j]) = y.xmed[j];
    next_bisection(y, s);
  }
}

__device__ void ray_init(RayState &y, const Search &s, int att, int node) {
  const BasinDev &b = s.b;
  for (int j = 0; j < 3; j++) y.xa[j] = b.att_x[3 * att + j], y.u[j] = b.ray_u[3 * node + j];
  y.typ = b.att_typ[att];
  const double rmin = b.att_rmin[att], rms = b.att_rminsame[att];
  const double ti[kNTries] = {2e-5, 0.9 * rmin, 0.99 * rmin, 0.0, 0.0, 0.0, 0.0};
  const double to[kNTries] = {b.amin, 0.99 * rms, 0.75 * rms, b.amax, b.amax, b.amax, b.amax};
  for (int i = 0; i < kNTries; i++) y.rin[i] = ti[i], y.rout[i] = to[i];
  sort7(y.rin);
  sort7(y.rout);
  y.riaprox = 0.0, y.raprox = DBL_MAX, y.rother = DBL_MAX;
  y.rlim = -1.0;
  y.npath = y.nwarn = y.nrestart = y.err = 0;
  y.nevals = 0;
  y.tracing = false, y.own_rb = false;
  y.phase = 0;
  y.k = kNTries - 1;
  next_inner(y, s);
}

// Advances the ray until it needs the field at a point (true, x) or is done.
// pre: the beta-sphere candidate for the path's position, or null.
__device__ bool ray_request(RayState &y, const Search &s, double x[3], const Nearest *pre) {
  while (y.tracing) {
    Path &p = y.path;
    if (p.stage == 0) {
      if (head(p, s.g, s.b.ncp, s.b.cpx, s.b.cptyp, y.own_rb ? s.rb : nullptr, pre)) {
        request_stage1(p);
        break;
      }
      p.done = true;
    }
    if (p.done) {
      y.tracing = false;
      if (p.incstep) p.nstep++;
      path_done(y, s);
      continue;
    }
    break;
  }
  if (!y.tracing) return false;
  if (y.nevals >= kMaxRayEvals) {
    y.err = 3;
    y.tracing = false;
    y.phase = 3;
    return false;
  }
  for (int j = 0; j < 3; j++) x[j] = y.path.req[j];
  return true;
}

// The block's evaluation of rho and its gradient at x (wrapped into the
// cell), into q[0..3] of thread 0.  Per chunk of 256 primitives (atom-major,
// so they span at most 256 atoms unless atoms without primitives lie
// between): the offsets to the chunk's atoms once per atom, the range tests
// of all primitives, those in range compacted in primitive order, their chi
// (the FP64 exponential and the Cartesian factors) on the first threads,
// then the contraction.  s_d holds the per-atom offsets and squared
// distances (or, for a chunk spanning more atoms, the compacted primitives').
template <int MPT>
__device__ void eval_block(const DevWfn &w, const double (&xin)[3], double *s_chi, double *s_d, int *s_k,
                           int *s_wn, double *s_red, double (&q)[4]) {
  const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
  double x[3] = {xin[0], xin[1], xin[2]};
  wrap_cell(w, x);
  double r[4] = {0.0, 0.0, 0.0, 0.0};
  // MOs in chunks of 256 MPT (one chunk up to 1024 MOs; above that the
  // primitives are evaluated again for each chunk)
  for (int mo0 = 0; mo0 < w.nmo; mo0 += 256 * MPT) {
    double acc[MPT][4];
#pragma unroll
    for (int m = 0; m < MPT; m++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[m][c] = 0.0;
    for (int k0 = 0; k0 < w.npri; k0 += 256) {
      const int ip = k0 + tid;
      const int a0 = w.prim[k0].atom, a1 = w.prim[min(k0 + 255, w.npri - 1)].atom;
      const bool per_atom = a1 - a0 < 256;  // uniform over the block
      if (per_atom && tid <= a1 - a0) {
        const double4 A = w.atoms[a0 + tid];
        const double dx = x[0] - A.x, dy = x[1] - A.y, dz = x[2] - A.z;
        s_d[4 * tid] = dx, s_d[4 * tid + 1] = dy, s_d[4 * tid + 2] = dz;
        const double dd = dx * dx + dy * dy + dz * dz;
        // beyond the atom's cutoff: marked by a negative squared distance
        s_d[4 * tid + 3] = dd <= A.w ? dd : -1.0;
      }
      if (per_atom) __syncthreads();
      double dx = 0.0, dy = 0.0, dz = 0.0, dd = 0.0;
      bool in = false;
      if (ip < w.npri) {
        const PrimF64 pr = w.prim[ip];
        if (per_atom) {
          dd = s_d[4 * (pr.atom - a0) + 3];
          in = dd >= 0.0 && within_dran(dd, pr.dran);
        } else {
          const double4 A = w.atoms[pr.atom];
          dx = x[0] - A.x, dy = x[1] - A.y, dz = x[2] - A.z;
          dd = dx * dx + dy * dy + dz * dz;
          in = dd <= A.w && within_dran(dd, pr.dran);
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, in);
      if (lane == 0) s_wn[wp] = __popc(bal);
      __syncthreads();
      int base = 0, nact = 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        base += i < wp ? s_wn[i] : 0;
        nact += s_wn[i];
      }
      const int slot = base + __popc(bal & ((1u << lane) - 1u));
      if (in) s_k[slot] = ip;
      if (!per_atom) {
        if (in) s_d[4 * slot] = dx, s_d[4 * slot + 1] = dy, s_d[4 * slot + 2] = dz, s_d[4 * slot + 3] = dd;
      }
      __syncthreads();
      if (tid < nact) {
        const PrimF64 pr = w.prim[s_k[tid]];
        const double *o = s_d + 4 * (per_atom ? pr.atom - a0 : tid);
        const double dist = sqrt(o[3]);
        double chi[4];
        chi_eval<4>(o[0], o[1], o[2], pr.e, pr.lpack, exp(-pr.e * (dist * dist)), chi);
#pragma unroll
        for (int c = 0; c < 4; c++) s_chi[tid * 4 + c] = chi[c];
      }
      __syncthreads();
      // threads without an MO skip the contraction (their sums stay zero)
#pragma unroll 2
      for (int j = 0; j < (mo0 + tid < w.nmo ? nact : 0); j++) {
        const double *crow = w.cmo + (size_t)s_k[j] * w.nmo_pad;
        double ch[4];
#pragma unroll
        for (int c = 0; c < 4; c++) ch[c] = s_chi[j * 4 + c];
#pragma unroll
        for (int m = 0; m < MPT; m++) {
          const int mo = mo0 + tid + 256 * m;
          const double cm = mo < w.nmo ? __ldg(crow + mo) : 0.0;
#pragma unroll
          for (int c = 0; c < 4; c++) acc[m][c] = fma(cm, ch[c], acc[m][c]);
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < MPT; m++) {
      const int mo = mo0 + tid + 256 * m;
      const double o = mo < w.nmo ? w.occ[mo] : 0.0;
      const double p0 = acc[m][0];
      r[0] += o * p0 * p0;
      r[1] += 2.0 * o * p0 * acc[m][1];
      r[2] += 2.0 * o * p0 * acc[m][2];
      r[3] += 2.0 * o * p0 * acc[m][3];
    }
  }
#pragma unroll
  for (int c = 0; c < 4; c++)
    for (int off = 16; off; off >>= 1) r[c] += __shfl_xor_sync(0xffffffffu, r[c], off);
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < 4; c++) s_red[wp * 4 + c] = r[c];
  __syncthreads();
  if (wp == 0) {
    double core_c = 0.0;
    if (w.nedf) {
      double core[10];
      edf_core_warp(w, x, core);
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (c == lane) core_c = core[c];
    }
    if (lane < 4) {
      double sum = 0.0;
      for (int i = 0; i < 8; i++) sum += s_red[i * 4 + lane];
      s_red[32 + lane] = sum + core_c;
    }
  }
  __syncthreads();
  if (wp == 0) {
    // the nucleus rule at the wrapped point, the nuclei spread over warp 0
    // (the square root only where the squared distance can pass)
    bool near = false;
    for (int a = lane; a < w.natom; a += 32) {
      const double4 A = w.atoms[a];
      const double dx = x[0] - A.x, dy = x[1] - A.y, dz = x[2] - A.z;
      const double dd = dx * dx + dy * dy + dz * dz;
      if (dd <= 1.000001e-10 && sqrt(dd) <= 1e-5) near = true;
    }
    near = __any_sync(0xffffffffu, near);
    if (lane == 0) {
      for (int c = 0; c < 4; c++) q[c] = s_red[32 + c];
      if (near) q[1] = q[2] = q[3] = 0.0;
    }
  }
  __syncthreads();
}

// Lexicographic minimum of (v, i) over the warp: the smallest value, and of
// equal values the smallest index.
__device__ void warp_min_first(double &v, int &i) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, off);
    const int oi = __shfl_xor_sync(0xffffffffu, i, off);
    if (ov < v || (ov == v && oi < i)) v = ov, i = oi;
  }
}

// nearest_serial by one warp (all 32 lanes, the same x): each lane scans
// every 32nd nucleus and CP keeping its first minimum, and the lanes' minima
// are merged by (value, index), so the candidate is the serial scan's.
__device__ void nearest_warp(const double x[3], int iup, const PathGeom &w, int ncp, const double *cpx,
                             const int *cptyp, Nearest &n) {
  const int lane = threadIdx.x & 31;
  double sph2 = 1e60;
  int idnuc = 0;
  for (int a = lane; a < w.natom; a += 32) {
    const double dx = x[0] - w.xyz[3 * a], dy = x[1] - w.xyz[3 * a + 1], dz = x[2] - w.xyz[3 * a + 2];
    const double d2a = dx * dx + dy * dy + dz * dz;
    if (d2a < sph2) sph2 = d2a, idnuc = a;
  }
  warp_min_first(sph2, idnuc);
  double c2 = CUDART_INF;
  int ci = INT_MAX;
  for (int i = lane; i < ncp; i += 32) {
    if (!((cptyp[i] == -3 && iup == 1) || (cptyp[i] == 3 && iup == -1))) continue;
    const double dx = x[0] - cpx[3 * i], dy = x[1] - cpx[3 * i + 1], dz = x[2] - cpx[3 * i + 2];
    const double d2i = dx * dx + dy * dy + dz * dz;
    if (d2i < c2) c2 = d2i, ci = i;
  }
  warp_min_first(c2, ci);
  for (int j = 0; j < 3; j++) n.x[j] = x[j];
  n.have = n.isnuc = false;
  n.idcp = -1;
  n.cp2 = 1e30;
  if (iup == 1 && w.z[idnuc] != 1) n.have = n.isnuc = true, n.idcp = idnuc, n.cp2 = sph2;
  if (c2 < n.cp2) n.have = true, n.isnuc = false, n.idcp = ci, n.cp2 = c2;
}

// Three blocks per SM (at most 85 registers a thread): the chain is
// latency-bound on small molecules, FP64-bound on large ones.
template <int MPT>
__global__ void __launch_bounds__(256, 3) k_basin_rays(DevWfn w, PathGeom g, BasinDev b) {
  __shared__ double s_chi[256 * 4];
  __shared__ double s_d[256 * 4];
  __shared__ int s_k[256];
  __shared__ int s_wn[8];
  __shared__ double s_red[8 * 4 + 4];
  __shared__ double s_x[3];
  __shared__ int s_more;
  // the ray's state, used by thread 0 only (set by ray_init)
  __shared__ __align__(16) unsigned char s_ray[sizeof(RayState)];
  RayState &y = *reinterpret_cast<RayState *>(s_ray);
  __shared__ long s_next;
  const Search s{g, b, b.rbeta_scratch + (size_t)blockIdx.x * (b.ncp > 0 ? b.ncp : 1)};
  const long nr = (long)b.natt * b.nray;
  // rays are handed out in order by a counter: their costs differ severalfold
  for (;;) {
    if (threadIdx.x == 0) s_next = (long)atomicAdd(b.ray_next, 1ull);
    __syncthreads();
    const long ray = s_next;
    if (ray >= nr) break;
    if (threadIdx.x == 0) ray_init(y, s, (int)(ray / b.nray), (int)(ray % b.nray));
    for (;;) {
      // a path about to take a step: its beta-sphere candidate by warp 0
      Nearest nc;
      bool pre = false;
      if (threadIdx.x < 32) {
        __syncwarp();
        pre = y.tracing && y.path.stage == 0;
        if (pre) nearest_warp(y.path.x, y.path.iup, g, b.ncp, b.cpx, b.cptyp, nc);
      }
      if (threadIdx.x == 0) {
        double x[3];
        s_more = ray_request(y, s, x, pre ? &nc : nullptr) ? 1 : 0;
        if (s_more) s_x[0] = x[0], s_x[1] = x[1], s_x[2] = x[2];
      }
      __syncthreads();
      if (!s_more) break;
      const double xx[3] = {s_x[0], s_x[1], s_x[2]};
      double q[4];
      eval_block<MPT>(w, xx, s_chi, s_d, s_k, s_wn, s_red, q);
      if (threadIdx.x == 0) {
        y.nevals++;
        double rec[4] = {q[0], q[1], q[2], q[3]};
        if (y.path.stage == -1) take_start(y.path, rec);
        else advance(y.path, rec);
      }
    }
    if (threadIdx.x == 0) {
      b.rsurf[ray] = y.rlim;
      b.ray_npath[ray] = y.npath;
      b.ray_nwarn[ray] = y.nwarn;
      b.ray_nrestart[ray] = y.nrestart;
      b.ray_err[ray] = y.err;
      b.ray_nevals[ray] = y.nevals;
    }
    __syncthreads();
  }
}

// Single gradient paths (makegraph's), one block per path at a time: thread
// 0 steps the path, the block evaluates the field it asks for.
template <int MPT>
__global__ void __launch_bounds__(256, 3) k_trace_paths(DevWfn w, PathGeom g, PathsDev d) {
  __shared__ double s_chi[256 * 4];
  __shared__ double s_d[256 * 4];
  __shared__ int s_k[256];
  __shared__ int s_wn[8];
  __shared__ double s_red[8 * 4 + 4];
  __shared__ double s_x[3];
  __shared__ int s_more;
  __shared__ __align__(16) unsigned char s_path[sizeof(Path)];
  Path &p = *reinterpret_cast<Path *>(s_path);
  for (int i = blockIdx.x; i < d.n; i += gridDim.x) {
    long nev = 0;
    if (threadIdx.x == 0) start_path(p, d.x0 + 3 * i, d.iup[i], d.pathini + 3 * i);
    for (;;) {
      // a path about to take a step: its beta-sphere candidate by warp 0
      Nearest nc;
      bool pre = false;
      if (threadIdx.x < 32) {
        __syncwarp();
        pre = !p.done && p.stage == 0;
        if (pre) nearest_warp(p.x, p.iup, g, d.ncp, d.cpx, d.cptyp, nc);
      }
      if (threadIdx.x == 0) {
        bool need = p.stage == -1;
        while (!need && !p.done) {
          if (p.stage == 0 && !head(p, g, d.ncp, d.cpx, d.cptyp, nullptr, pre ? &nc : nullptr)) {
            p.done = true;
            break;
          }
          if (p.stage == 0) request_stage1(p);
          need = true;
        }
        if (need && nev >= kMaxRayEvals) need = false, p.ier = 2, p.done = true;
        s_more = need ? 1 : 0;
        if (need) s_x[0] = p.req[0], s_x[1] = p.req[1], s_x[2] = p.req[2];
      }
      __syncthreads();
      if (!s_more) break;
      const double xx[3] = {s_x[0], s_x[1], s_x[2]};
      double q[4];
      eval_block<MPT>(w, xx, s_chi, s_d, s_k, s_wn, s_red, q);
      if (threadIdx.x == 0) {
        nev++;
        if (p.stage == -1) take_start(p, q);
        else advance(p, q);
      }
    }
    if (threadIdx.x == 0) {
      if (p.incstep) p.nstep++;
      for (int j = 0; j < 3; j++) d.xend[3 * i + j] = p.x[j];
      d.ier[i] = p.ier;
      d.nstep[i] = p.nstep;
      d.plen[i] = p.plen;
      d.nevals[i] = nev;
    }
    __syncthreads();
  }
}

}  // namespace

void launch_trace_paths(const DevWfn &w, const PathGeom &g, const PathsDev &d, int grid, cudaStream_t st) {
  if (w.nmo <= 256) k_trace_paths<1><<<grid, 256, 0, st>>>(w, g, d);
  else if (w.nmo <= 512) k_trace_paths<2><<<grid, 256, 0, st>>>(w, g, d);
  else k_trace_paths<4><<<grid, 256, 0, st>>>(w, g, d);
  C2G_CUDA(cudaGetLastError());
}

void launch_basin_rays(const DevWfn &w, const PathGeom &g, const BasinDev &b, int grid, cudaStream_t st) {
  if (w.nmo <= 256) k_basin_rays<1><<<grid, 256, 0, st>>>(w, g, b);
  else if (w.nmo <= 512) k_basin_rays<2><<<grid, 256, 0, st>>>(w, g, b);
  else k_basin_rays<4><<<grid, 256, 0, st>>>(w, g, b);
  C2G_CUDA(cudaGetLastError());
}

}  // namespace c2g
