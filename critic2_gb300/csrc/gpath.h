// Gradient paths of a molecular wavefunction field: field%gradient
// (src/fieldmod@proc.f90:2500-2732) with critic2's default navigation: the
// Bogacki-Shampine 2(3) stepper (:2860-2890) inside adaptive_stepper
// (:2737-2830), step 0.3, maxerr 1e-4, gradeps 1e-7, beta spheres 0.1
// (src/global@proc.F90:858-861, src/global.f90:41).
//
// A path is a small state machine: head() does the part of a step before
// the Runge-Kutta stages (path length, beta spheres, molecular cell, new
// CP), each stage asks for the field at one point (req) and advance() takes
// it, in the reference's order of operations, so the decisions are the ones
// a serial trace makes with the same field values.  The functions compile
// for host and device: the device kernels (k_gpath.cu) run whole paths
// without a host round trip.  BatchGrd evaluates the field at a batch of
// host points (the FP64 per-point kernel, then the nucleus rule).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "c2g_internal.h"

#if defined(__CUDACC__)
#define C2G_HD __host__ __device__
#else
#define C2G_HD
#endif

namespace c2g {
namespace gpath {

// What a path needs of the molecule (host or device arrays): the nuclei,
// their atomic numbers and the molecular cell.
struct PathGeom {
  int natom;
  const double *xyz;  // 3 * natom
  const int *z;
  double cell_lo[3], cell_aa[3], molborder[3];
};

inline PathGeom host_geom(const HostWfn &w) {
  PathGeom g;
  g.natom = w.natom;
  g.xyz = w.xyz.data();
  g.z = w.z.data();
  for (int j = 0; j < 3; j++) g.cell_lo[j] = w.cell_lo[j], g.cell_aa[j] = w.cell_aa[j], g.molborder[j] = w.molborder[j];
  return g;
}

constexpr double kNavStep = 0.3, kNavMaxErr = 1e-4, kNavGradEps = 1e-7, kRBeta = 0.1;
constexpr double kVSmall = 1e-80, kMinStep = 1e-12, kHFirst = 0.01;
constexpr int kMHist = 5;

// field%grd (value, gradient, Hessian) at a batch of host points: FP64
// per-point kernel, then the nucleus rule (|grad| := 0 within 1e-5 bohr of
// a nucleus, on the wrapped position) on the host.
class BatchGrd {
 public:
  // One staging buffer each way in pinned memory and one stream: a batch is
  // one upload (count + points), the kernel, one download and one sync.
  BatchGrd(Handle &h, int cap) : h_(h), cap_(std::max(cap, 1)) {
    try {
      allocate();
    } catch (...) {
      release();
      throw;
    }
  }
  ~BatchGrd() { release(); }
  BatchGrd(const BatchGrd &) = delete;
  BatchGrd &operator=(const BatchGrd &) = delete;

 private:
  void allocate() {
    C2G_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    C2G_CUDA(cudaMalloc(&d_in_, sizeof(double) * (1 + 3 * (size_t)cap_)));
    C2G_CUDA(cudaMalloc(&d_idx_, sizeof(int) * cap_));
    C2G_CUDA(cudaMalloc(&d_rec_, sizeof(double) * kRecNci * cap_));
    C2G_CUDA(cudaMallocHost(&h_in_, sizeof(double) * (1 + 3 * (size_t)cap_)));
    C2G_CUDA(cudaMallocHost(&h_rec_, sizeof(double) * kRecNci * cap_));
    std::vector<int> iota(cap_);
    std::iota(iota.begin(), iota.end(), 0);
    C2G_CUDA(cudaMemcpy(d_idx_, iota.data(), sizeof(int) * cap_, cudaMemcpyHostToDevice));
  }
  void release() {
    if (st_) cudaStreamSynchronize(st_);
    if (d_in_) cudaFree(d_in_);
    if (d_idx_) cudaFree(d_idx_);
    if (d_rec_) cudaFree(d_rec_);
    if (h_in_) cudaFreeHost(h_in_);
    if (h_rec_) cudaFreeHost(h_rec_);
    if (st_) cudaStreamDestroy(st_);
    st_ = nullptr, d_in_ = d_rec_ = h_in_ = h_rec_ = nullptr, d_idx_ = nullptr;
  }

 public:
  // xyz(3, n) -> rec(10, n) with the nucleus rule applied to the gradient
  const double *eval(const double *xyz, int n) {
    if (n <= 0) return h_rec_;
    if (n > cap_) fail(C2G_ERR_ARG, "gradient-path batch larger than its buffers");
    std::memcpy(h_in_, &n, sizeof(int));
    std::memcpy(h_in_ + 1, xyz, sizeof(double) * 3 * n);
    C2G_CUDA(cudaMemcpyAsync(d_in_, h_in_, sizeof(double) * (1 + 3 * (size_t)n), cudaMemcpyHostToDevice, st_));
    launch_fp64_index(h_.dev, d_in_ + 1, d_idx_, reinterpret_cast<const int *>(d_in_), n, d_rec_, st_);
    C2G_CUDA(cudaMemcpyAsync(h_rec_, d_rec_, sizeof(double) * kRecNci * n, cudaMemcpyDeviceToHost, st_));
    C2G_CUDA(cudaStreamSynchronize(st_));
    evals_ += n;
    launches_++;
    const HostWfn &w = h_.host;
    const auto nucleus_rule = [&](long b, long e) {
      for (long i = b; i < e; i++) {
        double x[3];
        for (int j = 0; j < 3; j++) {
          double fr = (xyz[3 * i + j] - w.cell_lo[j]) / w.cell_aa[j];
          if (fr < -1e-4 || fr > 1.0 + 1e-4) fr -= std::floor(fr);
          x[j] = w.cell_lo[j] + fr * w.cell_aa[j];
        }
        for (int a = 0; a < w.natom; a++) {
          const double dx = x[0] - w.xyz[3 * a], dy = x[1] - w.xyz[3 * a + 1], dz = x[2] - w.xyz[3 * a + 2];
          if (std::sqrt(dx * dx + dy * dy + dz * dz) <= 1e-5) {
            double *q = h_rec_ + (size_t)i * kRecNci;
            q[1] = q[2] = q[3] = 0.0;
            break;
          }
        }
      }
    };
    nucleus_rule(0, n);
    return h_rec_;
  }
  long evals() const { return evals_; }
  long launches() const { return launches_; }

 private:
  Handle &h_;
  int cap_;
  cudaStream_t st_ = nullptr;
  double *d_in_ = nullptr, *d_rec_ = nullptr, *h_in_ = nullptr, *h_rec_ = nullptr;
  int *d_idx_ = nullptr;
  long evals_ = 0, launches_ = 0;
};

// One gradient path (field%gradient's local state).
struct Path {
  double x[3], xlast[3], xlast2[3];
  double h0, hini, plen;
  double scal[kMHist];
  int nhist = 0, iup, nstep = 1, mstep, ier = 0;
  bool incstep = false, done = false, first = true;
  double gf[3] = {0, 0, 0}, gfmod = 0.0;  // field at x
  double grdt[3], ak2[3], ak3[3], xout[3];
  int stage = 0;  // -1 waiting for the field at the start; 0 head of a step; 1-3 the BS stages
  double req[3];  // point whose evaluation this path waits for
};

C2G_HD inline void unit(const double *q, double g[3]) {
  const double m = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int j = 0; j < 3; j++) g[j] = q[1 + j] / (m + kVSmall);
}

// The beta-sphere candidate of head(): the nearest nucleus, then the CPs of
// the kind the path goes to (maxima up, minima down) when nearer, with the
// nucleus as the first candidate if the path goes up and it is not hydrogen.
// Squared distances are compared (the square root of the minimum is the
// same value); ties keep the first candidate.
struct Nearest {
  double x[3];  // the point it was found for
  bool have;    // a candidate exists
  bool isnuc;   // the candidate is nucleus idcp (else CP idcp)
  int idcp;
  double cp2;   // its squared distance
};

C2G_HD inline void nearest_serial(const double x[3], int iup, const PathGeom &w, int ncp, const double *cpx,
                                  const int *cptyp, Nearest &n) {
  int idnuc = 0;
  double sph2 = 1e60;
  for (int a = 0; a < w.natom; a++) {
    const double dx = x[0] - w.xyz[3 * a], dy = x[1] - w.xyz[3 * a + 1], dz = x[2] - w.xyz[3 * a + 2];
    const double d2a = dx * dx + dy * dy + dz * dz;
    if (d2a < sph2) sph2 = d2a, idnuc = a;
  }
  for (int j = 0; j < 3; j++) n.x[j] = x[j];
  n.have = n.isnuc = false;
  n.idcp = -1;
  n.cp2 = 1e30;
  if (iup == 1 && w.z[idnuc] != 1) n.have = n.isnuc = true, n.idcp = idnuc, n.cp2 = sph2;
  for (int i = 0; i < ncp; i++) {
    if (!((cptyp[i] == -3 && iup == 1) || (cptyp[i] == 3 && iup == -1))) continue;
    const double dx = x[0] - cpx[3 * i], dy = x[1] - cpx[3 * i + 1], dz = x[2] - cpx[3 * i + 2];
    const double d2i = dx * dx + dy * dy + dz * dz;
    if (d2i < n.cp2) n.have = true, n.isnuc = false, n.idcp = i, n.cp2 = d2i;
  }
}

// The part of one field%gradient iteration before the step
// (src/fieldmod@proc.f90:2582-2680): path length, beta spheres, molecular
// cell, new CP.  Returns true when the path goes on with a step.  rbeta:
// null for the default sphere (min(Rbetadef, |hini| / 2) = 0.1 bohr), or
// per-CP radii (up2beta; the CP list then starts with the nuclei in atom
// order, so that a nucleus found first is CP idnuc).  pre: the candidate
// already found for the path's position (by a warp on the device), or null.
C2G_HD inline bool head(Path &p, const PathGeom &w, int ncp, const double *cpx, const int *cptyp,
                        const double *rbeta = nullptr, const Nearest *pre = nullptr) {
  if (p.nstep > p.mstep) {
    p.nstep = p.mstep;
    p.ier = 2;
    return false;
  }
  double d2 = 0.0;
  for (int j = 0; j < 3; j++) d2 += (p.x[j] - p.xlast[j]) * (p.x[j] - p.xlast[j]);
  p.plen += sqrt(d2);
  Nearest n;
  if (pre && pre->x[0] == p.x[0] && pre->x[1] == p.x[1] && pre->x[2] == p.x[2]) n = *pre;
  else nearest_serial(p.x, p.iup, w, ncp, cpx, cptyp, n);
  const bool have = n.have;
  const int idcp = n.idcp;
  const double cp2 = n.cp2;
  double xcp[3] = {0, 0, 0};
  if (have)
    for (int j = 0; j < 3; j++) xcp[j] = n.isnuc ? w.xyz[3 * idcp + j] : cpx[3 * idcp + j];
  const double cprad = sqrt(cp2);
  if (have && cprad <= (rbeta ? rbeta[idcp] : kRBeta)) {
    p.incstep = true;
    double e2 = 0.0;
    for (int j = 0; j < 3; j++) e2 += (p.x[j] - xcp[j]) * (p.x[j] - xcp[j]);
    p.plen += sqrt(e2);
    for (int j = 0; j < 3; j++) p.x[j] = xcp[j];
    p.ier = 0;
    return false;
  }
  if (p.iup == -1)
    for (int j = 0; j < 3; j++) {
      const double xf = (p.x[j] - w.cell_lo[j]) / w.cell_aa[j];
      if (xf < w.molborder[j] || xf > 1.0 - w.molborder[j]) {
        p.ier = 3;
        return false;
      }
    }
  if (p.gfmod < kNavGradEps) {
    p.ier = 0;
    return false;
  }
  for (int j = 0; j < 3; j++) p.xlast2[j] = p.xlast[j], p.xlast[j] = p.x[j];
  // adaptive_stepper: the first trial starts from the unit gradient at x
  for (int j = 0; j < 3; j++) p.grdt[j] = p.gf[j] / (p.gfmod + kVSmall);
  p.first = true;
  return true;
}

C2G_HD inline void request_stage1(Path &p) {
  for (int j = 0; j < 3; j++) p.req[j] = p.x[j] + p.h0 * (0.5 * p.grdt[j]);
  p.stage = 1;
}

// After adaptive_stepper (:2672-2690): bounce history and step floor.
C2G_HD inline void after_step(Path &p, bool ok) {
  p.nhist = p.nhist % kMHist + 1;
  double sc = 0.0;
  for (int j = 0; j < 3; j++) sc += (p.xlast[j] - p.xlast2[j]) * (p.x[j] - p.xlast[j]);
  p.scal[p.nhist - 1] = sc;
  bool allneg = true;
  for (int k = 0; k < kMHist; k++) allneg = allneg && p.scal[k] < 0.0;
  ok = ok && !allneg;
  if (!ok || fabs(p.h0) < kMinStep) {
    for (int j = 0; j < 3; j++) p.x[j] = p.xlast[j];
    p.ier = 1;
    p.done = true;
    return;
  }
  p.nstep++;
  p.stage = 0;
}

// One evaluated BS stage of a path.
C2G_HD inline void advance(Path &p, const double *q) {
  if (p.stage == 1) {
    unit(q, p.ak2);
    for (int j = 0; j < 3; j++) p.req[j] = p.x[j] + p.h0 * (0.75 * p.ak2[j]);
    p.stage = 2;
  } else if (p.stage == 2) {
    unit(q, p.ak3);
    for (int j = 0; j < 3; j++)
      p.xout[j] = p.x[j] + p.h0 * (2.0 / 9.0 * p.grdt[j] + 1.0 / 3.0 * p.ak2[j] + 4.0 / 9.0 * p.ak3[j]);
    for (int j = 0; j < 3; j++) p.req[j] = p.xout[j];
    p.stage = 3;
  } else {
    double ak4[3], xerr[3];
    unit(q, ak4);
    for (int j = 0; j < 3; j++)
      xerr[j] = p.x[j] + p.h0 * (7.0 / 24.0 * p.grdt[j] + 1.0 / 4.0 * p.ak2[j] + 1.0 / 3.0 * p.ak3[j] +
                                 1.0 / 8.0 * ak4[j]) - p.xout[j];
    for (int j = 0; j < 3; j++) p.gf[j] = q[1 + j], p.grdt[j] = ak4[j];
    p.gfmod = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    const double nerr = sqrt(xerr[0] * xerr[0] + xerr[1] * xerr[1] + xerr[2] * xerr[2]);
    if (nerr < kNavMaxErr) {
      for (int j = 0; j < 3; j++) p.x[j] = p.xout[j];
      if (p.first && nerr < kNavMaxErr / 10.0)
        p.h0 = copysign(fmin(fabs(p.hini), fabs(1.6 * p.h0)), p.hini);
      after_step(p, true);
    } else {
      p.h0 = 0.9 * p.h0 * kNavMaxErr / nerr;
      if (fabs(p.h0) < kVSmall) {
        after_step(p, false);
      } else {
        // the rejected trial's end-point gradient starts the next trial
        p.first = false;
        request_stage1(p);
      }
    }
  }
}

// A path from x going up (iup = 1) or down (iup = -1), field%gradient's
// initial state; plen starts at |x - pathini| (pathini null: 0).  Its first
// request is the field at x (stage -1).
C2G_HD inline void start_path(Path &p, const double x[3], int iup, const double *pathini = nullptr) {
  p = Path();
  p.iup = iup;
  p.hini = kNavStep * iup;
  p.h0 = kHFirst * iup;
  p.mstep = (int)lround(10000 * 0.1 / fabs(p.hini));
  for (int k = 0; k < kMHist; k++) p.scal[k] = 1.0;
  double d2 = 0.0;
  for (int k = 0; k < 3; k++) {
    p.x[k] = p.xlast[k] = p.xlast2[k] = p.req[k] = x[k];
    if (pathini) d2 += (x[k] - pathini[k]) * (x[k] - pathini[k]);
  }
  p.plen = sqrt(d2);
  p.stage = -1;
}

// The field at a path's start point (the answer to its stage -1 request).
C2G_HD inline void take_start(Path &p, const double *q) {
  for (int j = 0; j < 3; j++) p.gf[j] = q[1 + j];
  p.gfmod = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  p.stage = 0;
}

}  // namespace gpath
}  // namespace c2g
