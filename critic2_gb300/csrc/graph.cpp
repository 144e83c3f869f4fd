// Molecular graph after the CP search: critic2's makegraph
// (src/autocp@proc.f90:2116-2268) with every gradient path of the CP list
// traced at once.  Each path follows field%gradient
// (src/fieldmod@proc.f90:2500-2732) with the default navigation: the
// Bogacki-Shampine 2(3) stepper (:2860-2890) inside adaptive_stepper
// (:2737-2830), step 0.3, maxerr 1e-4, gradeps 1e-7, beta spheres 0.1
// (src/global@proc.F90:858-861, src/global.f90:41).
//
// The paths advance in lockstep: every Runge-Kutta stage of every live path
// is one batch of field evaluations, done on the GPU by the FP64 per-point
// kernel (k_eval_fp64_pt through launch_fp64_index); the step logic (error
// control, beta spheres, bounce detection) is O(1) per path and runs on the
// host between batches, in the reference's order of operations, so the
// decisions are the ones a serial trace makes with the same field values.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "c2g_internal.h"

namespace c2g {
namespace {

constexpr double kNavStep = 0.3, kNavMaxErr = 1e-4, kNavGradEps = 1e-7, kRBeta = 0.1;
constexpr double kVSmall = 1e-80, kMinStep = 1e-12, kHFirst = 0.01;
constexpr int kMHist = 5;

// Symmetric 3x3 eigen-decomposition (column-major input): cyclic Jacobi,
// eigenvalues ascending, vec + 3 j = eigenvector j, each scaled so that its
// component of largest magnitude (the first such) is positive.  The role of
// eigsym (LAPACK dsyev 'V', src/tools_math@proc.f90:1005-1039); dsyev's
// own sign choice is not reproduced.
void eigvec3(const double m[9], double ev[3], double vec[9]) {
  double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = 0.5 * (m[3 * j + i] + m[3 * i + j]);
  for (int sweep = 0; sweep < 60; sweep++) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    const double dia = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off == 0.0 || off < 1e-34 * dia) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {
          const double kp = a[k][p], kq = a[k][q];
          a[k][p] = c * kp - s * kq;
          a[k][q] = s * kp + c * kq;
        }
        for (int k = 0; k < 3; k++) {
          const double pk = a[p][k], qk = a[q][k];
          a[p][k] = c * pk - s * qk;
          a[q][k] = s * pk + c * qk;
        }
        for (int k = 0; k < 3; k++) {
          const double vp = v[k][p], vq = v[k][q];
          v[k][p] = c * vp - s * vq;
          v[k][q] = s * vp + c * vq;
        }
      }
  }
  int ord[3] = {0, 1, 2};
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2 - i; j++)
      if (a[ord[j]][ord[j]] > a[ord[j + 1]][ord[j + 1]]) std::swap(ord[j], ord[j + 1]);
  for (int j = 0; j < 3; j++) {
    const int c = ord[j];
    ev[j] = a[c][c];
    int big = 0;
    for (int k = 1; k < 3; k++)
      if (std::fabs(v[k][c]) > std::fabs(v[big][c])) big = k;
    const double sg = v[big][c] < 0.0 ? -1.0 : 1.0;
    for (int k = 0; k < 3; k++) vec[3 * j + k] = sg * v[k][c];
  }
}

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
    for (int i = 0; i < n; i++) {
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

}  // namespace
}  // namespace c2g

namespace c2g {
namespace {

// One gradient path (field%gradient's local state).
struct Path {
  double x[3], xlast[3], xlast2[3];
  double h0, hini, plen;
  double scal[kMHist];
  int nhist = 0, iup, nstep = 1, mstep, ier = 0;
  bool incstep = false, done = false, first = true;
  double gf[3] = {0, 0, 0}, gfmod = 0.0;  // field at x
  double grdt[3], ak2[3], ak3[3], xout[3];
  int stage = 0;  // 0 head of a step; 1, 2, 3: waiting for the BS stage
  double req[3];  // point whose evaluation this path waits for
};

void unit(const double *q, double g[3]) {
  const double m = std::sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int j = 0; j < 3; j++) g[j] = q[1 + j] / (m + kVSmall);
}

// The part of one field%gradient iteration before the step
// (src/fieldmod@proc.f90:2582-2680): path length, beta spheres, molecular
// cell, new CP.  Returns true when the path goes on with a step.
bool head(Path &p, const HostWfn &w, int ncp, const double *cpx, const int *cptyp) {
  if (p.nstep > p.mstep) {
    p.nstep = p.mstep;
    p.ier = 2;
    return false;
  }
  double d2 = 0.0;
  for (int j = 0; j < 3; j++) d2 += (p.x[j] - p.xlast[j]) * (p.x[j] - p.xlast[j]);
  p.plen += std::sqrt(d2);
  int idnuc = 0;
  double sphrad = 1e30;
  for (int a = 0; a < w.natom; a++) {
    const double dx = p.x[0] - w.xyz[3 * a], dy = p.x[1] - w.xyz[3 * a + 1], dz = p.x[2] - w.xyz[3 * a + 2];
    const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (d < sphrad) sphrad = d, idnuc = a;
  }
  bool have = false;
  double cprad = 1e15, xcp[3] = {0, 0, 0};
  if (p.iup == 1 && w.z[idnuc] != 1) {
    have = true;
    cprad = sphrad;
    for (int j = 0; j < 3; j++) xcp[j] = w.xyz[3 * idnuc + j];
  }
  for (int i = 0; i < ncp; i++) {
    if (!((cptyp[i] == -3 && p.iup == 1) || (cptyp[i] == 3 && p.iup == -1))) continue;
    const double dx = p.x[0] - cpx[3 * i], dy = p.x[1] - cpx[3 * i + 1], dz = p.x[2] - cpx[3 * i + 2];
    const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (d < cprad) {
      have = true;
      cprad = d;
      for (int j = 0; j < 3; j++) xcp[j] = cpx[3 * i + j];
    }
  }
  if (have && cprad <= kRBeta) {
    p.incstep = true;
    double e2 = 0.0;
    for (int j = 0; j < 3; j++) e2 += (p.x[j] - xcp[j]) * (p.x[j] - xcp[j]);
    p.plen += std::sqrt(e2);
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

void request_stage1(Path &p) {
  for (int j = 0; j < 3; j++) p.req[j] = p.x[j] + p.h0 * (0.5 * p.grdt[j]);
  p.stage = 1;
}

// After adaptive_stepper (:2672-2690): bounce history and step floor.
void after_step(Path &p, bool ok) {
  p.nhist = p.nhist % kMHist + 1;
  double sc = 0.0;
  for (int j = 0; j < 3; j++) sc += (p.xlast[j] - p.xlast2[j]) * (p.x[j] - p.xlast[j]);
  p.scal[p.nhist - 1] = sc;
  bool allneg = true;
  for (int k = 0; k < kMHist; k++) allneg = allneg && p.scal[k] < 0.0;
  ok = ok && !allneg;
  if (!ok || std::fabs(p.h0) < kMinStep) {
    for (int j = 0; j < 3; j++) p.x[j] = p.xlast[j];
    p.ier = 1;
    p.done = true;
    return;
  }
  p.nstep++;
  p.stage = 0;
}

// One evaluated BS stage of a path.
void advance(Path &p, const double *q) {
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
    p.gfmod = std::sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    const double nerr = std::sqrt(xerr[0] * xerr[0] + xerr[1] * xerr[1] + xerr[2] * xerr[2]);
    if (nerr < kNavMaxErr) {
      for (int j = 0; j < 3; j++) p.x[j] = p.xout[j];
      if (p.first && nerr < kNavMaxErr / 10.0)
        p.h0 = std::copysign(std::min(std::fabs(p.hini), std::fabs(1.6 * p.h0)), p.hini);
      after_step(p, true);
    } else {
      p.h0 = 0.9 * p.h0 * kNavMaxErr / nerr;
      if (std::fabs(p.h0) < kVSmall) {
        after_step(p, false);
      } else {
        // the rejected trial's end-point gradient starts the next trial
        p.first = false;
        request_stage1(p);
      }
    }
  }
}

// Traces the paths to their ends (x, ier, nstep, plen in each Path).
void trace_paths(Handle &h, std::vector<Path> &paths, int ncp, const double *cpx, const int *cptyp, BatchGrd &bg) {
  const HostWfn &w = h.host;
  const int n = (int)paths.size();
  std::vector<double> xs(3 * (size_t)n);
  std::vector<int> who(n);
  // field at the start points
  for (int i = 0; i < n; i++)
    for (int j = 0; j < 3; j++) xs[3 * i + j] = paths[i].x[j];
  const double *rec = bg.eval(xs.data(), n);
  for (int i = 0; i < n; i++) {
    const double *q = rec + (size_t)i * kRecNci;
    for (int j = 0; j < 3; j++) paths[i].gf[j] = q[1 + j];
    paths[i].gfmod = std::sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  }
  for (;;) {
    int m = 0;
    for (int i = 0; i < n; i++) {
      Path &p = paths[i];
      if (p.done) continue;
      if (p.stage == 0) {
        if (!head(p, w, ncp, cpx, cptyp)) {
          p.done = true;
          continue;
        }
        request_stage1(p);
      }
      for (int j = 0; j < 3; j++) xs[3 * m + j] = p.req[j];
      who[m++] = i;
    }
    if (m == 0) break;
    rec = bg.eval(xs.data(), m);
    for (int k = 0; k < m; k++) advance(paths[who[k]], rec + (size_t)k * kRecNci);
  }
  for (Path &p : paths)
    if (p.incstep) p.nstep++;
}

}  // namespace
}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_cp_graph(c2g_wfn *hp, int ncp, const double *cp_xyz, const int *cp_typ, int *ipath, double *brdist,
                 double *brpathlen, double *brang, double *brvec, int *ier, int *nstep, c2g_graph_stats *stats) {
  return guarded([&] {
    if (!hp) fail(C2G_ERR_ARG, "null handle");
    Handle &h = *reinterpret_cast<Handle *>(hp);
    if (ncp < 0) fail(C2G_ERR_ARG, "negative CP count");
    if (ncp > 0 && (!cp_xyz || !cp_typ || !ipath || !brdist || !brpathlen || !brang || !brvec))
      fail(C2G_ERR_ARG, "null output array");
    for (int i = 0; i < ncp; i++)
      if (cp_typ[i] != -3 && cp_typ[i] != -1 && cp_typ[i] != 1 && cp_typ[i] != 3)
        fail(C2G_ERR_ARG, "CP types must be -3, -1, 1 or 3");
    const auto t0 = std::chrono::steady_clock::now();
    struct Dev {  // the handle's device for the call, the caller's afterwards
      int old = 0;
      explicit Dev(int d) {
        C2G_CUDA(cudaGetDevice(&old));
        if (old != d) C2G_CUDA(cudaSetDevice(d));
      }
      ~Dev() { cudaSetDevice(old); }
    } guard(h.device);
    const HostWfn &w = h.host;
    std::vector<int> bcp;
    for (int i = 0; i < ncp; i++) {
      for (int j = 0; j < 2; j++) {
        ipath[2 * i + j] = 0, brdist[2 * i + j] = 0.0, brpathlen[2 * i + j] = 0.0;
        if (ier) ier[2 * i + j] = 0;
        if (nstep) nstep[2 * i + j] = 0;
      }
      brang[i] = 0.0;
      for (int k = 0; k < 3; k++) brvec[3 * i + k] = 0.0;
      if (std::abs(cp_typ[i]) == 1) bcp.push_back(i);
    }
    const int nb = (int)bcp.size();
    BatchGrd bg(h, std::max(2 * nb, 1));
    std::vector<Path> paths(2 * (size_t)nb);
    if (nb > 0) {
      // Hessians at the bond and ring CPs, eigenvector of the unique
      // curvature (largest eigenvalue at a bond CP, smallest at a ring CP)
      std::vector<double> xs(3 * (size_t)nb);
      for (int b = 0; b < nb; b++)
        for (int k = 0; k < 3; k++) xs[3 * b + k] = cp_xyz[3 * bcp[b] + k];
      const double *rec = bg.eval(xs.data(), nb);
      for (int b = 0; b < nb; b++) {
        const int i = bcp[b];
        const double *q = rec + (size_t)b * kRecNci;
        const double H[9] = {q[4], q[7], q[8], q[7], q[5], q[9], q[8], q[9], q[6]};
        double ev[3], vec[9];
        eigvec3(H, ev, vec);
        const double *e = cp_typ[i] == -1 ? vec + 6 : vec;
        const double nn = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        for (int k = 0; k < 3; k++) brvec[3 * i + k] = e[k] / nn;
        for (int j = 0; j < 2; j++) {
          Path &p = paths[2 * b + j];
          p.iup = cp_typ[i] == -1 ? 1 : -1;
          p.hini = kNavStep * p.iup;
          p.h0 = kHFirst * p.iup;
          p.mstep = (int)std::lround(10000 * 0.1 / std::fabs(p.hini));
          for (int k = 0; k < kMHist; k++) p.scal[k] = 1.0;
          double d2 = 0.0;
          for (int k = 0; k < 3; k++) {
            p.x[k] = cp_xyz[3 * i + k] + (j == 0 ? 1.0 : -1.0) * 0.01 * brvec[3 * i + k];
            p.xlast[k] = p.xlast2[k] = p.x[k];
            d2 += (p.x[k] - cp_xyz[3 * i + k]) * (p.x[k] - cp_xyz[3 * i + k]);
          }
          p.plen = std::sqrt(d2);  // pathini = the CP
        }
      }
      trace_paths(h, paths, ncp, cp_xyz, cp_typ, bg);
    }
    // end points -> terminating CPs, distances, angle (makegraph :2196-2262)
    for (int b = 0; b < nb; b++) {
      const int i = bcp[b];
      const double *r = cp_xyz + 3 * i;
      double xdif[2][3];
      for (int j = 0; j < 2; j++) {
        const Path &p = paths[2 * b + j];
        double dd = 0.0;
        for (int k = 0; k < 3; k++) xdif[j][k] = p.x[k] - r[k], dd += xdif[j][k] * xdif[j][k];
        brdist[2 * i + j] = std::sqrt(dd);
        brpathlen[2 * i + j] = p.plen;
        if (ier) ier[2 * i + j] = p.ier;
        if (nstep) nstep[2 * i + j] = p.nstep;
        double xf[3];
        bool outside = false;
        for (int k = 0; k < 3; k++) {
          const double f = (p.x[k] - w.cell_lo[k]) / w.cell_aa[k];
          outside = outside || f < w.molborder[k] || f > 1.0 - w.molborder[k];
          xf[k] = f - std::floor(f);
        }
        int wcp = 0;
        double best = 1e30;
        for (int c = 0; c < ncp; c++) {
          if (cp_typ[c] != 3 * cp_typ[i]) continue;
          double d2 = 0.0;
          for (int k = 0; k < 3; k++) {
            const double t = ((cp_xyz[3 * c + k] - w.cell_lo[k]) / w.cell_aa[k] - xf[k]) * w.cell_aa[k];
            d2 += t * t;
          }
          const double d = std::sqrt(d2);
          if (d < best) best = d, wcp = c + 1;
        }
        ipath[2 * i + j] = wcp ? wcp : (outside ? -1 : 0);
      }
      double ca = 0.0;
      if (brdist[2 * i] > 1e-12) {
        for (int k = 0; k < 3; k++) ca += xdif[0][k] * xdif[1][k];
        ca = ca / brdist[2 * i] / brdist[2 * i + 1];
      }
      if (std::fabs(ca) > 1.0) ca = ca / std::fabs(ca);
      brang[i] = std::acos(ca) * 180.0 / M_PI;
    }
    if (stats) {
      stats->npath = 2 * nb;
      stats->nbatch = (int)bg.launches();
      stats->nevals = bg.evals();
      stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

}  // extern "C"
