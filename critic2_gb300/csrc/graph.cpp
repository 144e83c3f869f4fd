// Molecular graph after the CP search: critic2's makegraph
// (src/autocp@proc.f90:2116-2268) with every gradient path of the CP list
// traced at once.  Each path follows field%gradient
// (src/fieldmod@proc.f90:2500-2732) with the default navigation: the
// Bogacki-Shampine 2(3) stepper (:2860-2890) inside adaptive_stepper
// (:2737-2830), step 0.3, maxerr 1e-4, gradeps 1e-7, beta spheres 0.1
// (src/global@proc.F90:858-861, src/global.f90:41).
//
// The paths run on the GPU (k_gpath.cu), one block per path: thread 0
// takes field%gradient's steps (error control, beta spheres, bounce
// detection, in the reference's order of operations) and the block
// evaluates the FP64 field each step needs, with the per-point kernel's
// arithmetic, so no step waits for the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "c2g_internal.h"
#include "gpath.h"
#include "k_gpath.h"

namespace c2g {
namespace {

using namespace gpath;

// Device copy of a host array, freed with the object.
template <class T>
struct DevArr {
  T *p = nullptr;
  explicit DevArr(const std::vector<T> &v) : DevArr(v.size()) {
    if (!v.empty()) C2G_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  }
  explicit DevArr(size_t n) {
    const cudaError_t e = cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
    if (e != cudaSuccess) fail(C2G_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  ~DevArr() {
    if (p) cudaFree(p);
  }
  DevArr(const DevArr &) = delete;
  DevArr &operator=(const DevArr &) = delete;
  std::vector<T> get(size_t n) const {
    std::vector<T> v(n);
    if (n) C2G_CUDA(cudaMemcpy(v.data(), p, sizeof(T) * n, cudaMemcpyDeviceToHost));
    return v;
  }
};

// Traces the paths (start x, iup, path length from pathini) to their ends on
// the device; returns the field evaluations made.
long trace_paths_dev(Handle &h, std::vector<Path> &paths, const std::vector<double> &pathini, int ncp,
                     const double *cpx, const int *cptyp) {
  const int n = (int)paths.size();
  if (n == 0) return 0;
  const HostWfn &w = h.host;
  std::vector<double> x0(3 * (size_t)n);
  std::vector<int> iup(n);
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) x0[3 * i + k] = paths[i].x[k];
    iup[i] = paths[i].iup;
  }
  DevArr<double> dx0(x0), dpi(pathini), dcp(std::vector<double>(cpx, cpx + 3 * (size_t)ncp)), dxyz(w.xyz);
  DevArr<int> diup(iup), dtyp(std::vector<int>(cptyp, cptyp + ncp)), dz(w.z);
  DevArr<double> dxe(3 * (size_t)n), dpl(n);
  DevArr<int> dier(n), dns(n);
  DevArr<long> dev(n);
  PathGeom g = host_geom(w);
  g.xyz = dxyz.p;
  g.z = dz.p;
  PathsDev d{n, dx0.p, dpi.p, diup.p, ncp, dcp.p, dtyp.p, dxe.p, dpl.p, dier.p, dns.p, dev.p};
  int dev_id = 0, sms = 0;
  C2G_CUDA(cudaGetDevice(&dev_id));
  C2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
  launch_trace_paths(h.dev, g, d, std::min(n, 3 * sms), 0);
  C2G_CUDA(cudaDeviceSynchronize());
  const std::vector<double> xe = dxe.get(3 * (size_t)n), pl = dpl.get(n);
  const std::vector<int> ie = dier.get(n), ns = dns.get(n);
  const std::vector<long> ev = dev.get(n);
  long nev = 0;
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) paths[i].x[k] = xe[3 * i + k];
    paths[i].ier = ie[i], paths[i].nstep = ns[i], paths[i].plen = pl[i];
    nev += ev[i];
  }
  return nev;
}

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
    long path_evals = 0;
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
      std::vector<double> pathini(6 * (size_t)nb);
      for (int b = 0; b < nb; b++)
        for (int j = 0; j < 2; j++)
          for (int k = 0; k < 3; k++) pathini[3 * (2 * b + j) + k] = cp_xyz[3 * bcp[b] + k];
      path_evals = trace_paths_dev(h, paths, pathini, ncp, cp_xyz, cp_typ);
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
      stats->nbatch = (int)bg.launches() + (nb > 0 ? 1 : 0);
      stats->nevals = bg.evals() + path_evals;
      stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

}  // extern "C"
