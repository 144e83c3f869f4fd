// critic2's AUTO critical-point search core for a molecular wavefunction:
// pair seeding (src/autocp@proc.f90:423-437, 665-729), batched Newton
// (k_newton.cu), addcp (src/fieldmod@proc.f90:2288-2439), sortcps
// (src/fieldmod@proc.f90:2441-2466) and the Poincare-Hopf count
// (src/autocp@proc.f90:1395-1420).
//
// critic2 calls addcp inside an omp critical section in whatever order the
// threads finish; here the converged seeds are offered in seed order, one
// of the orders the reference can produce.  Molecules carry no symmetry
// here, so every CP has multiplicity 1.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "c2g_internal.h"

namespace c2g {
namespace {

struct Cp {
  double x[3];  // cell-fractional
  double r[3];  // Cartesian
  double f;
  int typ, typind;
};

// critic2's molecular seeds: npts points on every ordered atom pair closer
// than maxdist.  With distinct, each unordered pair once: the k-th point of
// i -> j is the (npts + 1 - k)-th point of j -> i, so critic2's list holds
// every seed twice (equal up to rounding); one of each halves Newton's work.
std::vector<double> pair_seeds(const HostWfn &w, double maxdist, int npts, bool distinct = false) {
  std::vector<double> out;
  for (int i1 = 0; i1 < w.natom; i1++)
    for (int i2 = distinct ? i1 + 1 : 0; i2 < w.natom; i2++) {
      if (i1 == i2) continue;
      const double *a = &w.xyz[3 * i1], *b = &w.xyz[3 * i2];
      const double d = std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                                 (a[2] - b[2]) * (a[2] - b[2]));
      if (d > maxdist) continue;
      for (int k = 1; k <= npts; k++) {
        double x[3];
        bool keep = true;
        for (int c = 0; c < 3; c++) {
          const double xa = (a[c] - w.cell_lo[c]) / w.cell_aa[c];
          const double xb = (b[c] - w.cell_lo[c]) / w.cell_aa[c];
          double xf = xa + (double)k / (double)(npts + 1) * (xb - xa);
          xf -= std::floor(xf);
          if (xf < w.molborder[c] || xf > 1.0 - w.molborder[c]) keep = false;
          x[c] = w.cell_lo[c] + xf * w.cell_aa[c];
        }
        if (keep) out.insert(out.end(), x, x + 3);
      }
    }
  return out;
}

struct GrdOut {
  std::vector<double> f, gfmod;
  std::vector<int> r, s;
};

GrdOut grd_batch(c2g_wfn *hp, const std::vector<double> &xyz, int prec) {
  const int n = (int)(xyz.size() / 3);
  GrdOut o;
  o.f.resize(n);
  o.gfmod.resize(n);
  o.r.resize(n);
  o.s.resize(n);
  if (n == 0) return o;
  const int rc = c2g_grd(hp, n, xyz.data(), 2, prec, o.f.data(), nullptr, o.gfmod.data(), nullptr,
                         nullptr, o.r.data(), o.s.data(), nullptr);
  if (rc != C2G_OK) fail(rc, last_error());
  return o;
}

}  // namespace
}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_pair_seeds(const c2g_wfn *hp, double maxdist, int npts, double *xseed, int *nseed) {
  return guarded([&] {
    if (!hp || !nseed || npts < 1) fail(C2G_ERR_ARG, "null handle/nseed or npts < 1");
    const Handle *h = reinterpret_cast<const Handle *>(hp);
    std::vector<double> s = pair_seeds(h->host, maxdist, npts);
    const int n = (int)(s.size() / 3);
    if (!xseed) {
      *nseed = n;
      return;
    }
    const int m = std::min(n, *nseed);
    std::copy(s.begin(), s.begin() + 3 * (size_t)m, xseed);
    *nseed = m;
  });
}

int c2g_newton(c2g_wfn *hp, int n, double *xyz, double gfnormeps, int maxit, int prec, int *ier) {
  return guarded([&] {
    if (!hp || n < 0 || (n > 0 && (!xyz || !ier)) || maxit < 0) fail(C2G_ERR_ARG, "bad argument");
    if (prec != C2G_PREC_FP64 && prec != C2G_PREC_TF32X3 && prec != C2G_PREC_BF16X3)
      fail(C2G_ERR_ARG, "unknown precision mode");
    if (n == 0) return;
    Handle *h = reinterpret_cast<Handle *>(hp);
    int prev = 0;
    C2G_CUDA(cudaGetDevice(&prev));
    if (prev != h->device) C2G_CUDA(cudaSetDevice(h->device));
    double *dx = nullptr;
    int *di = nullptr;
    auto cleanup = [&] {
      cudaFree(dx);
      cudaFree(di);
      if (prev != h->device) cudaSetDevice(prev);
    };
    try {
      if (cudaMalloc(&dx, sizeof(double) * 3 * (size_t)n) != cudaSuccess ||
          cudaMalloc(&di, sizeof(int) * (size_t)n) != cudaSuccess)
        fail(C2G_ERR_ALLOC, "cudaMalloc (newton seeds)");
      C2G_CUDA(cudaMemcpy(dx, xyz, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice));
      newton_batch_dev(*h, n, dx, di, gfnormeps, maxit, prec, 0);
      C2G_CUDA(cudaMemcpy(xyz, dx, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost));
      C2G_CUDA(cudaMemcpy(ier, di, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int c2g_autocritic(c2g_wfn *hp, int nseed, const double *xseed, int prec, int maxcp,
                   double *cp_xyz, int *cp_typ, double *cp_f, c2g_cp_report *report) {
  return guarded([&] {
    if (!hp || maxcp < 0 || (maxcp > 0 && (!cp_xyz || !cp_typ || !cp_f))) fail(C2G_ERR_ARG, "bad argument");
    const auto t0 = std::chrono::steady_clock::now();
    Handle *h = reinterpret_cast<Handle *>(hp);
    const HostWfn &w = h->host;
    std::vector<double> seeds;
    if (xseed) seeds.assign(xseed, xseed + 3 * (size_t)std::max(nseed, 0));
    else seeds = pair_seeds(w, 15.0, 5, true);  // same CP list as critic2's doubled seed list
    const int ns = (int)(seeds.size() / 3);
    std::vector<int> ier(std::max(ns, 1), 2);
    const double gfnormeps = 1e-12, cpeps = 1e-2, nuceps = 1e-1, nucepsh = 2e-1;
    const double gradcheck = std::max(1e-4, gfnormeps);
    const int rc = c2g_newton(hp, ns, seeds.data(), gfnormeps, 200, prec, ier.data());
    if (rc != C2G_OK) fail(rc, last_error());
    // candidate positions mapped into the cell, evaluated in one batch
    std::vector<double> cand;
    std::vector<double> candx;
    std::vector<int> cand_seed;
    int nconv = 0;
    for (int i = 0; i < ns; i++) {
      if (ier[i] > 0) continue;
      nconv++;
      double xc[3], x1[3];
      bool inside = true;
      for (int j = 0; j < 3; j++) {
        xc[j] = (seeds[3 * i + j] - w.cell_lo[j]) / w.cell_aa[j];
        xc[j] -= std::floor(xc[j]);
        if (xc[j] < w.molborder[j] || xc[j] > 1.0 - w.molborder[j]) inside = false;
        x1[j] = w.cell_lo[j] + xc[j] * w.cell_aa[j];
      }
      if (!inside) continue;
      cand.insert(cand.end(), x1, x1 + 3);
      candx.insert(candx.end(), xc, xc + 3);
      cand_seed.push_back(i);
    }
    GrdOut gc = grd_batch(hp, cand, C2G_PREC_FP64);
    // nuclei first (init_cplist), with their density (init_cplist_deferred)
    std::vector<Cp> cps;
    std::vector<double> nx(w.xyz);
    GrdOut gn = grd_batch(hp, nx, C2G_PREC_FP64);
    for (int a = 0; a < w.natom; a++) {
      Cp c;
      for (int j = 0; j < 3; j++) {
        c.r[j] = w.xyz[3 * a + j];
        c.x[j] = (c.r[j] - w.cell_lo[j]) / w.cell_aa[j];
        c.x[j] -= std::floor(c.x[j]);
      }
      c.f = gn.f[a];
      c.typ = -3;
      c.typind = 0;
      cps.push_back(c);
    }
    const int nc = (int)cand_seed.size();
    for (int q = 0; q < nc; q++) {
      const double *xc = &candx[3 * q], *x1 = &cand[3 * q];
      // nearest CP in the list
      int nid = -1;
      double dmin = 1e30;
      for (int i = 0; i < (int)cps.size(); i++) {
        double dd = 0.0;
        for (int j = 0; j < 3; j++) {
          const double t = (cps[i].x[j] - xc[j]) * w.cell_aa[j];
          dd += t * t;
        }
        dd = std::sqrt(dd);
        if (dd < dmin) dmin = dd, nid = i;
      }
      if (nid >= w.natom && dmin < cpeps) continue;
      // nearest nucleus within max(nuceps, nucepsh)
      int at = -1;
      double dat = 1e30;
      for (int a = 0; a < w.natom; a++) {
        const double dx = x1[0] - w.xyz[3 * a], dy = x1[1] - w.xyz[3 * a + 1], dz = x1[2] - w.xyz[3 * a + 2];
        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (d < dat) dat = d, at = a;
      }
      if (at >= 0 && dat <= std::max(nuceps, nucepsh)) {
        if (w.z[at] == 1 ? dat < nucepsh : dat < nuceps) continue;
      }
      if (gc.gfmod[q] >= gradcheck) continue;
      if (gc.r[q] != 3) continue;  // degenerate CP discarded
      Cp c;
      std::memcpy(c.x, xc, sizeof(c.x));
      std::memcpy(c.r, x1, sizeof(c.r));
      c.f = gc.f[q];
      c.typ = gc.s[q];
      c.typind = (gc.s[q] + 3) / 2;
      cps.push_back(c);
    }
    // sortcps: stable by decreasing density, then stable by type
    std::stable_sort(cps.begin() + w.natom, cps.end(), [](const Cp &a, const Cp &b) { return -a.f < -b.f; });
    std::stable_sort(cps.begin() + w.natom, cps.end(), [](const Cp &a, const Cp &b) { return a.typind < b.typind; });
    int cnt[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < cps.size(); i++) {
      cnt[cps[i].typind]++;
      if ((int)i < maxcp) {
        std::memcpy(cp_xyz + 3 * i, cps[i].r, sizeof(double) * 3);
        cp_typ[i] = cps[i].typ;
        cp_f[i] = cps[i].f;
      }
    }
    if (report) {
      report->ncp = std::min((int)cps.size(), maxcp);
      for (int k = 0; k < 4; k++) report->count[k] = cnt[k];
      report->poincare_hopf = cnt[0] - cnt[1] + cnt[2] - cnt[3];
      report->nseed = ns;
      report->nconverged = nconv;
      report->ms_total =
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

}  // extern "C"
