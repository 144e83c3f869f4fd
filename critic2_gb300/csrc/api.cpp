// C-ABI entry points of critic2_gb300 (declared in include/critic2_gb300.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>

#include "c2g_internal.h"
#include "k_cube.h"
#include "k_tc.h"

namespace c2g {

namespace {
thread_local std::string g_last_error;

// Keeps the caller's current device and restores it on exit.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    C2G_CUDA(cudaGetDevice(&prev));
    if (prev != dev) C2G_CUDA(cudaSetDevice(dev));
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

template <class T>
T *dev_alloc(Handle &h, size_t n) {
  void *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) fail(C2G_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h.allocations.push_back(p);
  return static_cast<T *>(p);
}

template <class T>
T *upload(Handle &h, const std::vector<T> &v) {
  T *d = dev_alloc<T>(h, v.size());
  if (!v.empty()) C2G_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return d;
}

// Scratch device buffer owned by one call.
struct DevBuf {
  void *p = nullptr;
  explicit DevBuf(size_t bytes) {
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) fail(C2G_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

void require(bool ok, const char *msg) {
  if (!ok) fail(C2G_ERR_ARG, msg);
}

void build_device(Handle &h) {
  HostWfn &w = h.host;
  C2G_CUDA(cudaGetDevice(&h.device));
  DevWfn &d = h.dev;
  d.natom = w.natom;
  d.npri = w.npri;
  d.nmo = w.nmo;
  d.nmo_pad = (w.nmo + 63) / 64 * 64;
  std::vector<double4> atoms(w.natom);
  for (int a = 0; a < w.natom; a++)
    atoms[a] = make_double4(w.xyz[3 * a], w.xyz[3 * a + 1], w.xyz[3 * a + 2],
                            w.spcutoff[a] * w.spcutoff[a]);
  d.atoms = upload(h, atoms);
  d.atom_z = upload(h, w.z);
  std::vector<PrimF64> prim(w.npri);
  std::vector<double> cmo((size_t)w.npri * d.nmo_pad, 0.0);
  for (int k = 0; k < w.npri; k++) {
    const int ip = w.icord[k];
    const int *l = kLi[w.itype[ip] - 1];
    prim[k] = PrimF64{w.e[ip], w.dran[ip], l[0] | (l[1] << 4) | (l[2] << 8), w.icenter[ip], 0, 0};
    std::copy(w.cmo.begin() + (size_t)ip * w.nmo, w.cmo.begin() + (size_t)(ip + 1) * w.nmo,
              cmo.begin() + (size_t)k * d.nmo_pad);
  }
  d.prim = upload(h, prim);
  d.cmo = upload(h, cmo);
  std::vector<double> occ(d.nmo_pad, 0.0), wup(d.nmo_pad, 0.0), wdn(d.nmo_pad, 0.0);
  for (int m = 0; m < w.nmo; m++) {
    occ[m] = w.occ[m];
    const bool alpha = m < w.nalpha;
    if (w.wfntyp == C2G_WFN_UHF) (alpha ? wup : wdn)[m] = w.occ[m];
    else if (w.wfntyp == C2G_WFN_ROHF) {
      wup[m] = w.occ[m];
      if (alpha) wdn[m] = w.occ[m];
    }
  }
  d.occ = upload(h, occ);
  d.spin = (w.wfntyp == C2G_WFN_UHF || w.wfntyp == C2G_WFN_ROHF);
  d.wup = d.spin ? upload(h, wup) : nullptr;
  d.wdn = d.spin ? upload(h, wdn) : nullptr;
  for (int j = 0; j < 3; j++) d.cell_lo[j] = w.cell_lo[j], d.cell_aa[j] = w.cell_aa[j];
  d.edf = nullptr;
  d.nedf = 0;
}

// Uploads the EDF core primitives in centre-major order (critic2's
// icord_edf, src/wfn_private@proc.F90:3758-3776) and refreshes the atoms'
// spcutoff^2, which the EDF cutoffs widen.
void upload_edf(Handle &h) {
  HostWfn &w = h.host;
  DevWfn &d = h.dev;
  std::vector<double4> atoms(w.natom);
  for (int a = 0; a < w.natom; a++)
    atoms[a] = make_double4(w.xyz[3 * a], w.xyz[3 * a + 1], w.xyz[3 * a + 2],
                            w.spcutoff[a] * w.spcutoff[a]);
  C2G_CUDA(cudaMemcpy(const_cast<double4 *>(d.atoms), atoms.data(), sizeof(double4) * w.natom,
                      cudaMemcpyHostToDevice));
  if (h.edf_buf) {
    C2G_CUDA(cudaFree(h.edf_buf));
    h.edf_buf = nullptr;
  }
  d.edf = nullptr;
  d.nedf = 0;
  if (w.nedf == 0) return;
  std::vector<int> ord(w.nedf);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int a, int b) { return w.edf_icenter[a] < w.edf_icenter[b]; });
  std::vector<PrimEDF> prim(w.nedf);
  for (int k = 0; k < w.nedf; k++) {
    const int i = ord[k];
    const int *l = kLi[w.edf_itype[i] - 1];
    prim[k] = PrimEDF{w.edf_e[i], w.edf_dran[i], w.edf_c[i], l[0] | (l[1] << 4) | (l[2] << 8),
                      w.edf_icenter[i]};
  }
  C2G_CUDA(cudaMalloc(&h.edf_buf, sizeof(PrimEDF) * prim.size()));
  C2G_CUDA(cudaMemcpy(h.edf_buf, prim.data(), sizeof(PrimEDF) * prim.size(), cudaMemcpyHostToDevice));
  d.edf = static_cast<const PrimEDF *>(h.edf_buf);
  d.nedf = w.nedf;
}

// Replaces the EDF core of a handle (host arrays, cutoffs, device copy).
void set_edf(Handle &h, int nedf, const int *icenter, const int *itype, const double *e, const double *c) {
  HostWfn &w = h.host;
  require(nedf >= 0, "nedf must be non-negative");
  require(nedf == 0 || (icenter && itype && e && c), "null EDF array");
  for (int i = 0; i < nedf; i++) {
    require(icenter[i] >= 1 && icenter[i] <= w.natom, "EDF icenter out of range");
    require(itype[i] >= 1 && itype[i] <= 56, "EDF itype out of range (1..56)");
    require(e[i] > 0.0, "EDF exponents must be positive");
  }
  w.nedf = nedf;
  w.edf_icenter.resize(nedf);
  for (int i = 0; i < nedf; i++) w.edf_icenter[i] = icenter[i] - 1;
  w.edf_itype.assign(itype, itype + nedf);
  w.edf_e.assign(e, e + nedf);
  w.edf_c.assign(c, c + nedf);
  complete_struct(w);
  DeviceGuard g(h.device);
  upload_edf(h);
}

Handle *check_handle(c2g_wfn *hp) {
  require(hp != nullptr, "null handle");
  return reinterpret_cast<Handle *>(hp);
}

int check_prec(int prec) {
  require(prec == C2G_PREC_FP64 || prec == C2G_PREC_TF32X3 || prec == C2G_PREC_BF16X3,
          "unknown precision mode");
  return prec;
}

// Evaluates the FP64 record (kRecFull when full) at n host points.
std::vector<double> eval_records_fp64(Handle &h, int n, const double *xyz, int nder, bool full,
                                      bool valence = false) {
  const int nr = full ? kRecFull : kRecNci;
  DevBuf dx(sizeof(double) * 3 * (size_t)n), dr(sizeof(double) * nr * (size_t)n);
  C2G_CUDA(cudaMemcpy(dx.p, xyz, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice));
  DevWfn dw = h.dev;
  if (valence) dw.nedf = 0;  // the EDF core left out: rho2's rhoval/gradval/hval
  launch_fp64_points(dw, n, dx.as<double>(), nder, full, dr.as<double>(), 0);
  std::vector<double> rec((size_t)nr * n);
  C2G_CUDA(cudaMemcpy(rec.data(), dr.p, sizeof(double) * rec.size(), cudaMemcpyDeviceToHost));
  return rec;
}

// Records at n host points in the requested precision; the split modes give
// the kRecNci quantities only.
std::vector<double> eval_records(Handle &h, int n, const double *xyz, int nder, int prec, bool full) {
  if (prec == C2G_PREC_FP64) return eval_records_fp64(h, n, xyz, nder, full);
  const int nr = kRecNci;
  // The split kernel evaluates 32 points per tile relative to the tile's
  // centroid; ordering the batch along a Morton curve keeps tiles compact.
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) lo[c] = std::min(lo[c], xyz[3 * i + c]), hi[c] = std::max(hi[c], xyz[3 * i + c]);
  std::vector<uint64_t> key(n);
  for (int i = 0; i < n; i++) {
    uint64_t q[3], k = 0;
    for (int c = 0; c < 3; c++) {
      const double sp = hi[c] - lo[c];
      q[c] = (uint64_t)(sp > 0 ? std::min(2097151.0, (xyz[3 * i + c] - lo[c]) / sp * 2097151.0) : 0.0);
    }
    for (int b = 0; b < 21; b++)
      for (int c = 0; c < 3; c++) k |= ((q[c] >> b) & 1ull) << (3 * b + c);
    key[i] = k;
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; i++) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return key[a] < key[b]; });
  std::vector<double> sorted(3 * (size_t)n);
  for (int i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) sorted[3 * (size_t)i + c] = xyz[3 * (size_t)ord[i] + c];
  DevBuf dx(sizeof(double) * 3 * (size_t)n), dr(sizeof(double) * nr * (size_t)n);
  C2G_CUDA(cudaMemcpy(dx.p, sorted.data(), sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice));
  tc_points(h, prec, n, dx.as<double>(), dr.as<double>(), 0);
  std::vector<double> srec((size_t)nr * n), rec((size_t)nr * n);
  C2G_CUDA(cudaMemcpy(srec.data(), dr.p, sizeof(double) * srec.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; i++)
    std::copy(srec.begin() + (size_t)i * nr, srec.begin() + (size_t)(i + 1) * nr, rec.begin() + (size_t)ord[i] * nr);
  if (full) {
    std::vector<double> out((size_t)kRecFull * n, 0.0);
    for (int i = 0; i < n; i++)
      std::copy(rec.begin() + (size_t)i * nr, rec.begin() + (size_t)(i + 1) * nr,
                out.begin() + (size_t)i * kRecFull);
    return out;
  }
  return rec;
}

}  // namespace

void set_last_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

void fail(int code, const std::string &msg) { throw Failure(code, msg); }

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) fail(C2G_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Symmetric 3x3 eigenvalues (column-major input), ascending; cyclic Jacobi.
void eigsym3(const double m[9], double ev[3]) {
  double a[3][3];
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
      }
  }
  double e[3] = {a[0][0], a[1][1], a[2][2]};
  std::sort(e, e + 3);
  ev[0] = e[0], ev[1] = e[1], ev[2] = e[2];
}

// The rho2 output assembly (src/wfn_private@proc.F90:2636-2703) from a
// kRecFull record, for one point.
static void assemble_rho2(const HostWfn &w, const double *r, int nder, double *rho, double *grad,
                          double *hess, double *gkin, double *stress, double *vir) {
  const bool spin = (w.wfntyp == C2G_WFN_UHF || w.wfntyp == C2G_WFN_ROHF);
  double rh[3], g[3][3], hh[3][6], gk[3];
  rh[0] = r[0];
  for (int j = 0; j < 3; j++) g[0][j] = r[1 + j];
  for (int j = 0; j < 6; j++) hh[0][j] = r[4 + j];
  gk[0] = r[10];
  if (spin) {
    for (int s = 0; s < 2; s++) {
      const double *b = r + 17 + 11 * s;
      rh[1 + s] = b[0];
      for (int j = 0; j < 3; j++) g[1 + s][j] = b[1 + j];
      gk[1 + s] = b[4];
      for (int j = 0; j < 6; j++) hh[1 + s][j] = b[5 + j];
    }
  } else {
    rh[1] = rh[2] = 0.5 * rh[0];
    for (int j = 0; j < 3; j++) g[1][j] = g[2][j] = 0.5 * g[0][j];
    for (int j = 0; j < 6; j++) hh[1][j] = hh[2][j] = 0.5 * hh[0][j];
    gk[1] = gk[2] = gk[0] / 2.0;
  }
  if (rho)
    for (int s = 0; s < 3; s++) rho[s] = rh[s];
  if (grad && nder > 0)
    for (int s = 0; s < 3; s++)
      for (int j = 0; j < 3; j++) grad[3 * s + j] = g[s][j];
  if (gkin && nder > 0)
    for (int s = 0; s < 3; s++) gkin[s] = 0.5 * gk[s];
  if (hess && nder > 1)
    for (int s = 0; s < 3; s++) {
      double *H = hess + 9 * s;
      H[0] = hh[s][0], H[4] = hh[s][1], H[8] = hh[s][2];
      H[1] = H[3] = hh[s][3], H[2] = H[6] = hh[s][4], H[5] = H[7] = hh[s][5];
    }
  if (nder > 1 && (stress || vir)) {
    // r[11..16] = xx, xy, xz, yy, yz, zz, halved at the end
    const double sxx = 0.5 * r[11], sxy = 0.5 * r[12], sxz = 0.5 * r[13];
    const double syy = 0.5 * r[14], syz = 0.5 * r[15], szz = 0.5 * r[16];
    if (stress) {
      stress[0] = sxx, stress[1] = sxy, stress[2] = sxz;
      stress[3] = sxy, stress[4] = syy, stress[5] = syz;
      stress[6] = sxz, stress[7] = syz, stress[8] = szz;
    }
    if (vir) *vir = sxx + syy + szz;
  }
}

}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_abi_version(void) { return C2G_ABI_VERSION; }

int c2g_last_error(char *buf, int len) {
  const int n = (int)g_last_error.size();
  if (buf && len > 0) {
    const int m = std::min(n, len - 1);
    std::memcpy(buf, g_last_error.data(), m);
    buf[m] = 0;
  }
  return n;
}

int c2g_wfn_create(int natom, const double *atom_xyz, const int *atom_z, int npri, int nmo,
                   const int *icenter, const int *itype, const double *e, const double *occ,
                   const double *cmo, int wfntyp, int nalpha, c2g_wfn **out) {
  return guarded([&] {
    require(out != nullptr, "null output handle pointer");
    *out = nullptr;
    require(natom > 0 && npri > 0 && nmo > 0, "natom, npri and nmo must be positive");
    require(atom_xyz && atom_z && icenter && itype && e && occ && cmo, "null input array");
    require(wfntyp >= 0 && wfntyp <= 3, "unknown wavefunction type");
    auto h = std::make_unique<Handle>();
    HostWfn &w = h->host;
    w.natom = natom, w.npri = npri, w.nmo = nmo, w.wfntyp = wfntyp, w.nalpha = nalpha;
    w.xyz.assign(atom_xyz, atom_xyz + 3 * (size_t)natom);
    w.z.assign(atom_z, atom_z + natom);
    w.icenter.resize(npri);
    w.itype.assign(itype, itype + npri);
    w.e.assign(e, e + npri);
    w.occ.assign(occ, occ + nmo);
    w.cmo.assign(cmo, cmo + (size_t)npri * nmo);
    for (int i = 0; i < npri; i++) {
      require(icenter[i] >= 1 && icenter[i] <= natom, "icenter out of range");
      require(itype[i] >= 1 && itype[i] <= 56, "itype out of range (1..56)");
      require(e[i] > 0.0, "exponents must be positive");
      w.icenter[i] = icenter[i] - 1;
    }
    prune_primitives(w);
    complete_struct(w);
    molecular_cell(w);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(C2G_ERR_CUDA, "no CUDA device available");
    }
    try {
      build_device(*h);
      h->tc = tc_create(*h);
    } catch (...) {
      for (void *p : h->allocations) cudaFree(p);
      if (h->tc) tc_destroy(h->tc);
      throw;
    }
    *out = reinterpret_cast<c2g_wfn *>(h.release());
  });
}

int c2g_wfn_read_wfx(const char *path, c2g_wfn **out) {
  return guarded([&] {
    require(path && out, "null argument");
    HostWfn w;
    std::string err;
    if (!read_wfx(path, w, err)) fail(C2G_ERR_IO, err);
    // read_wfx already pruned; create re-runs prune (idempotent) on the
    // original-order arrays.
    std::vector<int> icenter1(w.npri);
    for (int i = 0; i < w.npri; i++) icenter1[i] = w.icenter[i] + 1;
    int rc = c2g_wfn_create(w.natom, w.xyz.data(), w.z.data(), w.npri, w.nmo, icenter1.data(),
                            w.itype.data(), w.e.data(), w.occ.data(), w.cmo.data(), w.wfntyp,
                            w.nalpha, out);
    if (rc != C2G_OK) fail(rc, g_last_error);
    if (w.nedf > 0) {
      std::vector<int> ic(w.nedf);
      for (int i = 0; i < w.nedf; i++) ic[i] = w.edf_icenter[i] + 1;
      try {
        set_edf(*reinterpret_cast<Handle *>(*out), w.nedf, ic.data(), w.edf_itype.data(), w.edf_e.data(),
                w.edf_c.data());
      } catch (...) {
        c2g_wfn_destroy(*out);
        *out = nullptr;
        throw;
      }
    }
  });
}

int c2g_wfn_read_molden(const char *path, c2g_wfn **out) {
  return guarded([&] {
    require(path && out, "null argument");
    HostWfn w;
    std::string err;
    if (!read_molden(path, w, err)) fail(C2G_ERR_IO, err);
    std::vector<int> icenter1(w.npri);
    for (int i = 0; i < w.npri; i++) icenter1[i] = w.icenter[i] + 1;
    int rc = c2g_wfn_create(w.natom, w.xyz.data(), w.z.data(), w.npri, w.nmo, icenter1.data(),
                            w.itype.data(), w.e.data(), w.occ.data(), w.cmo.data(), w.wfntyp,
                            w.nalpha, out);
    if (rc != C2G_OK) fail(rc, g_last_error);
  });
}

int c2g_wfn_read_fchk(const char *path, c2g_wfn **out) {
  return guarded([&] {
    require(path && out, "null argument");
    HostWfn w;
    std::string err;
    if (!read_fchk(path, w, err)) fail(C2G_ERR_IO, err);
    std::vector<int> icenter1(w.npri);
    for (int i = 0; i < w.npri; i++) icenter1[i] = w.icenter[i] + 1;
    int rc = c2g_wfn_create(w.natom, w.xyz.data(), w.z.data(), w.npri, w.nmo, icenter1.data(),
                            w.itype.data(), w.e.data(), w.occ.data(), w.cmo.data(), w.wfntyp,
                            w.nalpha, out);
    if (rc != C2G_OK) fail(rc, g_last_error);
  });
}

int c2g_wfn_read_wfn(const char *path, c2g_wfn **out) {
  return guarded([&] {
    require(path && out, "null argument");
    HostWfn w;
    std::string err;
    if (!read_wfn(path, w, err)) fail(C2G_ERR_IO, err);
    std::vector<int> icenter1(w.npri);
    for (int i = 0; i < w.npri; i++) icenter1[i] = w.icenter[i] + 1;
    int rc = c2g_wfn_create(w.natom, w.xyz.data(), w.z.data(), w.npri, w.nmo, icenter1.data(),
                            w.itype.data(), w.e.data(), w.occ.data(), w.cmo.data(), w.wfntyp,
                            w.nalpha, out);
    if (rc != C2G_OK) fail(rc, g_last_error);
  });
}

int c2g_wfn_destroy(c2g_wfn *hp) {
  return guarded([&] {
    if (!hp) return;
    Handle *h = reinterpret_cast<Handle *>(hp);
    {
      DeviceGuard g(h->device);
      if (h->tc) tc_destroy(h->tc);
      for (void *p : h->allocations) cudaFree(p);
      if (h->edf_buf) cudaFree(h->edf_buf);
    }
    delete h;
  });
}

int c2g_wfn_set_edf(c2g_wfn *hp, int nedf, const int *icenter, const int *itype, const double *e,
                    const double *c) {
  return guarded([&] { set_edf(*check_handle(hp), nedf, icenter, itype, e, c); });
}

int c2g_wfn_set_param(c2g_wfn *hp, int param, double value) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    if (param == C2G_PARAM_RECHECK_REL) {
      require(value < 1.0, "re-check threshold must be below 1 (negative: the default)");
      tc_set_recheck(*h, value < 0.0 ? -1.0 : value);
    } else if (param == C2G_PARAM_NEWTON_STALL) {
      require(value >= 0.0 && value <= 1e6, "stall count must be in [0, 1e6]");
      h->newton_stall = (int)value;
    } else if (param == C2G_PARAM_WAIT_NS) {
      require(value >= 1.0 && value <= 6e11, "wait limit must be in [1, 6e11] ns");
      tc_set_wait_ns(*h, (uint64_t)value);
    } else {
      fail(C2G_ERR_ARG, "unknown parameter");
    }
  });
}

int c2g_wfn_info(const c2g_wfn *hp, int *natom, int *npri, int *nmo, int *wfntyp, int *nalpha) {
  return guarded([&] {
    require(hp != nullptr, "null handle");
    const Handle *h = reinterpret_cast<const Handle *>(hp);
    if (natom) *natom = h->host.natom;
    if (npri) *npri = h->host.npri;
    if (nmo) *nmo = h->host.nmo;
    if (wfntyp) *wfntyp = h->host.wfntyp;
    if (nalpha) *nalpha = h->host.nalpha;
  });
}

int c2g_rho2(c2g_wfn *hp, int n, const double *xyz, int nder, int prec, double *rho, double *grad,
             double *hess, double *gkin, double *stress, double *vir) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(n >= 0, "negative point count");
    require(nder >= 0 && nder <= 2, "nder must be 0, 1 or 2");
    check_prec(prec);
    if (n == 0) return;
    require(xyz != nullptr, "null xyz");
    DeviceGuard g(h->device);
    const bool full = (prec == C2G_PREC_FP64);
    std::vector<double> rec = eval_records(*h, n, xyz, nder, prec, true);
    (void)full;
    for (int i = 0; i < n; i++)
      assemble_rho2(h->host, rec.data() + (size_t)i * kRecFull, nder, rho ? rho + 3 * i : nullptr,
                    grad ? grad + 9 * i : nullptr, hess ? hess + 27 * i : nullptr,
                    gkin ? gkin + 3 * i : nullptr, stress ? stress + 9 * i : nullptr,
                    vir ? vir + i : nullptr);
  });
}

int c2g_rho2_valence(c2g_wfn *hp, int n, const double *xyz, int nder, double *rho, double *grad, double *hess) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(n >= 0, "negative point count");
    require(nder >= 0 && nder <= 2, "nder must be 0, 1 or 2");
    if (n == 0) return;
    require(xyz != nullptr, "null xyz");
    DeviceGuard g(h->device);
    std::vector<double> rec = eval_records_fp64(*h, n, xyz, nder, true, true);
    for (int i = 0; i < n; i++)
      assemble_rho2(h->host, rec.data() + (size_t)i * kRecFull, nder, rho ? rho + 3 * i : nullptr,
                    grad ? grad + 9 * i : nullptr, hess ? hess + 27 * i : nullptr, nullptr, nullptr, nullptr);
  });
}

int c2g_grd(c2g_wfn *hp, int n, const double *xyz, int nder, int prec, double *f, double *gf,
            double *gfmod, double *hf, double *hfeval, int *r, int *s, int *isnuc) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(n >= 0, "negative point count");
    require(nder >= 0 && nder <= 2, "nder must be 0, 1 or 2");
    check_prec(prec);
    if (n == 0) return;
    require(xyz != nullptr, "null xyz");
    DeviceGuard g(h->device);
    std::vector<double> rec = eval_records(*h, n, xyz, nder, prec, false);
    const HostWfn &w = h->host;
    for (int i = 0; i < n; i++) {
      const double *q = rec.data() + (size_t)i * kRecNci;
      // wrapped position (as the kernel evaluated it) for the nucleus test
      double x[3];
      for (int j = 0; j < 3; j++) {
        double fr = (xyz[3 * i + j] - w.cell_lo[j]) / w.cell_aa[j];
        if (fr < -1e-4 || fr > 1.0 + 1e-4) fr -= std::floor(fr);
        x[j] = w.cell_lo[j] + fr * w.cell_aa[j];
      }
      bool nuc = false;
      for (int a = 0; a < w.natom && !nuc; a++) {
        const double dx = x[0] - w.xyz[3 * a], dy = x[1] - w.xyz[3 * a + 1], dz = x[2] - w.xyz[3 * a + 2];
        nuc = std::sqrt(dx * dx + dy * dy + dz * dz) <= 1e-5;
      }
      if (f) f[i] = q[0];
      if (isnuc) isnuc[i] = nuc;
      double gg[3] = {q[1], q[2], q[3]};
      if (nuc) gg[0] = gg[1] = gg[2] = 0.0;
      if (gf && nder > 0)
        for (int j = 0; j < 3; j++) gf[3 * i + j] = gg[j];
      if (gfmod) gfmod[i] = nder > 0 ? std::sqrt(gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2]) : 0.0;
      if (nder > 1) {
        double H[9] = {q[4], q[7], q[8], q[7], q[5], q[9], q[8], q[9], q[6]};
        if (hf) std::copy(H, H + 9, hf + 9 * i);
        double ev[3];
        eigsym3(H, ev);
        if (hfeval) std::copy(ev, ev + 3, hfeval + 3 * i);
        int np = 0, nm = 0;
        for (double v : ev) np += v > 1e-8, nm += v < -1e-8;
        if (r) r[i] = np + nm;
        if (s) s[i] = np - nm;
      }
    }
  });
}

int c2g_nciplot_dev(c2g_wfn *hp, const double *x0, const double *xmat, const int *nstep, int prec,
                    double *d_crho, double *d_cgrad, void *stream, c2g_nci_stats *stats) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(x0 && xmat && nstep && d_crho && d_cgrad, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    require((long)nstep[0] * nstep[1] * nstep[2] < (1L << 31), "grid too large (2^31 points)");
    check_prec(prec);
    DeviceGuard g(h->device);
    GridSpec gs;
    for (int j = 0; j < 3; j++) gs.x0[j] = x0[j], gs.nstep[j] = nstep[j];
    for (int j = 0; j < 9; j++) gs.xmat[j] = xmat[j];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (stats) {
      C2G_CUDA(cudaEventCreate(&e0));
      C2G_CUDA(cudaEventCreate(&e1));
      C2G_CUDA(cudaEventCreate(&e2));
      C2G_CUDA(cudaEventRecord(e0, st));
    }
    long nrecheck = 0;
    double stage_frac = 1.0;
    if (prec == C2G_PREC_FP64) {
      launch_fp64_nci_grid(h->dev, gs, d_crho, d_cgrad, st);
      if (stats) C2G_CUDA(cudaEventRecord(e1, st));
    } else {
      nrecheck = tc_nci_grid(*h, prec, gs, d_crho, d_cgrad, st, stats ? e1 : nullptr, &stage_frac);
    }
    if (stats) {
      C2G_CUDA(cudaEventRecord(e2, st));
      C2G_CUDA(cudaEventSynchronize(e2));
      float a = 0.f, b = 0.f;
      C2G_CUDA(cudaEventElapsedTime(&a, e0, e1));
      C2G_CUDA(cudaEventElapsedTime(&b, e1, e2));
      stats->npoints = (long)nstep[0] * nstep[1] * nstep[2];
      stats->nrecheck = nrecheck;
      stats->ms_kernel = a;
      stats->ms_recheck = b;
      stats->stage_frac = stage_frac;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cudaEventDestroy(e2);
    }
  });
}

int c2g_nciplot_dev_noalloc(c2g_wfn *hp, const double *x0, const double *xmat, const int *nstep, int prec,
                            double *d_crho, double *d_cgrad, void *stream) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(x0 && xmat && nstep && d_crho && d_cgrad, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    const long np = (long)nstep[0] * nstep[1] * nstep[2];
    if (np > tc_noalloc_max_points())
      fail(C2G_ERR_ARG, "grid has " + std::to_string(np) + " points; the no-allocation entry takes at most " +
                            std::to_string(tc_noalloc_max_points()) + " per call (split the grid into slabs)");
    check_prec(prec);
    DeviceGuard g(h->device);
    GridSpec gs;
    for (int j = 0; j < 3; j++) gs.x0[j] = x0[j], gs.nstep[j] = nstep[j];
    for (int j = 0; j < 9; j++) gs.xmat[j] = xmat[j];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (prec == C2G_PREC_FP64) {
      launch_fp64_nci_grid(h->dev, gs, d_crho, d_cgrad, st);  // uses no scratch
      C2G_CUDA(cudaStreamSynchronize(st));
    } else {
      tc_nci_grid_noalloc(*h, prec, gs, d_crho, d_cgrad, st);
    }
  });
}

int c2g_nciplot(c2g_wfn *hp, const double *x0, const double *xmat, const int *nstep, int prec,
                double *crho, double *cgrad, c2g_nci_stats *stats) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(x0 && xmat && nstep && crho && cgrad, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    DeviceGuard g(h->device);
    const size_t np = (size_t)nstep[0] * nstep[1] * nstep[2];
    DevBuf dr(sizeof(double) * np), dg(sizeof(double) * np);
    int rc = c2g_nciplot_dev(hp, x0, xmat, nstep, prec, dr.as<double>(), dg.as<double>(), nullptr, stats);
    if (rc != C2G_OK) fail(rc, g_last_error);
    C2G_CUDA(cudaMemcpy(crho, dr.p, sizeof(double) * np, cudaMemcpyDeviceToHost));
    C2G_CUDA(cudaMemcpy(cgrad, dg.p, sizeof(double) * np, cudaMemcpyDeviceToHost));
  });
}

}  // extern "C"

namespace {

c2g::NciCut to_cut(const c2g_nci_cut *c) {
  c2g::NciCut k;
  if (c) {
    k.rhocut = c->rhocut, k.dimcut = c->dimcut, k.rhoplot = c->rhoplot;
    k.srho_lo = c->srho_lo, k.srho_hi = c->srho_hi, k.onlyneg = c->onlyneg;
  } else {
    // critic2's defaults for a density field (src/nci@proc.f90:141-168)
    k.rhocut = 0.2, k.dimcut = 2.0, k.rhoplot = 0.1, k.srho_lo = -1e30, k.srho_hi = 1e30, k.onlyneg = 0;
  }
  return k;
}

void put_cube_header(std::string &o, const char *l1, const char *l2, const HostWfn &w, const double *x0,
                     const double *xmat, const int *nstep) {
  // src/nci@proc.f90:818-914 for a molecule without fragments: the atoms
  // inside the cube (0.1 bohr margin), or all atoms when none is inside
  char b[160];
  double x1[3];
  for (int c = 0; c < 3; c++)
    x1[c] = x0[c] + (nstep[0] - 1) * xmat[c] + (nstep[1] - 1) * xmat[3 + c] + (nstep[2] - 1) * xmat[6 + c];
  std::vector<int> in;
  for (int a = 0; a < w.natom; a++) {
    bool ok = true;
    for (int c = 0; c < 3; c++) {
      const double lo = std::min(x0[c], x1[c]) - 0.1, hi = std::max(x0[c], x1[c]) + 0.1;
      ok = ok && w.xyz[3 * a + c] > lo && w.xyz[3 * a + c] < hi;
    }
    if (ok) in.push_back(a);
  }
  if (in.empty())
    for (int a = 0; a < w.natom; a++) in.push_back(a);
  o += " ";
  o += l1;
  o += "\n ";
  o += l2;
  o += "\n";
  std::snprintf(b, sizeof b, "%5d%12.6f%12.6f%12.6f\n", (int)in.size(), x0[0], x0[1], x0[2]);
  o += b;
  for (int c = 0; c < 3; c++) {
    std::snprintf(b, sizeof b, "%5d%12.6f%12.6f%12.6f\n", nstep[c], xmat[3 * c], xmat[3 * c + 1], xmat[3 * c + 2]);
    o += b;
  }
  for (int a : in) {
    std::snprintf(b, sizeof b, "%4d%5.1f%11.6f%11.6f%11.6f\n", w.z[a], 0.0, w.xyz[3 * a], w.xyz[3 * a + 1],
                  w.xyz[3 * a + 2]);
    o += b;
  }
}

void write_file(const std::string &path, const std::string &head, const char *body, size_t nbody) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) fail(C2G_ERR_IO, "cannot open " + path + " for writing");
  const bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size() &&
                  (nbody == 0 || std::fwrite(body, 1, nbody, f) == nbody);
  if (std::fclose(f) != 0 || !ok) fail(C2G_ERR_IO, "write failed: " + path);
}

// writegrid_cube's precise header (src/crystalmod@write.f90:3527-3545): all
// atoms, in the frame of the handle
void put_precise_header(std::string &o, const HostWfn &w, const double *x0, const double *xmat,
                        const int *nstep) {
  char f[3][24], b[160];
  auto e22 = [&](double x, char *out) {
    fmt_E22_14E3(x, out);
    out[22] = 0;
  };
  o += "critic2-cube\ncritic2-cube\n";
  for (int c = 0; c < 3; c++) e22(x0[c], f[c]);
  std::snprintf(b, sizeof b, "%5d %s %s %s \n", w.natom, f[0], f[1], f[2]);
  o += b;
  for (int i = 0; i < 3; i++) {
    for (int c = 0; c < 3; c++) e22(xmat[3 * i + c], f[c]);
    std::snprintf(b, sizeof b, "%5d %s %s %s \n", nstep[i], f[0], f[1], f[2]);
    o += b;
  }
  for (int a = 0; a < w.natom; a++) {
    for (int c = 0; c < 3; c++) e22(w.xyz[3 * a + c], f[c]);
    std::snprintf(b, sizeof b, "%5d %5.1f %s %s %s \n", w.z[a], 0.0, f[0], f[1], f[2]);
    o += b;
  }
}

double ms_since(std::chrono::steady_clock::time_point t) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

}  // namespace

extern "C" {

int c2g_nci_post_dev(const int *nstep, const double *d_crho, double *d_cgrad, const c2g_nci_cut *cut,
                     double *d_dat, long cap, long *ndat, void *stream) {
  return guarded([&] {
    require(nstep && d_crho && d_cgrad && ndat && (cap == 0 || d_dat), "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    const long n = (long)nstep[0] * nstep[1] * nstep[2];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf bc(sizeof(int) * ((n + 255) / 256)), tot(sizeof(long));
    *ndat = nci_post_dev(nstep, d_crho, d_cgrad, to_cut(cut), d_dat, cap, bc.as<int>(), tot.as<long>(), st);
  });
}

int c2g_cube_text(const int *nstep, const double *d_values, char *text, long cap, long *nbytes, void *stream) {
  return guarded([&] {
    require(nstep && d_values && nbytes, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    const long nb = cube_body_bytes(nstep);
    *nbytes = nb;
    if (!text) return;
    if (cap < nb) fail(C2G_ERR_ARG, "text buffer too small (" + std::to_string(nb) + " bytes needed)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf dt(nb), sc(sizeof(int) * cube_flag_scratch_ints());
    cube_text_dev(nstep, d_values, dt.as<char>(), text, sc.as<int>(), st);
  });
}

int c2g_dat_text(const double *d_dat, long ndat, char *text, long cap, long *nbytes, void *stream) {
  return guarded([&] {
    require(ndat >= 0 && nbytes && (ndat == 0 || d_dat), "bad argument");
    const long nb = 31 * ndat;
    *nbytes = nb;
    if (!text || ndat == 0) return;
    if (cap < nb) fail(C2G_ERR_ARG, "text buffer too small (" + std::to_string(nb) + " bytes needed)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf dt(nb), sc(sizeof(int) * cube_flag_scratch_ints());
    dat_text_dev(d_dat, ndat, dt.as<char>(), text, sc.as<int>(), st);
  });
}

int c2g_grid_field_dev(c2g_wfn *hp, const double *x0, const double *xmat, const int *nstep, int prec, int prop,
                       double *d_out, void *stream) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(x0 && xmat && nstep && d_out, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    require(prop >= 0 && prop <= 11, "unknown field property");
    check_prec(prec);
    DeviceGuard g(h->device);
    GridSpec gs;
    for (int j = 0; j < 3; j++) gs.x0[j] = x0[j], gs.nstep[j] = nstep[j];
    for (int j = 0; j < 9; j++) gs.xmat[j] = xmat[j];
    field_grid_dev(*h, gs, prec, prop, d_out, static_cast<cudaStream_t>(stream));
  });
}

int c2g_cube_precise_text(const int *nstep, const double *d_values, char *text, long cap, long *nbytes,
                          void *stream) {
  return guarded([&] {
    require(nstep && d_values && nbytes, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    const long nb = precise_body_bytes(nstep);
    *nbytes = nb;
    if (!text) return;
    if (cap < nb) fail(C2G_ERR_ARG, "text buffer too small (" + std::to_string(nb) + " bytes needed)");
    DevBuf dt(nb), sc(sizeof(int) * cube_flag_scratch_ints());
    precise_text_dev(nstep, d_values, dt.as<char>(), text, sc.as<int>(), static_cast<cudaStream_t>(stream));
  });
}

int c2g_cube_field_file(c2g_wfn *hp, const double *x0, const double *xmat, const int *nstep, int prec, int prop,
                        const char *path, double *ms_parts) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(x0 && xmat && nstep && path, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    DeviceGuard g(h->device);
    const long n = (long)nstep[0] * nstep[1] * nstep[2];
    auto t0 = std::chrono::steady_clock::now();
    DevBuf dv(sizeof(double) * n);
    int rc = c2g_grid_field_dev(hp, x0, xmat, nstep, prec, prop, dv.as<double>(), nullptr);
    if (rc != C2G_OK) fail(rc, g_last_error);
    const double t_eval = ms_since(t0);
    auto t1 = std::chrono::steady_clock::now();
    const long nb = precise_body_bytes(nstep);
    std::vector<char> ht(nb);
    {
      DevBuf dt(nb), sc(sizeof(int) * cube_flag_scratch_ints());
      precise_text_dev(nstep, dv.as<double>(), dt.as<char>(), ht.data(), sc.as<int>(), nullptr);
    }
    const double t_fmt = ms_since(t1);
    auto t2 = std::chrono::steady_clock::now();
    std::string head;
    put_precise_header(head, h->host, x0, xmat, nstep);
    write_file(path, head, ht.data(), nb);
    if (ms_parts) {
      ms_parts[0] = t_eval;
      ms_parts[1] = t_fmt;
      ms_parts[2] = ms_since(t2);
    }
  });
}

int c2g_nciplot_files(c2g_wfn *hp, const double *x0, const double *xmat, const int *nstep, int prec,
                      const char *root, const c2g_nci_cut *cut, c2g_nci_stats *stats, double *ms_parts) {
  return guarded([&] {
    Handle *h = check_handle(hp);
    require(x0 && xmat && nstep && root, "null argument");
    require(nstep[0] > 0 && nstep[1] > 0 && nstep[2] > 0, "nstep must be positive");
    DeviceGuard g(h->device);
    const long n = (long)nstep[0] * nstep[1] * nstep[2];
    auto t0 = std::chrono::steady_clock::now();
    DevBuf dr(sizeof(double) * n), dg(sizeof(double) * n);
    int rc = c2g_nciplot_dev(hp, x0, xmat, nstep, prec, dr.as<double>(), dg.as<double>(), nullptr, stats);
    if (rc != C2G_OK) fail(rc, g_last_error);
    C2G_CUDA(cudaDeviceSynchronize());
    const double t_eval = ms_since(t0);
    auto t1 = std::chrono::steady_clock::now();
    DevBuf dd(sizeof(double) * 2 * n), bc(sizeof(int) * ((n + 255) / 256)), tot(sizeof(long));
    const long ndat = nci_post_dev(nstep, dr.as<double>(), dg.as<double>(), to_cut(cut), dd.as<double>(), n,
                                   bc.as<int>(), tot.as<long>(), nullptr);
    const double t_post = ms_since(t1);
    auto t2 = std::chrono::steady_clock::now();
    const long nb = cube_body_bytes(nstep);
    std::vector<char> hd(nb), hg(nb), ht((size_t)std::max(1L, 31 * ndat));
    {
      DevBuf dt(std::max(nb, 31 * ndat)), sc(sizeof(int) * cube_flag_scratch_ints());
      cube_text_dev(nstep, dr.as<double>(), dt.as<char>(), hd.data(), sc.as<int>(), nullptr);
      cube_text_dev(nstep, dg.as<double>(), dt.as<char>(), hg.data(), sc.as<int>(), nullptr);
      dat_text_dev(dd.as<double>(), ndat, dt.as<char>(), ht.data(), sc.as<int>(), nullptr);
    }
    const double t_fmt = ms_since(t2);
    auto t3 = std::chrono::steady_clock::now();
    std::string hdens, hgrad;
    put_cube_header(hdens, "dens_cube", "3d plot, density", h->host, x0, xmat, nstep);
    put_cube_header(hgrad, "grad_cube", "3d plot, reduced density gradient", h->host, x0, xmat, nstep);
    const std::string r(root);
    write_file(r + "-dens.cube", hdens, hd.data(), nb);
    write_file(r + "-grad.cube", hgrad, hg.data(), nb);
    write_file(r + ".dat", std::string(), ht.data(), (size_t)(31 * ndat));
    if (ms_parts) {
      ms_parts[0] = t_eval;
      ms_parts[1] = t_post;
      ms_parts[2] = t_fmt;
      ms_parts[3] = ms_since(t3);
    }
  });
}

}  // extern "C"
