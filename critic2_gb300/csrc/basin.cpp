// Atomic-basin integrals by bisection of the zero-flux surface: critic2's
// INTEGRALS keyword (src/bisect@proc.f90:862-1028) for a molecular
// wavefunction field, with every ray of every attractor traced at once.
//
// Per attractor (the nuclei, then the CPs of the nuclear type, -3) and ray
// (a Lebedev or Gauss-Legendre angular node), bisect_msurface
// (src/bisect@proc.f90:1208-1446) brackets the surface between an inner
// point whose upward gradient path ends at the attractor and an outer point
// whose path does not, and lim_surf (:1039-1126) bisects the bracket to
// within the IAS precision, restarting with a smaller beta sphere when the
// surface point falls inside one.  Every ray runs on the device
// (k_gpath.cu): its state machine, its gradient paths (gpath.h) and the
// FP64 evaluations they need, one block per ray, no host round trip.  The
// integrals follow integrals_lebedev / integrals_gauleg (:1638-1877): a
// beta sphere of 0.95 times the smallest surface radius integrated on a
// 170-point Lebedev rule (sphereintegrals_lebedev, :829-854), plus each
// ray's radial Gauss-Legendre quadrature (50 nodes) from the beta sphere to
// the surface (int_radialquad, src/integration@proc.f90:384-486), summed as
// lebedev_mquad (:591-642) or gauleg_mquad (:495-582).  The integrated
// properties are critic2's molecular defaults (set_default_integprop,
// src/systemmod@proc.f90:171-203): the valence density (Pop) and its
// Laplacian (Lap), evaluated in FP64 in one batch.
//
// One difference from the reference, for parallel rays: bisect_msurface
// seeds a ray's bracket from running means over the rays finished before it
// (OpenMP order); here every ray takes the bracket tries of the first ray
// (the same rule in every order), so the brackets, and with them the
// bisection's end points, can differ from a serial run by up to the IAS
// precision.  Beta-sphere shrinking (lim_surf's restart) acts on the ray's
// own copy of the radii (in the reference it persists for the rays and
// attractors that follow, in whatever order the threads reach them), so
// that every ray's result is independent of the others.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
#include <numeric>
#include <vector>

#include "c2g_internal.h"
#include "gpath.h"
#include "k_gpath.h"

namespace c2g {
namespace {

using namespace gpath;

// The handle's device for the call, the caller's afterwards.
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

// Device scratch owned by one call.
struct DevBuf {
  void *p = nullptr;
  explicit DevBuf(size_t bytes) {
    const cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) fail(C2G_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

constexpr int kSphereLeb = 170;                        // bs_spherequad_nleb
constexpr int kRadNodes = 50;                          // INT_radquad_nr (Gauss-Legendre)
constexpr double kVBig = std::numeric_limits<double>::max();
constexpr int kNProp = 2;                              // Pop, Lap

// good_lebedev (src/tools_math@lebedev.f90:105-124): the smallest rule with
// at least n points (5810 above that).
int good_lebedev(int n) {
  static const int sizes[] = {6,    14,   26,   38,   50,   74,   86,   110,  146,  170,  194,
                              230,  266,  302,  350,  434,  590,  770,  974,  1202, 1454, 1730,
                              2030, 2354, 2702, 3074, 3470, 3890, 4334, 4802, 5294, 5810};
  for (int s : sizes)
    if (n <= s) return s;
  return 5810;
}

// One angular node of the integration surface: the direction critic2
// rebuilds from (theta, phi) and the node's weight.
struct Node {
  double th, ph, u[3];
};

void set_unit(Node &n) {
  n.u[0] = std::sin(n.th) * std::cos(n.ph);
  n.u[1] = std::sin(n.th) * std::sin(n.ph);
  n.u[2] = std::cos(n.th);
}

// lebedev_nodes (src/surface@proc.f90:906-928); w: weights times 4 pi.
void lebedev_nodes(int n, std::vector<Node> &nodes, std::vector<double> &w) {
  const std::vector<double4> r = lebedev_points(n);
  nodes.resize(r.size());
  w.resize(r.size());
  for (size_t i = 0; i < r.size(); i++) {
    nodes[i].th = std::acos(r[i].z);
    nodes[i].ph = std::atan2(r[i].y, r[i].x);
    set_unit(nodes[i]);
    w[i] = r[i].w * (4.0 * M_PI);
  }
}

// gauleg_nodes (src/surface@proc.f90:863-896): ntheta Gauss-Legendre polar
// nodes on (0, pi), int(nphi |sin theta|) + 1 azimuthal ones on (0, 2 pi).
void gauleg_nodes(int ntheta, int nphi, std::vector<Node> &nodes, std::vector<int> &ring) {
  std::vector<double> tp, tw, pp, pw;
  gauleg(0.0, M_PI, ntheta, tp, tw);
  nodes.clear();
  ring.clear();
  for (int j = 0; j < ntheta; j++) {
    const int np = (int)(nphi * std::fabs(std::sin(tp[j]))) + 1;
    gauleg(0.0, 2.0 * M_PI, np, pp, pw);
    for (int k = 0; k < np; k++) {
      Node n;
      n.th = tp[j];
      n.ph = pp[k];
      set_unit(n);
      nodes.push_back(n);
      ring.push_back(j);
    }
  }
}

struct Attractor {
  int cp;           // index in the CP list
  double x[3];      // position
  int typ;          // its CP type
  double rmin, rminsame;
};

int num_sms() {
  int dev = 0, n = 0;
  C2G_CUDA(cudaGetDevice(&dev));
  C2G_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  return n;
}

template <class T>
T *upload(std::deque<DevBuf> &keep, const std::vector<T> &v) {
  keep.emplace_back(sizeof(T) * std::max<size_t>(v.size(), 1));
  if (!v.empty()) C2G_CUDA(cudaMemcpy(keep.back().p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return keep.back().as<T>();
}

template <class T>
std::vector<T> download(const T *d, size_t n) {
  std::vector<T> v(n);
  if (n) C2G_CUDA(cudaMemcpy(v.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost));
  return v;
}

struct SearchOut {
  std::vector<double> r;
  long npath = 0, nevals = 0;
  int nwarn = 0, nrestart = 0;
};

// The surfaces of every (attractor, node) ray, traced on the device
// (k_gpath.cu): one block per ray at a time.
SearchOut search_surfaces(Handle &h, int nc, const std::vector<double> &cpx, const std::vector<int> &typ,
                          const std::vector<Attractor> &att, const std::vector<Node> &nodes, double prec) {
  const HostWfn &w = h.host;
  const int natt = (int)att.size(), nray = (int)nodes.size();
  const long nr = (long)natt * nray;
  std::deque<DevBuf> keep;  // device arrays of the search (not relocated)
  std::vector<double> ax(3 * natt), rmin(natt), rms(natt), ru(3 * nray);
  std::vector<int> at(natt);
  for (int a = 0; a < natt; a++) {
    for (int j = 0; j < 3; j++) ax[3 * a + j] = att[a].x[j];
    rmin[a] = att[a].rmin, rms[a] = att[a].rminsame, at[a] = att[a].typ;
  }
  for (int i = 0; i < nray; i++)
    for (int j = 0; j < 3; j++) ru[3 * i + j] = nodes[i].u[j];
  PathGeom g = host_geom(w);
  g.xyz = upload(keep, w.xyz);
  g.z = upload(keep, w.z);
  BasinDev b{};
  b.ncp = nc;
  b.cpx = upload(keep, cpx);
  b.cptyp = upload(keep, typ);
  b.prec = prec;
  b.amin = std::min({w.cell_aa[0], w.cell_aa[1], w.cell_aa[2]});
  b.amax = std::max({w.cell_aa[0], w.cell_aa[1], w.cell_aa[2]});
  b.natt = natt;
  b.nray = nray;
  b.att_x = upload(keep, ax);
  b.att_typ = upload(keep, at);
  b.att_rmin = upload(keep, rmin);
  b.att_rminsame = upload(keep, rms);
  b.ray_u = upload(keep, ru);
  const int grid = (int)std::max(1L, std::min(nr, (long)num_sms() * 3));
  keep.emplace_back(sizeof(double) * (size_t)grid * std::max(nc, 1));
  b.rbeta_scratch = keep.back().as<double>();
  keep.emplace_back(sizeof(double) * std::max(nr, 1L));
  b.rsurf = keep.back().as<double>();
  int **ints[4] = {&b.ray_npath, &b.ray_nwarn, &b.ray_nrestart, &b.ray_err};
  for (int **q : ints) {
    keep.emplace_back(sizeof(int) * std::max(nr, 1L));
    *q = keep.back().as<int>();
  }
  keep.emplace_back(sizeof(long) * std::max(nr, 1L));
  b.ray_nevals = keep.back().as<long>();
  keep.emplace_back(sizeof(unsigned long long));
  b.ray_next = keep.back().as<unsigned long long>();
  C2G_CUDA(cudaMemset(b.ray_next, 0, sizeof(unsigned long long)));
  SearchOut out;
  if (nr > 0) {
    launch_basin_rays(h.dev, g, b, grid, 0);
    C2G_CUDA(cudaDeviceSynchronize());
  }
  out.r = download(b.rsurf, nr);
  const std::vector<int> np = download(b.ray_npath, nr), nw = download(b.ray_nwarn, nr),
                         rs = download(b.ray_nrestart, nr), er = download(b.ray_err, nr);
  const std::vector<long> ne = download(b.ray_nevals, nr);
  for (long i = 0; i < nr; i++) {
    if (er[i]) {
      static const char *why[4] = {"", "can not find ray limits", "too many beta-sphere restarts",
                                   "evaluation limit reached"};
      fail(C2G_ERR_NUMERIC, std::string("basin bisection: ") + why[er[i] & 3] + " (attractor " +
                                std::to_string(att[i / nray].cp) + ", ray " + std::to_string(i % nray) + ")");
    }
    out.npath += np[i], out.nevals += ne[i], out.nwarn += nw[i], out.nrestart += rs[i];
  }
  return out;
}

// Valence density and its Laplacian at n host points (FP64, the EDF core
// left out: grdall's fval and del2fval), in chunks.
void eval_props(Handle &h, const std::vector<double> &xyz, std::vector<double> &prop) {
  const size_t n = xyz.size() / 3;
  prop.assign(kNProp * n, 0.0);
  const size_t chunk = 1 << 20;
  DevBuf dx(sizeof(double) * 3 * std::min(n, chunk) + 8), dr(sizeof(double) * kRecNci * std::min(n, chunk) + 8);
  std::vector<double> rec(kRecNci * std::min(n, chunk));
  DevWfn dw = h.dev;
  dw.nedf = 0;
  for (size_t i0 = 0; i0 < n; i0 += chunk) {
    const int m = (int)std::min(chunk, n - i0);
    C2G_CUDA(cudaMemcpy(dx.p, xyz.data() + 3 * i0, sizeof(double) * 3 * m, cudaMemcpyHostToDevice));
    launch_fp64_points(dw, m, dx.as<double>(), 2, false, dr.as<double>(), 0);
    C2G_CUDA(cudaMemcpy(rec.data(), dr.p, sizeof(double) * kRecNci * m, cudaMemcpyDeviceToHost));
    for (int i = 0; i < m; i++) {
      const double *q = rec.data() + (size_t)i * kRecNci;
      prop[kNProp * (i0 + i)] = q[0];
      prop[kNProp * (i0 + i) + 1] = q[4] + q[5] + q[6];
    }
  }
}

// The attractors of INTEGRALS (:936-970): the nuclei, then the CPs of the
// nuclear type; cpid > 0 selects one (1-based, as critic2's CP keyword).
std::vector<int> attractor_list(const HostWfn &w, int ncp, const int *cptyp, int cpid) {
  std::vector<int> out;
  const int lo = cpid > 0 ? cpid - 1 : 0, hi = cpid > 0 ? cpid : ncp;
  for (int i = lo; i < hi; i++)
    if (i < w.natom || cptyp[i] == -3) out.push_back(i);
  return out;
}

void check_cp_list(const HostWfn &w, int ncp, const double *cpx, const int *cptyp) {
  if (ncp < w.natom) fail(C2G_ERR_ARG, "the CP list must start with the nuclei");
  for (int a = 0; a < w.natom; a++)
    for (int j = 0; j < 3; j++)
      if (std::fabs(cpx[3 * a + j] - w.xyz[3 * a + j]) > 1e-8)
        fail(C2G_ERR_ARG, "the CP list must start with the nuclei in atom order");
  for (int i = 0; i < ncp; i++)
    if (cptyp[i] != -3 && cptyp[i] != -1 && cptyp[i] != 1 && cptyp[i] != 3)
      fail(C2G_ERR_ARG, "CP types must be -3, -1, 1 or 3");
}

int ray_count(int meth, int n1, int n2) {
  if (meth == C2G_INT_LEBEDEV) {
    if (n1 <= 0) fail(C2G_ERR_ARG, "Lebedev rule size must be positive");
    return good_lebedev(n1);
  }
  if (meth == C2G_INT_GAULEG) {
    if (n1 <= 0 || n2 <= 0) fail(C2G_ERR_ARG, "ntheta and nphi must be positive");
    std::vector<Node> nodes;
    std::vector<int> ring;
    gauleg_nodes(n1, n2, nodes, ring);
    return (int)nodes.size();
  }
  fail(C2G_ERR_ARG, "unknown integration method");
  return 0;
}

}  // namespace
}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_basin_size(c2g_wfn *hp, int ncp, const int *cp_typ, int meth, int n1, int n2, int cpid, int *natt,
                   int *nray) {
  return guarded([&] {
    if (!hp) fail(C2G_ERR_ARG, "null handle");
    const Handle &h = *reinterpret_cast<Handle *>(hp);
    if (ncp < 0 || (ncp > 0 && !cp_typ)) fail(C2G_ERR_ARG, "bad CP list");
    if (cpid < 0 || cpid > std::max(ncp, h.host.natom)) fail(C2G_ERR_ARG, "cpid out of range");
    const int nr = ray_count(meth, n1, n2);
    std::vector<int> typ(cp_typ, cp_typ + ncp);
    if (ncp == 0) typ.assign(h.host.natom, -3);
    if (natt) *natt = (int)attractor_list(h.host, (int)typ.size(), typ.data(), cpid).size();
    if (nray) *nray = nr;
  });
}

int c2g_basin_integrals(c2g_wfn *hp, int ncp, const double *cp_xyz, const int *cp_typ, int meth, int n1, int n2,
                        int cpid, double iasprec, int *att_cp, double *props, double *iaserr, double *rays,
                        double *rsurf, double *rbeta_int, c2g_basin_stats *stats) {
  return guarded([&] {
    if (!hp) fail(C2G_ERR_ARG, "null handle");
    Handle &h = *reinterpret_cast<Handle *>(hp);
    const HostWfn &w = h.host;
    if (ncp < 0 || (ncp > 0 && (!cp_xyz || !cp_typ))) fail(C2G_ERR_ARG, "bad CP list");
    if (!props) fail(C2G_ERR_ARG, "null props");
    if (!(iasprec > 0.0)) fail(C2G_ERR_ARG, "iasprec must be positive");
    const auto t0 = std::chrono::steady_clock::now();
    DeviceGuard guard(h.device);
    // the CP list (the nuclei alone when none is given)
    std::vector<double> cpx(cp_xyz, cp_xyz + 3 * (size_t)ncp);
    std::vector<int> typ(cp_typ, cp_typ + ncp);
    if (ncp == 0) {
      cpx = w.xyz;
      typ.assign(w.natom, -3);
    }
    const int nc = (int)typ.size();
    check_cp_list(w, nc, cpx.data(), typ.data());
    if (cpid < 0 || cpid > nc) fail(C2G_ERR_ARG, "cpid out of range");
    // angular nodes of the surface
    std::vector<Node> nodes;
    std::vector<double> lw;
    std::vector<int> ring;
    if (meth == C2G_INT_LEBEDEV) lebedev_nodes(ray_count(meth, n1, n2), nodes, lw);
    else if (meth == C2G_INT_GAULEG) gauleg_nodes(n1, n2, nodes, ring);
    else fail(C2G_ERR_ARG, "unknown integration method");
    const int nray = (int)nodes.size();
    // attractors, with the distances to the nearest CP and the nearest one
    // of the same type (:1243-1255)
    const std::vector<int> ai = attractor_list(w, nc, typ.data(), cpid);
    std::vector<Attractor> att(ai.size());
    for (size_t a = 0; a < ai.size(); a++) {
      Attractor &t = att[a];
      t.cp = ai[a];
      t.typ = typ[ai[a]];
      for (int j = 0; j < 3; j++) t.x[j] = cpx[3 * ai[a] + j];
      t.rmin = t.rminsame = kVBig;
      for (int c = 0; c < nc; c++) {
        double d2 = 0.0;
        for (int j = 0; j < 3; j++) d2 += (cpx[3 * c + j] - t.x[j]) * (cpx[3 * c + j] - t.x[j]);
        const double d = std::sqrt(d2);
        if (d < 1e-5) continue;
        t.rmin = std::min(t.rmin, d);
        if (typ[c] == t.typ) t.rminsame = std::min(t.rminsame, d);
      }
    }
    // the surfaces
    const SearchOut so = search_surfaces(h, nc, cpx, typ, att, nodes, iasprec);
    const std::vector<double> &r = so.r;
    // quadrature points: each attractor's beta sphere, then its rays and the
    // rays' surface points (the IAS error estimate)
    std::vector<Node> snodes;
    std::vector<double> sw;
    lebedev_nodes(kSphereLeb, snodes, sw);
    const int natt = (int)att.size();
    std::vector<double> rb(natt), xyz;
    const size_t per_att = (size_t)kSphereLeb * kRadNodes + (size_t)nray * (kRadNodes + 1);
    xyz.reserve(3 * per_att * natt);
    std::vector<std::vector<double>> rad_r(natt * (size_t)(nray + 1)), rad_w(natt * (size_t)(nray + 1));
    for (int a = 0; a < natt; a++) {
      double rmin = kVBig;
      for (int j = 0; j < nray; j++) rmin = std::min(rmin, r[(size_t)a * nray + j]);
      rb[a] = 0.95 * rmin;
      // sphere: (0, rb) on every node of the 170-point rule
      std::vector<double> &sr = rad_r[(size_t)a * (nray + 1)], &swr = rad_w[(size_t)a * (nray + 1)];
      gauleg(0.0, rb[a], kRadNodes, sr, swr);
      for (int i = 0; i < kSphereLeb; i++)
        for (int k = 0; k < kRadNodes; k++)
          for (int j = 0; j < 3; j++) xyz.push_back(att[a].x[j] + sr[k] * snodes[i].u[j]);
      // rays: (rb, r_j) and the surface point
      for (int i = 0; i < nray; i++) {
        const double re = r[(size_t)a * nray + i];
        double r1 = rb[a], r2 = re;
        if (r2 < r1) std::swap(r1, r2);
        std::vector<double> &rr = rad_r[(size_t)a * (nray + 1) + 1 + i], &rw = rad_w[(size_t)a * (nray + 1) + 1 + i];
        gauleg(r1, r2, kRadNodes, rr, rw);
        for (int k = 0; k < kRadNodes; k++)
          for (int j = 0; j < 3; j++) xyz.push_back(att[a].x[j] + rr[k] * nodes[i].u[j]);
        for (int j = 0; j < 3; j++) xyz.push_back(att[a].x[j] + re * nodes[i].u[j]);
      }
    }
    std::vector<double> prop;
    eval_props(h, xyz, prop);
    // sums in the reference's order
    size_t ip = 0;
    for (int a = 0; a < natt; a++) {
      double sprop[kNProp] = {0, 0}, lprop[kNProp] = {0, 0}, ierr[kNProp] = {0, 0};
      const std::vector<double> &sr = rad_r[(size_t)a * (nray + 1)], &swr = rad_w[(size_t)a * (nray + 1)];
      for (int i = 0; i < kSphereLeb; i++) {
        double rp[kNProp] = {0, 0};
        for (int k = 0; k < kRadNodes; k++, ip++)
          for (int q = 0; q < kNProp; q++) rp[q] += sr[k] * sr[k] * swr[k] * prop[kNProp * ip + q];
        for (int q = 0; q < kNProp; q++) sprop[q] += rp[q] * sw[i];
      }
      std::vector<double> rp(kNProp * (size_t)nray), re(kNProp * (size_t)nray);
      for (int i = 0; i < nray; i++) {
        const std::vector<double> &rr = rad_r[(size_t)a * (nray + 1) + 1 + i],
                                  &rw = rad_w[(size_t)a * (nray + 1) + 1 + i];
        const double rend = r[(size_t)a * nray + i];
        const double sg = rend > rb[a] ? 1.0 : -1.0;
        double acc[kNProp] = {0, 0};
        for (int k = 0; k < kRadNodes; k++, ip++)
          for (int q = 0; q < kNProp; q++) acc[q] += rr[k] * rr[k] * rw[k] * prop[kNProp * ip + q];
        for (int q = 0; q < kNProp; q++) {
          rp[kNProp * i + q] = acc[q] * sg;
          re[kNProp * i + q] = std::fabs(prop[kNProp * ip + q] * rend * rend * iasprec);
        }
        ip++;
      }
      if (meth == C2G_INT_LEBEDEV) {
        for (int i = 0; i < nray; i++)
          for (int q = 0; q < kNProp; q++) lprop[q] += rp[kNProp * i + q] * lw[i], ierr[q] += re[kNProp * i + q] * lw[i];
      } else {
        // gauleg_mquad: per polar ring, the azimuthal sum, then sin(theta)
        // times the polar weight
        std::vector<double> tp, tw, pp, pw;
        gauleg(0.0, M_PI, n1, tp, tw);
        int v = 0;
        for (int t = 0; t < n1; t++) {
          const int np = (int)(n2 * std::fabs(std::sin(tp[t]))) + 1;
          gauleg(0.0, 2.0 * M_PI, np, pp, pw);
          double pr[kNProp] = {0, 0}, pe[kNProp] = {0, 0};
          for (int k = 0; k < np; k++, v++)
            for (int q = 0; q < kNProp; q++) pr[q] += rp[kNProp * v + q] * pw[k], pe[q] += re[kNProp * v + q] * pw[k];
          const double f = std::sin(nodes[v - 1].th) * tw[t];
          for (int q = 0; q < kNProp; q++) lprop[q] += f * pr[q], ierr[q] += f * pe[q];
        }
      }
      for (int q = 0; q < kNProp; q++) {
        props[kNProp * a + q] = lprop[q] + sprop[q];
        if (iaserr) iaserr[kNProp * a + q] = ierr[q];
      }
      if (att_cp) att_cp[a] = att[a].cp;
      if (rbeta_int) rbeta_int[a] = rb[a];
      if (rsurf)
        for (int i = 0; i < nray; i++) rsurf[(size_t)a * nray + i] = r[(size_t)a * nray + i];
    }
    if (rays)
      for (int i = 0; i < nray; i++)
        for (int j = 0; j < 3; j++) rays[3 * i + j] = nodes[i].u[j];
    if (stats) {
      stats->natt = natt;
      stats->nray = nray;
      stats->npath = so.npath;
      stats->nbatch = 1;
      stats->nevals = so.nevals + (long)xyz.size() / 3;
      stats->nwarn = so.nwarn;
      stats->nrestart = so.nrestart;
      stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

// SPHEREINTEGRALS (src/bisect@proc.f90:573-784): for each attractor, Pop
// and Lap inside spheres of nr radii r0 exp(h (n - 1)) up to rend (rend < 0:
// |rend| times half the distance to the nearest atom, get_rnn2), each
// sphere by sphereintegrals_lebedev / _gauleg (:793-854): the angular rule
// times 50 radial Gauss-Legendre nodes on (0, r), summed as lebedev_mquad /
// gauleg_mquad.
int c2g_sphere_integrals(c2g_wfn *hp, int ncp, const double *cp_xyz, const int *cp_typ, int meth, int n1, int n2,
                         int cpid, int nr, double r0, double rend, int *att_cp, double *radii, double *props) {
  return guarded([&] {
    if (!hp) fail(C2G_ERR_ARG, "null handle");
    Handle &hd = *reinterpret_cast<Handle *>(hp);
    const HostWfn &w = hd.host;
    if (ncp < 0 || (ncp > 0 && (!cp_xyz || !cp_typ))) fail(C2G_ERR_ARG, "bad CP list");
    if (!props || !radii) fail(C2G_ERR_ARG, "null output");
    if (nr < 1) fail(C2G_ERR_ARG, "nr must be positive");
    if (!(r0 > 0.0)) fail(C2G_ERR_ARG, "r0 must be positive");
    DeviceGuard guard(hd.device);
    std::vector<double> cpx(cp_xyz, cp_xyz + 3 * (size_t)ncp);
    std::vector<int> typ(cp_typ, cp_typ + ncp);
    if (ncp == 0) {
      cpx = w.xyz;
      typ.assign(w.natom, -3);
    }
    const int nc = (int)typ.size();
    check_cp_list(w, nc, cpx.data(), typ.data());
    if (cpid < 0 || cpid > nc) fail(C2G_ERR_ARG, "cpid out of range");
    std::vector<Node> nodes;
    std::vector<double> lw;
    std::vector<int> ring;
    if (meth == C2G_INT_LEBEDEV) lebedev_nodes(ray_count(meth, n1, n2), nodes, lw);
    else if (meth == C2G_INT_GAULEG) gauleg_nodes(n1, n2, nodes, ring);
    else fail(C2G_ERR_ARG, "unknown integration method");
    const int nray = (int)nodes.size();
    std::vector<double> tp, tw;
    if (meth == C2G_INT_GAULEG) gauleg(0.0, M_PI, n1, tp, tw);
    const std::vector<int> ai = attractor_list(w, nc, typ.data(), cpid);
    for (size_t a = 0; a < ai.size(); a++) {
      const double *xa = cpx.data() + 3 * ai[a];
      // get_rnn2: half the distance to the nearest atom (0 for a lone atom)
      double rnn = kVBig;
      for (int b = 0; b < w.natom; b++) {
        double d2 = 0.0;
        for (int j = 0; j < 3; j++) d2 += (w.xyz[3 * b + j] - xa[j]) * (w.xyz[3 * b + j] - xa[j]);
        if (d2 > 0.0) rnn = std::min(rnn, std::sqrt(d2));
      }
      const double rnn2 = w.natom <= 1 ? 0.0 : 0.5 * rnn;
      const double lh = nr > 1 ? std::log((rend < 0.0 ? rnn2 * std::fabs(rend) : rend) / r0) / (nr - 1) : 0.0;
      std::vector<double> xyz, rr((size_t)nr * kRadNodes), rw((size_t)nr * kRadNodes);
      xyz.reserve(3 * (size_t)nr * nray * kRadNodes);
      for (int n = 0; n < nr; n++) {
        const double rad = nr == 1 ? (rend < 0.0 ? rnn2 * std::fabs(rend) : r0) : r0 * std::exp(n * lh);
        radii[a * (size_t)nr + n] = rad;
        std::vector<double> gr, gw;
        gauleg(0.0, rad, kRadNodes, gr, gw);
        std::copy(gr.begin(), gr.end(), rr.begin() + (size_t)n * kRadNodes);
        std::copy(gw.begin(), gw.end(), rw.begin() + (size_t)n * kRadNodes);
        for (int i = 0; i < nray; i++)
          for (int k = 0; k < kRadNodes; k++)
            for (int j = 0; j < 3; j++) xyz.push_back(xa[j] + gr[k] * nodes[i].u[j]);
      }
      std::vector<double> prop;
      eval_props(hd, xyz, prop);
      size_t ip = 0;
      for (int n = 0; n < nr; n++) {
        const double *gr = rr.data() + (size_t)n * kRadNodes, *gw = rw.data() + (size_t)n * kRadNodes;
        std::vector<double> rp(kNProp * (size_t)nray);
        for (int i = 0; i < nray; i++) {
          double acc[kNProp] = {0, 0};
          for (int k = 0; k < kRadNodes; k++, ip++)
            for (int q = 0; q < kNProp; q++) acc[q] += gr[k] * gr[k] * gw[k] * prop[kNProp * ip + q];
          for (int q = 0; q < kNProp; q++) rp[kNProp * i + q] = acc[q];
        }
        double sp[kNProp] = {0, 0};
        if (meth == C2G_INT_LEBEDEV) {
          for (int i = 0; i < nray; i++)
            for (int q = 0; q < kNProp; q++) sp[q] += rp[kNProp * i + q] * lw[i];
        } else {
          std::vector<double> pp, pw;
          int v = 0;
          for (int t = 0; t < n1; t++) {
            const int np = (int)(n2 * std::fabs(std::sin(tp[t]))) + 1;
            gauleg(0.0, 2.0 * M_PI, np, pp, pw);
            double pr[kNProp] = {0, 0};
            for (int k = 0; k < np; k++, v++)
              for (int q = 0; q < kNProp; q++) pr[q] += rp[kNProp * v + q] * pw[k];
            const double f = std::sin(nodes[v - 1].th) * tw[t];
            for (int q = 0; q < kNProp; q++) sp[q] += f * pr[q];
          }
        }
        for (int q = 0; q < kNProp; q++) props[(a * (size_t)nr + n) * kNProp + q] = sp[q];
      }
      if (att_cp) att_cp[a] = ai[a];
    }
  });
}

}  // extern "C"
