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
// surface point falls inside one.  Each ray is a small state machine over
// gradient paths; all rays' paths advance in lockstep (gpath.h), so one
// Bogacki-Shampine stage of every live path is one batch of FP64
// evaluations on the GPU.  The integrals follow integrals_lebedev /
// integrals_gauleg (:1638-1877): a beta sphere of 0.95 times the smallest
// surface radius integrated on a 170-point Lebedev rule
// (sphereintegrals_lebedev, :829-854), plus each ray's radial Gauss-Legendre
// quadrature (50 nodes) from the beta sphere to the surface
// (int_radialquad, src/integration@proc.f90:384-486), summed as
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
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

#include "c2g_internal.h"
#include "forkjoin.h"
#include "gpath.h"

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

constexpr double kBsRNearNuc = 3.1622776601683794e-3;  // bs_rnearnuc = sqrt(1e-5)
constexpr int kNTries = 7;                             // bisect_msurface's bracket tries
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

// One (attractor, ray) of the surface search.
struct Ray {
  int att = 0, node = 0;
  int phase = 0;  // 0 inner tries, 1 outer tries, 2 bisection, 3 done
  int k = 0;      // position in the sorted tries
  double rin[kNTries], rout[kNTries];  // tries, ascending
  double riaprox = 0.0, raprox = kVBig, rother = kVBig;
  double xin[3], xfin[3], xi[3], xf[3], xmed[3];
  double rlim = -1.0;
  int nwarn = 0;      // paths of this ray that ended with ier > 0
  int npath = 0, nrestart = 0;
  bool tracing = false;
  std::vector<double> rbeta;  // the ray's beta radii once it has shrunk one (else the defaults)
  Path path;
};

struct Attractor {
  int cp;           // index in the CP list
  double x[3];      // position
  int typ;          // its CP type
  double rmin, rminsame;
};

class BasinSearch {
 public:
  BasinSearch(Handle &h, int ncp, const double *cpx, const int *cptyp, const std::vector<double> &rbeta,
              const std::vector<Attractor> &att, const std::vector<Node> &nodes, double prec)
      : h_(h), w_(h.host), ncp_(ncp), cpx_(cpx), cptyp_(cptyp), rbeta_(rbeta), att_(att), nodes_(nodes),
        prec_(prec) {}

  // Surface radii r[att * nray + ray]; counts of paths, warnings, restarts.
  void run(std::vector<double> &r) {
    const int nray = (int)nodes_.size(), natt = (int)att_.size();
    rays_.resize((size_t)natt * nray);
    const double amin = std::min({w_.cell_aa[0], w_.cell_aa[1], w_.cell_aa[2]});
    const double amax = std::max({w_.cell_aa[0], w_.cell_aa[1], w_.cell_aa[2]});
    for (int a = 0; a < natt; a++)
      for (int j = 0; j < nray; j++) {
        Ray &y = rays_[(size_t)a * nray + j];
        y.att = a, y.node = j;
        // bracket tries of bisect_msurface's first ray (:1290-1308,
        // :1332-1350), each list sorted ascending (qcksort)
        const double ti[kNTries] = {2e-5, 0.9 * att_[a].rmin, 0.99 * att_[a].rmin, 0.0, 0.0, 0.0, 0.0};
        const double to[kNTries] = {amin, 0.99 * att_[a].rminsame, 0.75 * att_[a].rminsame, amax, amax, amax, amax};
        std::copy(ti, ti + kNTries, y.rin);
        std::copy(to, to + kNTries, y.rout);
        std::sort(y.rin, y.rin + kNTries);
        std::sort(y.rout, y.rout + kNTries);
        y.phase = 0;
        y.k = kNTries - 1;
        next_inner(y);
      }
    const long nr = (long)rays_.size();
    BatchGrd bg(h_, std::max(1, (int)nr));
    std::vector<double> xs(3 * nr);
    std::vector<int> who(nr);
    std::vector<char> need(nr);
    // host threads for the rays' step logic (the rays are independent)
    const int hw = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
    ForkJoin pool((int)std::max(1L, std::min((long)hw, nr / 64)));
    for (;;) {
      pool.run(nr, [&](long b, long e) {
        for (long i = b; i < e; i++) {
          Ray &y = rays_[i];
          while (y.tracing) {
            Path &p = y.path;
            if (p.stage == 0) {
              if (head(p, w_, ncp_, cpx_, cptyp_, y.rbeta.empty() ? rbeta_.data() : y.rbeta.data())) {
                request_stage1(p);
                break;
              }
              p.done = true;
            }
            if (p.done) {
              y.tracing = false;
              if (p.incstep) p.nstep++;
              path_done(y);  // may start the ray's next path
              continue;
            }
            break;
          }
          need[i] = y.tracing;
        }
      });
      int m = 0;
      for (long i = 0; i < nr; i++)
        if (need[i]) who[m++] = (int)i;
      if (m == 0) break;
      pool.run(m, [&](long b, long e) {
        for (long k = b; k < e; k++)
          for (int j = 0; j < 3; j++) xs[3 * k + j] = rays_[who[k]].path.req[j];
      });
      const double *rec = bg.eval(xs.data(), m, &pool);
      pool.run(m, [&](long b, long e) {
        for (long k = b; k < e; k++) {
          Path &p = rays_[who[k]].path;
          const double *q = rec + (size_t)k * kRecNci;
          if (p.stage == -1) take_start(p, q);
          else advance(p, q);
        }
      });
    }
    r.resize(nr);
    for (long i = 0; i < nr; i++) {
      const Ray &y = rays_[i];
      r[i] = y.rlim;
      npath_ += y.npath;
      nwarn_ += y.nwarn;
      nrestart_ += y.nrestart;
    }
    nbatch_ = bg.launches();
    nevals_ = bg.evals();
    threads_ = pool.threads();
  }

  long npath() const { return npath_; }
  long nbatch() const { return nbatch_; }
  long nevals() const { return nevals_; }
  int nwarn() const { return nwarn_; }
  int nrestart() const { return nrestart_; }
  int threads() const { return threads_; }

 private:
  void trace_from(Ray &y, const double x[3]) {
    start_path(y.path, x, 1);
    y.tracing = true;
    y.npath++;
  }
  double end_dist(const Ray &y) const {
    const Attractor &a = att_[y.att];
    double d2 = 0.0;
    for (int j = 0; j < 3; j++) d2 += (y.path.x[j] - a.x[j]) * (y.path.x[j] - a.x[j]);
    return std::sqrt(d2);
  }
  void point_at(const Ray &y, double r, double x[3]) const {
    const Attractor &a = att_[y.att];
    const Node &n = nodes_[y.node];
    for (int j = 0; j < 3; j++) x[j] = a.x[j] + r * n.u[j];
  }

  // inner tries, largest radius first (:1309-1330)
  void next_inner(Ray &y) {
    if (y.k < 0) {
      begin_outer(y);
      return;
    }
    y.riaprox = y.rin[y.k];
    double x[3];
    point_at(y, y.riaprox, x);
    trace_from(y, x);
  }
  void begin_outer(Ray &y) {
    y.phase = 1;
    y.k = 0;
    y.raprox = y.rother;
    next_outer(y);
  }
  // outer tries, smallest radius first; a try must improve on a bisection
  // step of the bracket found so far (:1352-1394)
  void next_outer(Ray &y) {
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
    begin_bisection(y);
  }
  void begin_bisection(Ray &y) {
    if (y.raprox == kVBig || y.riaprox == 0.0)
      fail(C2G_ERR_NUMERIC, "basin bisection: can not find ray limits (attractor " + std::to_string(att_[y.att].cp) +
                                ", ray " + std::to_string(y.node) + ")");
    point_at(y, y.riaprox, y.xin);
    point_at(y, y.raprox, y.xfin);
    y.phase = 2;
    restart_bisection(y);
  }
  // lim_surf (:1039-1126) from its label 1
  void restart_bisection(Ray &y) {
    for (int j = 0; j < 3; j++) y.xi[j] = y.xin[j], y.xf[j] = y.xfin[j];
    next_bisection(y);
  }
  void next_bisection(Ray &y) {
    double d2 = 0.0;
    for (int j = 0; j < 3; j++) d2 += (y.xi[j] - y.xf[j]) * (y.xi[j] - y.xf[j]);
    if (std::sqrt(d2) > prec_) {
      for (int j = 0; j < 3; j++) y.xmed[j] = 0.5 * (y.xi[j] + y.xf[j]);
      trace_from(y, y.xmed);
      return;
    }
    for (int j = 0; j < 3; j++) y.xmed[j] = 0.5 * (y.xi[j] + y.xf[j]);
    // a surface point inside the beta sphere of a CP of the attractor's
    // type shrinks that sphere and restarts the bisection (:1110-1124)
    const int typ = att_[y.att].typ;
    for (int i = 0; i < ncp_; i++) {
      if (cptyp_[i] != typ) continue;
      double e2 = 0.0;
      for (int j = 0; j < 3; j++) e2 += (cpx_[3 * i + j] - y.xmed[j]) * (cpx_[3 * i + j] - y.xmed[j]);
      if (y.rbeta.empty()) y.rbeta = rbeta_;
      if (std::sqrt(e2) <= y.rbeta[i]) {
        y.rbeta[i] *= 0.75;
        y.nrestart++;
        restart_bisection(y);
        return;
      }
    }
    double r2 = 0.0;
    for (int j = 0; j < 3; j++) r2 += (y.xmed[j] - att_[y.att].x[j]) * (y.xmed[j] - att_[y.att].x[j]);
    y.rlim = std::sqrt(r2);
    y.phase = 3;
  }

  // nearest CP of the nuclear type (-3) to x: field%nearest_cp with type
  double nearest_attractor(const double x[3]) const {
    double best = kVBig;
    for (int i = 0; i < ncp_; i++) {
      if (cptyp_[i] != -3) continue;
      double d2 = 0.0;
      for (int j = 0; j < 3; j++) d2 += (cpx_[3 * i + j] - x[j]) * (cpx_[3 * i + j] - x[j]);
      best = std::min(best, std::sqrt(d2));
    }
    return best;
  }

  void path_done(Ray &y) {
    const Path &p = y.path;
    if (p.ier > 0) y.nwarn++;
    if (y.phase == 0) {
      // :1314-1329
      if (p.ier == 3) {
        y.rother = std::min(y.rother, y.rin[y.k]);
      } else {
        if (end_dist(y) <= kBsRNearNuc) {
          begin_outer(y);
          return;
        }
        y.rother = std::min(y.rother, y.rin[y.k]);
      }
      y.k--;
      next_inner(y);
    } else if (y.phase == 1) {
      // :1366-1393
      if (p.ier == 3) {
        if (y.raprox > y.riaprox) y.riaprox = y.raprox;
        y.raprox = y.rother;
      } else {
        if (end_dist(y) > kBsRNearNuc) {
          begin_bisection(y);
          return;
        }
        if (y.raprox > y.riaprox) y.riaprox = y.raprox;
        y.raprox = y.rother;
      }
      y.k++;
      next_outer(y);
    } else {
      // :1078-1105
      bool inside;
      if (p.ier <= 0) {
        inside = end_dist(y) <= kBsRNearNuc;
      } else if (p.ier == 3) {
        inside = false;
      } else {
        inside = nearest_attractor(p.x) <= kBsRNearNuc;
      }
      for (int j = 0; j < 3; j++) (inside ? y.xi[j] : y.xf[j]) = y.xmed[j];
      next_bisection(y);
    }
  }

  Handle &h_;
  const HostWfn &w_;
  int ncp_;
  const double *cpx_;
  const int *cptyp_;
  const std::vector<double> &rbeta_;
  const std::vector<Attractor> &att_;
  const std::vector<Node> &nodes_;
  double prec_;
  std::vector<Ray> rays_;
  long npath_ = 0, nbatch_ = 0, nevals_ = 0;
  int nwarn_ = 0, nrestart_ = 0, threads_ = 1;
};

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
    std::vector<double> rbeta(nc, kRBeta), r;
    BasinSearch bs(h, nc, cpx.data(), typ.data(), rbeta, att, nodes, iasprec);
    bs.run(r);
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
      stats->npath = bs.npath();
      stats->nbatch = bs.nbatch();
      stats->nevals = bs.nevals() + (long)xyz.size() / 3;
      stats->nwarn = bs.nwarn();
      stats->nrestart = bs.nrestart();
      stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

}  // extern "C"
