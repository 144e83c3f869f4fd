// Molecular integration meshes and molcalc (src/meshmod@proc.f90:45-627,
// src/molcalc@proc.F90:94-256): atom-centred radial x Lebedev angular grids
// with Becke's or Franchini's partition of space, filled with the field on
// the GPU and summed.
//
// Mesh order is critic2's: atoms in order, then radial shells (increasing
// r), then the angular points.  z2nang depends only on the level, so every
// shell has the same angular rule and point t lies on shell t / nang.
// The partition weights are computed on the GPU, one thread per point
// (Franchini: O(natom) per point; Becke: the pairwise cutoff products,
// O(natom^2) per point).  The field is the batched evaluator's
// (FP64 or split), the integral a fixed-order reduction.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "c2g_internal.h"
#include "k_tc.h"
#include "lebedev_tables.h"

namespace c2g {
namespace {

constexpr double kFourPi = 12.566370614359172953850573533118;
constexpr double kLog2 = 0.69314718055994530941723212145818;

// Franchini et al., J. Comput. Chem. 34 (2013) 1819, SI: radial scaling
// zeta(Z), Z = 1..103 (the table of rmesh_franchini, meshmod@proc.f90:541).
const double kZeta[103] = {
    0.8, 0.9, 1.8, 1.4, 1.3, 1.1, 0.9, 0.9, 0.9, 0.9, 1.4, 1.3, 1.3, 1.2, 1.1, 1.0, 1.0, 1.0, 1.5, 1.4,
    1.3, 1.2, 1.2, 1.2, 1.2, 1.2, 1.2, 1.1, 1.1, 1.1, 1.1, 1.0, 0.9, 0.9, 0.9, 0.9, 1.4, 1.4, 1.1, 1.3,
    1.0, 1.2, 0.9, 0.9, 0.9, 1.0, 0.9, 1.0, 1.0, 1.3, 1.2, 1.2, 0.9, 1.0, 1.7, 1.5, 1.5, 1.3, 1.3, 1.4,
    1.8, 1.4, 1.2, 1.3, 1.3, 1.4, 1.1, 1.1, 1.2, 1.6, 1.4, 1.3, 1.2, 1.0, 1.0, 0.9, 1.3, 1.2, 1.2, 1.0,
    1.2, 1.2, 1.1, 1.2, 1.1, 2.1, 2.2, 1.8, 1.7, 1.3, 1.4, 1.2, 1.2, 1.3, 1.4, 1.4, 1.7, 1.9, 1.9, 2.0,
    2.0, 1.6, 2.0};

// z2nr (:574-602).  critic2 scales the base count by a default-kind (single
// precision) literal; the product is formed in float here as well.
int z2nr(int z, int lvl) {
  int nr = 15;
  if (z > 2) nr = 20;
  if (z > 10) nr = 25;
  if (z > 18) nr = 35;
  if (z > 36) nr = 60;
  if (z > 54) nr = 85;
  if (z > 86) nr = 110;
  static const float f[6] = {0.f, 2.37f, 3.08f, 3.42f, 4.27f, 6.72f};
  return (int)std::ceil((float)nr * f[lvl]);
}

// z2nang (:607-627)
int z2nang(int lvl) {
  static const int n[6] = {0, 110, 194, 302, 590, 770};
  return n[lvl];
}

// The angular rule of n points (x, y, z, weight normalised to 1): every
// distinct signed permutation of each orbit representative.
std::vector<double4> lebedev(int n) {
  for (const LebedevRule &r : kLebedevRules) {
    if (r.npts != n) continue;
    std::vector<double4> pts;
    for (int o = 0; o < r.norb; o++) {
      const LebedevOrbit &q = r.orb[o];
      const double v[3] = {q.a, q.b, q.c};
      static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
      const size_t first = pts.size();
      for (const auto &p : perm)
        for (int sg = 0; sg < 8; sg++) {
          double x[3];
          for (int k = 0; k < 3; k++) x[k] = ((sg >> k) & 1 ? -1.0 : 1.0) * v[p[k]];
          bool dup = false;
          for (size_t i = first; i < pts.size() && !dup; i++)
            dup = pts[i].x == x[0] && pts[i].y == x[1] && pts[i].z == x[2];
          // -0.0 and 0.0 are the same point
          if (!dup) pts.push_back(make_double4(x[0] + 0.0, x[1] + 0.0, x[2] + 0.0, q.w));
        }
    }
    if ((int)pts.size() != n) fail(C2G_ERR_ARG, "Lebedev table expansion is inconsistent");
    return pts;
  }
  fail(C2G_ERR_UNSUPPORTED, "no Lebedev rule of that size");
}

// Gauss-Legendre nodes (ascending) and weights on (-1, 1): Newton on P_n
// from the asymptotic guesses, the role of gauleg.
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; j++) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) <= 1e-15) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

// rmesh_postg (:508-529): r = rmid q / (1 - q) on a uniform q mesh.
void rmesh_postg(int n, int z, std::vector<double> &r, std::vector<double> &w) {
  r.resize(n);
  w.resize(n);
  const double rmid = 1.0 / std::pow((double)z, 1.0 / 3.0), h = 1.0 / (n + 1);
  for (int i = 1; i <= n; i++) {
    const double q = h * i;
    r[i - 1] = rmid * q / (1.0 - q);
    w[i - 1] = kFourPi * h * r[i - 1] * r[i - 1] * rmid / ((1.0 - q) * (1.0 - q));
  }
}

// rmesh_franchini (:536-568): r = zeta/ln2 (1 + q) ln(2/(1 - q)), q Gauss-
// Legendre on (-1, 1).
void rmesh_franchini(int n, int z, std::vector<double> &r, std::vector<double> &w) {
  std::vector<double> q, wq;
  gauss_legendre(n, q, wq);
  r.resize(n);
  w.resize(n);
  const double zeta = kZeta[z - 1];
  for (int i = 0; i < n; i++) {
    const double l = std::log(2.0 / (1.0 - q[i]));
    r[i] = zeta / kLog2 * (1.0 + q[i]) * l;
    w[i] = kFourPi * r[i] * r[i] * wq[i] * zeta / kLog2 * (l + (1.0 + q[i]) / (1.0 - q[i]));
  }
}

}  // namespace
}  // namespace c2g

namespace c2g {
namespace {

constexpr int kBeckeMaxAtoms = 512;

// One radial shell of the mesh: centre atom, radius, radial weight and, for
// Franchini's partition, the atom's own unnormalised weight at r.
struct MeshShell {
  double r, wrad, vp0;
  int atom, pad;
};

struct MeshDev {
  const double4 *nuc;      // natom: x, y, z, Franchini scale (0.3 for H, else 1)
  const MeshShell *shell;  // nshell
  const double4 *ang;      // nang: x, y, z, weight (sum 1)
  const double *rr;        // natom x natom distances (Becke)
  int natom, nang, type;
  long npoints;
  double rmax2;            // Franchini: atoms within sqrt(rmax2) of the point
};

__device__ __forceinline__ double becke_step(double mu) {
  // four iterations of 1.5 mu - 0.5 mu^3 (genmesh_becke, :165-168)
#pragma unroll
  for (int k = 0; k < 4; k++) mu = 1.5 * mu - 0.5 * mu * mu * mu;
  return mu;
}

// Points p0 .. p0 + n - 1 of the mesh: position and weight.
__global__ void k_mesh(MeshDev m, long p0, int n, double *xyz, double *wt) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long p = p0 + t;
  const MeshShell s = m.shell[p / m.nang];
  const double4 a = m.ang[p % m.nang];
  const double4 c = m.nuc[s.atom];
  const double x = c.x + s.r * a.x, y = c.y + s.r * a.y, z = c.z + s.r * a.z;
  double part;
  if (m.type == C2G_MESH_FRANCHINI) {
    // genmesh_franchini (:300-330): p_j = f_j exp(-2 d_j) / d_j^3 over the
    // atoms within rmax, w = p_i / max(p_i, sum_j p_j)
    double vpsum = 0.0;
    for (int j = 0; j < m.natom; j++) {
      const double4 b = m.nuc[j];
      const double dx = x - b.x, dy = y - b.y, dz = z - b.z;
      const double dd = dx * dx + dy * dy + dz * dz;
      if (!(dd <= m.rmax2)) continue;
      const double d = sqrt(dd), dm = fmax(d, 1e-10);
      vpsum += b.w * exp(-2.0 * d) / (dm * dm * dm);
    }
    vpsum = fmax(s.vp0, vpsum);
    part = s.vp0 / fmax(vpsum, 1e-40);
  } else {
    // genmesh_becke (:150-186): cutoff(j,k) = (1 - h((d_j - d_k)/R_jk))/2
    double d[kBeckeMaxAtoms];
    for (int j = 0; j < m.natom; j++) {
      const double4 b = m.nuc[j];
      const double dx = x - b.x, dy = y - b.y, dz = z - b.z;
      d[j] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    double vp0 = 1.0, vpsum = 0.0;
    for (int j = 0; j < m.natom; j++) {
      double vpi = 1.0;
      for (int k = 0; k < m.natom; k++) {
        if (k == j) continue;
        // critic2 forms the pair (j > k) once: cutoff(j,k) = (1 - h)/2 and
        // cutoff(k,j) = (1 + h)/2 with h from (d_j - d_k)/R_jk, j > k
        const int hi = j > k ? j : k, lo = j > k ? k : j;
        const double h = becke_step((d[hi] - d[lo]) / m.rr[(size_t)hi * m.natom + lo]);
        vpi *= j > k ? (1.0 - h) / 2.0 : (1.0 + h) / 2.0;
      }
      if (j == s.atom) vp0 = vpi;
      vpsum += vpi;
    }
    part = vp0 / vpsum;
  }
  xyz[3 * t] = x;
  xyz[3 * t + 1] = y;
  xyz[3 * t + 2] = z;
  wt[t] = part * s.wrad * a.w;
}

// Host description of a mesh plus its device tables.
struct Mesh {
  std::vector<MeshShell> shell;
  std::vector<double4> ang, nuc;
  std::vector<double> rr;
  int type = 0, nang = 0;
  long npoints = 0;
  double rmax2 = 0.0;
};

Mesh build_mesh(const HostWfn &w, int type, int lvl) {
  if (type != C2G_MESH_BECKE && type != C2G_MESH_FRANCHINI) fail(C2G_ERR_ARG, "unknown mesh type");
  if (lvl < 1 || lvl > 5) fail(C2G_ERR_ARG, "mesh level must be 1..5");
  if (type == C2G_MESH_BECKE && w.natom > kBeckeMaxAtoms)
    fail(C2G_ERR_UNSUPPORTED, "Becke mesh limited to 512 atoms here");
  Mesh m;
  m.type = type;
  m.nang = z2nang(lvl);
  m.ang = lebedev(m.nang);
  m.nuc.resize(w.natom);
  for (int a = 0; a < w.natom; a++) {
    if (w.z[a] < 1 || w.z[a] > 103) fail(C2G_ERR_UNSUPPORTED, "atomic number outside 1..103");
    m.nuc[a] = make_double4(w.xyz[3 * a], w.xyz[3 * a + 1], w.xyz[3 * a + 2], w.z[a] == 1 ? 0.3 : 1.0);
  }
  if (type == C2G_MESH_FRANCHINI) {
    // rmax: the largest radius of the atom with the most radial points (ties:
    // the larger Z), at least 12 bohr (:262-287)
    int mr = -1, izmr = -1;
    for (int a = 0; a < w.natom; a++) {
      const int nr = z2nr(w.z[a], lvl);
      if (nr > mr || (nr == mr && w.z[a] > izmr)) mr = nr, izmr = w.z[a];
    }
    std::vector<double> r, wr;
    rmesh_franchini(mr, izmr, r, wr);
    const double rmax = std::max(r[mr - 1], 12.0);
    m.rmax2 = rmax * rmax;
  } else {
    m.rr.assign((size_t)w.natom * w.natom, 0.0);
    for (int i = 0; i < w.natom; i++)
      for (int j = i + 1; j < w.natom; j++) {
        double d2 = 0.0;
        for (int k = 0; k < 3; k++) d2 += (w.xyz[3 * i + k] - w.xyz[3 * j + k]) * (w.xyz[3 * i + k] - w.xyz[3 * j + k]);
        m.rr[(size_t)i * w.natom + j] = m.rr[(size_t)j * w.natom + i] = std::sqrt(d2);
      }
  }
  for (int a = 0; a < w.natom; a++) {
    const int nr = z2nr(w.z[a], lvl);
    std::vector<double> r, wr;
    if (type == C2G_MESH_FRANCHINI) rmesh_franchini(nr, w.z[a], r, wr);
    else rmesh_postg(nr, w.z[a], r, wr);
    const double fs = w.z[a] == 1 ? 0.3 : 1.0;
    for (int i = 0; i < nr; i++) {
      const double rm = std::max(r[i], 1e-10);
      m.shell.push_back(MeshShell{r[i], wr[i], fs * std::exp(-2.0 * r[i]) / (rm * rm * rm), a, 0});
    }
  }
  m.npoints = (long)m.shell.size() * m.nang;
  return m;
}

template <class T>
T *dev_copy(const std::vector<T> &v, std::vector<void *> &owned) {
  void *p = nullptr;
  C2G_CUDA(cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(T)));
  owned.push_back(p);
  if (!v.empty()) C2G_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return static_cast<T *>(p);
}

struct DevOwner {
  std::vector<void *> p;
  ~DevOwner() {
    for (void *q : p) cudaFree(q);
  }
};

MeshDev upload_mesh(const Mesh &m, int natom, DevOwner &own) {
  MeshDev d{};
  d.nuc = dev_copy(m.nuc, own.p);
  d.shell = dev_copy(m.shell, own.p);
  d.ang = dev_copy(m.ang, own.p);
  d.rr = dev_copy(m.rr, own.p);
  d.natom = natom;
  d.nang = m.nang;
  d.type = m.type;
  d.npoints = m.npoints;
  d.rmax2 = m.rmax2;
  return d;
}

}  // namespace
}  // namespace c2g

namespace c2g {
namespace {

constexpr int kSumThreads = 256;
constexpr int kMaxQuant = 8;

struct SumArgs {
  const double *w, *rec, *xyz;
  const double4 *atoms;  // x, y, z, spcutoff^2 (the handle's)
  int natom, nr, nq;
  int quant[kMaxQuant];
  double cell_lo[3], cell_aa[3];
};

// sum_t w_t f_q(t) over a chunk, one partial per block and quantity, each a
// fixed-order tree over the block's points.
__global__ void k_mesh_sum(SumArgs a, int n, double *partial) {
  __shared__ double s[kSumThreads];
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  for (int q = 0; q < a.nq; q++) {
    double v = 0.0;
    if (t < n) {
      const double *r = a.rec + (size_t)t * a.nr;
      double f = 0.0;
      switch (a.quant[q]) {
        case C2G_MOLCALC_VOLUME: f = 1.0; break;
        case C2G_MOLCALC_RHO: f = r[0]; break;
        case C2G_MOLCALC_GKIN: f = 0.5 * r[10]; break;
        default: {  // |grad rho| with grd's nucleus rule (points not wrapped)
          const double x[3] = {a.xyz[3 * t], a.xyz[3 * t + 1], a.xyz[3 * t + 2]};
          bool nuc = false;
          for (int k = 0; k < a.natom && !nuc; k++) {
            const double4 b = a.atoms[k];
            const double dx = x[0] - b.x, dy = x[1] - b.y, dz = x[2] - b.z;
            nuc = sqrt(dx * dx + dy * dy + dz * dz) <= 1e-5;
          }
          f = nuc ? 0.0 : sqrt(r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
        }
      }
      v = a.w[t] * f;
    }
    s[threadIdx.x] = v;
    __syncthreads();
    for (int h = kSumThreads / 2; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)blockIdx.x * a.nq + q] = s[0];
    __syncthreads();
  }
}

Handle *handle(c2g_wfn *hp) {
  if (!hp) fail(C2G_ERR_ARG, "null handle");
  return reinterpret_cast<Handle *>(hp);
}

double ms_since(const std::chrono::steady_clock::time_point &t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

struct DevSwitch {  // the handle's device for the call, the caller's afterwards
  int old = 0;
  explicit DevSwitch(int d) {
    C2G_CUDA(cudaGetDevice(&old));
    if (old != d) C2G_CUDA(cudaSetDevice(d));
  }
  ~DevSwitch() { cudaSetDevice(old); }
};

}  // namespace
}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_mesh_size(const c2g_wfn *hp, int type, int level, long *npoints) {
  return guarded([&] {
    if (!hp || !npoints) fail(C2G_ERR_ARG, "null argument");
    const HostWfn &w = reinterpret_cast<const Handle *>(hp)->host;
    *npoints = build_mesh(w, type, level).npoints;
  });
}

int c2g_mesh_dev(c2g_wfn *hp, int type, int level, double *d_xyz, double *d_w, void *stream) {
  return guarded([&] {
    Handle *h = handle(hp);
    if (!d_xyz || !d_w) fail(C2G_ERR_ARG, "null device buffer");
    DevSwitch ds(h->device);
    const Mesh m = build_mesh(h->host, type, level);
    DevOwner own;
    const MeshDev md = upload_mesh(m, h->host.natom, own);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    constexpr long kChunk = 1L << 22;
    for (long p0 = 0; p0 < m.npoints; p0 += kChunk) {
      const int n = (int)std::min(kChunk, m.npoints - p0);
      k_mesh<<<(n + 127) / 128, 128, 0, st>>>(md, p0, n, d_xyz + 3 * p0, d_w + p0);
      C2G_CUDA(cudaGetLastError());
    }
    C2G_CUDA(cudaStreamSynchronize(st));
  });
}

int c2g_molcalc(c2g_wfn *hp, int type, int level, int prec, int nq, const int *quant, double *integral,
                c2g_mesh_stats *stats) {
  return guarded([&] {
    Handle *h = handle(hp);
    if (nq < 1 || nq > kMaxQuant || !quant || !integral) fail(C2G_ERR_ARG, "bad quantity list");
    if (prec != C2G_PREC_FP64 && prec != C2G_PREC_TF32X3 && prec != C2G_PREC_BF16X3)
      fail(C2G_ERR_ARG, "unknown precision mode");
    bool need_grad = false, need_gkin = false;
    for (int q = 0; q < nq; q++) {
      if (quant[q] < C2G_MOLCALC_VOLUME || quant[q] > C2G_MOLCALC_GKIN) fail(C2G_ERR_ARG, "unknown quantity");
      need_grad = need_grad || quant[q] == C2G_MOLCALC_GRADRHO;
      need_gkin = need_gkin || quant[q] == C2G_MOLCALC_GKIN;
    }
    if (need_gkin && prec != C2G_PREC_FP64)
      fail(C2G_ERR_UNSUPPORTED, "the kinetic energy density needs C2G_PREC_FP64");
    const auto t0 = std::chrono::steady_clock::now();
    DevSwitch ds(h->device);
    const Mesh m = build_mesh(h->host, type, level);
    DevOwner own;
    const MeshDev md = upload_mesh(m, h->host.natom, own);
    const int nr = need_gkin ? kRecFull : kRecNci;
    const long chunk = need_gkin ? (1L << 19) : (1L << 20);
    const long nbuf = std::min(chunk, std::max(m.npoints, 1L));
    double *d_xyz = nullptr, *d_w = nullptr, *d_rec = nullptr, *d_part = nullptr;
    const int nblk = (int)((nbuf + kSumThreads - 1) / kSumThreads);
    C2G_CUDA(cudaMalloc(&d_xyz, sizeof(double) * 3 * nbuf));
    own.p.push_back(d_xyz);
    C2G_CUDA(cudaMalloc(&d_w, sizeof(double) * nbuf));
    own.p.push_back(d_w);
    C2G_CUDA(cudaMalloc(&d_rec, sizeof(double) * nr * nbuf));
    own.p.push_back(d_rec);
    C2G_CUDA(cudaMalloc(&d_part, sizeof(double) * nq * nblk));
    own.p.push_back(d_part);
    SumArgs sa{};
    sa.w = d_w, sa.rec = d_rec, sa.xyz = d_xyz, sa.atoms = h->dev.atoms;
    sa.natom = h->host.natom, sa.nr = nr, sa.nq = nq;
    for (int q = 0; q < nq; q++) sa.quant[q] = quant[q];
    for (int j = 0; j < 3; j++) sa.cell_lo[j] = h->host.cell_lo[j], sa.cell_aa[j] = h->host.cell_aa[j];
    std::vector<double> part((size_t)nq * nblk), acc(nq, 0.0);
    double ms_mesh = 0.0;
    for (long p0 = 0; p0 < m.npoints; p0 += chunk) {
      const int n = (int)std::min(chunk, m.npoints - p0);
      const auto tm = std::chrono::steady_clock::now();
      k_mesh<<<(n + 127) / 128, 128, 0, 0>>>(md, p0, n, d_xyz, d_w);
      C2G_CUDA(cudaGetLastError());
      C2G_CUDA(cudaDeviceSynchronize());
      ms_mesh += ms_since(tm);
      // fillmesh evaluates a molecule's field with periodic = .false.: no wrap
      if (prec == C2G_PREC_FP64)
        launch_fp64_points(h->dev, n, d_xyz, need_grad || need_gkin ? 1 : 0, need_gkin, d_rec, 0, false);
      else tc_points(*h, prec, n, d_xyz, d_rec, 0, false);
      const int nb = (n + kSumThreads - 1) / kSumThreads;
      k_mesh_sum<<<nb, kSumThreads, 0, 0>>>(sa, n, d_part);
      C2G_CUDA(cudaGetLastError());
      C2G_CUDA(cudaMemcpy(part.data(), d_part, sizeof(double) * nq * nb, cudaMemcpyDeviceToHost));
      for (int b = 0; b < nb; b++)
        for (int q = 0; q < nq; q++) acc[q] += part[(size_t)b * nq + q];
    }
    for (int q = 0; q < nq; q++) integral[q] = acc[q];
    if (stats) {
      stats->npoints = m.npoints;
      stats->ms_mesh = ms_mesh;
      stats->ms_total = ms_since(t0);
    }
  });
}

}  // extern "C"

namespace c2g {

std::vector<double4> lebedev_points(int n) { return lebedev(n); }

void gauleg(double a, double b, int n, std::vector<double> &x, std::vector<double> &w) {
  gauss_legendre(n, x, w);
  const double xm = 0.5 * (b + a), xl = 0.5 * (b - a);
  for (int i = 0; i < n; i++) x[i] = xm + xl * x[i], w[i] *= xl;
}

}  // namespace c2g
