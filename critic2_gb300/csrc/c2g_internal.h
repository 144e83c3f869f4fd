// Internal declarations of the critic2_gb300 library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/critic2_gb300.h"

namespace c2g {

// ---------------------------------------------------------------- errors
// Every entry point runs its body through guarded(): a Failure carries the
// C2G_ERR_* code, the message goes to the calling thread's last-error text.
struct Failure : std::runtime_error {
  int code;
  Failure(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
void set_last_error(const std::string &msg);
const std::string &last_error();
[[noreturn]] void fail(int code, const std::string &msg);
void cuda_check(cudaError_t e, const char *what);
#define C2G_CUDA(call) ::c2g::cuda_check((call), #call)

template <class F>
int guarded(F &&f) {
  try {
    f();
    return C2G_OK;
  } catch (const Failure &e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    set_last_error("host allocation failed");
    return C2G_ERR_ALLOC;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return C2G_ERR_ARG;
  }
}

// ------------------------------------------------------------- host model
// molwfn after prune_primitives + complete_struct, in critic2's layout.
struct HostWfn {
  int natom = 0, npri = 0, nmo = 0, wfntyp = 0, nalpha = 0;
  std::vector<double> xyz;      // 3*natom
  std::vector<int> z;           // natom
  std::vector<int> icenter;     // npri, 0-based
  std::vector<int> itype;       // npri, 1-based li index
  std::vector<double> e;        // npri
  std::vector<double> occ;      // nmo
  std::vector<double> cmo;      // npri*nmo, MO fastest
  // complete_struct
  std::vector<double> dran;     // npri
  std::vector<double> spcutoff; // natom
  std::vector<int> lmax;        // natom
  std::vector<int> icord;       // npri: primitives ordered by centre
  std::vector<int> iprilo, iprihi;  // natom, ranges in icord
  // EDF core density (nedf = 0 without one), in input order
  int nedf = 0;
  std::vector<int> edf_icenter;  // nedf, 0-based
  std::vector<int> edf_itype;    // nedf, 1-based li index
  std::vector<double> edf_e, edf_c, edf_dran;
  // molecular cell (bounding box grown by the 10 angstrom border)
  double cell_lo[3], cell_aa[3], molborder[3];
};

void prune_primitives(HostWfn &w);
void complete_struct(HostWfn &w);
void molecular_cell(HostWfn &w);
bool read_wfx(const char *path, HostWfn &w, std::string &err);
bool read_wfn(const char *path, HostWfn &w, std::string &err);
bool read_fchk(const char *path, HostWfn &w, std::string &err);
bool read_molden(const char *path, HostWfn &w, std::string &err);

// Cartesian exponents of critic2's li(3,56) table.
extern const int kLi[56][3];

// ----------------------------------------------------------- device model
// A primitive in the FP64 kernel's order (atom-major, critic2's icord).
struct __align__(16) PrimF64 {
  double e;      // exponent
  double dran;   // cutoff distance
  int lpack;     // lx | ly << 4 | lz << 8
  int atom;      // 0-based centre
  int pad0, pad1;
};

// An EDF core primitive (centre-major order).
struct __align__(16) PrimEDF {
  double e;      // exponent
  double dran;   // cutoff distance sqrt(-ln(1e-12)/e)
  double c;      // coefficient
  int lpack;     // lx | ly << 4 | lz << 8
  int atom;      // 0-based centre
};

struct DevWfn {
  int natom, npri, nmo, nmo_pad;
  const double4 *atoms;   // x, y, z, spcutoff^2
  const int *atom_z;
  const PrimF64 *prim;    // npri, atom-major
  const double *cmo;      // npri x nmo_pad (row = primitive, MO fastest)
  const double *occ;      // nmo_pad (0 for padding)
  const double *wup;      // nmo_pad spin weights (UHF/ROHF), else null
  const double *wdn;
  double cell_lo[3], cell_aa[3];
  int spin;               // 1 for UHF/ROHF
  const PrimEDF *edf;     // nedf core primitives, or null
  int nedf;
};

struct TcOperands;  // split-precision operands (k_tc.cu)

struct Handle {
  HostWfn host;
  int device = 0;
  DevWfn dev{};
  std::vector<void *> allocations;
  TcOperands *tc = nullptr;
  int newton_stall = 0;  // C2G_PARAM_NEWTON_STALL (0: critic2's maxit only)
  void *edf_buf = nullptr;  // device EDF primitives (replaced by c2g_wfn_set_edf)
};

// per-point record produced by the evaluator (FP64 path), quantities:
//  0 rho, 1-3 grad, 4-9 hess (xx,yy,zz,xy,xz,yz), 10 sum occ|grad phi|^2,
//  11-16 stress (xx,xy,xz,yy,yz,zz) before the 1/2 factor,
//  17-27 up channel (rho, grad3, gkin, hess6), 28-38 down channel.
constexpr int kRecNci = 10;
constexpr int kRecFull = 39;

// grid / point sources
struct GridSpec {
  double x0[3];
  double xmat[9];   // column-major
  int nstep[3];
};

// k_fp64.cu
// wrap = false evaluates the points as given, as grd does for a molecule
// with periodic = .false. (molecular meshes).
void launch_fp64_points(const DevWfn &w, int n, const double *d_xyz, int nder, bool full,
                        double *d_rec, cudaStream_t st, bool wrap = true);
// kRecNci records of the points x(3, idx[t]), t < *count, written at rec[t].
void launch_fp64_index(const DevWfn &w, const double *d_x, const int *d_idx, const int *d_count,
                       int maxn, double *d_rec, cudaStream_t st);
void launch_fp64_nci_grid(const DevWfn &w, const GridSpec &g, double *d_crho, double *d_cgrad,
                          cudaStream_t st);
void launch_fp64_nci_list(const DevWfn &w, const GridSpec &g, const int *d_list, const int *d_count,
                          int maxn, double *d_crho, double *d_cgrad, cudaStream_t st);

// mesh.cu: the n-point Lebedev rule (x, y, z, weight summing to 1; the
// sizes of good_lebedev, 6 to 5810) and Gauss-Legendre nodes and weights on
// (a, b), ascending (gauleg, src/tools_math@proc.f90:1765-1826).
std::vector<double4> lebedev_points(int n);
void gauleg(double a, double b, int n, std::vector<double> &x, std::vector<double> &w);

// k_newton.cu: batched field%newton on device arrays x(3,n), ier(n)
void newton_batch_dev(Handle &h, int n, double *d_x, int *d_ier, double gfnormeps, int maxit,
                      int prec, cudaStream_t st);

// host utilities shared by the entry points (api.cpp)
void eigsym3(const double h[9], double ev[3]);

}  // namespace c2g
