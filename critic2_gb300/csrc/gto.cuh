// Cartesian Gaussian basis functions in FP64 and the EDF core density.
//
// chi_eval gives a primitive x^lx y^ly z^lz exp(-al r^2) and its first and
// second derivatives with the per-axis factors of critic2's calculate_mo_gto
// (src/wfn_private@proc.F90:3218-3261): component order 0 value, 1-3 d/dx,
// d/dy, d/dz, 4-9 xx, yy, zz, xy, xz, yz.
//
// edf_core is calculate_edf (src/wfn_private@proc.F90:3275-3369): the
// electron density function of the pseudopotential cores, a linear sum
// sum_i c_i chi_i over the EDF primitives whose centre is in the point's
// environment (d^2 <= spcutoff^2, spcutoff including the EDF cutoffs) and
// with dist <= dran_edf = sqrt(-ln(1e-12)/al).  The EDF primitives are in
// centre-major order, so the sum runs in critic2's order.
#pragma once

#include "c2g_internal.h"

namespace c2g {

// x^l factors of one Cartesian axis and their first and second derivatives
// including the Gaussian's exp(-al r^2) chain rule:
//   f0 = x^l, f1 = l x^(l-1) - 2 al x^(l+1),
//   f2 = l(l-1) x^(l-2) - 2 al (2l+1) x^l + 4 al^2 x^(l+2).
__device__ __forceinline__ void axis_factors(double x, int l, double al, double &f0, double &f1,
                                             double &f2) {
  double a = 1.0, b = 0.0, c = 0.0;  // x^l, x^(l-1), x^(l-2)
  for (int i = 0; i < l; i++) {
    c = b;
    b = a;
    a *= x;
  }
  const double p1 = a * x, p2 = p1 * x;
  f0 = a;
  f1 = l * b - 2.0 * al * p1;
  f2 = (double)(l * (l - 1)) * c - 2.0 * al * (double)(2 * l + 1) * a + 4.0 * al * al * p2;
}

template <int NC>
__device__ __forceinline__ void chi_eval(double dx, double dy, double dz, double al, int lpack,
                                         double ex, double (&chi)[NC]) {
  double fx0, fx1, fx2, fy0, fy1, fy2, fz0, fz1, fz2;
  axis_factors(dx, lpack & 15, al, fx0, fx1, fx2);
  axis_factors(dy, (lpack >> 4) & 15, al, fy0, fy1, fy2);
  axis_factors(dz, (lpack >> 8) & 15, al, fz0, fz1, fz2);
  chi[0] = fx0 * fy0 * fz0 * ex;
  if constexpr (NC > 1) {
    chi[1] = fx1 * fy0 * fz0 * ex;
    chi[2] = fy1 * fx0 * fz0 * ex;
    chi[3] = fz1 * fx0 * fy0 * ex;
  }
  if constexpr (NC > 4) {
    chi[4] = fx2 * fy0 * fz0 * ex;
    chi[5] = fy2 * fz0 * fx0 * ex;
    chi[6] = fz2 * fx0 * fy0 * ex;
    chi[7] = fx1 * fy1 * fz0 * ex;
    chi[8] = fx1 * fz1 * fy0 * ex;
    chi[9] = fz1 * fy1 * fx0 * ex;
  }
}

// Whether a primitive at squared distance dd from its atom is within its
// cutoff: !(sqrt(dd) > dran), decided without the square root except
// within 1e-12 of the cutoff (the rounding of sqrt and of dran^2 is far
// below that margin, so the answer is the same).
__device__ __forceinline__ bool within_dran(double dd, double dran) {
  const double r2 = dran * dran;
  if (dd < r2 * (1.0 - 1e-12)) return true;
  if (dd > r2 * (1.0 + 1e-12)) return false;
  return !(sqrt(dd) > dran);
}

// Adds EDF primitive i's c chi (value, gradient, Hessian) at x to core.
__device__ __forceinline__ void edf_prim_add(const DevWfn &w, int i, const double (&x)[3], double (&core)[10]) {
  const PrimEDF pr = w.edf[i];
  const double4 A = w.atoms[pr.atom];
  const double dx = x[0] - A.x, dy = x[1] - A.y, dz = x[2] - A.z;
  const double dd = dx * dx + dy * dy + dz * dz;
  if (!(dd <= A.w)) return;
  const double dist = sqrt(dd);
  if (dist > pr.dran) return;
  double chi[10];
  chi_eval<10>(dx, dy, dz, pr.e, pr.lpack, exp(-pr.e * (dist * dist)), chi);
#pragma unroll
  for (int c = 0; c < 10; c++) core[c] = fma(pr.c, chi[c], core[c]);
}

// Core density, gradient and Hessian (xx, yy, zz, xy, xz, yz) at x.
__device__ __forceinline__ void edf_core(const DevWfn &w, const double (&x)[3], double (&core)[10]) {
#pragma unroll
  for (int c = 0; c < 10; c++) core[c] = 0.0;
  for (int i = 0; i < w.nedf; i++) edf_prim_add(w, i, x, core);
}

// The same sum spread over the 32 lanes of a warp (all lanes call it with
// the same x): lane j takes primitives j, j+32, ...; the partial sums are
// combined by a fixed butterfly, so the result is deterministic and the
// same on every lane.
__device__ __forceinline__ void edf_core_warp(const DevWfn &w, const double (&x)[3], double (&core)[10]) {
#pragma unroll
  for (int c = 0; c < 10; c++) core[c] = 0.0;
  for (int i = (int)(threadIdx.x & 31); i < w.nedf; i += 32) edf_prim_add(w, i, x, core);
#pragma unroll
  for (int c = 0; c < 10; c++)
    for (int o = 16; o; o >>= 1) core[c] += __shfl_xor_sync(0xffffffffu, core[c], o);
}

// Adds the core to a record r[q * stride] in the kRec* layout: the total
// density's 10 sums, and for spin-polarised records (UHF/ROHF, kRecFull)
// half the core to each spin channel (src/wfn_private@proc.F90:2636-2677);
// the kinetic energy density and stress have no core part.
__device__ __forceinline__ void edf_add_record(const DevWfn &w, const double (&x)[3], double *r, int stride,
                                               int nr, bool spin) {
  double core[10];
  edf_core(w, x, core);
#pragma unroll
  for (int c = 0; c < 10; c++) r[c * stride] += core[c];
  if (spin && nr == kRecFull) {
#pragma unroll
    for (int s = 0; s < 2; s++) {
      double *b = r + (17 + 11 * s) * stride;
      b[0] += 0.5 * core[0];
#pragma unroll
      for (int j = 0; j < 3; j++) b[(1 + j) * stride] += 0.5 * core[1 + j];
#pragma unroll
      for (int j = 0; j < 6; j++) b[(5 + j) * stride] += 0.5 * core[4 + j];
    }
  }
}

}  // namespace c2g
