// NCI post-pass and cube/dat text (k_cube.cu): internal interface.
#pragma once

#include <cuda_runtime.h>

#include "c2g_internal.h"

namespace c2g {

// critic2's nciplot cutoffs (src/nci@proc.f90:141-168, 612-645)
struct NciCut {
  double rhocut, dimcut, rhoplot, srho_lo, srho_hi;
  int onlyneg;
};

// Host formatters of the Fortran edit descriptors (correctly rounded):
// " " + 1p,e13.5e3 (14 characters) and 1p,E15.7 (15 characters).
void fmt_e13_5e3(double x, char *out);
void fmt_E15_7(double x, char *out);
void fmt_E22_14E3(double x, char *out);  // 22 characters, no scale factor

// Bytes of a cube record of n3 numbers and of a whole cube body.
long cube_record_bytes(int n3);
long cube_body_bytes(const int *nstep);
// the same for writegrid_cube's precise body (6(" ",E22.14E3))
long precise_record_bytes(int n3);
long precise_body_bytes(const int *nstep);

// Ints of device scratch the text functions need.
int cube_flag_scratch_ints();

// Cube body of d_v (k fastest) into d_text; copied to h_text (and fixed up
// there) when h_text is not null, else fixed up on the device.
void cube_text_dev(const int *nstep, const double *d_v, char *d_text, char *h_text, int *d_scratch,
                   cudaStream_t st);

// Precise cube body ((6(" ",E22.14E3)) records) of d_v, as cube_text_dev.
void precise_text_dev(const int *nstep, const double *d_v, char *d_text, char *h_text, int *d_scratch,
                      cudaStream_t st);

// dat lines (31 bytes each) of ndat (crho/100, s) pairs.
void dat_text_dev(const double *d_dat, long ndat, char *d_text, char *h_text, int *d_scratch, cudaStream_t st);

// Post-pass: writes up to cap dat pairs into d_dat in grid order, applies
// the s := 100 rules to d_cgrad, returns the number of dat pairs.
// d_bcount: (npoints + 255) / 256 ints; d_total: one long.
long nci_post_dev(const int *nstep, const double *d_crho, double *d_cgrad, const NciCut &cut, double *d_dat,
                  long cap, int *d_bcount, long *d_total, cudaStream_t st);

// One grd quantity (prop: 0 rho, 1-3 gradient x y z, 4 |grad|, 5-10 Hessian
// xx xy xz yy yz zz, 11 Laplacian) on a grid, (k,j,i) order, in slabs of
// i-planes (src/rhoplot@proc.f90:890-950).
void field_grid_dev(Handle &h, const GridSpec &g, int prec, int prop, double *d_out, cudaStream_t st);

}  // namespace c2g
