// Split-precision (tcgen05 tensor-core) evaluator: internal interface.
#pragma once

#include "c2g_internal.h"

namespace c2g {

// Builds the split operands of the coefficient matrix on the device.
TcOperands *tc_create(Handle &h);
void tc_destroy(TcOperands *t);

// Relative |lambda2| threshold below which split-precision NCI points are
// re-evaluated in FP64.
void tc_set_recheck(Handle &h, double rel);

// Limit (nanoseconds) of every pipeline wait of the split kernel; a wait
// that runs out ends the launch with C2G_ERR_CUDA.
void tc_set_wait_ns(Handle &h, uint64_t ns);

// Reports (and clears) a pipeline timeout recorded by an earlier split kernel.
void tc_check_error(Handle &h);

// kRecNci records (rho, grad, hess) at n device points, split precision.
void tc_points(Handle &h, int prec, int n, const double *d_xyz, double *d_rec, cudaStream_t st,
               bool wrap = true);

// kRecNci records of the points x(3, idx[t]), t < *d_count (<= maxn), split
// precision, written at rec[t].
void tc_points_index(Handle &h, int prec, const double *d_x, const int *d_idx, const int *d_count,
                     int maxn, double *d_rec, cudaStream_t st);

// NCI grid in split precision followed by the FP64 re-check of the points
// whose Hessian has a small |lambda2| relative to max|lambda| (threshold:
// C2G_PARAM_RECHECK_REL).  Records ev_split after the
// split pass when not null, and the fraction of active K-stages per tile in
// *stage_frac when not null.  Returns the number of re-checked points.
long tc_nci_grid(Handle &h, int prec, const GridSpec &g, double *d_crho, double *d_cgrad,
                 cudaStream_t st, cudaEvent_t ev_split, double *stage_frac);

// No-allocation variant of tc_nci_grid: the re-check list lives in static
// device memory (at most tc_noalloc_max_points() grid points per call), the
// nucleus rule runs on the device; no statistics.  Fails when the handle's
// split operands for prec were not built yet.
void tc_nci_grid_noalloc(Handle &h, int prec, const GridSpec &g, double *d_crho, double *d_cgrad,
                         cudaStream_t st);
long tc_noalloc_max_points();

}  // namespace c2g
