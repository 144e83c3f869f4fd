/*
 * CPU oracle for the critic2 molecular-wavefunction evaluator path.
 * TEST INFRASTRUCTURE ONLY: see oracle.h for its role and parity status.
 *
 * Each function restates the reference routine cited in its comment
 * (paths relative to the critic2 source tree).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Cartesian exponent table, critic2 li(3,56) order
 * (src/wfn_private@proc.F90:3186-3196): s; p; d; f; g; h. */
static const int LI[56][3] = {
    {0, 0, 0},
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
    {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1},
    {3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {0, 2, 1},
    {1, 2, 0}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1},
    {4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1}, {1, 0, 3},
    {0, 1, 3}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2},
    {0, 0, 5}, {0, 1, 4}, {0, 2, 3}, {0, 3, 2}, {0, 4, 1}, {0, 5, 0}, {1, 0, 4}, {1, 1, 3},
    {1, 2, 2}, {1, 3, 1}, {1, 4, 0}, {2, 0, 3}, {2, 1, 2}, {2, 2, 1}, {2, 3, 0}, {3, 0, 2},
    {3, 1, 1}, {3, 2, 0}, {4, 0, 1}, {4, 1, 0}, {5, 0, 0}};

#define RPRIM_THRES 1e-12   /* src/wfn_private@proc.F90:170 */
#define VSMALL 1e-80        /* src/param.F90:27 */
#define FLOOREPS 1e-4       /* src/fieldmod@proc.f90:31 */
#define BOHRTOA 0.52917720859 /* src/param.F90:42 */
#define CP_HDEGEN 1e-8      /* src/global.f90:149 */

struct owfn {
  int natom;
  double *xyz;
  int *z;
  int npri, nmo;
  int *icenter; /* 0-based */
  int *itype;   /* 1-based li index */
  double *e, *occ, *cmo;
  int wfntyp, nalpha;
  double *dran, *spcutoff;
  int *lmax, *icord, *iprilo, *iprihi;
  double cell_lo[3], aa[3], molborder[3];
  /* EDF core (src/wfn_private.f90 molwfn: nedf, icenter_edf, itype_edf,
   * e_edf, c_edf, dran_edf, icord_edf, iprilo_edf, iprihi_edf) */
  int nedf;
  int *icenter_edf, *itype_edf, *icord_edf, *iprilo_edf, *iprihi_edf;
  double *e_edf, *c_edf, *dran_edf;
};

static int limax_of(int itype) {
  const int *l = LI[itype - 1];
  int m = l[0] > l[1] ? l[0] : l[1];
  return m > l[2] ? m : l[2];
}

/* stable index sort by a double key (insertion into merge sort) */
static void msort_idx(int *idx, int n, const double *key, int *tmp) {
  if (n < 2) return;
  int h = n / 2;
  msort_idx(idx, h, key, tmp);
  msort_idx(idx + h, n - h, key, tmp);
  int i = 0, j = h, k = 0;
  while (i < h && j < n) tmp[k++] = (key[idx[j]] < key[idx[i]]) ? idx[j++] : idx[i++];
  while (i < h) tmp[k++] = idx[i++];
  while (j < n) tmp[k++] = idx[j++];
  memcpy(idx, tmp, sizeof(int) * n);
}

/* prune_primitives, src/wfn_private@proc.F90:3632-3684: merge primitives with
 * the same exponent (within 1e-12), type and centre, summing their MO
 * coefficient columns, then compact the arrays keeping the original order. */
static void prune_primitives(owfn *w) {
  int n = w->npri;
  int *iord = malloc(sizeof(int) * n), *tmp = malloc(sizeof(int) * n);
  char *keep = malloc(n);
  for (int i = 0; i < n; i++) iord[i] = i, keep[i] = 1;
  msort_idx(iord, n, w->e, tmp);
  for (int i = 0; i < n; i++) {
    int a = iord[i];
    if (!keep[a]) continue;
    for (int j = i + 1; j < n; j++) {
      int b = iord[j];
      if (fabs(w->e[b] - w->e[a]) > 1e-12) continue;
      if (w->itype[a] == w->itype[b] && w->icenter[a] == w->icenter[b] && keep[b]) {
        for (int m = 0; m < w->nmo; m++) w->cmo[(size_t)a * w->nmo + m] += w->cmo[(size_t)b * w->nmo + m];
        keep[b] = 0;
      }
    }
  }
  int j = 0;
  for (int i = 0; i < n; i++) {
    if (!keep[i]) continue;
    if (j != i) {
      memmove(w->cmo + (size_t)j * w->nmo, w->cmo + (size_t)i * w->nmo, sizeof(double) * w->nmo);
      w->e[j] = w->e[i];
      w->icenter[j] = w->icenter[i];
      w->itype[j] = w->itype[i];
    }
    j++;
  }
  w->npri = j;
  free(iord);
  free(tmp);
  free(keep);
}

/* complete_struct, src/wfn_private@proc.F90:3692-3785 (GTO branch):
 * dran = sqrt(-ln(thres)/alpha), per-atom cutoff = max dran, per-atom lmax
 * (largest single Cartesian exponent), primitives ordered by centre. */
static void complete_struct(owfn *w) {
  int n = w->npri, na = w->natom;
  w->dran = malloc(sizeof(double) * n);
  w->spcutoff = calloc(na, sizeof(double));
  w->lmax = calloc(na, sizeof(int));
  w->icord = malloc(sizeof(int) * n);
  w->iprilo = malloc(sizeof(int) * na);
  w->iprihi = malloc(sizeof(int) * na);
  for (int i = 0; i < n; i++) {
    w->dran[i] = sqrt(-log(RPRIM_THRES) / w->e[i]);
    int a = w->icenter[i];
    if (w->dran[i] > w->spcutoff[a]) w->spcutoff[a] = w->dran[i];
    int lm = limax_of(w->itype[i]);
    if (lm > w->lmax[a]) w->lmax[a] = lm;
  }
  /* stable sort by centre */
  int k = 0;
  for (int a = 0; a < na; a++) {
    w->iprilo[a] = -1;
    w->iprihi[a] = -2;
    for (int i = 0; i < n; i++)
      if (w->icenter[i] == a) {
        if (w->iprilo[a] < 0) w->iprilo[a] = k;
        w->iprihi[a] = k;
        w->icord[k++] = i;
      }
  }
}

/* Molecular cell (src/crystalmod@proc.f90:222-249, 545): bounding box of the
 * atoms grown by the default border (10 angstrom, src/global.f90:122); the
 * inner region that keeps CPs is the cell minus molborder on each side. */
static void molecular_cell(owfn *w) {
  double border = 10.0 / BOHRTOA;
  for (int j = 0; j < 3; j++) {
    double lo = 1e40, hi = -1e40;
    for (int a = 0; a < w->natom; a++) {
      double x = w->xyz[3 * a + j];
      if (x - border < lo) lo = x - border;
      if (x + border > hi) hi = x + border;
    }
    w->cell_lo[j] = lo;
    w->aa[j] = hi - lo;
    double b = border - fmax(2.0, 0.8 * border);
    w->molborder[j] = fmax(b, 0.0) / (hi - lo);
  }
}

owfn *o_wfn_new(int natom, const double *xyz, const int *z, int npri, int nmo,
                const int *icenter, const int *itype, const double *e,
                const double *occ, const double *cmo, int wfntyp, int nalpha) {
  owfn *w = calloc(1, sizeof(owfn));
  w->natom = natom;
  w->xyz = malloc(sizeof(double) * 3 * natom);
  memcpy(w->xyz, xyz, sizeof(double) * 3 * natom);
  w->z = malloc(sizeof(int) * natom);
  memcpy(w->z, z, sizeof(int) * natom);
  w->npri = npri;
  w->nmo = nmo;
  w->icenter = malloc(sizeof(int) * npri);
  w->itype = malloc(sizeof(int) * npri);
  w->e = calloc(npri, sizeof(double));
  w->occ = malloc(sizeof(double) * nmo);
  w->cmo = malloc(sizeof(double) * (size_t)npri * nmo);
  for (int i = 0; i < npri; i++) {
    w->icenter[i] = icenter[i] - 1;
    w->itype[i] = itype[i];
    w->e[i] = e[i];
  }
  memcpy(w->occ, occ, sizeof(double) * nmo);
  memcpy(w->cmo, cmo, sizeof(double) * (size_t)npri * nmo);
  w->wfntyp = wfntyp;
  w->nalpha = nalpha;
  prune_primitives(w);
  complete_struct(w);
  molecular_cell(w);
  return w;
}

static void free_edf(owfn *w) {
  free(w->icenter_edf); free(w->itype_edf); free(w->icord_edf); free(w->iprilo_edf);
  free(w->iprihi_edf); free(w->e_edf); free(w->c_edf); free(w->dran_edf);
  w->icenter_edf = w->itype_edf = w->icord_edf = w->iprilo_edf = w->iprihi_edf = NULL;
  w->e_edf = w->c_edf = w->dran_edf = NULL;
  w->nedf = 0;
}

void o_wfn_free(owfn *w) {
  if (!w) return;
  free(w->xyz); free(w->z); free(w->icenter); free(w->itype); free(w->e);
  free(w->occ); free(w->cmo); free(w->dran); free(w->spcutoff); free(w->lmax);
  free(w->icord); free(w->iprilo); free(w->iprihi);
  free_edf(w);
  free(w);
}

/* The EDF part of read_wfx + complete_struct (src/wfn_private@proc.F90:
 * 1185-1230, 3750-3776): dran_edf = sqrt(-ln(thres)/alpha), the atom's
 * spcutoff grows to cover its EDF primitives, EDF primitives ordered by
 * centre.  EDF primitives are not pruned.  icenter is 1-based.  nedf = 0
 * removes the core; the MO cutoffs are recomputed from scratch. */
void o_wfn_set_edf(owfn *w, int nedf, const int *icenter, const int *itype, const double *e,
                   const double *c) {
  free_edf(w);
  free(w->dran); free(w->spcutoff); free(w->lmax); free(w->icord); free(w->iprilo); free(w->iprihi);
  complete_struct(w);
  if (nedf <= 0) return;
  int na = w->natom;
  w->nedf = nedf;
  w->icenter_edf = malloc(sizeof(int) * nedf);
  w->itype_edf = malloc(sizeof(int) * nedf);
  w->e_edf = malloc(sizeof(double) * nedf);
  w->c_edf = malloc(sizeof(double) * nedf);
  w->dran_edf = malloc(sizeof(double) * nedf);
  w->icord_edf = malloc(sizeof(int) * nedf);
  w->iprilo_edf = malloc(sizeof(int) * na);
  w->iprihi_edf = malloc(sizeof(int) * na);
  for (int i = 0; i < nedf; i++) {
    w->icenter_edf[i] = icenter[i] - 1;
    w->itype_edf[i] = itype[i];
    w->e_edf[i] = e[i];
    w->c_edf[i] = c[i];
    w->dran_edf[i] = sqrt(-log(RPRIM_THRES) / e[i]);
    int a = w->icenter_edf[i];
    if (w->dran_edf[i] > w->spcutoff[a]) w->spcutoff[a] = w->dran_edf[i];
  }
  int k = 0;
  for (int a = 0; a < na; a++) {
    w->iprilo_edf[a] = -1;
    w->iprihi_edf[a] = -2;
    for (int i = 0; i < nedf; i++)
      if (w->icenter_edf[i] == a) {
        if (w->iprilo_edf[a] < 0) w->iprilo_edf[a] = k;
        w->iprihi_edf[a] = k;
        w->icord_edf[k++] = i;
      }
  }
}

int o_wfn_npri(const owfn *w) { return w->npri; }

void o_wfn_cell(const owfn *w, double lo[3], double aa[3], double mb[3]) {
  for (int j = 0; j < 3; j++) lo[j] = w->cell_lo[j], aa[j] = w->aa[j], mb[j] = w->molborder[j];
}

static double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; i++) r *= x;
  return r;
}

/* calculate_mo_gto, src/wfn_private@proc.F90:3161-3273.  The environment is
 * the set of atoms with d^2 <= spcutoff^2 (list_near_atoms with up2dcidx,
 * src/crystalmod@env.f90:409-410; for a molecule the block walk returns the
 * same set).  phi is (10, nmo): component-major, MO fastest. */
static void calculate_mo_gto(const owfn *w, const double xpos[3], int nder, double *phi) {
  static const int imax[3] = {1, 4, 10};
  int nmo = w->nmo, nc = imax[nder];
  memset(phi, 0, sizeof(double) * 10 * nmo);
  for (int a = 0; a < w->natom; a++) {
    double xx[3], dd = 0.0;
    for (int j = 0; j < 3; j++) {
      xx[j] = xpos[j] - w->xyz[3 * a + j];
      dd += xx[j] * xx[j];
    }
    if (!(dd <= w->spcutoff[a] * w->spcutoff[a])) continue;
    double dist = sqrt(dd);
    double d2 = dist * dist;
    double xl[3][3][6];
    int lm = w->lmax[a];
    for (int ix = 0; ix < 3; ix++) {
      xl[ix][0][0] = 1.0; xl[ix][1][0] = 0.0; xl[ix][2][0] = 0.0;
      if (lm < 1) continue;
      xl[ix][0][1] = xx[ix]; xl[ix][1][1] = 1.0; xl[ix][2][1] = 0.0;
      if (lm < 2) continue;
      xl[ix][0][2] = xl[ix][0][1] * xx[ix]; xl[ix][1][2] = 2.0 * xl[ix][0][1]; xl[ix][2][2] = 2.0;
      if (lm < 3) continue;
      xl[ix][0][3] = xl[ix][0][2] * xx[ix]; xl[ix][1][3] = 3.0 * xl[ix][0][2]; xl[ix][2][3] = 6.0 * xl[ix][0][1];
      if (lm < 4) continue;
      xl[ix][0][4] = xl[ix][0][3] * xx[ix]; xl[ix][1][4] = 4.0 * xl[ix][0][3]; xl[ix][2][4] = 12.0 * xl[ix][0][2];
      if (lm < 5) continue;
      xl[ix][0][5] = xl[ix][0][4] * xx[ix]; xl[ix][1][5] = 5.0 * xl[ix][0][4]; xl[ix][2][5] = 20.0 * xl[ix][0][3];
    }
    for (int j = w->iprilo[a]; j <= w->iprihi[a]; j++) {
      int ip = w->icord[j];
      if (dist > w->dran[ip]) continue;
      double al = w->e[ip];
      double ex = exp(-al * d2);
      const int *l = LI[w->itype[ip] - 1];
      double chi[10];
      chi[0] = xl[0][0][l[0]] * xl[1][0][l[1]] * xl[2][0][l[2]] * ex;
      if (nder > 0) {
        double f1x = xl[0][1][l[0]] - 2 * al * ipow(xx[0], l[0] + 1);
        double f1y = xl[1][1][l[1]] - 2 * al * ipow(xx[1], l[1] + 1);
        double f1z = xl[2][1][l[2]] - 2 * al * ipow(xx[2], l[2] + 1);
        chi[1] = f1x * xl[1][0][l[1]] * xl[2][0][l[2]] * ex;
        chi[2] = f1y * xl[0][0][l[0]] * xl[2][0][l[2]] * ex;
        chi[3] = f1z * xl[0][0][l[0]] * xl[1][0][l[1]] * ex;
        if (nder > 1) {
          chi[4] = (xl[0][2][l[0]] - 2 * al * (2 * l[0] + 1) * xl[0][0][l[0]] + 4 * al * al * ipow(xx[0], l[0] + 2)) *
                   xl[1][0][l[1]] * xl[2][0][l[2]] * ex;
          chi[5] = (xl[1][2][l[1]] - 2 * al * (2 * l[1] + 1) * xl[1][0][l[1]] + 4 * al * al * ipow(xx[1], l[1] + 2)) *
                   xl[2][0][l[2]] * xl[0][0][l[0]] * ex;
          chi[6] = (xl[2][2][l[2]] - 2 * al * (2 * l[2] + 1) * xl[2][0][l[2]] + 4 * al * al * ipow(xx[2], l[2] + 2)) *
                   xl[0][0][l[0]] * xl[1][0][l[1]] * ex;
          chi[7] = f1x * f1y * xl[2][0][l[2]] * ex;
          chi[8] = f1x * f1z * xl[1][0][l[1]] * ex;
          chi[9] = f1z * f1y * xl[0][0][l[0]] * ex;
        }
      }
      const double *c = w->cmo + (size_t)ip * nmo;
      for (int ix = 0; ix < nc; ix++) {
        double cx = chi[ix];
        double *p = phi + (size_t)ix * nmo;
        for (int m = 0; m < nmo; m++) p[m] += c[m] * cx;
      }
    }
  }
}

/* calculate_edf, src/wfn_private@proc.F90:3275-3369: the core density
 * rhoc = sum c_edf chi over the EDF primitives of the environment's atoms
 * (d^2 <= spcutoff^2) with dist <= dran_edf, its gradient and Hessian
 * hc = (xx, yy, zz, xy, xz, yz).  The reference tabulates the powers x^l
 * only up to the atom's MO lmax; here they are tabulated up to 5, which is
 * the same for every EDF type within lmax (s-type EDFs always are). */
static void calculate_edf(const owfn *w, const double xpos[3], int nder, double *rhoc, double gradc[3],
                          double hc[6]) {
  *rhoc = 0.0;
  for (int j = 0; j < 3; j++) gradc[j] = 0.0;
  for (int j = 0; j < 6; j++) hc[j] = 0.0;
  if (w->nedf == 0) return;
  for (int a = 0; a < w->natom; a++) {
    double xx[3], dd = 0.0;
    for (int j = 0; j < 3; j++) {
      xx[j] = xpos[j] - w->xyz[3 * a + j];
      dd += xx[j] * xx[j];
    }
    if (!(dd <= w->spcutoff[a] * w->spcutoff[a])) continue;
    if (w->iprilo_edf[a] < 0) continue;
    double dist = sqrt(dd), d2 = dist * dist;
    double xl[3][3][6];
    for (int ix = 0; ix < 3; ix++) {
      xl[ix][0][0] = 1.0; xl[ix][1][0] = 0.0; xl[ix][2][0] = 0.0;
      xl[ix][0][1] = xx[ix]; xl[ix][1][1] = 1.0; xl[ix][2][1] = 0.0;
      for (int l = 2; l <= 5; l++) {
        xl[ix][0][l] = xl[ix][0][l - 1] * xx[ix];
        xl[ix][1][l] = l * xl[ix][0][l - 1];
        xl[ix][2][l] = l * (l - 1) * xl[ix][0][l - 2];
      }
    }
    for (int j = w->iprilo_edf[a]; j <= w->iprihi_edf[a]; j++) {
      int ip = w->icord_edf[j];
      if (dist > w->dran_edf[ip]) continue;
      const int *l = LI[w->itype_edf[ip] - 1];
      double al = w->e_edf[ip];
      double ex = exp(-al * d2);
      double exc = w->c_edf[ip] * ex;
      *rhoc += w->c_edf[ip] * xl[0][0][l[0]] * xl[1][0][l[1]] * xl[2][0][l[2]] * ex;
      if (nder < 1) continue;
      double f1x = xl[0][1][l[0]] - 2 * al * ipow(xx[0], l[0] + 1);
      double f1y = xl[1][1][l[1]] - 2 * al * ipow(xx[1], l[1] + 1);
      double f1z = xl[2][1][l[2]] - 2 * al * ipow(xx[2], l[2] + 1);
      gradc[0] += f1x * xl[1][0][l[1]] * xl[2][0][l[2]] * exc;
      gradc[1] += f1y * xl[0][0][l[0]] * xl[2][0][l[2]] * exc;
      gradc[2] += f1z * xl[0][0][l[0]] * xl[1][0][l[1]] * exc;
      if (nder < 2) continue;
      hc[0] += (xl[0][2][l[0]] - 2 * al * (2 * l[0] + 1) * xl[0][0][l[0]] + 4 * al * al * ipow(xx[0], l[0] + 2)) *
               xl[1][0][l[1]] * xl[2][0][l[2]] * exc;
      hc[1] += (xl[1][2][l[1]] - 2 * al * (2 * l[1] + 1) * xl[1][0][l[1]] + 4 * al * al * ipow(xx[1], l[1] + 2)) *
               xl[2][0][l[2]] * xl[0][0][l[0]] * exc;
      hc[2] += (xl[2][2][l[2]] - 2 * al * (2 * l[2] + 1) * xl[2][0][l[2]] + 4 * al * al * ipow(xx[2], l[2] + 2)) *
               xl[0][0][l[0]] * xl[1][0][l[1]] * exc;
      hc[3] += f1x * f1y * xl[2][0][l[2]] * exc;
      hc[4] += f1x * f1z * xl[1][0][l[1]] * exc;
      hc[5] += f1z * f1y * xl[0][0][l[0]] * exc;
    }
  }
}

/* molwfn%rho2, src/wfn_private@proc.F90:2484-2705. Output
 * arrays are Fortran-ordered: rho(3) = total/up/down, grad(3,3) column j =
 * spin j, h(3,3,3) column-major per spin, stress(3,3). */
void o_rho2(const owfn *w, const double xpos[3], int nder, double rho[3], double rhoval[3],
            double grad[9], double gradval[9], double h[27], double hval[27],
            double gkin[3], double *vir, double stress[9]) {
  int nmo = w->nmo;
  double *phi = malloc(sizeof(double) * 10 * nmo);
  double hh[3][6] = {{0}}, hhval[3][6];
  double g[3][3] = {{0}}, gk[3] = {0}, st[3][3] = {{0}}, rh[3] = {0};
  calculate_mo_gto(w, xpos, nder, phi);
  const double *p0 = phi, *px = phi + nmo, *py = phi + 2 * nmo, *pz = phi + 3 * nmo;
  const double *pxx = phi + 4 * nmo, *pyy = phi + 5 * nmo, *pzz = phi + 6 * nmo;
  const double *pxy = phi + 7 * nmo, *pxz = phi + 8 * nmo, *pyz = phi + 9 * nmo;
  int uhf = (w->wfntyp == 1), rohf = (w->wfntyp == 2);
  for (int m = 0; m < nmo; m++) {
    double aocc = w->occ[m];
    int isalpha = (m < w->nalpha);
    double rs = aocc * p0[m] * p0[m];
    rh[0] += rs;
    if (uhf) rh[isalpha ? 1 : 2] += rs;
    else if (rohf) { rh[1] += rs; if (isalpha) rh[2] += rs; }
    if (nder > 0) {
      double gs[3] = {2 * aocc * p0[m] * px[m], 2 * aocc * p0[m] * py[m], 2 * aocc * p0[m] * pz[m]};
      double ks = aocc * (px[m] * px[m] + py[m] * py[m] + pz[m] * pz[m]);
      for (int j = 0; j < 3; j++) g[0][j] += gs[j];
      gk[0] += ks;
      if (uhf) { int s = isalpha ? 1 : 2; for (int j = 0; j < 3; j++) g[s][j] += gs[j]; gk[s] += ks; }
      else if (rohf) {
        for (int j = 0; j < 3; j++) g[1][j] += gs[j];
        gk[1] += ks;
        if (isalpha) { for (int j = 0; j < 3; j++) g[2][j] += gs[j]; gk[2] += ks; }
      }
    }
    if (nder > 1) {
      double hs[6];
      hs[0] = 2 * aocc * (p0[m] * pxx[m] + px[m] * px[m]);
      hs[1] = 2 * aocc * (p0[m] * pyy[m] + py[m] * py[m]);
      hs[2] = 2 * aocc * (p0[m] * pzz[m] + pz[m] * pz[m]);
      hs[3] = 2 * aocc * (p0[m] * pxy[m] + px[m] * py[m]);
      hs[4] = 2 * aocc * (p0[m] * pxz[m] + px[m] * pz[m]);
      hs[5] = 2 * aocc * (p0[m] * pyz[m] + py[m] * pz[m]);
      for (int j = 0; j < 6; j++) hh[0][j] += hs[j];
      if (uhf) { int s = isalpha ? 1 : 2; for (int j = 0; j < 6; j++) hh[s][j] += hs[j]; }
      else if (rohf) {
        for (int j = 0; j < 6; j++) hh[1][j] += hs[j];
        if (isalpha) for (int j = 0; j < 6; j++) hh[2][j] += hs[j];
      }
      st[0][0] += aocc * (p0[m] * pxx[m] - px[m] * px[m]);
      st[0][1] += aocc * (p0[m] * pxy[m] - px[m] * py[m]);
      st[0][2] += aocc * (p0[m] * pxz[m] - px[m] * pz[m]);
      st[1][1] += aocc * (p0[m] * pyy[m] - py[m] * py[m]);
      st[1][2] += aocc * (p0[m] * pyz[m] - py[m] * pz[m]);
      st[2][2] += aocc * (p0[m] * pzz[m] - pz[m] * pz[m]);
    }
  }
  free(phi);
  /* core contribution (:2626-2677): RHF-like types add it to the total and
   * halve; UHF/ROHF add it to the total and half to each spin channel */
  double rhoc, gradc[3], hhc[6];
  calculate_edf(w, xpos, nder, &rhoc, gradc, hhc);
  if (!uhf && !rohf) {
    rhoval[0] = rh[0]; rhoval[1] = 0.5 * rh[0]; rhoval[2] = rhoval[1];
    rh[0] += rhoc;
    rh[1] = 0.5 * rh[0]; rh[2] = rh[1];
    for (int j = 0; j < 3; j++) {
      gradval[j] = g[0][j]; gradval[3 + j] = 0.5 * g[0][j]; gradval[6 + j] = 0.5 * g[0][j];
      g[0][j] += gradc[j];
      g[1][j] = 0.5 * g[0][j]; g[2][j] = g[1][j];
    }
    gk[1] = gk[0] / 2; gk[2] = gk[1];
    for (int j = 0; j < 6; j++) {
      hhval[0][j] = hh[0][j]; hhval[1][j] = 0.5 * hh[0][j]; hhval[2][j] = hhval[1][j];
      hh[0][j] += hhc[j];
      hh[1][j] = 0.5 * hh[0][j]; hh[2][j] = hh[1][j];
    }
  } else {
    for (int s = 0; s < 3; s++) {
      rhoval[s] = rh[s];
      for (int j = 0; j < 3; j++) gradval[3 * s + j] = g[s][j];
      for (int j = 0; j < 6; j++) hhval[s][j] = hh[s][j];
    }
    rh[0] += rhoc;
    rh[1] += 0.5 * rhoc;
    rh[2] += 0.5 * rhoc;
    for (int j = 0; j < 3; j++) {
      g[0][j] += gradc[j];
      g[1][j] += 0.5 * gradc[j];
      g[2][j] += 0.5 * gradc[j];
    }
    for (int j = 0; j < 6; j++) {
      hh[0][j] += hhc[j];
      hh[1][j] += 0.5 * hhc[j];
      hh[2][j] += 0.5 * hhc[j];
    }
  }
  for (int s = 0; s < 3; s++) rho[s] = rh[s];
  for (int s = 0; s < 3; s++)
    for (int j = 0; j < 3; j++) grad[3 * s + j] = g[s][j];
  st[1][0] = st[0][1]; st[2][0] = st[0][2]; st[2][1] = st[1][2];
  double v = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { st[i][j] *= 0.5; stress[3 * j + i] = st[i][j]; }
  v = st[0][0] + st[1][1] + st[2][2];
  *vir = v;
  for (int s = 0; s < 3; s++) {
    gkin[s] = 0.5 * gk[s];
    double *H = h + 9 * s, *HV = hval + 9 * s;
    /* column-major H(i,j) at 3*j+i */
    H[0] = hh[s][0]; H[4] = hh[s][1]; H[8] = hh[s][2];
    H[3] = H[1] = hh[s][3]; H[6] = H[2] = hh[s][4]; H[7] = H[5] = hh[s][5];
    HV[0] = hhval[s][0]; HV[4] = hhval[s][1]; HV[8] = hhval[s][2];
    HV[3] = HV[1] = hhval[s][3]; HV[6] = HV[2] = hhval[s][4]; HV[7] = HV[5] = hhval[s][5];
  }
}

/* Symmetric 3x3 eigenvalues in ascending order (the role of LAPACK dsyev in
 * eigsym, src/tools_math@proc.f90:1005-1039).  Cyclic Jacobi rotations. */
void o_eigsym3(const double m[9], double ev[3]) {
  double a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = 0.5 * (m[3 * j + i] + m[3 * i + j]);
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    double dia = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off == 0.0 || off < 1e-34 * dia) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
      }
  }
  double e0 = a[0][0], e1 = a[1][1], e2 = a[2][2], t;
  if (e0 > e1) t = e0, e0 = e1, e1 = t;
  if (e1 > e2) t = e1, e1 = e2, e2 = t;
  if (e0 > e1) t = e0, e0 = e1, e1 = t;
  ev[0] = e0; ev[1] = e1; ev[2] = e2;
}

/* rsindex, src/tools_math@proc.f90:1084-1106: rank and signature with a
 * zero threshold eps. */
void o_rsindex(const double m[9], double ev[3], int *r, int *s, double eps) {
  o_eigsym3(m, ev);
  int np = 0, nm = 0;
  for (int i = 0; i < 3; i++) {
    if (ev[i] > eps) np++;
    if (ev[i] < -eps) nm++;
  }
  *r = np + nm;
  *s = np - nm;
}

/* matinvsym for n = 3 (src/tools_math@proc.f90:1276-1316): inverse of a
 * symmetric matrix; nonzero return when the matrix is exactly singular
 * (the LDL^T factor has a zero pivot). */
int o_matinvsym3(double m[9]) {
  double a = m[0], b = m[3], c = m[6], d = m[4], e = m[7], f = m[8];
  double A = d * f - e * e, B = c * e - b * f, C = b * e - c * d;
  double det = a * A + b * B + c * C;
  if (det == 0.0 || !isfinite(det)) return 1;
  double D = a * f - c * c, E = b * c - a * e, F = a * d - b * b;
  double id = 1.0 / det;
  m[0] = A * id; m[4] = D * id; m[8] = F * id;
  m[1] = m[3] = B * id; m[2] = m[6] = C * id; m[5] = m[7] = E * id;
  return 0;
}

/* nearest atom within distmax (identify_atom for a molecule,
 * src/crystalmod@env.f90:593-614). Returns the 0-based atom or -1. */
static int identify_atom(const owfn *w, const double x[3], double distmax, double *dist) {
  int best = -1;
  double dmin = 1e30;
  for (int a = 0; a < w->natom; a++) {
    double dx = x[0] - w->xyz[3 * a], dy = x[1] - w->xyz[3 * a + 1], dz = x[2] - w->xyz[3 * a + 2];
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d < dmin) dmin = d, best = a;
  }
  if (dist) *dist = dmin;
  return (dmin <= distmax) ? best : -1;
}

/* field%grd for a molecular wavefunction, src/fieldmod@proc.f90:808-1171:
 * wrap into the molecular cell (:921-943), rho2 (:1002-1047), nucleus
 * check within 1e-5 bohr -> zero gradient (:1148-1154), rank/signature with
 * CP_hdegen (:1157-1162). */
void o_grd(const owfn *w, const double v[3], int nder, ores *res) {
  memset(res, 0, sizeof(*res));
  res->valid = 1;
  double wc[3];
  for (int j = 0; j < 3; j++) {
    double x = (v[j] - w->cell_lo[j]) / w->aa[j];
    if (x < -FLOOREPS || x > 1.0 + FLOOREPS) x -= floor(x);
    wc[j] = w->cell_lo[j] + x * w->aa[j];
  }
  double rho[3], rhov[3], g[9], gv[9], h[27], hv[27], gk[3], vir, st[9];
  o_rho2(w, wc, nder, rho, rhov, g, gv, h, hv, gk, &vir, st);
  res->f = rho[0];
  res->fval = rhov[0];
  res->fspin[0] = rho[1];
  res->fspin[1] = rho[2];
  if (nder > 0) {
    for (int j = 0; j < 3; j++) res->gf[j] = g[j];
    res->gfmodval = sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
    res->gfmodspin[0] = sqrt(g[3] * g[3] + g[4] * g[4] + g[5] * g[5]);
    res->gfmodspin[1] = sqrt(g[6] * g[6] + g[7] * g[7] + g[8] * g[8]);
    res->gkin = gk[0];
    res->gkinspin[0] = gk[1];
    res->gkinspin[1] = gk[2];
  }
  if (nder > 1) {
    memcpy(res->hf, h, sizeof(double) * 9);
    res->del2fval = hv[0] + hv[4] + hv[8];
    res->lapspin[0] = h[9] + h[13] + h[17];
    res->lapspin[1] = h[18] + h[22] + h[26];
    memcpy(res->stress, st, sizeof(st));
    res->vir = vir;
  }
  res->isnuc = identify_atom(w, wc, 1e-5, NULL) >= 0;
  if (nder > 0) {
    if (res->isnuc) res->gf[0] = res->gf[1] = res->gf[2] = 0.0;
    res->gfmod = sqrt(res->gf[0] * res->gf[0] + res->gf[1] * res->gf[1] + res->gf[2] * res->gf[2]);
  }
  if (nder > 1) {
    res->del2f = res->hf[0] + res->hf[4] + res->hf[8];
    o_rsindex(res->hf, res->hfeval, &res->r, &res->s, CP_HDEGEN);
  }
}

/* NCI per-point body, src/nci@proc.f90:565-571 and 598-599:
 * s = |grad rho| / (2 (3 pi^2)^(1/3) max(rho,vsmall)^(4/3)),
 * crho = sign(rho, lambda2) * 100. */
static void nci_point(const owfn *w, const double x[3], double *crho, double *cgrad) {
  const double cst = 2.0 * pow(3.0 * M_PI * M_PI, 1.0 / 3.0);
  ores res;
  o_grd(w, x, 2, &res);
  double ev[3];
  o_eigsym3(res.hf, ev);
  *cgrad = res.gfmod / (cst * pow(fmax(res.f, VSMALL), 4.0 / 3.0));
  *crho = copysign(fabs(res.f), ev[1]) * 100.0;
}

void o_nci_points(const owfn *w, long n, const double *xyz, double *crho, double *cgrad,
                  int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < n; i++) nci_point(w, xyz + 3 * i, crho + i, cgrad + i);
}

/* The nciplot grid loop, src/nci@proc.f90:543-605: OpenMP dynamic over the
 * outermost index i; arrays laid out (k, j, i) with k fastest; x = x0 +
 * i*xmat(:,1) + j*xmat(:,2) + k*xmat(:,3).  Rows i0..i1-1 only (bounded
 * samples); outputs are indexed from row i0. */
void o_nciplot(const owfn *w, const double x0[3], const double xmat[9], const int nstep[3],
               int i0, int i1, double *crho, double *cgrad, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  int n2 = nstep[1], n3 = nstep[2];
#pragma omp parallel for schedule(dynamic)
  for (int i = i0; i < i1; i++)
    for (int j = 0; j < n2; j++)
      for (int k = 0; k < n3; k++) {
        double x[3];
        for (int c = 0; c < 3; c++) x[c] = x0[c] + i * xmat[c] + j * xmat[3 + c] + k * xmat[6 + c];
        size_t idx = ((size_t)(i - i0) * n2 + j) * n3 + k;
        nci_point(w, x, crho + idx, cgrad + idx);
      }
}

void o_rho2_points(const owfn *w, long n, const double *xyz, int nder, double *rho,
                   double *grad, double *hess, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < n; i++) {
    double r[3], rv[3], g[9], gv[9], h[27], hv[27], gk[3], vir, st[9];
    o_rho2(w, xyz + 3 * i, nder, r, rv, g, gv, h, hv, gk, &vir, st);
    rho[i] = r[0];
    if (grad) for (int j = 0; j < 3; j++) grad[3 * i + j] = g[j];
    if (hess) for (int j = 0; j < 9; j++) hess[9 * i + j] = h[j];
  }
}

/* field%newton, src/fieldmod@proc.f90:2238-2279: ier 0 converged,
 * 1 invalid/singular Hessian, 2 too many iterations. */
int o_newton(const owfn *w, double r[3], double gfnormeps, int maxit) {
  for (int it = 0; it < maxit; it++) {
    ores res;
    o_grd(w, r, 2, &res);
    if (!res.valid) return 1;
    if (res.gfmod < gfnormeps) return 0;
    if (o_matinvsym3(res.hf)) return 1;
    double *H = res.hf;
    double d0 = H[0] * res.gf[0] + H[3] * res.gf[1] + H[6] * res.gf[2];
    double d1 = H[1] * res.gf[0] + H[4] * res.gf[1] + H[7] * res.gf[2];
    double d2 = H[2] * res.gf[0] + H[5] * res.gf[1] + H[8] * res.gf[2];
    r[0] -= d0; r[1] -= d1; r[2] -= d2;
  }
  return 2;
}

void o_newton_batch(const owfn *w, long n, double *xyz, double gfnormeps, int maxit,
                    int *ier, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic)
  for (long i = 0; i < n; i++) ier[i] = o_newton(w, xyz + 3 * i, gfnormeps, maxit);
}

/* Default molecular seeding, src/autocp@proc.f90:423-437 (pairs within
 * maxdist, npts points at fractions k/(npts+1)), then the molecular-cell
 * border filter (:672-693).  Returns the number of seeds written. */
int o_pair_seeds(const owfn *w, double maxdist, int npts, double *xseed, int maxseed) {
  int nn = 0;
  for (int i1 = 0; i1 < w->natom; i1++)
    for (int i2 = 0; i2 < w->natom; i2++) {
      if (i1 == i2) continue;
      const double *a = w->xyz + 3 * i1, *b = w->xyz + 3 * i2;
      double d = sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                      (a[2] - b[2]) * (a[2] - b[2]));
      if (d > maxdist) continue;
      for (int k = 1; k <= npts; k++) {
        double x[3], keep = 1;
        for (int c = 0; c < 3; c++) {
          double xa = (a[c] - w->cell_lo[c]) / w->aa[c], xb = (b[c] - w->cell_lo[c]) / w->aa[c];
          double xf = xa + (double)k / (double)(npts + 1) * (xb - xa);
          xf -= floor(xf);
          if (xf < w->molborder[c] || xf > 1.0 - w->molborder[c]) keep = 0;
          x[c] = w->cell_lo[c] + xf * w->aa[c];
        }
        if (!keep) continue;
        if (nn < maxseed) memcpy(xseed + 3 * nn, x, sizeof(x));
        nn++;
      }
    }
  return nn;
}

typedef struct {
  double x[3]; /* cell-fractional */
  double r[3]; /* Cartesian */
  double f;
  int typ, typind, isnuc;
} ocp;

/* field%addcp for a molecule, src/fieldmod@proc.f90:2288-2439 (no
 * symmetry: every CP has multiplicity 1). Returns 1 when the CP is added. */
static int addcp(const owfn *w, const double x0[3], double cpeps, double nuceps,
                 double nucepsh, double gfnormeps, ocp *cps, int *ncp, int maxcp) {
  double xc[3], x1[3];
  for (int j = 0; j < 3; j++) {
    xc[j] = (x0[j] - w->cell_lo[j]) / w->aa[j];
    xc[j] -= floor(xc[j]);
    if (xc[j] < w->molborder[j] || xc[j] > 1.0 - w->molborder[j]) return 0;
    x1[j] = w->cell_lo[j] + xc[j] * w->aa[j];
  }
  /* nearest CP (nearest_cp, src/fieldmod@proc.f90:1883-1933) */
  int nid = -1;
  double dmin = 1e30;
  for (int i = 0; i < *ncp; i++) {
    double t[3], dd = 0;
    for (int j = 0; j < 3; j++) {
      t[j] = (cps[i].x[j] - (xc[j] - floor(xc[j]))) * w->aa[j];
      dd += t[j] * t[j];
    }
    dd = sqrt(dd);
    if (dd < dmin) dmin = dd, nid = i;
  }
  if (nid >= w->natom && dmin < cpeps) return 0;
  double dist;
  int at = identify_atom(w, x1, fmax(nuceps, nucepsh), &dist);
  if (at >= 0) {
    if (w->z[at] == 1) { if (dist < nucepsh) return 0; }
    else if (dist < nuceps) return 0;
  }
  ores res;
  o_grd(w, x1, 2, &res);
  if (!res.valid) return 0;
  if (res.gfmod >= gfnormeps) return 0;
  if (res.r != 3) return 0; /* degenerate CP discarded */
  if (*ncp >= maxcp) return 0;
  ocp *c = cps + (*ncp)++;
  memcpy(c->x, xc, sizeof(xc));
  memcpy(c->r, x1, sizeof(x1));
  c->f = res.f;
  c->typ = res.s;
  c->typind = (res.s + 3) / 2;
  c->isnuc = 0;
  return 1;
}

/* autocritic core, src/autocp@proc.f90:755-822: Newton from every seed
 * (parallel), addcp on the converged ones (serial, in seed order, which is
 * one valid order of the reference's omp critical section), then sortcps
 * (src/fieldmod@proc.f90:2441-2466): non-nuclear CPs by type, then by
 * decreasing density.  Outputs Cartesian positions, types and densities;
 * nuc_count[4] = n, b, r, c counts.  Returns ncp. */
int o_autocritic(const owfn *w, int nseed, const double *xseed, int nthreads, int maxcp,
                 double *cp_xyz, int *cp_typ, double *cp_f, int *nuc_count) {
  const double gfnormeps = 1e-12, cpeps = 1e-2, nuceps = 1e-1, nucepsh = 2e-1;
  double *x = malloc(sizeof(double) * 3 * (size_t)(nseed > 0 ? nseed : 1));
  int *ier = malloc(sizeof(int) * (size_t)(nseed > 0 ? nseed : 1));
  memcpy(x, xseed, sizeof(double) * 3 * (size_t)nseed);
  o_newton_batch(w, nseed, x, gfnormeps, 200, ier, nthreads);
  int cap = w->natom + nseed + 1;
  ocp *cps = calloc((size_t)cap, sizeof(ocp));
  int ncp = 0;
  /* init_cplist: nuclei first (src/fieldmod@proc.f90:1795-1852) */
  for (int a = 0; a < w->natom; a++) {
    ocp *c = cps + ncp++;
    for (int j = 0; j < 3; j++) {
      c->r[j] = w->xyz[3 * a + j];
      c->x[j] = (c->r[j] - w->cell_lo[j]) / w->aa[j];
      c->x[j] -= floor(c->x[j]);
    }
    c->typ = -3; c->typind = 0; c->isnuc = 1;
    ores res;
    o_grd(w, c->r, 2, &res);
    c->f = res.f;
  }
  for (int i = 0; i < nseed; i++)
    if (ier[i] <= 0) addcp(w, x + 3 * i, cpeps, nuceps, nucepsh, fmax(1e-4, gfnormeps), cps, &ncp, cap);
  /* sortcps: stable sort by -f, then stable sort by typind (non-nuclear part) */
  int nn = ncp - w->natom;
  ocp *tail = cps + w->natom;
  for (int pass = 0; pass < 2; pass++) {
    for (int i = 1; i < nn; i++) {
      ocp t = tail[i];
      int j = i - 1;
      while (j >= 0 && (pass == 0 ? (-tail[j].f > -t.f) : (tail[j].typind > t.typind))) {
        tail[j + 1] = tail[j];
        j--;
      }
      tail[j + 1] = t;
    }
  }
  for (int k = 0; k < 4; k++) nuc_count[k] = 0;
  for (int i = 0; i < ncp; i++) {
    nuc_count[cps[i].typind]++;
    if (i < maxcp) {
      memcpy(cp_xyz + 3 * i, cps[i].r, sizeof(double) * 3);
      cp_typ[i] = cps[i].typ;
      cp_f[i] = cps[i].f;
    }
  }
  free(x);
  free(ier);
  free(cps);
  return ncp;
}

/* ------------------------------------------------------- molecular graph */
/* Symmetric 3x3 eigenvalues and eigenvectors (column-major input), the role
 * of eigsym (LAPACK dsyev 'V', src/tools_math@proc.f90:1005-1039): cyclic
 * Jacobi, eigenvalues ascending, vec column j (vec[3*j..3*j+2]) for ev[j].
 * dsyev's sign of an eigenvector is not reproduced: each vector is scaled
 * so that its component of largest magnitude (the first such) is positive. */
void o_eigvec3(const double m[9], double ev[3], double vec[9]) {
  double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = 0.5 * (m[3 * j + i] + m[3 * i + j]);
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    double dia = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off == 0.0 || off < 1e-34 * dia) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; k++) {
          double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
  int ord[3] = {0, 1, 2};
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2 - i; j++)
      if (a[ord[j]][ord[j]] > a[ord[j + 1]][ord[j + 1]]) { int t = ord[j]; ord[j] = ord[j + 1]; ord[j + 1] = t; }
  for (int j = 0; j < 3; j++) {
    int c = ord[j];
    ev[j] = a[c][c];
    int big = 0;
    for (int k = 1; k < 3; k++)
      if (fabs(v[k][c]) > fabs(v[big][c])) big = k;
    double sg = v[big][c] < 0.0 ? -1.0 : 1.0;
    for (int k = 0; k < 3; k++) vec[3 * j + k] = sg * v[k][c];
  }
}

#define NAV_STEP 0.3      /* src/global@proc.F90:859 */
#define NAV_MAXERR 1e-4   /* :860 */
#define NAV_GRADEPS 1e-7  /* :861 */
#define RBETADEF 0.1      /* src/global.f90:41 */

static void unit_grad(const ores *r, double g[3]) {
  for (int j = 0; j < 3; j++) g[j] = r->gf[j] / (r->gfmod + VSMALL);
}

/* stepper_bs, src/fieldmod@proc.f90:2860-2890 (Bogacki-Shampine 2(3),
 * FSAL): res ends as the evaluation at xout. */
static void stepper_bs(const owfn *w, const double x[3], const double ak1[3], double h0, double xout[3],
                       double xerr[3], ores *res) {
  double ak2[3], ak3[3], ak4[3], xt[3];
  for (int j = 0; j < 3; j++) xt[j] = x[j] + h0 * (0.5 * ak1[j]);
  o_grd(w, xt, 2, res);
  unit_grad(res, ak2);
  for (int j = 0; j < 3; j++) xt[j] = x[j] + h0 * (0.75 * ak2[j]);
  o_grd(w, xt, 2, res);
  unit_grad(res, ak3);
  for (int j = 0; j < 3; j++) xout[j] = x[j] + h0 * (2.0 / 9.0 * ak1[j] + 1.0 / 3.0 * ak2[j] + 4.0 / 9.0 * ak3[j]);
  o_grd(w, xout, 2, res);
  unit_grad(res, ak4);
  for (int j = 0; j < 3; j++)
    xerr[j] = x[j] + h0 * (7.0 / 24.0 * ak1[j] + 1.0 / 4.0 * ak2[j] + 1.0 / 3.0 * ak3[j] + 1.0 / 8.0 * ak4[j]) -
              xout[j];
}

/* adaptive_stepper with the BS stepper, src/fieldmod@proc.f90:2737-2830.
 * As in the reference, a rejected trial leaves its end-point gradient as
 * the first stage of the next trial. */
static int adaptive_stepper(const owfn *w, double x[3], double *h0, double maxstep, ores *res) {
  double grdt[3], xtemp[3], xerr[3];
  unit_grad(res, grdt);
  int first = 1;
  for (;;) {
    stepper_bs(w, x, grdt, *h0, xtemp, xerr, res);
    unit_grad(res, grdt);
    double nerr = sqrt(xerr[0] * xerr[0] + xerr[1] * xerr[1] + xerr[2] * xerr[2]);
    if (nerr < NAV_MAXERR) {
      for (int j = 0; j < 3; j++) x[j] = xtemp[j];
      if (first && nerr < NAV_MAXERR / 10.0)
        *h0 = copysign(fmin(fabs(maxstep), fabs(1.6 * *h0)), maxstep);
      return 1;
    }
    *h0 = 0.9 * *h0 * NAV_MAXERR / nerr;
    if (fabs(*h0) < VSMALL) return 0;
    first = 0;
  }
}

/* field%gradient for a molecule, src/fieldmod@proc.f90:2500-2732, with
 * critic2's default navigation (BS stepper, step 0.3, maxerr 1e-4,
 * gradeps 1e-7) and up2beta: a path stops in the beta sphere (0.1 bohr) of
 * the nearest CP of the attracting kind (-3 up, +3 down; the nearest
 * non-hydrogen nucleus counts first when going up), at a new CP
 * (|grad| < gradeps), when it leaves the molecular cell's inner region
 * (going down, ier 3), when it bounces (5 reversals) or the step falls
 * under 1e-12 (ier 1), or after nint(1000/0.3) steps (ier 2).  x: start
 * (in) and end point (out); plen starts at |x - pathini|. */
static int o_gradient_rb(const owfn *w, double x[3], int iup, int ncp, const double *cpx, const int *cptyp,
                         const double *rbeta, const double pathini[3], int *nstep_out, double *plen_out);

int o_gradient(const owfn *w, double x[3], int iup, int ncp, const double *cpx, const int *cptyp,
               const double pathini[3], int *nstep_out, double *plen_out) {
  return o_gradient_rb(w, x, iup, ncp, cpx, cptyp, NULL, pathini, nstep_out, plen_out);
}

/* The same with up2beta and per-CP beta radii rbeta (the CP list starting
 * with the nuclei in atom order, so that a nucleus found first is CP
 * idnuc); rbeta NULL: the default sphere min(Rbetadef, |hini|/2) = 0.1. */
static int o_gradient_rb(const owfn *w, double x[3], int iup, int ncp, const double *cpx, const int *cptyp,
                         const double *rbeta, const double pathini[3], int *nstep_out, double *plen_out) {
  const double minstep = 1e-12, hfirst = 0.01;
  const int mhist = 5;
  double hini = NAV_STEP * iup, h0 = hfirst * iup;
  double scalhist[5] = {1, 1, 1, 1, 1};
  int nhist = 0, ier = 0, incstep = 0, nstep;
  double xlast[3], xlast2[3];
  for (int j = 0; j < 3; j++) xlast[j] = xlast2[j] = x[j];
  double plen = sqrt((x[0] - pathini[0]) * (x[0] - pathini[0]) + (x[1] - pathini[1]) * (x[1] - pathini[1]) +
                     (x[2] - pathini[2]) * (x[2] - pathini[2]));
  const int mstep = (int)lround(10000 * 0.1 / fabs(hini));
  ores res;
  o_grd(w, x, 2, &res);
  for (nstep = 1; nstep <= mstep; nstep++) {
    double d[3];
    for (int j = 0; j < 3; j++) d[j] = x[j] - xlast[j];
    plen += sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    /* nearest nucleus, then nearer CPs of the attracting kind */
    double sphrad;
    int idnuc = identify_atom(w, x, 1e300, &sphrad);
    int idcp = -1;
    double cprad = 1e15, xcp[3] = {0, 0, 0};
    if (iup == 1 && w->z[idnuc] != 1) {
      idcp = idnuc;
      cprad = sphrad;
      for (int j = 0; j < 3; j++) xcp[j] = w->xyz[3 * idnuc + j];
    }
    for (int i = 0; i < ncp; i++) {
      if (!((cptyp[i] == -3 && iup == 1) || (cptyp[i] == 3 && iup == -1))) continue;
      double dx = x[0] - cpx[3 * i], dy = x[1] - cpx[3 * i + 1], dz = x[2] - cpx[3 * i + 2];
      double dist = sqrt(dx * dx + dy * dy + dz * dz);
      if (dist < cprad) {
        cprad = dist;
        idcp = i;
        for (int j = 0; j < 3; j++) xcp[j] = cpx[3 * i + j];
      }
    }
    if (idcp >= 0 && cprad <= (rbeta ? rbeta[idcp] : RBETADEF)) {
      incstep = 1;
      double e2 = 0.0;
      for (int j = 0; j < 3; j++) e2 += (x[j] - xcp[j]) * (x[j] - xcp[j]);
      plen += sqrt(e2);
      for (int j = 0; j < 3; j++) x[j] = xcp[j];
      ier = 0;
      goto done;
    }
    if (iup == -1) {
      for (int j = 0; j < 3; j++) {
        double xf = (x[j] - w->cell_lo[j]) / w->aa[j];
        if (xf < w->molborder[j] || xf > 1.0 - w->molborder[j]) { ier = 3; goto done; }
      }
    }
    if (res.gfmod < NAV_GRADEPS) { ier = 0; goto done; }
    for (int j = 0; j < 3; j++) xlast2[j] = xlast[j], xlast[j] = x[j];
    int ok = adaptive_stepper(w, x, &h0, hini, &res);
    nhist = nhist % mhist + 1;
    double sc = 0.0;
    for (int j = 0; j < 3; j++) sc += (xlast[j] - xlast2[j]) * (x[j] - xlast[j]);
    scalhist[nhist - 1] = sc;
    int allneg = 1;
    for (int k = 0; k < mhist; k++) allneg &= scalhist[k] < 0.0;
    ok = ok && !allneg;
    if (!ok || fabs(h0) < minstep) {
      for (int j = 0; j < 3; j++) x[j] = xlast[j];
      ier = 1;
      goto done;
    }
  }
  nstep = mstep;
  ier = 2;
done:
  if (incstep) nstep++;
  *nstep_out = nstep;
  *plen_out = plen;
  return ier;
}

/* makegraph, src/autocp@proc.f90:2116-2268, for a molecule without
 * symmetry: for each bond (typ -1) and ring (typ +1) CP, two paths from
 * r +- 0.01 e (e: Hessian eigenvector of the largest eigenvalue for a bond
 * CP, of the smallest for a ring CP), up for bonds and down for rings;
 * ipath(j) = 1-based index of the CP of type 3 typ nearest to the end
 * point (no distance limit), -1 when there is none and the end point is
 * outside the molecular cell's inner region, else 0; brdist = |end - r|,
 * brpathlen = path length, brang = angle (degrees) between the two end
 * vectors.  Other CPs get zeros.  Arrays: ipath, brdist, brpathlen, ier,
 * nstep (2, ncp); brang (ncp); brvec (3, ncp). */
void o_makegraph(const owfn *w, int ncp, const double *cpx, const int *cptyp, int *ipath, double *brdist,
                 double *brpathlen, double *brang, double *brvec, int *ier, int *nstep, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < ncp; i++) {
    for (int j = 0; j < 2; j++) {
      ipath[2 * i + j] = 0, brdist[2 * i + j] = 0.0, brpathlen[2 * i + j] = 0.0;
      ier[2 * i + j] = 0, nstep[2 * i + j] = 0;
    }
    brang[i] = 0.0;
    for (int k = 0; k < 3; k++) brvec[3 * i + k] = 0.0;
    if (abs(cptyp[i]) != 1) continue;
    const int isbcp = cptyp[i] == -1;
    const double *r = cpx + 3 * i;
    ores res;
    o_grd(w, r, 2, &res);
    double ev[3], vec[9], xx[3];
    o_eigvec3(res.hf, ev, vec);
    const double *e = isbcp ? vec + 6 : vec;
    double nn = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    for (int k = 0; k < 3; k++) xx[k] = e[k] / nn;
    double xd[2][3], xdif[2][3];
    for (int j = 0; j < 2; j++) {
      for (int k = 0; k < 3; k++) xd[j][k] = r[k] + (j == 0 ? 1.0 : -1.0) * 0.01 * xx[k];
      ier[2 * i + j] = o_gradient(w, xd[j], isbcp ? 1 : -1, ncp, cpx, cptyp, r, &nstep[2 * i + j],
                                  &brpathlen[2 * i + j]);
    }
    for (int k = 0; k < 3; k++) brvec[3 * i + k] = xx[k];
    for (int j = 0; j < 2; j++) {
      double dd = 0.0;
      for (int k = 0; k < 3; k++) xdif[j][k] = xd[j][k] - r[k], dd += xdif[j][k] * xdif[j][k];
      brdist[2 * i + j] = sqrt(dd);
      /* nearest CP of type 3*typ, end point wrapped into the cell */
      double xf[3], best = 1e30;
      int wcp = 0, outside = 0;
      for (int k = 0; k < 3; k++) {
        double f = (xd[j][k] - w->cell_lo[k]) / w->aa[k];
        if (f < w->molborder[k] || f > 1.0 - w->molborder[k]) outside = 1;
        xf[k] = f - floor(f);
      }
      for (int c = 0; c < ncp; c++) {
        if (cptyp[c] != 3 * cptyp[i]) continue;
        double d2 = 0.0;
        for (int k = 0; k < 3; k++) {
          double t = ((cpx[3 * c + k] - w->cell_lo[k]) / w->aa[k] - xf[k]) * w->aa[k];
          d2 += t * t;
        }
        double dist = sqrt(d2);
        if (dist < best) best = dist, wcp = c + 1;
      }
      ipath[2 * i + j] = wcp ? wcp : (outside ? -1 : 0);
    }
    double ca = 0.0;
    if (brdist[2 * i] > 1e-12) {
      for (int k = 0; k < 3; k++) ca += xdif[0][k] * xdif[1][k];
      ca = ca / brdist[2 * i] / brdist[2 * i + 1];
    }
    if (fabs(ca) > 1.0) ca = ca / fabs(ca);
    brang[i] = acos(ca) * 180.0 / M_PI;
  }
}

/* ------------------------------------------------------ molecular meshes */
/* genmesh_becke / genmesh_franchini, src/meshmod@proc.f90:79-371, and the
 * radial helpers :508-627, for a molecule without lattice images.  The
 * angular rule (nang points x, y, z, w with w summing to 1) is given by the
 * caller.  Output in critic2's order: atoms, radial shells, angular points. */
static const double O_ZETA[103] = {
    0.8, 0.9, 1.8, 1.4, 1.3, 1.1, 0.9, 0.9, 0.9, 0.9, 1.4, 1.3, 1.3, 1.2, 1.1, 1.0, 1.0, 1.0, 1.5, 1.4,
    1.3, 1.2, 1.2, 1.2, 1.2, 1.2, 1.2, 1.1, 1.1, 1.1, 1.1, 1.0, 0.9, 0.9, 0.9, 0.9, 1.4, 1.4, 1.1, 1.3,
    1.0, 1.2, 0.9, 0.9, 0.9, 1.0, 0.9, 1.0, 1.0, 1.3, 1.2, 1.2, 0.9, 1.0, 1.7, 1.5, 1.5, 1.3, 1.3, 1.4,
    1.8, 1.4, 1.2, 1.3, 1.3, 1.4, 1.1, 1.1, 1.2, 1.6, 1.4, 1.3, 1.2, 1.0, 1.0, 0.9, 1.3, 1.2, 1.2, 1.0,
    1.2, 1.2, 1.1, 1.2, 1.1, 2.1, 2.2, 1.8, 1.7, 1.3, 1.4, 1.2, 1.2, 1.3, 1.4, 1.4, 1.7, 1.9, 1.9, 2.0,
    2.0, 1.6, 2.0};

int o_z2nr(int z, int lvl) {
  int nr = 15;
  if (z > 2) nr = 20;
  if (z > 10) nr = 25;
  if (z > 18) nr = 35;
  if (z > 36) nr = 60;
  if (z > 54) nr = 85;
  if (z > 86) nr = 110;
  /* default-kind (single precision) literals in critic2 */
  static const float f[6] = {0.f, 2.37f, 3.08f, 3.42f, 4.27f, 6.72f};
  return (int)ceilf((float)nr * f[lvl]);
}

/* gauleg on (-1, 1): ascending nodes, Newton on the Legendre recurrence */
static void o_gauleg(int n, double *x, double *w) {
  for (int i = 1; i <= (n + 1) / 2; i++) {
    double z = cos(M_PI * (i - 0.25) / (n + 0.5)), pp = 0.0, z1;
    do {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; j++) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (fabs(z - z1) > 1e-15);
    x[i - 1] = -z;
    x[n - i] = z;
    w[i - 1] = w[n - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

static void o_radial(int type, int n, int z, double *r, double *wr) {
  const double fourpi = 4.0 * M_PI;
  if (type == 1) { /* rmesh_postg */
    double rmid = 1.0 / pow((double)z, 1.0 / 3.0), h = 1.0 / (n + 1);
    for (int i = 1; i <= n; i++) {
      double q = h * i;
      r[i - 1] = rmid * q / (1.0 - q);
      wr[i - 1] = fourpi * h * r[i - 1] * r[i - 1] * rmid / ((1.0 - q) * (1.0 - q));
    }
  } else { /* rmesh_franchini */
    double *q = malloc(sizeof(double) * n), *wq = malloc(sizeof(double) * n);
    o_gauleg(n, q, wq);
    double zeta = O_ZETA[z - 1], l2 = log(2.0);
    for (int i = 0; i < n; i++) {
      double l = log(2.0 / (1.0 - q[i]));
      r[i] = zeta / l2 * (1.0 + q[i]) * l;
      wr[i] = fourpi * r[i] * r[i] * wq[i] * zeta / l2 * (l + (1.0 + q[i]) / (1.0 - q[i]));
    }
    free(q);
    free(wq);
  }
}

long o_mesh_size(const owfn *w, int lvl, int nang) {
  long n = 0;
  for (int a = 0; a < w->natom; a++) n += (long)o_z2nr(w->z[a], lvl) * nang;
  return n;
}

void o_mesh(const owfn *w, int type, int lvl, int nang, const double *ang, double *xyz, double *wt,
            int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  int na = w->natom;
  long *off = malloc(sizeof(long) * (na + 1));
  off[0] = 0;
  for (int a = 0; a < na; a++) off[a + 1] = off[a] + (long)o_z2nr(w->z[a], lvl) * nang;
  double rmax = 0.0, *rr = NULL;
  if (type == 2) {
    int mr = -1, izmr = -1;
    for (int a = 0; a < na; a++) {
      int nr = o_z2nr(w->z[a], lvl);
      if (nr > mr || (nr == mr && w->z[a] > izmr)) mr = nr, izmr = w->z[a];
    }
    double *r = malloc(sizeof(double) * mr), *wr = malloc(sizeof(double) * mr);
    o_radial(2, mr, izmr, r, wr);
    rmax = fmax(r[mr - 1], 12.0);
    free(r);
    free(wr);
  } else {
    rr = calloc((size_t)na * na, sizeof(double));
    for (int i = 0; i < na; i++)
      for (int j = i + 1; j < na; j++) {
        const double *a = w->xyz + 3 * i, *b = w->xyz + 3 * j;
        rr[(size_t)i * na + j] = rr[(size_t)j * na + i] =
            sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
      }
  }
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < na; i++) {
    int nr = o_z2nr(w->z[i], lvl);
    double *r = malloc(sizeof(double) * nr), *wr = malloc(sizeof(double) * nr);
    double *cut = type == 1 ? malloc(sizeof(double) * (size_t)na * na) : NULL;
    o_radial(type, nr, w->z[i], r, wr);
    double fscal = w->z[i] == 1 ? 0.3 : 1.0;
    const double *c = w->xyz + 3 * i;
    for (int ir = 0; ir < nr; ir++) {
      double vp0f = fscal * exp(-2.0 * r[ir]) / pow(fmax(r[ir], 1e-10), 3);
      for (int il = 0; il < nang; il++) {
        long p = off[i] + (long)ir * nang + il;
        double x[3];
        for (int k = 0; k < 3; k++) x[k] = c[k] + r[ir] * ang[4 * il + k];
        double part;
        if (type == 2) {
          double vpsum = 0.0;
          for (int j = 0; j < na; j++) {
            const double *b = w->xyz + 3 * j;
            double dd = (x[0] - b[0]) * (x[0] - b[0]) + (x[1] - b[1]) * (x[1] - b[1]) + (x[2] - b[2]) * (x[2] - b[2]);
            if (!(dd <= rmax * rmax)) continue;
            double d = sqrt(dd), dm = fmax(d, 1e-10);
            vpsum += (w->z[j] == 1 ? 0.3 : 1.0) * exp(-2.0 * d) / (dm * dm * dm);
          }
          vpsum = fmax(vp0f, vpsum);
          part = vp0f / fmax(vpsum, 1e-40);
        } else {
          for (int j = 1; j < na; j++) {
            for (int k = 0; k < j; k++) {
              const double *bj = w->xyz + 3 * j, *bk = w->xyz + 3 * k;
              double r1 = sqrt((x[0] - bj[0]) * (x[0] - bj[0]) + (x[1] - bj[1]) * (x[1] - bj[1]) + (x[2] - bj[2]) * (x[2] - bj[2]));
              double r2 = sqrt((x[0] - bk[0]) * (x[0] - bk[0]) + (x[1] - bk[1]) * (x[1] - bk[1]) + (x[2] - bk[2]) * (x[2] - bk[2]));
              double h = (r1 - r2) / rr[(size_t)j * na + k];
              for (int it = 0; it < 4; it++) h = 1.5 * h - 0.5 * h * h * h;
              cut[(size_t)j * na + k] = (1.0 - h) / 2.0;
              cut[(size_t)k * na + j] = (1.0 + h) / 2.0;
            }
            cut[(size_t)j * na + j] = 1.0;
          }
          cut[0] = 1.0;
          double vp0 = 1.0, vpsum = 0.0;
          for (int j = 0; j < na; j++) {
            vp0 *= cut[(size_t)i * na + j];
            double vpi = 1.0;
            for (int k = 0; k < na; k++) vpi *= cut[(size_t)j * na + k];
            vpsum += vpi;
          }
          part = vp0 / vpsum;
        }
        for (int k = 0; k < 3; k++) xyz[3 * p + k] = x[k];
        wt[p] = part * wr[ir] * ang[4 * il + 3];
      }
    }
    free(r);
    free(wr);
    free(cut);
  }
  free(off);
  free(rr);
}

/* ------------------------------------------------------------ NCI output */
/* Fortran list output of (" ",1p,e13.5e3): blank, then the number right-
 * justified in 13 columns with 6 significant digits and a 3-digit
 * exponent (the C library's conversion is correctly rounded). */
void o_fmt_e13_5e3(double x, char *out) {
  char buf[64], t[96];
  snprintf(buf, sizeof buf, "%.5E", x);
  char *p = strchr(buf, 'E');
  int e = atoi(p + 1);
  *p = 0;
  snprintf(t, sizeof t, " %8sE%c%03d", buf, e < 0 ? '-' : '+', e < 0 ? -e : e);
  memcpy(out, t, 14);
}

/* 1p,E15.7: 8 significant digits right-justified in 15 columns; an
 * exponent beyond +-99 is written as sign and three digits, without E. */
void o_fmt_E15_7(double x, char *out) {
  char buf[64], t[96];
  snprintf(buf, sizeof buf, "%.7E", x);
  char *p = strchr(buf, 'E');
  int e = atoi(p + 1);
  *p = 0;
  int ae = e < 0 ? -e : e;
  if (ae > 99) snprintf(t, sizeof t, "%11s%c%03d", buf, e < 0 ? '-' : '+', ae);
  else snprintf(t, sizeof t, "%11sE%c%02d", buf, e < 0 ? '-' : '+', ae);
  memcpy(out, t, 15);
}

/* write_cube_body: do i; do j; write (lu,'(6(" ",1p,e13.5e3))') c(:,j,i)
 * (src/nci@proc.f90:916-932) */
long o_cube_body(const int nstep[3], const double *v, char *out) {
  long o = 0;
  for (long r = 0; r < (long)nstep[0] * nstep[1]; r++)
    for (int k = 0; k < nstep[2]; k++) {
      o_fmt_e13_5e3(v[r * nstep[2] + k], out + o);
      o += 14;
      /* a line with fewer than 6 numbers keeps the blank of the next
       * (" ",...) item before the format runs out of data */
      if (k == nstep[2] - 1 && nstep[2] % 6 != 0) out[o++] = ' ';
      if (k % 6 == 5 || k == nstep[2] - 1) out[o++] = '\n';
    }
  return o;
}

/* nciplot's cutoff pass without fragments or void (nci@proc.f90:612-645) */
long o_nci_post(const int nstep[3], const double *crho, double *cgrad, double rhocut, double dimcut,
                double rhoplot, double srho_lo, double srho_hi, int onlyneg, double *dat) {
  long nd = 0;
  const long n = (long)nstep[0] * nstep[1] * nstep[2];
  for (long v = 0; v < n; v++) {
    if (fabs(crho[v]) < rhocut * 100.0 && cgrad[v] < dimcut) {
      dat[2 * nd] = crho[v] / 100.0;
      dat[2 * nd + 1] = cgrad[v];
      nd++;
    }
    if (fabs(crho[v]) > rhoplot * 100.0) cgrad[v] = 100.0;
    if (crho[v] < srho_lo * 100.0 || crho[v] > srho_hi * 100.0) cgrad[v] = 100.0;
    if (crho[v] > 0 && onlyneg) cgrad[v] = 100.0;
  }
  return nd;
}

/* E22.14E3 without scale factor (writegrid_cube's precise format,
 * src/crystalmod@write.f90:3536-3563): 0.dddddddddddddd (14 digits) and
 * a 3-digit exponent, right-justified in 22 columns. */
void o_fmt_E22_14E3(double x, char *out) {
  char buf[64], t[96];
  snprintf(buf, sizeof buf, "%.13E", x);
  char *p = strchr(buf, 'E');
  int e = atoi(p + 1) + (x != 0.0 ? 1 : 0);
  *p = 0;
  const int neg = buf[0] == '-';
  const char *m = buf + neg; /* d.ddddddddddddd */
  char dig[16];
  dig[0] = m[0];
  memcpy(dig + 1, m + 2, 13);
  dig[14] = 0;
  snprintf(t, sizeof t, "%c0.%sE%c%03d", neg ? '-' : ' ', dig, e < 0 ? '-' : '+', e < 0 ? -e : e);
  memcpy(out, t, 22);
}

/* ------------------------------------------------------------------ */
/* Atomic-basin integrals by bisection (critic2's INTEGRALS for a molecule,
 * src/bisect@proc.f90:862-1028), the surface search of bisect_msurface
 * (:1208-1446) and lim_surf (:1039-1126), the radial quadrature of
 * int_radialquad (src/integration@proc.f90:384-486, Gauss-Legendre, 50
 * nodes) and the angular sums of lebedev_mquad / gauleg_mquad (:495-642),
 * with a 170-point Lebedev beta sphere (sphereintegrals_lebedev,
 * src/bisect@proc.f90:829-854).  Integrated: the valence density and its
 * Laplacian (grdall's fval and del2fval for critic2's molecular default
 * properties Pop and Lap). */

#define BS_RNEARNUC 3.1622776601683794e-3 /* sqrt(1e-5), src/bisect@proc.f90:50 */
#define BS_NTRIES 7
#define BS_NRAD 50

typedef struct {
  int idone;
  double rnearsum, rfarsum, rzfssum, rnearmin, rfarmax;
} o_bstats;

static int cmp_dbl(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

static double dist3(const double *a, const double *b) {
  double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
  return sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

/* up-path from x; returns ier, end point in x */
static int o_uppath(const owfn *w, double x[3], int ncp, const double *cpx, const int *cptyp, const double *rbeta) {
  int nstep;
  double plen;
  return o_gradient_rb(w, x, 1, ncp, cpx, cptyp, rbeta, x, &nstep, &plen);
}

/* lim_surf: bisection between xin and xfin to within delta; restarts with
 * a smaller beta sphere when the result lies in one of the attractor's
 * type.  Returns the surface point in xmed. */
static void o_lim_surf(const owfn *w, int ncp, const double *cpx, const int *cptyp, double *rbeta, const double *xnuc,
                       int typ, const double xin[3], const double xfin[3], double delta, double xmed[3], int *nwarn,
                       int *nrestart) {
  for (;;) {
    double xi[3], xf[3];
    for (int j = 0; j < 3; j++) xi[j] = xin[j], xf[j] = xfin[j];
    while (dist3(xi, xf) > delta) {
      double xp[3];
      for (int j = 0; j < 3; j++) xmed[j] = xp[j] = 0.5 * (xi[j] + xf[j]);
      int ier = o_uppath(w, xp, ncp, cpx, cptyp, rbeta), inside;
      if (ier <= 0) {
        inside = dist3(xp, xnuc) <= BS_RNEARNUC;
      } else if (ier == 3) {
        inside = 0;
      } else {
        double best = 1e300;
        (*nwarn)++;
        for (int i = 0; i < ncp; i++)
          if (cptyp[i] == -3) best = fmin(best, dist3(cpx + 3 * i, xp));
        inside = best <= BS_RNEARNUC;
      }
      for (int j = 0; j < 3; j++) {
        if (inside) xi[j] = xmed[j];
        else xf[j] = xmed[j];
      }
    }
    for (int j = 0; j < 3; j++) xmed[j] = 0.5 * (xi[j] + xf[j]);
    int again = 0;
    for (int i = 0; i < ncp && !again; i++) {
      if (cptyp[i] != typ) continue;
      if (dist3(cpx + 3 * i, xmed) <= rbeta[i]) {
        rbeta[i] *= 0.75;
        (*nrestart)++;
        again = 1;
      }
    }
    if (!again) return;
  }
}

/* bisect_msurface for one ray u of the attractor at xcar; st NULL: every
 * ray takes the first ray's bracket tries.  Returns the surface radius, or
 * -1 when no bracket is found ("Can not find ray limits"). */
static double o_bisect_ray(const owfn *w, int ncp, const double *cpx, const int *cptyp, double *rbeta,
                           const double *xcar, int typ, double rmin, double rminsame, const double u[3], double prec,
                           o_bstats *st, int *nwarn, int *nrestart) {
  const double vbig = DBL_MAX;
  double amin = fmin(w->aa[0], fmin(w->aa[1], w->aa[2])), amax = fmax(w->aa[0], fmax(w->aa[1], w->aa[2]));
  int idone = st ? st->idone : 0;
  double rtry[BS_NTRIES], x[3];
  double rother = vbig, raprox = vbig, riaprox = 0.0;
  rtry[0] = 2e-5, rtry[1] = 0.9 * rmin, rtry[2] = 0.99 * rmin;
  if (idone > 0) {
    rtry[3] = 0.99 * st->rnearmin, rtry[4] = st->rnearsum / idone, rtry[5] = 0.8 * st->rzfssum / idone, rtry[6] = 0.0;
  } else {
    rtry[3] = rtry[4] = rtry[5] = rtry[6] = 0.0;
  }
  qsort(rtry, BS_NTRIES, sizeof(double), cmp_dbl);
  for (int k = BS_NTRIES - 1; k >= 0; k--) {
    riaprox = rtry[k];
    for (int j = 0; j < 3; j++) x[j] = xcar[j] + riaprox * u[j];
    int ier = o_uppath(w, x, ncp, cpx, cptyp, rbeta);
    if (ier == 3) {
      if (rtry[k] < rother) rother = rtry[k];
    } else {
      if (ier > 0) (*nwarn)++;
      if (dist3(x, xcar) <= BS_RNEARNUC) break;
      if (rtry[k] < rother) rother = rtry[k];
    }
  }
  rtry[0] = amin, rtry[1] = 0.99 * rminsame, rtry[2] = 0.75 * rminsame;
  if (idone > 0) {
    rtry[3] = 1.01 * st->rfarmax, rtry[4] = st->rfarsum / idone, rtry[5] = 1.2 * st->rzfssum / idone, rtry[6] = amax;
  } else {
    rtry[3] = rtry[4] = rtry[5] = rtry[6] = amax;
  }
  qsort(rtry, BS_NTRIES, sizeof(double), cmp_dbl);
  raprox = rother;
  for (int k = 0; k < BS_NTRIES; k++) {
    raprox = rtry[k];
    if (raprox > (rother + riaprox) / 2.0 || raprox < riaprox) {
      raprox = rother;
      continue;
    }
    for (int j = 0; j < 3; j++) x[j] = xcar[j] + raprox * u[j];
    int ier = o_uppath(w, x, ncp, cpx, cptyp, rbeta);
    if (ier == 3) {
      if (raprox > riaprox) riaprox = raprox;
      raprox = rother;
    } else {
      if (ier > 0) (*nwarn)++;
      if (dist3(x, xcar) > BS_RNEARNUC) break;
      if (raprox > riaprox) riaprox = raprox;
      raprox = rother;
    }
  }
  if (raprox == vbig || riaprox == 0.0) return -1.0;
  double xin[3], xfin[3], xmed[3];
  for (int j = 0; j < 3; j++) xin[j] = xcar[j] + riaprox * u[j], xfin[j] = xcar[j] + raprox * u[j];
  o_lim_surf(w, ncp, cpx, cptyp, rbeta, xcar, typ, xin, xfin, prec, xmed, nwarn, nrestart);
  double rlim = dist3(xmed, xcar);
  if (st) {
    st->rnearsum += riaprox, st->rfarsum += raprox, st->rzfssum += rlim;
    st->rnearmin = fmin(st->rnearmin, riaprox), st->rfarmax = fmax(st->rfarmax, raprox);
    st->idone++;
  }
  return rlim;
}

/* gauleg on (a, b), ascending */
static void o_gauleg_ab(double a, double b, int n, double *x, double *wt) {
  o_gauleg(n, x, wt);
  double xm = 0.5 * (b + a), xl = 0.5 * (b - a);
  for (int i = 0; i < n; i++) x[i] = xm + xl * x[i], wt[i] *= xl;
}

/* int_radialquad with Gauss-Legendre: integral of r^2 (fval, del2fval)
 * from r0 to rend along u; iaserr from the end point */
static void o_radialquad(const owfn *w, const double *x0, const double u[3], double r0, double rend, double prec,
                         double lp[2], double ie[2]) {
  double rr[BS_NRAD], rw[BS_NRAD], r1 = r0, r2 = rend, sg = 1.0;
  if (rend <= r0) r1 = rend, r2 = r0, sg = -1.0;
  o_gauleg_ab(r1, r2, BS_NRAD, rr, rw);
  lp[0] = lp[1] = 0.0;
  for (int k = 0; k < BS_NRAD; k++) {
    double x[3];
    ores res;
    for (int j = 0; j < 3; j++) x[j] = x0[j] + rr[k] * u[j];
    o_grd(w, x, 2, &res);
    lp[0] += rr[k] * rr[k] * rw[k] * res.fval;
    lp[1] += rr[k] * rr[k] * rw[k] * res.del2fval;
  }
  lp[0] *= sg, lp[1] *= sg;
  if (ie) {
    double x[3];
    ores res;
    for (int j = 0; j < 3; j++) x[j] = x0[j] + rend * u[j];
    o_grd(w, x, 2, &res);
    ie[0] = fabs(res.fval * rend * rend * prec);
    ie[1] = fabs(res.del2fval * rend * rend * prec);
  }
}

/* INTEGRALS for the attractors of the CP list (the nuclei, which it must
 * start with in atom order, and the CPs of type -3; cpid > 0: that CP
 * alone, 1-based).  Rays: unit vectors u(3, nray) with angular weights
 * wang; ring NULL sums them as lebedev_mquad (weights times 4 pi), else
 * ray i belongs to polar ring ring[i] whose factor sin(theta) w_theta is
 * ringw[ring[i]] and wang is the azimuthal weight (gauleg_mquad).  The beta
 * sphere uses usph/wsph (nsph points, weights times 4 pi).  stats: critic2's
 * running bracket statistics over the rays in order and beta radii shared
 * by all rays and attractors (serial, as critic2 with one thread); else
 * every ray takes the first ray's tries and shrinks its own copy of the
 * beta radii (rays in parallel).  Outputs per
 * attractor a: props(2, natt) Pop, Lap; iaserr(2, natt); rsurf(nray, natt);
 * rbeta_int(natt); att_cp(natt).  Returns the attractor count, or -1 when
 * a ray has no bracket. */
int o_basin_integrals(const owfn *w, int ncp, const double *cpx, const int *cptyp, int cpid, int nray,
                      const double *u, const double *wang, const int *ring, int nring, const double *ringw, int nsph,
                      const double *usph, const double *wsph, double prec, int stats, int nthreads, int *att_cp,
                      double *props, double *iaserr, double *rsurf, double *rbeta_int, int *nwarn_out,
                      int *nrestart_out) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  int lo = cpid > 0 ? cpid - 1 : 0, hi = cpid > 0 ? cpid : ncp, natt = 0, fail = 0, nwarn = 0, nrestart = 0;
  double *rbeta = malloc(sizeof(double) * (ncp > 0 ? ncp : 1));
  for (int i = 0; i < ncp; i++) rbeta[i] = RBETADEF;
  for (int c = lo; c < hi; c++) {
    if (!(c < w->natom || cptyp[c] == -3)) continue;
    const double *xcar = cpx + 3 * c;
    double rmin = DBL_MAX, rminsame = DBL_MAX;
    for (int i = 0; i < ncp; i++) {
      double d = dist3(cpx + 3 * i, xcar);
      if (d < 1e-5) continue;
      rmin = fmin(rmin, d);
      if (cptyp[i] == cptyp[c]) rminsame = fmin(rminsame, d);
    }
    double *r = rsurf + (size_t)natt * nray;
    if (stats) {
      o_bstats st = {0, 0.0, 0.0, 0.0, DBL_MAX, 0.0};
      for (int i = 0; i < nray && !fail; i++) {
        r[i] = o_bisect_ray(w, ncp, cpx, cptyp, rbeta, xcar, cptyp[c], rmin, rminsame, u + 3 * i, prec, &st, &nwarn,
                            &nrestart);
        if (r[i] < 0) fail = 1;
      }
    } else {
      /* every ray on its own copy of the beta radii */
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nwarn, nrestart)
      for (int i = 0; i < nray; i++) {
        double *rb = malloc(sizeof(double) * (ncp > 0 ? ncp : 1));
        for (int k = 0; k < ncp; k++) rb[k] = RBETADEF;
        r[i] = o_bisect_ray(w, ncp, cpx, cptyp, rb, xcar, cptyp[c], rmin, rminsame, u + 3 * i, prec, NULL, &nwarn,
                            &nrestart);
        free(rb);
      }
      for (int i = 0; i < nray; i++)
        if (r[i] < 0) fail = 1;
    }
    if (fail) break;
    double rmn = DBL_MAX;
    for (int i = 0; i < nray; i++) rmn = fmin(rmn, r[i]);
    double rb = 0.95 * rmn;
    /* the beta sphere */
    double sp[2] = {0, 0};
    for (int i = 0; i < nsph; i++) {
      double lp[2];
      o_radialquad(w, xcar, usph + 3 * i, 0.0, rb, prec, lp, NULL);
      sp[0] += lp[0] * wsph[i], sp[1] += lp[1] * wsph[i];
    }
    /* the rays */
    double *rp = malloc(sizeof(double) * 4 * (size_t)nray);
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < nray; i++) o_radialquad(w, xcar, u + 3 * i, rb, r[i], prec, rp + 4 * i, rp + 4 * i + 2);
    double lp[2] = {0, 0}, ie[2] = {0, 0};
    if (!ring) {
      for (int i = 0; i < nray; i++)
        for (int q = 0; q < 2; q++) lp[q] += rp[4 * i + q] * wang[i], ie[q] += rp[4 * i + 2 + q] * wang[i];
    } else {
      for (int t = 0; t < nring; t++) {
        double pr[2] = {0, 0}, pe[2] = {0, 0};
        for (int i = 0; i < nray; i++) {
          if (ring[i] != t) continue;
          for (int q = 0; q < 2; q++) pr[q] += rp[4 * i + q] * wang[i], pe[q] += rp[4 * i + 2 + q] * wang[i];
        }
        for (int q = 0; q < 2; q++) lp[q] += ringw[t] * pr[q], ie[q] += ringw[t] * pe[q];
      }
    }
    free(rp);
    for (int q = 0; q < 2; q++) {
      props[2 * natt + q] = lp[q] + sp[q];
      iaserr[2 * natt + q] = ie[q];
    }
    rbeta_int[natt] = rb;
    att_cp[natt] = c;
    natt++;
  }
  free(rbeta);
  if (nwarn_out) *nwarn_out = nwarn;
  if (nrestart_out) *nrestart_out = nrestart;
  return fail ? -1 : natt;
}

/* SPHEREINTEGRALS (src/bisect@proc.f90:573-784) for the attractors of the
 * CP list (as o_basin_integrals selects them): Pop and Lap inside nr
 * spheres of radius r0 exp(h (n - 1)), the last radius rend (rend < 0:
 * |rend| times half the distance to the nearest atom), each by the angular
 * rule (u, wang; ring/ringw as in o_basin_integrals) times 50 radial
 * Gauss-Legendre nodes on (0, r).  Outputs radii(nr, natt), props(2, nr,
 * natt), att_cp(natt).  Returns natt. */
int o_sphere_integrals(const owfn *w, int ncp, const double *cpx, const int *cptyp, int cpid, int nray,
                       const double *u, const double *wang, const int *ring, int nring, const double *ringw, int nr,
                       double r0, double rend, int nthreads, int *att_cp, double *radii, double *props) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  int lo = cpid > 0 ? cpid - 1 : 0, hi = cpid > 0 ? cpid : ncp, natt = 0;
  double *rp = malloc(sizeof(double) * 2 * (size_t)(nray > 0 ? nray : 1));
  for (int c = lo; c < hi; c++) {
    if (!(c < w->natom || cptyp[c] == -3)) continue;
    const double *xa = cpx + 3 * c;
    double rnn = DBL_MAX;
    for (int b = 0; b < w->natom; b++) {
      double d = dist3(w->xyz + 3 * b, xa);
      if (d > 0.0) rnn = fmin(rnn, d);
    }
    double rnn2 = w->natom <= 1 ? 0.0 : 0.5 * rnn;
    double h = nr > 1 ? log((rend < 0.0 ? rnn2 * fabs(rend) : rend) / r0) / (nr - 1) : 0.0;
    for (int n = 0; n < nr; n++) {
      double rad = nr == 1 ? (rend < 0.0 ? rnn2 * fabs(rend) : r0) : r0 * exp(n * h);
      radii[(size_t)natt * nr + n] = rad;
#pragma omp parallel for schedule(dynamic, 4)
      for (int i = 0; i < nray; i++) o_radialquad(w, xa, u + 3 * i, 0.0, rad, 1e-5, rp + 2 * i, NULL);
      double sp[2] = {0, 0};
      if (!ring) {
        for (int i = 0; i < nray; i++) sp[0] += rp[2 * i] * wang[i], sp[1] += rp[2 * i + 1] * wang[i];
      } else {
        for (int t = 0; t < nring; t++) {
          double pr[2] = {0, 0};
          for (int i = 0; i < nray; i++)
            if (ring[i] == t) pr[0] += rp[2 * i] * wang[i], pr[1] += rp[2 * i + 1] * wang[i];
          sp[0] += ringw[t] * pr[0], sp[1] += ringw[t] * pr[1];
        }
      }
      props[((size_t)natt * nr + n) * 2] = sp[0];
      props[((size_t)natt * nr + n) * 2 + 1] = sp[1];
    }
    att_cp[natt++] = c;
  }
  free(rp);
  return natt;
}
