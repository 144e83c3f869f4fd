/*
 * CPU oracle for the critic2 molecular-wavefunction evaluator path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C (+OpenMP) restatement of
 * critic2's FP64 algorithm for the path (rho2 / calculate_mo_gto, field%grd,
 * the NCI grid loop, field%newton, field%addcp, autocritic pair seeding and
 * the Poincare-Hopf count).  It is what the GPU library's results are
 * compared against in the tests, and the timed CPU baseline ("port") in bench.py.  The
 * product library never links, loads or calls it.
 *
 * Parity status: the post-processing (3x3 eigen-solve, rank/signature, spin
 * halves, Laplacian, |grad|, NCI reduced gradient) is pinned against the
 * POINT records in critic2's own test references (tests/golden).  The GTO
 * evaluator itself is pinned only by known-answer tests (analytic single
 * primitives, finite differences, normalisation integrals): the reference
 * cannot be compiled on these machines (no Fortran compiler) and its
 * wavefunction test inputs are not distributed with the source.
 *
 * Conventions: Cartesian bohr; cmo is (npri, nmo) C order = Fortran
 * cmo(nmo,npri); icenter/itype are 1-based on input.
 */
#ifndef CRITIC2_ORACLE_H
#define CRITIC2_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct owfn owfn;

/* scalar_value subset (src/types.f90:218-258) */
typedef struct {
  double f, fval;
  double gf[3];
  double gfmod, gfmodval;
  double hf[9];          /* column-major 3x3 */
  double hfeval[3];      /* ascending */
  double del2f, del2fval;
  double gkin;
  double fspin[2], gkinspin[2], lapspin[2], gfmodspin[2];
  double stress[9];
  double vir;
  int r, s, isnuc, valid;
} ores;

owfn *o_wfn_new(int natom, const double *xyz, const int *z, int npri, int nmo,
                const int *icenter, const int *itype, const double *e,
                const double *occ, const double *cmo, int wfntyp, int nalpha);
void o_wfn_free(owfn *w);
/* EDF core density (1-based icenter; nedf = 0 removes it) */
void o_wfn_set_edf(owfn *w, int nedf, const int *icenter, const int *itype, const double *e,
                   const double *c);
int o_wfn_npri(const owfn *w);
void o_wfn_cell(const owfn *w, double lo[3], double aa[3], double molborder[3]);

void o_rho2(const owfn *w, const double xpos[3], int nder, double rho[3], double rhoval[3],
            double grad[9], double gradval[9], double h[27], double hval[27],
            double gkin[3], double *vir, double stress[9]);
void o_grd(const owfn *w, const double v[3], int nder, ores *res);

void o_eigsym3(const double m[9], double ev[3]);
void o_rsindex(const double m[9], double ev[3], int *r, int *s, double eps);
int o_matinvsym3(double m[9]);

void o_nci_points(const owfn *w, long n, const double *xyz, double *crho, double *cgrad,
                  int nthreads);
void o_nciplot(const owfn *w, const double x0[3], const double xmat[9], const int nstep[3],
               int i0, int i1, double *crho, double *cgrad, int nthreads);
void o_rho2_points(const owfn *w, long n, const double *xyz, int nder, double *rho,
                   double *grad, double *hess, int nthreads);

int o_newton(const owfn *w, double r[3], double gfnormeps, int maxit);
void o_newton_batch(const owfn *w, long n, double *xyz, double gfnormeps, int maxit,
                    int *ier, int nthreads);

/* autocritic with default molecular pair seeding.  Outputs the CP list in
 * critic2's final order (nuclei first, then sortcps order).  Returns ncp. */
int o_pair_seeds(const owfn *w, double maxdist, int npts, double *xseed, int maxseed);
int o_autocritic(const owfn *w, int nseed, const double *xseed, int nthreads, int maxcp,
                 double *cp_xyz, int *cp_typ, double *cp_f, int *nuc_count);

/* NCI output (src/nci@proc.f90:612-645, 916-932).  o_fmt_e13_5e3 writes
 * the 14 characters of (" ",1p,e13.5e3), o_fmt_E15_7 the 15 of 1p,E15.7
 * (three-digit exponents without the E).  o_cube_body writes a cube body
 * (records of nstep[2] numbers, 6 a line) and returns its length.
 * o_nci_post applies the cutoff pass to cgrad in place and writes the .dat
 * pairs into dat (room for every point); returns their number. */
void o_fmt_e13_5e3(double x, char *out);
void o_fmt_E15_7(double x, char *out);
void o_fmt_E22_14E3(double x, char *out);
long o_cube_body(const int nstep[3], const double *v, char *out);
long o_nci_post(const int nstep[3], const double *crho, double *cgrad, double rhocut, double dimcut,
                double rhoplot, double srho_lo, double srho_hi, int onlyneg, double *dat);

/* Molecular graph: Hessian eigenvectors, field%gradient, makegraph
 * (src/fieldmod@proc.f90:2500-2890, src/autocp@proc.f90:2116-2268). */
void o_eigvec3(const double m[9], double ev[3], double vec[9]);
int o_gradient(const owfn *w, double x[3], int iup, int ncp, const double *cpx, const int *cptyp,
               const double pathini[3], int *nstep, double *plen);
void o_makegraph(const owfn *w, int ncp, const double *cpx, const int *cptyp, int *ipath, double *brdist,
                 double *brpathlen, double *brang, double *brvec, int *ier, int *nstep, int nthreads);
int o_basin_integrals(const owfn *w, int ncp, const double *cpx, const int *cptyp, int cpid, int nray,
                      const double *u, const double *wang, const int *ring, int nring, const double *ringw, int nsph,
                      const double *usph, const double *wsph, double prec, int stats, int nthreads, int *att_cp,
                      double *props, double *iaserr, double *rsurf, double *rbeta_int, int *nwarn_out,
                      int *nrestart_out);
int o_sphere_integrals(const owfn *w, int ncp, const double *cpx, const int *cptyp, int cpid, int nray,
                       const double *u, const double *wang, const int *ring, int nring, const double *ringw, int nr,
                       double r0, double rend, int nthreads, int *att_cp, double *radii, double *props);

/* Molecular meshes (src/meshmod@proc.f90:79-627): type 1 Becke, 2
 * Franchini; ang(4, nang) the angular rule (weights sum to 1). */
int o_z2nr(int z, int lvl);
long o_mesh_size(const owfn *w, int lvl, int nang);
void o_mesh(const owfn *w, int type, int lvl, int nang, const double *ang, double *xyz, double *wt,
            int nthreads);

#ifdef __cplusplus
}
#endif
#endif
