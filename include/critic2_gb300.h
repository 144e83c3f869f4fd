/*
 * critic2_gb300 -- C ABI of the GB300 molecular-wavefunction field evaluator.
 *
 * The library evaluates critic2's GTO molecular-wavefunction field (density,
 * gradient, Hessian and derived quantities) on one GPU and runs the two
 * consumers of that evaluator that critic2 drives from it: the NCI grid
 * (reduced density gradient s and sign(lambda2)*rho) and the AUTO Newton
 * critical-point search.
 *
 * Conventions (identical to critic2's internal ones):
 *   - Cartesian coordinates in bohr, in the frame of the wavefunction file.
 *   - Arrays are Fortran-ordered where critic2 passes Fortran arrays:
 *     cmo is cmo(nmo, npri) (MO index fastest), a 3x3 matrix is column-major,
 *     a batch of n points is xyz(3, n).
 *   - icenter and itype are 1-based, itype indexes critic2's li(3,56) table.
 *   - Every entry point returns an int status (C2G_OK = 0).  No exception
 *     crosses the ABI; c2g_last_error() gives the calling thread's message.
 *   - A handle may be used by one host thread at a time.
 *
 * Reference interfaces replaced (paths within the critic2 source tree):
 *   c2g_wfn_create / c2g_wfn_read_wfx / c2g_wfn_read_wfn : molwfn%read_wfx,
 *       read_wfn + prune_primitives + complete_struct
 *       (src/wfn_private@proc.F90:981-1284, 3632-3785)
 *   c2g_rho2      : molwfn%rho2 (src/wfn_private.f90:293-307,
 *                   src/wfn_private@proc.F90:2484-2705), batched over points
 *   c2g_grd       : field%grd for a wavefunction field
 *                   (src/fieldmod.f90:178-184, src/fieldmod@proc.f90:808-1171)
 *   c2g_nciplot   : the nciplot grid loop (src/nci@proc.f90:540-605)
 *   c2g_newton    : field%newton (src/fieldmod.f90:264-269,
 *                   src/fieldmod@proc.f90:2238-2279), batched over seeds
 *   c2g_autocritic: autocritic's seed / Newton / addcp / sortcps core
 *                   (src/autocp@proc.f90:423-437, 755-822,
 *                   src/fieldmod@proc.f90:2288-2466)
 */
#ifndef CRITIC2_GB300_H
#define CRITIC2_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define C2G_ABI_VERSION 1

/* status codes */
#define C2G_OK 0
#define C2G_ERR_ARG 1         /* bad argument (null pointer, size, mode) */
#define C2G_ERR_CUDA 2        /* a CUDA call failed, or no usable GPU */
#define C2G_ERR_ALLOC 3       /* host or device allocation failed */
#define C2G_ERR_IO 4          /* file could not be read or parsed */
#define C2G_ERR_UNSUPPORTED 5 /* valid request this library does not support */
#define C2G_ERR_NUMERIC 6     /* the algorithm cannot complete on this input (critic2 stops there too) */

/* arithmetic of the evaluation */
#define C2G_PREC_FP64 0   /* FP64 everywhere (the plain form) */
#define C2G_PREC_TF32X3 1 /* TF32 split (3 products), FP32 accumulation */
#define C2G_PREC_BF16X3 2 /* BF16 split (3 products), FP32 accumulation */

/* wavefunction types (src/wfn_private.f90:156-159) */
#define C2G_WFN_RHF 0
#define C2G_WFN_UHF 1
#define C2G_WFN_ROHF 2
#define C2G_WFN_FRAC 3

typedef struct c2g_wfn c2g_wfn;

/* Library ABI version (C2G_ABI_VERSION). */
int c2g_abi_version(void);

/* Message of the last failed call on this host thread (always NUL-ended).
 * Returns the length of the full message. */
int c2g_last_error(char *buf, int len);

/* Creates a wavefunction handle from molwfn arrays.  The arrays are copied
 * (the caller keeps ownership); duplicate primitives are merged and the
 * primitive cutoffs computed exactly as critic2's prune_primitives and
 * complete_struct do; the result is uploaded to the current CUDA device.
 *   atom_xyz(3,natom), atom_z(natom): nuclei (atomic numbers; 1 = H)
 *   icenter(npri), itype(npri): 1-based centre and li type (1..56)
 *   e(npri): exponents; occ(nmo): occupations; cmo(nmo,npri): coefficients
 *   wfntyp: C2G_WFN_*; nalpha: number of alpha MOs (UHF/ROHF split)
 * Replaces src/wfn_private@proc.F90:3632-3785 (prune_primitives,
 * complete_struct) following read_wfx. */
int c2g_wfn_create(int natom, const double *atom_xyz, const int *atom_z, int npri, int nmo,
                   const int *icenter, const int *itype, const double *e, const double *occ,
                   const double *cmo, int wfntyp, int nalpha, c2g_wfn **out);

/* Reads a wfx file (nuclei, primitives, occupied MOs) like critic2's
 * `molecule file.wfx` + `load file.wfx` and creates a handle.  Replaces
 * read_wfx, src/wfn_private@proc.F90:1121-1284. */
int c2g_wfn_read_wfx(const char *path, c2g_wfn **out);

/* Reads an AIMPAC wfn file (its fixed columns: nuclei, primitives, MOs;
 * element symbols give the atomic numbers) like critic2's `molecule
 * file.wfn` + `load file.wfn`, and creates a handle.  RHF/UHF/ROHF/
 * fractional from the occupations; a UHF file's alpha count from the first
 * drop of the orbital energies.  Replaces read_wfn,
 * src/wfn_private@proc.F90:981-1118. */
int c2g_wfn_read_wfn(const char *path, c2g_wfn **out);

/* Reads a Gaussian formatted checkpoint (fchk) file's occupied orbitals like
 * critic2's `load file.fchk`, and creates a handle: sp shells unfolded,
 * pure d, f and g shells (real solid harmonics, m = 0, 1, -1, 2, -2, ...)
 * transformed to Cartesian Gaussians, each Cartesian component normalised
 * by its primitive and contraction factors; RHF, UHF (Beta Orbital
 * Energies present) or ROHF (alpha and beta counts differ).  h shells are
 * rejected as in critic2.  Replaces read_fchk without virtual orbitals,
 * src/wfn_private@proc.F90:1287-1812. */
int c2g_wfn_read_fchk(const char *path, c2g_wfn **out);

/* Reads a molden file with Gaussian-type orbitals (occupied MOs; [Atoms]
 * in AU or Angs, [GTO], [5D]/[5D7F]/[5D10F]/[7F]/[9G], [MO]) like critic2's
 * `load file.molden`, and creates a handle.  ORCA files (title "created by
 * orca_2mkl") are spherical throughout, with ORCA's per-l primitive
 * normalisation and opposite sign of the |m| >= 3 functions.  STO basis
 * sets, sp shells, ROHF and fractional occupations are rejected, as in
 * critic2.  Replaces read_molden, src/wfn_private@proc.F90:1819-2478. */
int c2g_wfn_read_molden(const char *path, c2g_wfn **out);

/* Frees the handle and its device memory. */
int c2g_wfn_destroy(c2g_wfn *h);

/* Sets (or, with nedf = 0, removes) the EDF core density of a handle: the
 * electron density functions of pseudopotential cores, a linear sum
 * sum_i c(i) chi_i(r) of Cartesian Gaussians added to the MO density in
 * every evaluation (total density, and half of it to each spin channel of
 * a UHF/ROHF wavefunction; kinetic energy density and stress have no core
 * part).  Arrays as in the wfx <EDF Primitive *> sections:
 *   icenter(nedf), itype(nedf): 1-based centre and li type (1..56)
 *   e(nedf): exponents, c(nedf): coefficients
 * The cutoffs are critic2's: dran_edf = sqrt(-ln(1e-12)/e), and each atom's
 * environment radius grows to cover its EDF primitives.  c2g_wfn_read_wfx
 * calls this for files with <Number of EDF Primitives> > 0.  Replaces the
 * EDF part of read_wfx and complete_struct and calculate_edf
 * (src/wfn_private@proc.F90:1185-1230, 3750-3776, 3275-3369, 2626-2677);
 * critic2 builds the EDF polynomial powers only up to the atom's MO lmax
 * (s-type EDFs, the usual case, are unaffected), this library evaluates the
 * full polynomial of every type. */
int c2g_wfn_set_edf(c2g_wfn *h, int nedf, const int *icenter, const int *itype, const double *e,
                    const double *c);

/* Tunable parameters of a handle. */
#define C2G_PARAM_RECHECK_REL 1 /* split-precision NCI: points with
                                   |lambda2| < value * max|lambda| are
                                   re-evaluated in FP64.  Default (or any
                                   negative value): 1e-4 for TF32X3, 1e-3
                                   for BF16X3; 0 disables the re-check;
                                   values above 1e-3 act as 1e-3 */
#define C2G_PARAM_NEWTON_STALL 2 /* Newton (c2g_newton, c2g_autocritic): stop a
                                    seed with ier = 2 after this many FP64
                                    steps without a new minimum of |grad|.
                                    Default 0: off, critic2's semantics (only
                                    maxit ends a seed).  Such seeds sit at the
                                    FP64 rounding floor of |grad| above
                                    gfnormeps and would otherwise run to maxit;
                                    this option has no counterpart in the
                                    reference. */
#define C2G_PARAM_WAIT_NS 3 /* split-precision kernel: limit, in nanoseconds,
                               of every wait between its pipeline stages
                               (default 4e9).  A wait that runs out stops the
                               kernel cleanly (its MMAs in flight are
                               drained, its tensor memory is freed) and the
                               call returns C2G_ERR_CUDA with "a pipeline
                               wait timed out"; the handle stays usable.
                               Range [1, 6e11]; this option has no
                               counterpart in the reference. */
int c2g_wfn_set_param(c2g_wfn *h, int param, double value);

/* Sizes after pruning. */
int c2g_wfn_info(const c2g_wfn *h, int *natom, int *npri, int *nmo, int *wfntyp, int *nalpha);

/* molwfn%rho2 over a batch of n points (src/wfn_private@proc.F90:2484-2705).
 * xyz(3,n).  Outputs (any may be NULL; nder >= the order each needs):
 *   rho(3,n)      total, up, down density
 *   grad(3,3,n)   gradient per spin channel (columns total, up, down)  [nder>=1]
 *   hess(3,3,3,n) Hessian per spin channel                             [nder>=2]
 *   gkin(3,n)     kinetic energy density G per spin channel            [nder>=1]
 *   stress(3,3,n) Schrodinger stress tensor; vir(n) its trace          [nder>=2]
 * prec: C2G_PREC_FP64 gives every output; the split modes give rho, grad
 * and hess totals only (spin channels are then the RHF halves). */
int c2g_rho2(c2g_wfn *h, int n, const double *xyz, int nder, int prec, double *rho,
             double *grad, double *hess, double *gkin, double *stress, double *vir);

/* The valence outputs of molwfn%rho2 (rhoval, gradval, hval: the density
 * without the EDF core, src/wfn_private@proc.F90:2484-2705), FP64, in the
 * layout of c2g_rho2's rho, grad and hess (any may be NULL).  Equal to
 * c2g_rho2's for a wavefunction without EDF primitives. */
int c2g_rho2_valence(c2g_wfn *h, int n, const double *xyz, int nder, double *rho, double *grad,
                     double *hess);

/* field%grd for the wavefunction field at n points: molecular-cell wrap,
 * rho2, nucleus check (|grad| := 0 within 1e-5 bohr of a nucleus),
 * Hessian eigenvalues (ascending), rank r and signature s with the 1e-8
 * degeneracy threshold (src/fieldmod@proc.f90:808-1171).  Outputs may be
 * NULL: f(n), gf(3,n), gfmod(n), hf(3,3,n), hfeval(3,n), r(n), s(n),
 * isnuc(n). */
int c2g_grd(c2g_wfn *h, int n, const double *xyz, int nder, int prec, double *f, double *gf,
            double *gfmod, double *hf, double *hfeval, int *r, int *s, int *isnuc);

/* Error statistics of a split-precision NCI evaluation, filled when the
 * caller asks for an FP64 re-check (see c2g_nciplot). */
typedef struct {
  long npoints;
  long nrecheck;        /* points re-evaluated in FP64 (|l2| < 1e-3 |l1|) */
  double ms_kernel;     /* device time of the evaluation, milliseconds */
  double ms_recheck;    /* device time of the FP64 re-check pass */
  double stage_frac;    /* split modes: fraction of the K-stages of a 32-point
                           tile that some point of the tile can see */
} c2g_nci_stats;

/* The nciplot grid loop (src/nci@proc.f90:540-605) over the grid
 * x = x0 + i*xmat(:,1) + j*xmat(:,2) + k*xmat(:,3), i < nstep(1), j <
 * nstep(2), k < nstep(3).  Writes crho(k,j,i) = sign(rho, lambda2)*100 and
 * cgrad(k,j,i) = s (k fastest), host arrays of nstep(1)*nstep(2)*nstep(3)
 * doubles.  xmat is column-major (column i = step vector of axis i).
 * In the split modes the points whose Hessian eigenvalues satisfy
 * |lambda2| < recheck max|lambda| (C2G_PARAM_RECHECK_REL) are re-evaluated
 * in FP64.  stats may be NULL. */
int c2g_nciplot(c2g_wfn *h, const double *x0, const double *xmat, const int *nstep, int prec,
                double *crho, double *cgrad, c2g_nci_stats *stats);

/* As c2g_nciplot, writing device arrays on the given CUDA stream (NULL =
 * legacy default stream).  Returns after the work is enqueued and, when
 * stats is not NULL, after it finishes. */
int c2g_nciplot_dev(c2g_wfn *h, const double *x0, const double *xmat, const int *nstep,
                    int prec, double *d_crho, double *d_cgrad, void *stream,
                    c2g_nci_stats *stats);

/* No-allocation form of c2g_nciplot_dev (this entry has no counterpart in
 * the reference).  For callers that cannot let the library allocate device
 * memory during a run: codes whose memory is reserved up front by their own
 * pool (a caching allocator that holds the GPU's memory, or an MPI job that
 * sizes everything at start-up) and codes that stream grid slabs on their
 * own streams, where cudaFree -- which synchronises the whole device --
 * would stall their other work.  c2g_nciplot_dev allocates its FP64
 * re-check list (kept on the handle, grown on demand); this entry keeps the
 * re-check list in a static device array of 4 MiB + 256 B, and makes no
 * cudaMalloc/cudaFree or allocating-library call.
 *   - At most C2G_NOALLOC_MAX_POINTS grid points per call; larger grids are
 *     rejected with C2G_ERR_ARG (split them into i-slabs and call per slab).
 *   - The split operands of the requested mode must already be on the
 *     device: they are allocated by the first split-precision call of an
 *     allocating entry (e.g. c2g_nciplot_dev on a 1-point grid); otherwise
 *     the call returns C2G_ERR_UNSUPPORTED.  C2G_PREC_FP64 needs nothing.
 *   - The first call on each device looks up the scratch array's address
 *     (cudaGetSymbolAddress, with that device current).  Every call reads
 *     the kernels' error word back and synchronises its stream, so no call
 *     can be captured into a CUDA graph.  That first call (like the first call
 *     of any entry, with CUDA's default lazy module loading) also loads the
 *     library's GPU code together with the 4 MiB static array, which takes
 *     device memory once: make it before a pool of the caller's reserves
 *     the GPU's memory.
 *   - The address is kept per device ordinal for the life of the process.
 *     After cudaDeviceReset (or any teardown of the device's primary
 *     context) it is stale: do not call this entry again in that process.
 *   - The re-check counter, which must start at zero, is cleared by the call
 *     itself on the given stream.
 *   - The scratch is shared by all calls on a device: calls that overlap in
 *     time (other host threads, or other streams, on the same device) race
 *     on it and must be serialised by the caller.
 *   - Returns after the work on `stream` has finished (a pipeline timeout of
 *     the split kernel is reported as C2G_ERR_CUDA).  No statistics. */
#define C2G_NOALLOC_MAX_POINTS 1048576
int c2g_nciplot_dev_noalloc(c2g_wfn *h, const double *x0, const double *xmat, const int *nstep,
                            int prec, double *d_crho, double *d_cgrad, void *stream);

/* NCI post-pass cutoffs (src/nci@proc.f90:141-168): .dat gets the points
 * with |rho| < rhocut and s < dimcut; then s := 100 where |rho| > rhoplot,
 * where sign(lambda2)*rho is outside [srho_lo, srho_hi], or (onlyneg) where
 * it is positive.  A NULL cut means critic2's defaults for a density field:
 * 0.2, 2.0, 0.1, -1e30, 1e30, 0. */
typedef struct {
  double rhocut, dimcut, rhoplot, srho_lo, srho_hi;
  int onlyneg;
} c2g_nci_cut;

/* The cutoff pass of nciplot (src/nci@proc.f90:612-645, no fragments, no
 * void) on device cubes in (k,j,i) order: writes the .dat pairs
 * (sign(lambda2)*rho, s) of the selected points in grid order into
 * d_dat(2, cap) (up to cap pairs), sets *ndat to their number, and applies
 * the s := 100 rules to d_cgrad in place. */
int c2g_nci_post_dev(const int *nstep, const double *d_crho, double *d_cgrad, const c2g_nci_cut *cut,
                     double *d_dat, long cap, long *ndat, void *stream);

/* write_cube_body (src/nci@proc.f90:916-932) of a device cube in (k,j,i)
 * order into the host buffer text: records of nstep(3) numbers in
 * Fortran's (6(" ",1p,e13.5e3)) layout.  *nbytes = size of the text; with
 * text NULL only *nbytes is set.  Formatted on the GPU, correctly rounded. */
int c2g_cube_text(const int *nstep, const double *d_values, char *text, long cap, long *nbytes, void *stream);

/* The .dat lines (1p,E15.7,E15.7; src/nci@proc.f90:638) of ndat device
 * pairs d_dat(2, ndat) into the host buffer text (31 bytes a line). */
int c2g_dat_text(const double *d_dat, long ndat, char *text, long cap, long *nbytes, void *stream);

/* nciplot end to end: the grid (c2g_nciplot), the cutoff pass and the
 * files root-dens.cube, root-grad.cube (headers as write_cube_header,
 * src/nci@proc.f90:818-914, atoms in the frame of the handle) and root.dat.
 * ms_parts (may be NULL) receives 4 wall times in ms: evaluation, cutoff
 * pass, text formatting (device) + copies, file writes. */
int c2g_nciplot_files(c2g_wfn *h, const double *x0, const double *xmat, const int *nstep, int prec,
                      const char *root, const c2g_nci_cut *cut, c2g_nci_stats *stats, double *ms_parts);

/* nciplot's checkpoint file <root>.chk_nci (writechk / readchk,
 * src/nci@proc.f90:1019-1117), byte-compatible with critic2's (gfortran
 * unformatted sequential records): the grid (x0(3), xmat(3,3) columns,
 * nstep(3)) and the host cubes crho, cgrad in (k,j,i) order, without
 * promolecular or fragment densities.  c2g_nci_chk_read loads the cubes
 * when the file exists and matches x0 and xmat to 1e-13 and nstep exactly
 * (*found = 1); a missing or non-matching file gives *found = 0 and
 * C2G_OK, as readchk restarts the calculation; a truncated or malformed
 * file gives C2G_ERR_IO (crho and cgrad are then undefined). */
int c2g_nci_chk_write(const char *path, const double *x0, const double *xmat, const int *nstep,
                      const double *crho, const double *cgrad);
int c2g_nci_chk_read(const char *path, const double *x0, const double *xmat, const int *nstep, double *crho,
                     double *cgrad, int *found);

/* Molecular integration meshes (src/meshmod@proc.f90:45-627): atom-centred
 * radial x Lebedev angular grids with Becke's or Franchini's partition of
 * space, in critic2's point order (atoms, radial shells, angular points).
 * Becke: rmesh_postg radial grid, Becke's fuzzy cells (four smoothing
 * iterations, no size adjustment).  Franchini (critic2's default): Gauss-
 * Legendre radial grid scaled by the tabulated zeta(Z), weights from
 * f exp(-2 d)/d^3 (f = 0.3 for H) over the atoms within max(r_max, 12 bohr).
 * Levels set the radial counts (z2nr) and Lebedev sizes 110, 194, 302, 590,
 * 770 (z2nang); the default is good (302).  Lattice images of the atoms,
 * which critic2's molecular cell adds to the partition of points farther
 * than the cell border, are not included (those points carry no density). */
#define C2G_MESH_BECKE 1
#define C2G_MESH_FRANCHINI 2
#define C2G_MESH_SMALL 1
#define C2G_MESH_NORMAL 2
#define C2G_MESH_GOOD 3
#define C2G_MESH_VGOOD 4
#define C2G_MESH_AMAZING 5
/* quantities integrated by c2g_molcalc (fillmesh's im_*) */
#define C2G_MOLCALC_VOLUME 0  /* 1 */
#define C2G_MOLCALC_RHO 1     /* rho (molcalc_nelec, molcalc "$1") */
#define C2G_MOLCALC_GRADRHO 2 /* |grad rho| */
#define C2G_MOLCALC_GKIN 3    /* kinetic energy density G (FP64 only) */

typedef struct {
  long npoints;    /* mesh points */
  double ms_mesh;  /* building the mesh on the GPU */
  double ms_total; /* the whole call */
} c2g_mesh_stats;

/* Number of points of the mesh (genmesh's m%n). */
int c2g_mesh_size(const c2g_wfn *h, int type, int level, long *npoints);
/* The mesh into caller device buffers d_xyz(3, n) and d_w(n) (genmesh). */
int c2g_mesh_dev(c2g_wfn *h, int type, int level, double *d_xyz, double *d_w, void *stream);
/* molcalc: integral(q) = sum_i w_i f_q(x_i) over the mesh for nq quantities
 * (fillmesh + molcalc_nelec / molcalc_expression, src/molcalc@proc.F90:
 * 94-256), the field evaluated in precision prec.  stats may be NULL. */
int c2g_molcalc(c2g_wfn *h, int type, int level, int prec, int nq, const int *quant, double *integral,
                c2g_mesh_stats *stats);

/* Quantities of field%grd for CUBE plots (rhoplot_cube's nti selectors,
 * src/rhoplot@proc.f90:905-930). */
#define C2G_FIELD_RHO 0
#define C2G_FIELD_GX 1
#define C2G_FIELD_GY 2
#define C2G_FIELD_GZ 3
#define C2G_FIELD_GMOD 4
#define C2G_FIELD_HXX 5
#define C2G_FIELD_HXY 6
#define C2G_FIELD_HXZ 7
#define C2G_FIELD_HYY 8
#define C2G_FIELD_HYZ 9
#define C2G_FIELD_HZZ 10
#define C2G_FIELD_LAP 11

/* rhoplot_cube's evaluation (src/rhoplot@proc.f90:890-950): one
 * C2G_FIELD_* quantity of grd at x0 + i*xmat(:,1) + j*xmat(:,2) +
 * k*xmat(:,3) into the device array d_out, (k,j,i) order (k fastest). */
int c2g_grid_field_dev(c2g_wfn *h, const double *x0, const double *xmat, const int *nstep, int prec, int prop,
                       double *d_out, void *stream);

/* writegrid_cube's precise body (src/crystalmod@write.f90:3557-3567,
 * (6(" ",E22.14E3)) records) of a device cube into the host buffer text,
 * as c2g_cube_text. */
int c2g_cube_precise_text(const int *nstep, const double *d_values, char *text, long cap, long *nbytes,
                          void *stream);

/* CUBE plot end to end: c2g_grid_field_dev + a precise cube file (header as
 * writegrid_cube, all atoms, in the frame of the handle).  ms_parts (may be
 * NULL) receives 3 wall times in ms: evaluation, text, file write. */
int c2g_cube_field_file(c2g_wfn *h, const double *x0, const double *xmat, const int *nstep, int prec, int prop,
                        const char *path, double *ms_parts);

/* field%newton for n seeds at once (src/fieldmod@proc.f90:2238-2279):
 * xyz(3,n) in/out; ier(n): 0 converged (|grad| < gfnormeps), 1 invalid or
 * singular Hessian, 2 maxit reached.  In the split modes the iterations run
 * in split precision until the Newton step is shorter than 1e-5 bohr and
 * finish in FP64 (convergence is only declared from an FP64 evaluation). */
int c2g_newton(c2g_wfn *h, int n, double *xyz, double gfnormeps, int maxit, int prec, int *ier);

/* Default molecular pair seeds of critic2's AUTO (src/autocp@proc.f90:
 * 423-437, 665-729): for every ordered atom pair closer than maxdist, npts
 * points at fractions k/(npts+1), filtered by the molecular-cell border.
 * With xseed NULL returns the count in *nseed; otherwise writes up to
 * *nseed seeds xseed(3,*) and sets *nseed to the number written. */
int c2g_pair_seeds(const c2g_wfn *h, double maxdist, int npts, double *xseed, int *nseed);

/* CP list result of c2g_autocritic. */
typedef struct {
  int ncp;              /* CPs written (nuclei first, then sortcps order) */
  int count[4];         /* n, b, r, c */
  int poincare_hopf;    /* n - b + r - c (1 for a molecule) */
  int nseed;            /* seeds searched */
  int nconverged;       /* Newton runs with ier == 0 */
  double ms_total;      /* wall time of the search, milliseconds */
} c2g_cp_report;

/* autocritic core: Newton from every seed (c2g_newton), addcp on the
 * converged ones (cpeps 1e-2, nuceps 0.1, nucepsh 0.2, gradient check
 * max(1e-4, gfnormeps), degenerate CPs dropped), sortcps.  Outputs up to
 * maxcp CPs: cp_xyz(3,*), cp_typ(*) (signature: -3 n, -1 b, 1 r, 3 c),
 * cp_f(*) density.  With xseed NULL the default pair seeds are used, each
 * unordered atom pair once: critic2 seeds both ordered pairs, whose points
 * coincide (the k-th point of i->j is the (6-k)-th of j->i), so its list
 * (c2g_pair_seeds) holds every seed twice; taking one of each gives the same
 * CP list with half the Newton work. */
int c2g_autocritic(c2g_wfn *h, int nseed, const double *xseed, int prec, int maxcp,
                   double *cp_xyz, int *cp_typ, double *cp_f, c2g_cp_report *report);

/* The molecular graph that autocritic builds after the CP search
 * (makegraph, src/autocp@proc.f90:2116-2268; autocritic runs it by
 * default, dograph = 1).  From every bond CP (typ -1) two gradient paths go
 * up the density from r +- 0.01 e, e the Hessian eigenvector of the
 * positive curvature; from every ring CP (typ +1) two go down along the
 * negative one.  Paths follow field%gradient (src/fieldmod@proc.f90:
 * 2500-2732) with critic2's default navigation: Bogacki-Shampine stepper,
 * step 0.3 bohr, maxerr 1e-4, gradeps 1e-7, beta spheres 0.1 bohr; they end
 * in the beta sphere of the nearest nucleus or CP of type 3 typ, at a new
 * CP, on leaving the molecular cell (down paths), on bouncing, or after
 * 3333 steps.  The CP list is c2g_autocritic's (nuclei included, typ -3).
 * Outputs, column-major (j = 1, 2 are the two paths):
 *   ipath(2,ncp)     1-based CP index of type 3 typ nearest to the end
 *                    point (no distance limit); -1 when there is none and
 *                    the end point is outside the molecular cell's inner
 *                    region; 0 otherwise, and for CPs with |typ| /= 1
 *   brdist(2,ncp)    |end point - CP|;  brpathlen(2,ncp) path length
 *   brang(ncp)       angle (degrees) between the two end vectors
 *   brvec(3,ncp)     the unit eigenvector e
 *   ier(2,ncp), nstep(2,ncp)   field%gradient's ier and step count (may be NULL)
 * The paths are traced on the GPU, one block per path (the steps and their
 * FP64 evaluations on the device).  The sign of e follows a fixed rule (largest
 * component positive), not LAPACK's, so the two paths of a CP may be
 * listed in the other order than critic2 lists them. */
typedef struct {
  int npath;       /* gradient paths traced */
  int nbatch;      /* GPU launches (Hessians at the CPs, the paths) */
  long nevals;     /* field evaluations */
  double ms_total; /* wall time of the call */
} c2g_graph_stats;

int c2g_cp_graph(c2g_wfn *h, int ncp, const double *cp_xyz, const int *cp_typ, int *ipath, double *brdist,
                 double *brpathlen, double *brang, double *brvec, int *ier, int *nstep, c2g_graph_stats *stats);

/* Atomic-basin integrals by bisection of the zero-flux surface: critic2's
 * INTEGRALS keyword for a molecular wavefunction field
 * (src/bisect@proc.f90:862-1028; INTEGRALS LEBEDEV n / GAULEG ntheta nphi,
 * CP id).  The attractors are the nuclei and the CPs of type -3 of the CP
 * list (cpid = 0), or the one CP cpid (1-based).  For each attractor and
 * angular node the surface radius is found as bisect_msurface does
 * (:1208-1446): a bracket from critic2's tries at 2e-5 bohr, 0.9 and 0.99
 * of the distance to the nearest CP (inner; the largest whose upward
 * gradient path ends within sqrt(1e-5) bohr of the attractor) and the cell
 * size, 0.75 and 0.99 of the distance to the nearest CP of the same type
 * (outer; the smallest whose path does not), then bisection to iasprec
 * bohr (lim_surf, :1039-1126; critic2's default INT_iasprec 1e-5), with
 * field%gradient's navigation and beta spheres of 0.1 bohr shrunk by 0.75
 * when a surface point falls inside one.  The integral is a beta sphere of
 * 0.95 times the smallest surface radius (170-point Lebedev rule) plus the
 * radial Gauss-Legendre quadrature (50 nodes) of each ray from the sphere to
 * the surface, summed as lebedev_mquad / gauleg_mquad
 * (src/integration@proc.f90:495-642).  Integrated properties are critic2's
 * molecular defaults: the valence density (Pop) and its Laplacian (Lap).
 *   meth C2G_INT_LEBEDEV: n1 = rule size (rounded up to the next of
 *        critic2's 32 sizes, 6-5810); C2G_INT_GAULEG: n1 = ntheta,
 *        n2 = nphi (int(nphi |sin theta|) + 1 nodes per polar ring).
 *   CP list: c2g_autocritic's (the nuclei first, in atom order), or ncp = 0
 *        for the nuclei alone.
 * Outputs (natt and nray from c2g_basin_size):
 *   att_cp(natt)          0-based CP index of each attractor (may be NULL)
 *   props(2, natt)        Pop, Lap per attractor
 *   iaserr(2, natt)       critic2's IAS error estimate (may be NULL)
 *   rays(3, nray)         unit direction of each node (may be NULL)
 *   rsurf(nray, natt)     surface radius per attractor and node (may be NULL)
 *   rbeta_int(natt)       beta-sphere radius (may be NULL)
 * Rays are independent: unlike a serial critic2 run, a ray's bracket does
 * not depend on running means over the rays done before it (every ray
 * takes the first ray's tries), so end points can differ from critic2's by
 * up to iasprec; and a beta sphere shrunk by a ray's restart stays shrunk for
 * that ray only.  A ray without a bracket returns C2G_ERR_NUMERIC (critic2:
 * "Can not find ray limits"). */
#define C2G_INT_LEBEDEV 0
#define C2G_INT_GAULEG 1
typedef struct {
  int natt;        /* attractors integrated */
  int nray;        /* rays per attractor */
  long npath;      /* gradient paths traced */
  long nbatch;     /* GPU launches of the surface search */
  long nevals;     /* field evaluations (paths and quadrature) */
  int nwarn;       /* paths that ended with field%gradient's ier > 0 */
  int nrestart;    /* beta-sphere shrinks (bisection restarts) */
  double ms_total; /* wall time of the call */
} c2g_basin_stats;

int c2g_basin_size(c2g_wfn *h, int ncp, const int *cp_typ, int meth, int n1, int n2, int cpid, int *natt,
                   int *nray);

/* Integrals over spheres around the attractors: critic2's SPHEREINTEGRALS
 * (src/bisect@proc.f90:573-784; SPHEREINTEGRALS GAULEG ntheta nphi |
 * LEBEDEV n, NR nr, R0 r0, REND rend, CP id).  For each attractor (as
 * c2g_basin_integrals selects them; natt from c2g_basin_size) Pop and Lap
 * inside nr spheres of radius r0 exp(h (n - 1)), n = 1..nr, the last
 * radius rend (rend < 0: |rend| times half the distance to the nearest
 * atom, get_rnn2; critic2's defaults are nr = 100, r0 = 1e-3 bohr,
 * rend = -1, GAULEG 20 20 or LEBEDEV 770).  Each sphere is the angular rule
 * times 50 radial Gauss-Legendre nodes on (0, r), FP64.  Outputs:
 * att_cp(natt) (may be NULL), radii(nr, natt), props(2, nr, natt). */
int c2g_sphere_integrals(c2g_wfn *h, int ncp, const double *cp_xyz, const int *cp_typ, int meth, int n1, int n2,
                         int cpid, int nr, double r0, double rend, int *att_cp, double *radii, double *props);
int c2g_basin_integrals(c2g_wfn *h, int ncp, const double *cp_xyz, const int *cp_typ, int meth, int n1, int n2,
                        int cpid, double iasprec, int *att_cp, double *props, double *iaserr, double *rays,
                        double *rsurf, double *rbeta_int, c2g_basin_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
