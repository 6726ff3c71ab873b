/*
 * mo_ed.h -- C-ABI of the GB300 exact-diagonalization impurity solver.
 *
 * Drop-in boundary for the ED hot path of MO-DMFT (sector basis, matrix-free
 * H*v, Lanczos, continued-fraction G(i w_n), chi^2 bath fit).  Each entry
 * point names the reference routine it replaces (file:line in the reference
 * project).  A Fortran host binds these with ISO_C_BINDING (see
 * mo-dmft_gb300/fortran/mo_ed_bind.f90); every Fortran array argument is
 * passed as a plain pointer with the Fortran (column-major, 1-based) layout
 * described per function.
 *
 * Conventions
 *   - Every function returns an int status (MO_ED_OK == 0).  The reference
 *     has no status codes: it calls die -> MPI_Abort or STOP; a Fortran shim
 *     maps a nonzero status to die.  mo_ed_last_error() gives the message.
 *   - One context per host thread; a context is not re-entrant.  All device
 *     work of a context is issued on its stream (mo_ed_create).
 *   - Sites: 1..nsite with impurity orbitals 1..norb first, then bath levels
 *     norb+1..nsite.  ek[nsite] is ek(1:nsite); vk[norb*nbath] is Fortran
 *     vk(1:norb, norb+1:nsite) column-major (norb fastest).
 *   - State word: bit (ispin-1)*nsite + isite-1 is occupation of (isite,
 *     ispin); row index of a sector vector = iup + (idown-1)*nup (1-based,
 *     up-spin fastest), as in the reference.
 *   - Complex arrays are interleaved (re, im) doubles, Fortran order
 *     (norb, nw): element (iorb, iw) at 2*((iw-1)*norb + iorb-1).
 *   - Host-pointer entry points copy in/out through the context's stream and
 *     synchronize it; *_dev entry points take device pointers and do not
 *     synchronize.
 *   - There is no CPU fallback: without a usable CUDA device, mo_ed_create
 *     fails with MO_ED_ERR_CUDA.
 */
#ifndef MO_ED_H
#define MO_ED_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define MO_ED_OK 0
#define MO_ED_ERR_ARG 1        /* invalid argument (null pointer, bad size, NaN input) */
#define MO_ED_ERR_SECTOR 2     /* (ne_up, ne_down) outside [0, nsite] or nsite > 15 */
#define MO_ED_ERR_CUDA 3       /* CUDA runtime error, or no device */
#define MO_ED_ERR_NOMEM 4      /* device allocation failed */
#define MO_ED_ERR_NOCONV 5     /* eigensolver did not converge within its limits */
#define MO_ED_ERR_FIT 6        /* frprmn / brent iteration limit (reference: STOP) */
#define MO_ED_ERR_STATE 7      /* call order: model, sectors or omega not set */
#define MO_ED_ERR_CAPACITY 8   /* caller buffer smaller than required */

/* ---- precision of the sector vectors --------------------------------- */
#define MO_ED_FP64 0           /* plain FP64 device path */
#define MO_ED_FP32 1           /* FP32 vectors and H*v, FP64 reductions / small solves */

typedef struct mo_ed_ctx mo_ed_ctx;

/* Solver options.  Defaults (mo_ed_default_options) follow ed_config.f90:116-126. */
typedef struct {
    int nstep;          /* Lanczos steps of the Green's function (DMFT.ContinuedFractionSteps, 50) */
    int nev;            /* eigenpairs per sector (DMFT.Nev, 30) */
    double beta;        /* inverse temperature (DMFT.beta, 100) */
    int precision;      /* MO_ED_FP32 (default) or MO_ED_FP64 */
    int fortran_cmplx;  /* 1 (default): round E and w_n to float inside CMPLX as the
                           reference does (ed_green.F90:161,177); 0: exact doubles */
    int gs_ncv;         /* Krylov basis size of the eigensolver per restart cycle (0: auto) */
    int gs_maxcycles;   /* restart cycles before MO_ED_ERR_NOCONV (default 200) */
    double gs_tol;      /* relative residual tolerance of converged Ritz pairs (0: auto) */
    int green_reorth;   /* must be 0: the Green's-function Lanczos is the reference
                           recurrence without reorthogonalisation (ed_lanczos.F90:53-68);
                           other values are rejected with MO_ED_ERR_ARG */
    int green_fp64;     /* 0 (default): the Green's-function Lanczos runs in `precision`;
                           1: it runs in FP64 whatever `precision` is (FP32 eigenvectors
                           of ed_solve are widened to FP64 before c / c^dagger) */
    int solve_threads;  /* host threads of mo_ed_solve over the sector list.  0 (default):
                           automatic -- 4 for lists of at least 8 sectors of fewer
                           than 2^18 elements each (small eigensolves are bound by their
                           chains of short launches), one otherwise; 1: one thread; n: up
                           to n.  Each thread solves its sectors through a worker context
                           of its own (stream and workspace); every sector's result is
                           the same as in one thread. */
    int fit_quantum;    /* bath fits (mo_ed_fit_batch, mo_ed_minimization): CG
                           iterations between a fit's looks for waiting fits, to which
                           it then gives up its thread-block cluster (0: 256).  Results
                           do not depend on it. */
    int reserved[5];
} mo_ed_options;

/* ---- context ----------------------------------------------------------- */
/* stream: a cudaStream_t, or NULL to create a private non-blocking stream. */
int mo_ed_create(mo_ed_ctx **ctx, int device, void *stream);
int mo_ed_destroy(mo_ed_ctx *ctx);
const char *mo_ed_last_error(const mo_ed_ctx *ctx);
/* Library version string. */
const char *mo_ed_version(void);
int mo_ed_default_options(mo_ed_options *opt);
int mo_ed_set_options(mo_ed_ctx *ctx, const mo_ed_options *opt);

/* Model globals of ed_config.f90:11-36 (Norb, Nbath, U, Jex, ek, vk).
 * Replaces ed_read_options' model part (ed_config.f90:53-114).  Invalidates
 * cached sector tables. */
int mo_ed_set_model(mo_ed_ctx *ctx, int norb, int nbath, double U, double Jex,
                    const double *ek, const double *vk);
/* Sector list (ed_config.f90:66-80: Nsector, Nelec(:), Nup(:)). */
int mo_ed_set_sectors(mo_ed_ctx *ctx, int nsector, const int *nelec, const int *nup);
/* Local Matsubara grid omega(1:nwloc) (ed_green.F90:41-52). */
int mo_ed_set_omega(mo_ed_ctx *ctx, int nw, const double *omega);

/* ---- a1: binomials (ed_utils.f90:54-69 iCom) --------------------------- */
long long mo_ed_icom(int n, int m);

/* ---- a2-a5: sector basis (ed_basis.F90) -------------------------------- */
/* Sector dimensions (ed_basis.F90:44-46). */
int mo_ed_sector_dims(mo_ed_ctx *ctx, int ne_up, int ne_down, int *nup, int *ndown,
                      long long *ntot);
/* generate_basis (ed_basis.F90:35-107), computed by the combinadic unrank /
 * rank kernels.  Outputs (any may be NULL): up[nup], down[ndown] state words
 * in ascending order; idx_up[2^nsite], idx_down[2^nsite] 1-based ranks, 0
 * for words outside the sector (the reference allocates only
 * [minrange, maxrange] and leaves other words undefined). */
int mo_ed_generate_basis(mo_ed_ctx *ctx, int ne_up, int ne_down, int *up, int *down,
                         int *idx_up, int *idx_down);
/* ed_basis_get (ed_basis.F90:110-124) for n 1-based rows -> state words. */
int mo_ed_basis_get(mo_ed_ctx *ctx, int ne_up, int ne_down, long long n, const long long *idx,
                    unsigned int *state);
/* ed_basis_idx (ed_basis.F90:127-139) for n state words -> 1-based rows
 * (0 for a word outside the sector). */
int mo_ed_basis_idx(mo_ed_ctx *ctx, int ne_up, int ne_down, long long n,
                    const unsigned int *state, long long *idx);

/* Device layout of a sector vector: ndown rows of nup elements (the
 * reference's order) with row stride *ld = roundup(nup, 32) elements, so
 * *nelem = ndown * ld; pad elements must be zero.  The *_dev entry points
 * take vectors in this layout; host entry points use the reference layout. */
int mo_ed_vector_layout(mo_ed_ctx *ctx, int ne_up, int ne_down, int *ld, long long *nelem);

/* ---- a6-a10: matrix-free H*v (ed_hamiltonian.F90:88-191 multiply_H) ------ */
/* B = H*A on host FP64 arrays of ntot entries, computed on the FP64 device path. */
int mo_ed_multiply_h(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *A, double *B);
/* Host FP32 arrays, computed on the FP32 device path. */
int mo_ed_multiply_h_f32(mo_ed_ctx *ctx, int ne_up, int ne_down, const float *A, float *B);
/* Device pointers in the device layout (mo_ed_vector_layout); dtype
 * MO_ED_FP64 (double) or MO_ED_FP32 (float).  Issues the H*v kernel on the
 * context's stream; no synchronization. */
int mo_ed_multiply_h_dev(mo_ed_ctx *ctx, int ne_up, int ne_down, int dtype, const void *dA,
                         void *dB);
/* FP32 input, FP64-accumulated FP64 output (the refinement operator);
 * device layout. */
int mo_ed_multiply_h_mixed_dev(mo_ed_ctx *ctx, int ne_up, int ne_down, const float *dA,
                               double *dB);

/* H*v tile-shape autotuner of a sector (no reference counterpart: the
 * reference has one CPU loop).  The first H*v of each (precision, Nup, Ndn)
 * times every variant on that sector and keeps the fastest; this call runs
 * the tuning if needed and reports *nvariant variants: shape[4*i..4*i+3] =
 * (rows per item, threads per CTA, CTAs per SM, kernel: 0 k_hv, 1 the
 * double-buffered staged k_hv_async, 2 / 3 split: k_hv_down over down-spin
 * blocks on 128- / 64-byte row slices, then k_hv_async for the other terms),
 * ms[i] (negative: does not fit this sector or model), and the *chosen
 * index.  Arrays hold capacity variants.  Pinning a split variant on a model
 * whose down-spin blocks do not fit one CTA fails with MO_ED_ERR_ARG. */
int mo_ed_hv_tuning(mo_ed_ctx *ctx, int ne_up, int ne_down, int dtype, int capacity, int *nvariant,
                    int *shape, float *ms, int *chosen);
/* Pin the H*v variant (index into the list mo_ed_hv_tuning reports) of a
 * sector and precision, replacing the autotuner's choice.  Every variant
 * computes the same sums; the order of the up-spin terms differs between
 * the shared-memory schedules, so FP32 results agree to rounding. */
int mo_ed_hv_set_variant(mo_ed_ctx *ctx, int ne_up, int ne_down, int dtype, int variant);

/* ---- a11: apply_c (ed_operators.F90:10-61) ------------------------------ */
/* vec_out = c^dagger_(iorb,ispin) vec (pm = 1) or c_(iorb,ispin) vec (pm = 2).
 * The reference allocates vec_out; here the caller passes its capacity
 * (query the target sector with mo_ed_sector_dims).  *ntot_out receives the
 * target dimension; MO_ED_ERR_SECTOR if the target sector does not exist. */
int mo_ed_apply_c(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *vec, int pm, int iorb,
                  int ispin, double *vec_out, long long capacity, long long *ntot_out);

/* ---- a12: lanczos_iteration (ed_lanczos.F90:14-68) ---------------------- */
/* The reference three-term recurrence on the device.  a, b have nstep+1
 * entries (0:nstep); b holds squared norms; *nstep_calc as the reference.
 * Precision per options. */
int mo_ed_lanczos_iteration(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *vec,
                            int *nstep_calc, double *a, double *b);

/* No counterpart in the reference.  mo_ed_lanczos_iteration without device
 * allocation, for hosts that own all of the GPU's memory through their own
 * pool (a DMFT driver that reserves the device up front for the arrays of its
 * self-consistency loop) or cannot afford the device-wide synchronisation of
 * cudaFree inside their loop.  Same arguments and results; the Krylov vectors,
 * coefficients and partial sums live in one fixed 32 MiB region that the
 * library reserves statically on every GPU that loads it, held until the
 * process exits.  Limits: sectors up to about 1.0e6 padded elements in FP64
 * (2.0e6 in FP32, mo_ed_vector_layout gives the count); larger ones return
 * MO_ED_ERR_CAPACITY.  The sector must have been prepared in the same
 * precision by an earlier mo_ed_lanczos_iteration, mo_ed_multiply_h_dev or
 * mo_ed_hv_tuning call (those build its tables and may allocate); otherwise
 * MO_ED_ERR_STATE.  mo_ed_create looks up the region's address on its
 * device, which commits the region there before the host's pool takes the
 * device; if that look-up failed, the first call on the device repeats it,
 * so make that call before any stream capture.  A device reset after the
 * look-up is not supported.  All calls share the region, which keeps the
 * previous call's contents (this call clears what must start at zero); calls
 * that overlap on the GPU race on it, so serialise them. */
int mo_ed_lanczos_iteration_noalloc(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *vec,
                                    int *nstep_calc, double *a, double *b);

/* ---- a13: diag (ed_solver.F90:107-191) ---------------------------------- */
/* nev lowest eigenpairs of one sector (thick-restart Lanczos with full
 * reorthogonalisation; FP64 Rayleigh quotients).  eigval[nev] (unconverged /
 * nonexistent levels: DBL_MAX, like the reference's huge()); eigvec may be
 * NULL or a host (ntot, nev) column-major FP64 array. */
int mo_ed_diag(mo_ed_ctx *ctx, int ne_up, int ne_down, int nev, double *eigval, double *eigvec);

/* Statistics of the last eigensolve (like ARPACK's iparam(3) / iparam(9)):
 * restart cycles, H*v applications, the largest Ritz residual estimate and
 * the largest FP64 residual ||H x - E x|| / ||x|| of the returned vectors. */
int mo_ed_diag_stats(mo_ed_ctx *ctx, int *cycles, long long *matvecs, double *res_est,
                     double *res_true);

/* Statistics of the last mo_ed_calc_green_ftn (no counterpart in the
 * reference): with green_fp64 over FP32 eigenvectors, the largest Ritz
 * residual ||H x - E x|| of their FP64 refinement; 0 when none ran. */
int mo_ed_green_stats(mo_ed_ctx *ctx, double *refine_res);

/* ---- a14: ed_solve (ed_solver.F90:28-105) ------------------------------- */
/* All sectors of mo_ed_set_sectors: eigenpairs, heapsort, Boltzmann weights,
 * nev_calc and normalized probabilities.  Eigenvectors of the kept states stay
 * on the device for mo_ed_calc_green_ftn.  Outputs have capacity entries;
 * sector / level are 1-based as eigval_t (ed_solver.F90:15-20). */
int mo_ed_solve(mo_ed_ctx *ctx, int *nev_calc, double *val, double *prob, int *sector,
                int *level, int capacity);

/* ---- a15-a16: Green's function (ed_green.F90:60-185) -------------------- */
/* Gr(norb, nw) after mo_ed_solve: for every kept state and orbital/spin,
 * c^dagger psi and c psi, Lanczos, and the continued fractions, all
 * excitations batched per Lanczos step.  Gr is overwritten (Gr(:,:) = 0 at
 * ed_green.F90:78). */
int mo_ed_calc_green_ftn(mo_ed_ctx *ctx, double *Gr);
/* The continued-fraction coefficients of the last mo_ed_calc_green_ftn, in
 * the order the reference writes apbpanbn.dat (ed_green.F90:112-115,
 * 125-128): for record r, nstep_calc[2r] (particle) and nstep_calc[2r+1]
 * (hole), coefficients ab[r][4][nstep+1] = ap, bp, an, bn.  nstep_calc = -1
 * marks a run whose excitation leaves the Fock space (c+ on a full or c on an
 * empty spin species): it adds nothing to G or A.  *nrec receives the record
 * count; ab / nstep_calc may be NULL to query it. */
int mo_ed_green_coeffs(mo_ed_ctx *ctx, int *nrec, int *nstep_calc, double *ab, int capacity);

/* ---- DMFT self-consistency (ed_hamiltonian.F90:29-85, ed_green.F90:187-253) -- */
/* ed_set_band_structure: the square-lattice band Hk(i,i,k) = -0.5 (cos kx +
 * cos ky) on a sqrt(Nq) x sqrt(Nq) grid, kept on the device for
 * mo_ed_delta_new; ef(norb) = its k-average (the reference also copies ef
 * into ek(1:norb)).  Nq must be a perfect square (the reference stops). */
int mo_ed_set_band_structure(mo_ed_ctx *ctx, int nq, double *ef);
/* ed_delta_new: for every orbital and w_n, Gksum = (1/Nq) sum_k 1 / (1/Gr +
 * D_ev + mu - Hk(k)) and D_ev <- 1/Gr - 1/Gksum + D_ev.  Gr, D_ev (in/out)
 * and Gksum (out, may be NULL) are complex (norb, nwloc), interleaved re/im. */
int mo_ed_delta_new(mo_ed_ctx *ctx, int nwloc, double rmu, const double *Gr, double *D_ev,
                    double *Gksum);
/* n_from_gksum: nocc(iorb) = 2 sum_w Re Gksum(iorb, w) / beta + 0.5. */
int mo_ed_n_from_gksum(mo_ed_ctx *ctx, int nw, const double *Gksum, double beta, double *nocc);

/* ---- real-frequency spectral function (dos.f90:1-106) ------------------------ */
/* A(iorb, w) = -Im(G+ + G-) / pi from the records of the last
 * mo_ed_calc_green_ftn (the apbpanbn.dat content), z+ = CMPLX(E + w, small),
 * z- = CMPLX(w - E, small) (default-REAL rounding with fortran_cmplx).
 * weighted = 0: as dos_diag, each record assigns A(iorb, :), so the last
 * record of an orbital sets it; weighted = 1: sum of pev * factor * A over
 * the records.  omega_real(nw); Aff real (norb, nw). */
int mo_ed_dos(mo_ed_ctx *ctx, int nw, const double *omega_real, double small, int weighted,
              double *Aff);

/* ---- eigenpair and coefficient files (ed_io.F90:13-147, ed_green.F90:112-115) -- */
/* Fortran unformatted sequential files as gfortran writes them (4-byte record
 * length markers before and after each record, LOGICAL as a 4-byte 1/0).
 * export: eigenvalues.dat (export_eigval's layout: nev_calc, then
 * {ind, eigenvalue, Boltzmann factor} per kept state) and eigvec-SS-LLL-0000
 * (nloc, then the vector in the reference's row order) for every state kept
 * by the last mo_ed_solve, into directory dir (NULL or "": the current one).
 * import: reads them back as the kept states (same model, sectors and nev),
 * so mo_ed_calc_green_ftn can run without mo_ed_solve; *nev_calc receives the
 * state count. */
int mo_ed_export_eigvec(mo_ed_ctx *ctx, const char *dir);
int mo_ed_import_eigvec(mo_ed_ctx *ctx, const char *dir, int *nev_calc);
/* apbpanbn.dat: the records of the last mo_ed_calc_green_ftn in the
 * reference's layout ({nstep_calcp, nstep_calcn}, then {iev, iorb, E, prob,
 * even, ap, bp, an, bn}; nstep_calc = -1: no run).  read replaces the
 * context's records (for mo_ed_dos, as dos.f90 reads the file); *nrec
 * receives the record count. */
int mo_ed_write_apbpanbn(mo_ed_ctx *ctx, const char *path);
int mo_ed_read_apbpanbn(mo_ed_ctx *ctx, const char *path, int *nrec);

/* ---- a18-a22: bath fit (func.f90, frprmn.f90, ed_green.F90:260-273) ------ */
/* FUNC (func.f90:1-45): chi^2 at x(nxsize); D_ev (norb, nwloc) complex. */
int mo_ed_func(mo_ed_ctx *ctx, const double *x, int ns, int nwloc, int nxsize,
               const double *omega, const double *D_ev, int nbath, int norb, double *f);
/* dfunc (func.f90:47-142): gradient p(nxsize) (argument order as the reference). */
int mo_ed_dfunc(mo_ed_ctx *ctx, const double *x, double *p, int nwloc, int ns, int nxsize,
                const double *omega, const double *D_ev, int nbath, int norb);
/* minimization (func.f90:144-163): Polak-Ribiere CG (frprmn.f90) from x, in
 * place, with FTOL = 1e-7; *fret = final chi^2, *iter = CG iterations. */
int mo_ed_minimization(mo_ed_ctx *ctx, double *x, int nwloc, int ns, int nxsize,
                       const double *omega, const double *D_ev, int nbath, int norb,
                       double *fret, int *iter);
/* nbatch independent fits (the reference runs one per call) in one launch:
 * each fit runs on a thread-block cluster that splits every FUNC / dfunc
 * over its CTAs by w_n; the clusters share the fits out and take turns on
 * long ones.  Each fit's result equals that of the same fit run alone, bit
 * for bit.  x[nbatch][nxsize] in place; fret, iter, status have nbatch
 * entries (status: 0, or MO_ED_ERR_FIT). */
int mo_ed_fit_batch(mo_ed_ctx *ctx, int nbatch, double *x, int nwloc, int ns, int nxsize,
                    const double *omega, const double *D_ev, int nbath, int norb, double ftol,
                    double *fret, int *iter, int *status);
/* Statistics of the last mo_ed_fit_batch / mo_ed_minimization (no
 * counterpart in the reference): how often a fit gave up its cluster to a
 * waiting fit, and the number of clusters launched. */
int mo_ed_fit_stats(mo_ed_ctx *ctx, long long *suspensions, int *clusters);
/* chi^2 and gradient of nbatch parameter sets on device pointers
 * (x[nbatch][nxsize], f[nbatch], g[nbatch][nxsize]); dev is the device copy
 * of D_ev, omega of the grid.  No synchronization. */
int mo_ed_chi2_grad_dev(mo_ed_ctx *ctx, int nbatch, const double *x, int nwloc, int ns,
                        int nxsize, const double *omega, const double *D_ev, int nbath,
                        int norb, double *f, double *g);
/* calc_dev (ed_green.F90:260-273): D_ev(norb, nwloc) from ek(nsite), vk, ef(norb). */
int mo_ed_calc_dev(mo_ed_ctx *ctx, int norb, int nsite, int nwloc, const double *omega,
                   const double *ek, const double *vk, const double *ef, double *D_ev);

/* ---- host helpers of the same path (no device work) --------------------- */
/* ev_to_x / x_to_ev (func.f90:165-216). */
int mo_ed_ev_to_x(const double *ek, const double *vk, const double *ef, int ns, int nbath,
                  int nxsize, double *x);
int mo_ed_x_to_ev(const double *x, int nxsize, int ns, int nbath, int norb, double *ef,
                  double *ek, double *vk);

/* ---- instrumentation -------------------------------------------------- */
/* Number of kernels this context has launched since creation. */
long long mo_ed_kernel_launches(const mo_ed_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
