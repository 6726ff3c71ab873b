/*
 * ed_oracle.h -- CPU restatement of the MO-DMFT exact-diagonalization hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity reference for the CUDA solver
 * and the timed CPU baseline ("port") of bench.py.  It is never linked into,
 * loaded by or called from the product library; only tests/, the smoke check
 * of __graft_entry__.py and the CPU-baseline leg of bench.py may use it.
 *
 * Every function restates one routine of the reference Fortran (single MPI
 * rank, so every MPI_Allgatherv is a copy and every MPI_Allreduce the
 * identity), in FP64, following the reference's loop order.  File:line
 * citations are into the reference project.
 *
 * Conventions (mirroring the Fortran):
 *   - sites are 1-based (1..nsite), spins 1 (up) / 2 (down), orbitals 1..norb,
 *     bath levels 1..nbath (site norb+ibath);
 *   - ek[nsite]: ek(1:nsite) (ed_config.f90:25);
 *   - vk[norb*nbath]: Fortran vk(1:norb, norb+1:nsite), column-major, i.e.
 *     vk[(ibath-1)*norb + (iorb-1)] (ed_config.f90:26,97);
 *   - row indices returned by or_basis_idx / taken by or_basis_get are
 *     1-based (ed_basis.F90:110-139);
 *   - complex arrays are interleaved (re, im), Fortran column-major
 *     (norb, nw), i.e. element (iorb, iw) at 2*((iw-1)*norb + iorb-1).
 */
#ifndef ED_ORACLE_H
#define ED_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int norb, nbath, nsite;
    double U, Jex;
    const double *ek;   /* nsite */
    const double *vk;   /* norb*nbath, column-major (norb fastest) */
} or_model;

typedef struct {
    int nsite, ne_up, ne_down;
    int nup, ndown;
    int64_t ntot;
    int *up, *down;          /* words, ascending (ed_basis.F90:69-105) */
    int *idx_up, *idx_down;  /* dense inverse tables over [0, 2^nsite) */
} or_basis;

/* ed_utils.f90:28-69 (int32 arithmetic, as in the reference) */
int or_ifact(int n);
int or_iP(int n, int m);
int or_icom(int n, int m);

/* ed_basis.F90:35-107.  Returns 0 on success. */
int or_generate_basis(int nsite, int ne_up, int ne_down, or_basis *b);
void or_free_basis(or_basis *b);
/* ed_basis.F90:110-124 (idx 1-based) */
uint32_t or_basis_get(const or_basis *b, int64_t idx);
/* ed_basis.F90:127-139 (returns 1-based row) */
int64_t or_basis_idx(const or_basis *b, uint32_t state);

/* ed_operators.F90:273-348: return sgn (0, +1, -1) and the new state */
int or_number_op(uint32_t in, int isite, int ispin, int nsite, uint32_t *out);
int or_destruction_op(uint32_t in, int isite, int ispin, int nsite, uint32_t *out);
int or_creation_op(uint32_t in, int isite, int ispin, int nsite, uint32_t *out);

/* ed_hamiltonian.F90:88-191.  B = H*A over the whole sector. */
void or_multiply_H(const or_model *m, const or_basis *b, const double *A, double *B);
/* Same restatement, rows split over nthreads OpenMP threads (the MPI row
 * split of ed_basis.F90:52-62 on one node).  nthreads <= 0: all cores. */
void or_multiply_H_omp(const or_model *m, const or_basis *b, const double *A,
                       double *B, int nthreads);
/* Rows [row0, row1) (0-based) of B = H*A with nthreads OpenMP threads: a
 * bounded sample of one H*v for the CPU baseline. */
void or_multiply_H_rows(const or_model *m, const or_basis *b, const double *A, double *B,
                        int64_t row0, int64_t row1, int nthreads);
/* Dense H of the sector (row-major ntot x ntot), built column by column
 * with or_multiply_H; for small sectors only. */
int or_dense_H(const or_model *m, const or_basis *b, double *Hd);

/* ed_operators.F90:10-61.  vec_out has basis_out->ntot entries; basis_out
 * must be freed by the caller.  Returns 0, or 2 if the target sector does
 * not exist (ne out of [0, nsite]). */
int or_apply_c(const or_model *m, const or_basis *b, const double *vec, int pm,
               int iorb, int ispin, or_basis *bout, double **vec_out);

/* ed_lanczos.F90:14-68.  a, b have nstep+1 entries (0:nstep). b holds the
 * squared norms.  Returns nstep_calc.  nthreads as or_multiply_H_omp. */
int or_lanczos_iteration(const or_model *m, const or_basis *bs, const double *vec,
                         int nstep, double *a, double *b, int nthreads);

/* ed_green.F90:160-168 (particle) and :176-184 (hole) continued fractions,
 * accumulated into gr (interleaved complex, nw entries of one orbital) as
 * gr += pev*factor*G.  sgn = +1 particle (z = E + i w, -a), -1 hole
 * (z = -E + i w, +a). */
void or_green_cf(int sgn, double eigval, double pev, double factor, int nstep_calc,
                 const double *a, const double *b, int nw, const double *omega,
                 double *gr);

/* ed_solver.F90:193-219 */
void or_boltzmann_factor(const double *elv, int nev, double beta, double *p);
/* func.f90:301-353 (heapsort, 1-based indices written to indx) */
void or_sort(int n, const double *arrin, int *indx);

/* func.f90:165-216 */
void or_ev_to_x(const double *ek, const double *vk, const double *ef, int ns,
                int nbath, int nxsize, double *x);
void or_x_to_ev(const double *x, int nxsize, int ns, int nbath, int norb,
                double *ef, double *ek, double *vk);
/* func.f90:1-45 and :47-142 (one rank: nw == nwloc) */
double or_func(const double *x, int ns, int nwloc, int nxsize, const double *omega,
               const double *dev, int nbath, int norb);
void or_dfunc(const double *x, double *p, int nwloc, int ns, int nxsize,
              const double *omega, const double *dev, int nbath, int norb);
/* frprmn.f90:1-310 with the reference's default-REAL constants.
 * Returns 0 on convergence, 1 if itmax was exceeded (the reference
 * stops the program), 2 if brent exceeded its iteration limit. */
int or_frprmn(double *p, int n, double ftol, int *iter, double *fret, int nxsize,
              int nwloc, int ns, const double *omega, const double *dev, int nbath,
              int norb);
/* ed_green.F90:260-273 */
void or_calc_dev(int norb, int nsite, int nwloc, const double *omega,
                 const double *ek, const double *vk, const double *ef, double *dev);

/* ed_hamiltonian.F90:29-85: square-lattice band hk[nq] and ef[norb]. */
int or_set_band_structure(int norb, int nq, double *hk, double *ef);
/* ed_green.F90:187-214: Gksum and the updated D_ev (complex (norb, nwloc)). */
void or_delta_new(int norb, int nwloc, int nq, const double *hk, double rmu, const double *gr,
                  double *dev, double *gksum);
/* ed_green.F90:227-253 */
void or_n_from_gksum(int norb, int nw, const double *gksum, double beta, double *nocc);
/* dos.f90:1-106 over apbpanbn.dat records (weighted = 0: the reference's
 * assignment; 1: probability-weighted sum). */
void or_dos(int norb, int nrec, const int *iorb, const double *ev, const double *prob,
            const int *even, const int *np, const int *nn, const double *ab, int ld, int nw,
            const double *omega_real, double small, int weighted, double *aff);

/* Number of FUNC evaluations performed by or_frprmn since the last reset. */
int64_t or_func_calls(void);
void or_reset_func_calls(void);

#ifdef __cplusplus
}
#endif
#endif
