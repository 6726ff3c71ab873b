/*
 * ed_oracle.c -- FP64 CPU restatement of the MO-DMFT ED hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity reference of the tests and the "port" CPU baseline); see
 * ed_oracle.h.  Nothing in the product links or loads this file.
 *
 * Each routine follows the cited reference routine loop for loop on a single
 * MPI rank.  Two reference behaviours are restated on purpose:
 *   - Fortran CMPLX(x, y) without KIND yields a default (single precision)
 *     complex, so every `cmplx(a, b)` of the reference rounds a and b to
 *     float before use (ed_green.F90:161,177,268; func.f90:25,80,96-97,110-112).
 *     fcmplx() below does exactly that.
 *   - Default-REAL literals (1.e-12 in ed_lanczos.F90:62, the frprmn.f90
 *     constants) are single-precision values widened to double.
 * Complex division uses Smith's (1962) scaled algorithm.
 */
#include "ed_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* small complex helpers                                               */
/* ------------------------------------------------------------------ */
typedef struct { double re, im; } cplx;

static cplx c_make(double re, double im) { cplx z = {re, im}; return z; }
/* Fortran CMPLX(re, im) without KIND: default (single-precision) complex */
static cplx fcmplx(double re, double im) { return c_make((double)(float)re, (double)(float)im); }
static cplx c_add(cplx a, cplx b) { return c_make(a.re + b.re, a.im + b.im); }
static cplx c_sub(cplx a, cplx b) { return c_make(a.re - b.re, a.im - b.im); }
static cplx c_scale(cplx a, double s) { return c_make(a.re * s, a.im * s); }
static cplx c_conj(cplx a) { return c_make(a.re, -a.im); }
/* Smith's algorithm for a/b */
static cplx c_div(cplx a, cplx b)
{
    if (fabs(b.re) >= fabs(b.im)) {
        double r = b.im / b.re, den = b.re + b.im * r;
        return c_make((a.re + a.im * r) / den, (a.im - a.re * r) / den);
    } else {
        double r = b.re / b.im, den = b.re * r + b.im;
        return c_make((a.re * r + a.im) / den, (a.im * r - a.re) / den);
    }
}
static double c_abs(cplx a) { return hypot(a.re, a.im); }

/* ------------------------------------------------------------------ */
/* ed_utils.f90:28-69                                                   */
/* ------------------------------------------------------------------ */
int or_ifact(int n)
{
    int32_t f = 1;
    for (int i = 1; i <= n; ++i) f = (int32_t)((uint32_t)f * (uint32_t)i);
    return f;
}

int or_iP(int n, int m)
{
    int32_t p = 1;
    for (int i = n - m + 1; i <= n; ++i) p = (int32_t)((uint32_t)p * (uint32_t)i);
    return p;
}

int or_icom(int n, int m)
{
    if (n == m || m == 0) return 1;
    if (m > n / 2) {
        int k = n - m;
        return or_iP(n, k) / or_ifact(k);
    }
    return or_iP(n, m) / or_ifact(m);
}

/* ------------------------------------------------------------------ */
/* ed_basis.F90                                                         */
/* ------------------------------------------------------------------ */
static int btest(uint32_t w, int bit) { return (int)((w >> bit) & 1u); }

/* ed_basis.F90:35-107: enumerate [minrange, maxrange], keep popcount == ne */
static int build_species(int nsite, int ne, int n_expected, int **words, int **idx)
{
    int64_t minrange = 0, maxrange = 0;
    for (int i = 1; i <= ne; ++i) {
        minrange += (int64_t)1 << (i - 1);
        maxrange += (nsite - i >= 0) ? ((int64_t)1 << (nsite - i)) : 0;
    }
    *words = (int *)calloc((size_t)(n_expected > 0 ? n_expected : 1), sizeof(int));
    *idx = (int *)calloc((size_t)1 << nsite, sizeof(int));
    if (!*words || !*idx) return 1;
    int counts = 0;
    for (int64_t i = minrange; i <= maxrange; ++i) {
        int nbit = 0;
        for (int j = 0; j <= nsite - 1; ++j)
            if (btest((uint32_t)i, j)) nbit++;
        if (nbit == ne) {
            counts++;
            if (counts > n_expected) return 1;
            (*words)[counts - 1] = (int)i;
            (*idx)[i] = counts;
        }
    }
    return counts == n_expected ? 0 : 1;
}

int or_generate_basis(int nsite, int ne_up, int ne_down, or_basis *b)
{
    memset(b, 0, sizeof(*b));
    if (nsite < 1 || nsite > 15 || ne_up < 0 || ne_up > nsite || ne_down < 0 || ne_down > nsite)
        return 2;
    b->nsite = nsite;
    b->ne_up = ne_up;
    b->ne_down = ne_down;
    b->nup = or_icom(nsite, ne_up);
    b->ndown = or_icom(nsite, ne_down);
    b->ntot = (int64_t)b->nup * b->ndown;
    if (build_species(nsite, ne_up, b->nup, &b->up, &b->idx_up)) return 1;
    if (build_species(nsite, ne_down, b->ndown, &b->down, &b->idx_down)) return 1;
    return 0;
}

void or_free_basis(or_basis *b)
{
    free(b->up); free(b->down); free(b->idx_up); free(b->idx_down);
    memset(b, 0, sizeof(*b));
}

uint32_t or_basis_get(const or_basis *b, int64_t idx)
{
    int64_t iup = (idx - 1) % b->nup + 1;
    int64_t idown = (idx - 1) / b->nup + 1;
    return (uint32_t)b->up[iup - 1] + ((uint32_t)1 << b->nsite) * (uint32_t)b->down[idown - 1];
}

int64_t or_basis_idx(const or_basis *b, uint32_t state)
{
    uint32_t s_up = state % (1u << b->nsite);
    uint32_t s_dn = state / (1u << b->nsite);
    return (int64_t)(b->idx_down[s_dn] - 1) * b->nup + b->idx_up[s_up];
}

/* ------------------------------------------------------------------ */
/* ed_operators.F90                                                     */
/* ------------------------------------------------------------------ */
static int get_bitidx(int isite, int ispin, int nsite) { return (ispin - 1) * nsite + isite - 1; }

int or_number_op(uint32_t in, int isite, int ispin, int nsite, uint32_t *out)
{
    int bit = get_bitidx(isite, ispin, nsite);
    if (btest(in, bit)) { *out = in; return 1; }
    *out = 0;
    return 0;
}

int or_destruction_op(uint32_t in, int isite, int ispin, int nsite, uint32_t *out)
{
    int bit = get_bitidx(isite, ispin, nsite);
    if (btest(in, bit)) {
        int n = 0;
        for (int i = 0; i <= bit - 1; ++i)
            if (btest(in, i)) n++;
        *out = in & ~(1u << bit);
        return (n % 2 == 1) ? -1 : 1;
    }
    *out = 0;
    return 0;
}

int or_creation_op(uint32_t in, int isite, int ispin, int nsite, uint32_t *out)
{
    int bit = get_bitidx(isite, ispin, nsite);
    if (!btest(in, bit)) {
        int n = 0;
        for (int i = 0; i <= bit - 1; ++i)
            if (btest(in, i)) n++;
        *out = in | (1u << bit);
        return (n % 2 == 1) ? -1 : 1;
    }
    *out = 0;
    return 0;
}

static double vk_at(const or_model *m, int iorb, int isite)
{
    /* vk(iorb, isite), isite in norb+1..nsite */
    return m->vk[(size_t)(isite - m->norb - 1) * m->norb + (iorb - 1)];
}

/* ed_operators.F90:68-84 */
static double op_onsite(const or_model *m, uint32_t in, int isite, int ispin)
{
    uint32_t out;
    if (or_number_op(in, isite, ispin, m->nsite, &out) == 0) return 0.0;
    return m->ek[isite - 1];
}

/* ed_operators.F90:86-107 */
static double op_hyb1(const or_model *m, uint32_t in, int iorb, int ibath, int ispin, uint32_t *out)
{
    double coeff = 1.0;
    int sgn = or_destruction_op(in, m->norb + ibath, ispin, m->nsite, out);
    if (sgn == 0) return 0.0;
    coeff *= sgn;
    sgn = or_creation_op(*out, iorb, ispin, m->nsite, out);
    if (sgn == 0) return 0.0;
    coeff *= sgn;
    return coeff * vk_at(m, iorb, m->norb + ibath);
}

/* ed_operators.F90:109-130 */
static double op_hyb2(const or_model *m, uint32_t in, int iorb, int ibath, int ispin, uint32_t *out)
{
    double coeff = 1.0;
    int sgn = or_destruction_op(in, iorb, ispin, m->nsite, out);
    if (sgn == 0) return 0.0;
    coeff *= sgn;
    sgn = or_creation_op(*out, m->norb + ibath, ispin, m->nsite, out);
    if (sgn == 0) return 0.0;
    coeff *= sgn;
    return coeff * vk_at(m, iorb, m->norb + ibath);
}

/* ed_operators.F90:132-165 */
static double op_dens_dens(const or_model *m, uint32_t in, int iorb, int jorb, int ispin, int jspin)
{
    uint32_t out;
    int n1 = or_number_op(in, iorb, ispin, m->nsite, &out);
    int n2 = or_number_op(in, jorb, jspin, m->nsite, &out);
    if (n1 * n2 == 0) return 0.0;
    if (iorb == jorb) {
        if (ispin == jspin) return 0.0;
        return m->U;
    } else if (ispin == jspin) {
        return m->U - 3 * m->Jex;
    }
    return m->U - 2 * m->Jex;
}

/* ed_operators.F90:167-218 */
static double op_spin_flip(const or_model *m, uint32_t in, int iorb, int jorb, uint32_t *out)
{
    int sgn_tot = 1, sgn;
    *out = 0;
    if (iorb == jorb) return 0.0;
    sgn = or_destruction_op(in, jorb, 1, m->nsite, out);      /* c_j,u   */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    sgn = or_creation_op(*out, jorb, 2, m->nsite, out);       /* c+_j,d  */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    sgn = or_destruction_op(*out, iorb, 2, m->nsite, out);    /* c_i,d   */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    sgn = or_creation_op(*out, iorb, 1, m->nsite, out);       /* c+_i,u  */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    return -m->Jex * sgn_tot;
}

/* ed_operators.F90:220-271 */
static double op_pair_exchange(const or_model *m, uint32_t in, int iorb, int jorb, uint32_t *out)
{
    int sgn_tot = 1, sgn;
    *out = 0;
    if (iorb == jorb) return 0.0;
    sgn = or_destruction_op(in, jorb, 2, m->nsite, out);      /* c_j,d   */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    sgn = or_destruction_op(*out, jorb, 1, m->nsite, out);    /* c_j,u   */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    sgn = or_creation_op(*out, iorb, 2, m->nsite, out);       /* c+_i,d  */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    sgn = or_creation_op(*out, iorb, 1, m->nsite, out);       /* c+_i,u  */
    if (sgn == 0) return 0.0;
    sgn_tot *= sgn;
    return -m->Jex * sgn_tot;
}

/* ------------------------------------------------------------------ */
/* ed_hamiltonian.F90:88-191 -- one row of B = H*A                      */
/* ------------------------------------------------------------------ */
static double multiply_H_row(const or_model *m, const or_basis *b, const double *A_all, int64_t i)
{
    const int norb = m->norb, nbath = m->nbath;
    uint32_t basis_i = or_basis_get(b, i), basis_j;
    double coeff_sum = 0.0, coeff, Bi;

    /* 1. onsite */
    for (int ispin = 1; ispin <= 2; ++ispin) {
        for (int iorb = 1; iorb <= norb; ++iorb) coeff_sum = coeff_sum + op_onsite(m, basis_i, iorb, ispin);
        for (int ibath = 1; ibath <= nbath; ++ibath)
            coeff_sum = coeff_sum + op_onsite(m, basis_i, norb + ibath, ispin);
    }
    /* 2. density-density: intra-orbital */
    for (int iorb = 1; iorb <= norb; ++iorb) coeff_sum = coeff_sum + op_dens_dens(m, basis_i, iorb, iorb, 1, 2);
    /* 3. density-density: inter-orbital */
    for (int iorb = 1; iorb <= norb; ++iorb)
        for (int jorb = iorb + 1; jorb <= norb; ++jorb)
            for (int ispin = 1; ispin <= 2; ++ispin)
                for (int jspin = 1; jspin <= 2; ++jspin)
                    coeff_sum = coeff_sum + op_dens_dens(m, basis_i, iorb, jorb, ispin, jspin);

    Bi = coeff_sum * A_all[i - 1];

    /* off-diagonal 1. hybridization */
    for (int ispin = 1; ispin <= 2; ++ispin)
        for (int iorb = 1; iorb <= norb; ++iorb)
            for (int ibath = 1; ibath <= nbath; ++ibath) {
                coeff = op_hyb1(m, basis_i, iorb, ibath, ispin, &basis_j);
                if (basis_j != 0) Bi = Bi + coeff * A_all[or_basis_idx(b, basis_j) - 1];
                coeff = op_hyb2(m, basis_i, iorb, ibath, ispin, &basis_j);
                if (basis_j != 0) Bi = Bi + coeff * A_all[or_basis_idx(b, basis_j) - 1];
            }
    /* 2. spin-flip */
    for (int iorb = 1; iorb <= norb; ++iorb)
        for (int jorb = 1; jorb <= norb; ++jorb) {
            if (iorb == jorb) continue;
            coeff = op_spin_flip(m, basis_i, iorb, jorb, &basis_j);
            if (basis_j != 0) Bi = Bi + coeff * A_all[or_basis_idx(b, basis_j) - 1];
        }
    /* 3. pair-exchange */
    for (int iorb = 1; iorb <= norb; ++iorb)
        for (int jorb = 1; jorb <= norb; ++jorb) {
            if (iorb == jorb) continue;
            coeff = op_pair_exchange(m, basis_i, iorb, jorb, &basis_j);
            if (basis_j != 0) Bi = Bi + coeff * A_all[or_basis_idx(b, basis_j) - 1];
        }
    return Bi;
}

void or_multiply_H(const or_model *m, const or_basis *b, const double *A, double *B)
{
    for (int64_t i = 1; i <= b->ntot; ++i) B[i - 1] = multiply_H_row(m, b, A, i);
}

void or_multiply_H_omp(const or_model *m, const or_basis *b, const double *A, double *B, int nthreads)
{
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 1; i <= b->ntot; ++i) B[i - 1] = multiply_H_row(m, b, A, i);
#else
    (void)nthreads;
    or_multiply_H(m, b, A, B);
#endif
}

void or_multiply_H_rows(const or_model *m, const or_basis *b, const double *A, double *B,
                        int64_t row0, int64_t row1, int nthreads)
{
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = row0 + 1; i <= row1; ++i) B[i - 1] = multiply_H_row(m, b, A, i);
#else
    (void)nthreads;
    for (int64_t i = row0 + 1; i <= row1; ++i) B[i - 1] = multiply_H_row(m, b, A, i);
#endif
}

int or_dense_H(const or_model *m, const or_basis *b, double *Hd)
{
    int64_t n = b->ntot;
    double *e = (double *)calloc((size_t)n, sizeof(double));
    double *col = (double *)malloc((size_t)n * sizeof(double));
    if (!e || !col) { free(e); free(col); return 1; }
    for (int64_t j = 0; j < n; ++j) {
        e[j] = 1.0;
        or_multiply_H(m, b, e, col);
        for (int64_t i = 0; i < n; ++i) Hd[i * n + j] = col[i];
        e[j] = 0.0;
    }
    free(e); free(col);
    return 0;
}

/* ------------------------------------------------------------------ */
/* ed_operators.F90:10-61                                               */
/* ------------------------------------------------------------------ */
int or_apply_c(const or_model *m, const or_basis *b, const double *vec, int pm, int iorb, int ispin,
               or_basis *bout, double **vec_out)
{
    int nu = b->ne_up, nd = b->ne_down;
    if (ispin == 1) nu += (pm == 1) ? 1 : -1;
    else nd += (pm == 1) ? 1 : -1;
    *vec_out = NULL;
    int rc = or_generate_basis(m->nsite, nu, nd, bout);
    if (rc) return rc;
    double *out = (double *)calloc((size_t)bout->ntot, sizeof(double));
    if (!out) return 1;
    for (int64_t i = 1; i <= bout->ntot; ++i) {
        uint32_t basis_i = or_basis_get(bout, i), basis_j;
        int sgn = (pm == 1) ? or_destruction_op(basis_i, iorb, ispin, m->nsite, &basis_j)
                            : or_creation_op(basis_i, iorb, ispin, m->nsite, &basis_j);
        if (sgn == 0) continue;
        int64_t j = or_basis_idx(b, basis_j);
        out[i - 1] = out[i - 1] + vec[j - 1] * sgn;
    }
    *vec_out = out;
    return 0;
}

/* ------------------------------------------------------------------ */
/* ed_utils.f90:7-18 (one rank)                                         */
/* ------------------------------------------------------------------ */
static double dot(const double *x, const double *y, int64_t n)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

/* ------------------------------------------------------------------ */
/* ed_lanczos.F90:14-68                                                 */
/* ------------------------------------------------------------------ */
int or_lanczos_iteration(const or_model *m, const or_basis *bs, const double *vec, int nstep,
                         double *a, double *b, int nthreads)
{
    const double tiny = (double)1.e-12f; /* default-REAL literal, ed_lanczos.F90:62 */
    int64_t n = bs->ntot;
    double *v1 = (double *)malloc((size_t)n * sizeof(double));
    double *v2 = (double *)calloc((size_t)n, sizeof(double));
    double *v3 = (double *)malloc((size_t)n * sizeof(double));
    double *w = (double *)calloc((size_t)n, sizeof(double));
    int nstep_calc = nstep;
    for (int j = 0; j <= nstep; ++j) { a[j] = 0.0; b[j] = 0.0; }

    memcpy(v1, vec, (size_t)n * sizeof(double));
    double norm_v = dot(v1, v1, n);
    for (int64_t i = 0; i < n; ++i) v1[i] = v1[i] / sqrt(norm_v);
    or_multiply_H_omp(m, bs, v1, w, nthreads);
    a[0] = dot(v1, w, n);
    b[0] = 0.0;

    for (int64_t i = 0; i < n; ++i) v2[i] = w[i] - a[0] * v1[i];
    b[1] = dot(v2, v2, n);
    or_multiply_H_omp(m, bs, v2, w, nthreads);
    a[1] = dot(w, v2, n);
    a[1] = a[1] / b[1];
    for (int64_t i = 0; i < n; ++i) v2[i] = v2[i] / sqrt(b[1]);

    for (int j = 2; j <= nstep; ++j) {
        double sb = sqrt(b[j - 1]);
        for (int64_t i = 0; i < n; ++i) v3[i] = w[i] / sb - a[j - 1] * v2[i] - sb * v1[i];
        b[j] = dot(v3, v3, n);
        or_multiply_H_omp(m, bs, v3, w, nthreads);
        a[j] = dot(v3, w, n);
        a[j] = a[j] / b[j];
        for (int64_t i = 0; i < n; ++i) v3[i] = v3[i] / sqrt(b[j]);
        if (b[j] < tiny) { nstep_calc = j; break; }
        double *t = v1; v1 = v2; v2 = v3; v3 = t;
    }
    free(v1); free(v2); free(v3); free(w);
    return nstep_calc;
}

/* ------------------------------------------------------------------ */
/* ed_green.F90:160-168 / 176-184                                       */
/* ------------------------------------------------------------------ */
void or_green_cf(int sgn, double eigval, double pev, double factor, int nstep_calc, const double *a,
                 const double *b, int nw, const double *omega, double *gr)
{
    for (int i = 0; i < nw; ++i) {
        cplx z, grx;
        if (sgn > 0) {
            z = fcmplx(eigval, omega[i]);
            grx = c_div(c_make(b[nstep_calc], 0.0), c_sub(z, c_make(a[nstep_calc], 0.0)));
            for (int j = nstep_calc - 1; j >= 0; --j)
                grx = c_div(c_make(b[j], 0.0), c_sub(c_sub(z, c_make(a[j], 0.0)), grx));
        } else {
            z = fcmplx(-eigval, omega[i]);
            grx = c_div(c_make(b[nstep_calc], 0.0), c_add(z, c_make(a[nstep_calc], 0.0)));
            for (int j = nstep_calc - 1; j >= 0; --j)
                grx = c_div(c_make(b[j], 0.0), c_sub(c_add(z, c_make(a[j], 0.0)), grx));
        }
        double s = pev * factor;
        gr[2 * i] += s * grx.re;
        gr[2 * i + 1] += s * grx.im;
    }
}

/* ------------------------------------------------------------------ */
/* ed_solver.F90:193-219                                                */
/* ------------------------------------------------------------------ */
void or_boltzmann_factor(const double *elv, int nev, double beta, double *p)
{
    for (int i = 0; i < nev; ++i) {
        double Z = 0.0, en = elv[i];
        int zero = 0;
        for (int k = 0; k < nev; ++k) {
            if (-beta * (elv[k] - en) > 10.0) { zero = 1; break; }
            Z = Z + exp(-beta * (elv[k] - en));
        }
        p[i] = zero ? 0.0 : 1.0 / Z;
    }
}

/* ------------------------------------------------------------------ */
/* func.f90:301-353 (Numerical Recipes heapsort of an index)            */
/* ------------------------------------------------------------------ */
void or_sort(int n, const double *arrin, int *indx)
{
    /* 1-based views */
    const double *A = arrin - 1;
    int *X = indx - 1;
    if (n == 1) { X[1] = 1; return; }
    for (int j = 1; j <= n; ++j) X[j] = j;
    int l = n / 2 + 1, ir = n, indxt, i, j;
    double q;
    for (;;) {
        if (l > 1) {
            l = l - 1;
            indxt = X[l];
            q = A[indxt];
        } else {
            indxt = X[ir];
            q = A[indxt];
            X[ir] = X[1];
            ir = ir - 1;
            if (ir == 1) { X[1] = indxt; return; }
        }
        i = l;
        j = l + l;
        while (j <= ir) {
            if (j < ir && A[X[j]] < A[X[j + 1]]) j = j + 1;
            if (q < A[X[j]]) {
                X[i] = X[j];
                i = j;
                j = j + j;
            } else {
                j = ir + 1;
            }
        }
        X[i] = indxt;
    }
}

/* ------------------------------------------------------------------ */
/* func.f90:165-216                                                     */
/* ------------------------------------------------------------------ */
void or_ev_to_x(const double *ek, const double *vk, const double *ef, int ns, int nbath, int nxsize,
                double *x)
{
    int norb = ns - nbath;
    for (int i = 1; i <= nbath; ++i) x[i - 1] = ek[norb + i - 1];
    for (int iorb = 1; iorb <= norb; ++iorb) {
        int iinit = nbath + 1 + (iorb - 1) * nbath;
        int ifina = nbath + iorb * nbath;
        for (int k = iinit; k <= ifina; ++k) x[k - 1] = vk[(size_t)(k - iinit) * norb + (iorb - 1)];
    }
    for (int i = 1; i <= norb; ++i) x[nxsize - norb + i - 1] = ef[i - 1];
}

void or_x_to_ev(const double *x, int nxsize, int ns, int nbath, int norb, double *ef, double *ek,
                double *vk)
{
    for (int i = 1; i <= norb; ++i) {
        ek[i - 1] = x[nxsize - norb + i - 1];
        ef[i - 1] = ek[i - 1];
    }
    for (int i = norb + 1; i <= norb + nbath; ++i) ek[i - 1] = x[i - norb - 1];
    for (int iorb = 1; iorb <= norb; ++iorb) {
        int ia = (iorb - 1) * nbath;
        for (int i = norb + 1; i <= ns; ++i) vk[(size_t)(i - norb - 1) * norb + (iorb - 1)] = x[i + nbath + ia - norb - 1];
    }
}

/* ------------------------------------------------------------------ */
/* func.f90:1-45 / 47-142                                               */
/* ------------------------------------------------------------------ */
static int64_t g_func_calls = 0;
int64_t or_func_calls(void) { return g_func_calls; }
void or_reset_func_calls(void) { g_func_calls = 0; }

static void fit_delta(const double *x, int ns, int nwloc, int nxsize, const double *omega, int nbath,
                      int norb, double *ek, double *vk, double *ef, cplx *delta)
{
    or_x_to_ev(x, nxsize, ns, nbath, norb, ef, ek, vk);
    for (int iw = 0; iw < nwloc; ++iw)
        for (int korb = 1; korb <= norb; ++korb) {
            cplx d = c_make(0.0, 0.0);
            for (int ksite = norb + 1; ksite <= ns; ++ksite) {
                double v = vk[(size_t)(ksite - norb - 1) * norb + (korb - 1)];
                d = c_add(d, c_div(c_make(v * v, 0.0), c_sub(fcmplx(0.0, omega[iw]), c_make(ek[ksite - 1], 0.0))));
            }
            delta[(size_t)iw * norb + (korb - 1)] = c_add(d, c_make(ef[korb - 1], 0.0));
        }
}

double or_func(const double *x, int ns, int nwloc, int nxsize, const double *omega, const double *dev,
               int nbath, int norb)
{
    double *ek = (double *)malloc((size_t)ns * sizeof(double));
    double *vk = (double *)malloc((size_t)norb * nbath * sizeof(double));
    double *ef = (double *)malloc((size_t)norb * sizeof(double));
    cplx *delta = (cplx *)malloc((size_t)norb * nwloc * sizeof(cplx));
    fit_delta(x, ns, nwloc, nxsize, omega, nbath, norb, ek, vk, ef, delta);
    double func_loc = 0.0;
    for (int iw = 0; iw < nwloc; ++iw)
        for (int korb = 0; korb < norb; ++korb) {
            size_t k = (size_t)iw * norb + korb;
            cplx t = c_sub(delta[k], c_make(dev[2 * k], dev[2 * k + 1]));
            func_loc = func_loc + c_abs(t) * c_abs(t) / omega[iw];
        }
    int nw = nwloc;
    double func = func_loc / (double)(float)(norb * norb * nw);
    free(ek); free(vk); free(ef); free(delta);
    g_func_calls++;
    return func;
}

void or_dfunc(const double *x, double *p, int nwloc, int ns, int nxsize, const double *omega,
              const double *dev, int nbath, int norb)
{
    double *ek = (double *)malloc((size_t)ns * sizeof(double));
    double *vk = (double *)malloc((size_t)norb * nbath * sizeof(double));
    double *ef = (double *)malloc((size_t)norb * sizeof(double));
    cplx *delta = (cplx *)malloc((size_t)norb * nwloc * sizeof(cplx));
    fit_delta(x, ns, nwloc, nxsize, omega, nbath, norb, ek, vk, ef, delta);
    int nek = nbath;
    for (int ibath = 1; ibath <= nek; ++ibath) {
        double acc = 0.0;
        for (int korb = 1; korb <= norb; ++korb)
            for (int iw = 0; iw < nwloc; ++iw) {
                size_t k = (size_t)iw * norb + (korb - 1);
                cplx r = c_conj(c_sub(delta[k], c_make(dev[2 * k], dev[2 * k + 1])));
                double v = vk[(size_t)(ibath - 1) * norb + (korb - 1)];
                cplx den = c_sub(fcmplx(0.0, omega[iw]), c_make(ek[norb + ibath - 1], 0.0));
                /* conjg(r)*vk*vk/(z)/(z), evaluated left to right */
                cplx t = c_div(c_div(c_scale(c_scale(r, v), v), den), den);
                acc = acc + 2.0 * t.re / omega[iw];
            }
        p[ibath - 1] = acc;
    }
    for (int iorb = 1; iorb <= norb; ++iorb)
        for (int ksite = norb + 1; ksite <= ns; ++ksite) {
            int i = nek + ksite - norb + (iorb - 1) * nbath;
            double acc = 0.0;
            for (int iw = 0; iw < nwloc; ++iw) {
                size_t k = (size_t)iw * norb + (iorb - 1);
                cplx r = c_conj(c_sub(delta[k], c_make(dev[2 * k], dev[2 * k + 1])));
                double v = vk[(size_t)(ksite - norb - 1) * norb + (iorb - 1)];
                cplx den = c_sub(fcmplx(0.0, omega[iw]), c_make(ek[ksite - 1], 0.0));
                cplx t1 = c_div(c_scale(r, v), den);
                cplx t2 = c_div(c_scale(r, v), den);
                acc = acc + 2.0 * c_add(t1, t2).re / omega[iw];
            }
            p[i - 1] = acc;
        }
    for (int iorb = 1; iorb <= norb; ++iorb) {
        int i = nxsize - norb + iorb;
        double acc = 0.0;
        for (int iw = 0; iw < nwloc; ++iw) {
            size_t k = (size_t)iw * norb + (iorb - 1);
            acc = acc + 2.0 * (delta[k].re - dev[2 * k]) / omega[iw];
        }
        p[i - 1] = acc;
    }
    int nw = nwloc;
    for (int i = 0; i < nxsize; ++i) p[i] = p[i] / (double)(float)(norb * norb) / (double)(float)nw;
    free(ek); free(vk); free(ef); free(delta);
}

/* ------------------------------------------------------------------ */
/* frprmn.f90:1-310                                                     */
/* ------------------------------------------------------------------ */
typedef struct {
    int nxsize, nwloc, ns, nbath, norb;
    const double *omega, *dev;
    const double *pcom, *xicom;
    double *xt;
} fit_ctx;

static double f1dim(const fit_ctx *c, double x)   /* frprmn.f90:212-234 */
{
    for (int j = 0; j < c->nxsize; ++j) c->xt[j] = c->pcom[j] + x * c->xicom[j];
    return or_func(c->xt, c->ns, c->nwloc, c->nxsize, c->omega, c->dev, c->nbath, c->norb);
}

static double fsign(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

static void mnbrak(const fit_ctx *c, double *ax, double *bx, double *cx, double *fa, double *fb,
                   double *fc)   /* frprmn.f90:236-310 */
{
    const double GOLD = (double)1.618034f, GLIMIT = (double)100.f, TINY = (double)1.e-20f;
    double dum, fu, q, r, u, ulim;
    *fa = f1dim(c, *ax);
    *fb = f1dim(c, *bx);
    if (*fb > *fa) {
        dum = *ax; *ax = *bx; *bx = dum;
        dum = *fb; *fb = *fa; *fa = dum;
    }
    *cx = *bx + GOLD * (*bx - *ax);
    *fc = f1dim(c, *cx);
    while (*fb >= *fc) {
        r = (*bx - *ax) * (*fb - *fc);
        q = (*bx - *cx) * (*fb - *fa);
        u = *bx - ((*bx - *cx) * q - (*bx - *ax) * r) / (2. * fsign(fmax(fabs(q - r), TINY), q - r));
        ulim = *bx + GLIMIT * (*cx - *bx);
        if ((*bx - u) * (u - *cx) > 0.) {
            fu = f1dim(c, u);
            if (fu < *fc) {
                *ax = *bx; *fa = *fb; *bx = u; *fb = fu;
                return;
            } else if (fu > *fb) {
                *cx = u; *fc = fu;
                return;
            }
            u = *cx + GOLD * (*cx - *bx);
            fu = f1dim(c, u);
        } else if ((*cx - u) * (u - ulim) > 0.) {
            fu = f1dim(c, u);
            if (fu < *fc) {
                *bx = *cx; *cx = u; u = *cx + GOLD * (*cx - *bx);
                *fb = *fc; *fc = fu;
                fu = f1dim(c, u);
            }
        } else if ((u - ulim) * (ulim - *cx) >= 0.) {
            u = ulim;
            fu = f1dim(c, u);
        } else {
            u = *cx + GOLD * (*cx - *bx);
            fu = f1dim(c, u);
        }
        *ax = *bx; *bx = *cx; *cx = u;
        *fa = *fb; *fb = *fc; *fc = fu;
    }
}

static int brent(const fit_ctx *c, double ax, double bx, double cx, double tol, double *xmin,
                 double *fret)   /* frprmn.f90:119-210 */
{
    const int ITMAX = 100;
    const double CGOLD = (double).3819660f, ZEPS = (double)1.0e-10f;
    double a, b, d = 0.0, e, etemp, fu, fv, fw, fx, p, q, r, tol1, tol2, u, v, w, x, xm;
    a = fmin(ax, cx);
    b = fmax(ax, cx);
    v = bx; w = v; x = v;
    e = 0.;
    fx = f1dim(c, x);
    fv = fx; fw = fx;
    for (int iter = 1; iter <= ITMAX; ++iter) {
        xm = 0.5 * (a + b);
        tol1 = tol * fabs(x) + ZEPS;
        tol2 = 2. * tol1;
        if (fabs(x - xm) <= (tol2 - .5 * (b - a))) { *xmin = x; *fret = fx; return 0; }
        int golden = 1;
        if (fabs(e) > tol1) {
            r = (x - w) * (fx - fv);
            q = (x - v) * (fx - fw);
            p = (x - v) * q - (x - w) * r;
            q = 2. * (q - r);
            if (q > 0.) p = -p;
            q = fabs(q);
            etemp = e;
            e = d;
            if (!(fabs(p) >= fabs(.5 * q * etemp) || p <= q * (a - x) || p >= q * (b - x))) {
                d = p / q;
                u = x + d;
                if (u - a < tol2 || b - u < tol2) d = fsign(tol1, xm - x);
                golden = 0;
            }
        }
        if (golden) {
            e = (x >= xm) ? a - x : b - x;
            d = CGOLD * e;
        }
        u = (fabs(d) >= tol1) ? x + d : x + fsign(tol1, d);
        fu = f1dim(c, u);
        if (fu <= fx) {
            if (u >= x) a = x; else b = x;
            v = w; fv = fw; w = x; fw = fx; x = u; fx = fu;
        } else {
            if (u < x) a = u; else b = u;
            if (fu <= fw || w == x) {
                v = w; fv = fw; w = u; fw = fu;
            } else if (fu <= fv || v == x || v == w) {
                v = u; fv = fu;
            }
        }
    }
    *xmin = x;
    *fret = fx;
    return 2;
}

static int linmin(fit_ctx *c, double *p, double *xi, int n, double *fret)   /* frprmn.f90:86-117 */
{
    const double TOL = (double)1.e-8f;
    double pcom[60], xicom[60], ax, xx, bx, fa, fx, fb, xmin = 0.0;
    for (int j = 0; j < n; ++j) { pcom[j] = p[j]; xicom[j] = xi[j]; }
    c->pcom = pcom;
    c->xicom = xicom;
    ax = 0.;
    xx = 1.;
    mnbrak(c, &ax, &xx, &bx, &fa, &fx, &fb);
    int rc = brent(c, ax, xx, bx, TOL, &xmin, fret);
    for (int j = 0; j < n; ++j) {
        xi[j] = xmin * xi[j];
        p[j] = p[j] + xi[j];
    }
    return rc;
}

int or_frprmn(double *p, int n, double ftol, int *iter, double *fret, int nxsize, int nwloc, int ns,
              const double *omega, const double *dev, int nbath, int norb)
{
    const int itmax = 20000;
    const double eps = 1.e-10;
    double g[60], h[60], xi[60], xt[60], dgg, fp, gam, gg;
    if (n > 60 || nxsize > 60) return 3;
    fit_ctx c = {nxsize, nwloc, ns, nbath, norb, omega, dev, NULL, NULL, xt};
    fp = or_func(p, ns, nwloc, nxsize, omega, dev, nbath, norb);
    or_dfunc(p, xi, nwloc, ns, nxsize, omega, dev, nbath, norb);
    for (int j = 0; j < n; ++j) {
        g[j] = -xi[j];
        h[j] = g[j];
        xi[j] = h[j];
    }
    for (int its = 1; its <= itmax; ++its) {
        *iter = its;
        int rc = linmin(&c, p, xi, n, fret);
        if (rc) return rc;
        if (2. * fabs(*fret - fp) <= ftol * (fabs(*fret) + fabs(fp) + eps)) return 0;
        fp = *fret;
        or_dfunc(p, xi, nwloc, ns, nxsize, omega, dev, nbath, norb);
        gg = 0.;
        dgg = 0.;
        for (int j = 0; j < n; ++j) {
            gg = gg + g[j] * g[j];
            dgg = dgg + (xi[j] + g[j]) * xi[j];
        }
        if (gg == 0.) return 0;
        gam = dgg / gg;
        for (int j = 0; j < n; ++j) {
            g[j] = -xi[j];
            h[j] = g[j] + gam * h[j];
            xi[j] = h[j];
        }
    }
    return 1;
}

/* ------------------------------------------------------------------ */
/* ed_green.F90:260-273                                                 */
/* ------------------------------------------------------------------ */
void or_calc_dev(int norb, int nsite, int nwloc, const double *omega, const double *ek, const double *vk,
                 const double *ef, double *dev)
{
    for (int i = 0; i < nwloc; ++i)
        for (int korb = 1; korb <= norb; ++korb) {
            cplx d = c_make(0.0, 0.0);
            for (int k = norb + 1; k <= nsite; ++k) {
                double v = vk[(size_t)(k - norb - 1) * norb + (korb - 1)];
                d = c_add(d, c_div(c_make(v * v, 0.0), c_sub(fcmplx(0.0, omega[i]), c_make(ek[k - 1], 0.0))));
            }
            d = c_add(d, c_make(ef[korb - 1], 0.0));
            size_t k = (size_t)i * norb + (korb - 1);
            dev[2 * k] = d.re;
            dev[2 * k + 1] = d.im;
        }
}

/* ------------------------------------------------------------------ */
/* DMFT self-consistency and real-frequency spectra                    */
/* ------------------------------------------------------------------ */
/* ed_hamiltonian.F90:29-85: Hk(i,i,ik) = -0.5 (cos kx + cos ky) for every
 * orbital on an nk x nk grid (nk = int(sqrt(Nq)), kx outer), dq = 2 pi /
 * float(nk); ef(i) = sum_k Hk(i,i,k) / float(Nq).  hk[nq] is the diagonal
 * (the same for every orbital).  Returns -1 if nk*nk != nq (the reference
 * stops). */
int or_set_band_structure(int norb, int nq, double *hk, double *ef)
{
    const double pi = 4.0 * atan(1.0);
    const int nk = (int)sqrt((double)nq);
    const double dq = 2.0 * pi / (double)(float)nk;
    int ik = 0;
    for (int i = 1; i <= nk; ++i)
        for (int j = 1; j <= nk; ++j) {
            const double kx = dq * (double)(float)(i - 1), ky = dq * (double)(float)(j - 1);
            hk[ik++] = -0.5 * (cos(kx) + cos(ky));
        }
    if (ik != nq) return -1;
    for (int i = 0; i < norb; ++i) {
        double s = 0.0;
        for (int k = 0; k < nq; ++k) s += hk[k];
        ef[i] = s / (double)(float)nq;
    }
    return 0;
}

/* ed_green.F90:187-214 (H(k) diagonal): per w_n and orbital,
 * Gksum = (1/Nq) sum_q 1 / (1/Gr + D_ev + mu - Hk(q)), then
 * D_ev <- 1/Gr - 1/Gksum + D_ev.  Gr, D_ev, Gksum: complex (norb, nwloc). */
void or_delta_new(int norb, int nwloc, int nq, const double *hk, double rmu, const double *gr, double *dev,
                  double *gksum)
{
    for (int iw = 0; iw < nwloc; ++iw) {
        for (int iorb = 0; iorb < norb; ++iorb) {
            const size_t k = (size_t)iw * norb + iorb;
            const cplx g = c_make(gr[2 * k], gr[2 * k + 1]), d = c_make(dev[2 * k], dev[2 * k + 1]);
            const cplx ginv = c_div(c_make(1.0, 0.0), g);
            cplx acc = c_make(0.0, 0.0);
            for (int jq = 0; jq < nq; ++jq) {
                const cplx tmp = c_sub(c_add(c_add(ginv, d), c_make(rmu, 0.0)), c_make(hk[jq], 0.0));
                acc = c_add(acc, c_div(c_make(1.0, 0.0), tmp));
            }
            acc = c_make(acc.re / (double)(float)nq, acc.im / (double)(float)nq);
            const cplx dn = c_add(c_sub(ginv, c_div(c_make(1.0, 0.0), acc)), d);
            gksum[2 * k] = acc.re;
            gksum[2 * k + 1] = acc.im;
            dev[2 * k] = dn.re;
            dev[2 * k + 1] = dn.im;
        }
    }
}

/* ed_green.F90:227-253: nocc(iorb) = 2 sum_w Re Gksum(iorb, w) / beta + 0.5 */
void or_n_from_gksum(int norb, int nw, const double *gksum, double beta, double *nocc)
{
    for (int iorb = 0; iorb < norb; ++iorb) {
        double s = 0.0;
        for (int iw = 0; iw < nw; ++iw) s += gksum[2 * ((size_t)iw * norb + iorb)];
        nocc[iorb] = 2.0 * s / beta + 0.5;
    }
}

/* dos.f90:1-106 over the records of apbpanbn.dat in file order: record r has
 * orbital iorb[r] (1-based), energy ev[r], nstep_calc np[r] / nn[r] and
 * coefficients ab[r][4][ld] = ap, bp, an, bn.  For each w:
 *   G+ = bp(0)/(z+ - ap(0) - bp(1)/(z+ - ap(1) - ...)), z+ = CMPLX(ev + w, small),
 *   G- = bn(0)/(z- + an(0) - bn(1)/(z- + an(1) - ...)), z- = CMPLX(w - ev, small),
 *   A(iorb, w) = -Im(G+ + G-) / pi.
 * As in dos_diag, A(iorb, :) is assigned, not accumulated, so the last
 * record of each orbital sets it (weighted = 0).  weighted = 1 instead sums
 * prob[r] * factor (1 if even[r], else 0.5) * (-Im(G+ + G-) / pi) over the
 * records.  A run with nstep_calc < 0 (its excitation leaves the Fock
 * space) adds nothing.  aff: real (norb, nw). */
void or_dos(int norb, int nrec, const int *iorb, const double *ev, const double *prob, const int *even,
            const int *np, const int *nn, const double *ab, int ld, int nw, const double *omega_real,
            double small, int weighted, double *aff)
{
    const double pi = 4.0 * atan(1.0);
    for (size_t i = 0; i < (size_t)norb * nw; ++i) aff[i] = 0.0;
    for (int r = 0; r < nrec; ++r) {
        const double *ap = ab + (size_t)(4 * r + 0) * ld, *bp = ab + (size_t)(4 * r + 1) * ld;
        const double *an = ab + (size_t)(4 * r + 2) * ld, *bn = ab + (size_t)(4 * r + 3) * ld;
        for (int iw = 0; iw < nw; ++iw) {
            cplx grx = c_make(0.0, 0.0);
            if (np[r] >= 0) {
                const cplx z = fcmplx(ev[r] + omega_real[iw], small);
                cplx g = c_div(c_make(bp[np[r]], 0.0), c_sub(z, c_make(ap[np[r]], 0.0)));
                for (int is = np[r] - 1; is >= 0; --is)
                    g = c_div(c_make(bp[is], 0.0), c_sub(c_sub(z, c_make(ap[is], 0.0)), g));
                grx = g;
            }
            if (nn[r] >= 0) {
                const cplx z = fcmplx(omega_real[iw] - ev[r], small);
                cplx g = c_div(c_make(bn[nn[r]], 0.0), c_add(z, c_make(an[nn[r]], 0.0)));
                for (int is = nn[r] - 1; is >= 0; --is)
                    g = c_div(c_make(bn[is], 0.0), c_sub(c_add(z, c_make(an[is], 0.0)), g));
                grx = c_add(grx, g);
            }
            const double a = -grx.im / pi;
            double *out = aff + (size_t)iw * norb + (iorb[r] - 1);
            if (weighted) *out += prob[r] * (even[r] ? 1.0 : 0.5) * a;
            else *out = a;
        }
    }
}
