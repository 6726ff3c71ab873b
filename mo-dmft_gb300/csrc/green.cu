// green.cu -- excitations, ed_solve and the continued-fraction Green's function.
//
//  apply_c        ed_operators.F90:10-61  (one thread per target element)
//  ed_solve       ed_solver.F90:28-105    (sectors -> eigenpairs, heapsort,
//                                          Boltzmann weights, nev_calc)
//  ed_calc_green  ed_green.F90:60-185     (all c+psi / c psi starts of all
//                                          kept states advance together in
//                                          the batched reference recurrence;
//                                          G(i w_n) from one CF kernel)
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>

#include "krylov.cuh"

namespace moed {

// ---------------------------------------------------------------------------
// apply_c
// ---------------------------------------------------------------------------
// Row i of the target sector: apply the opposite operator to its state
// (destruction for pm = 1, creation for pm = 2) and gather the source
// element with the operator's sign; zero where the operator annihilates the
// state (ed_operators.F90:44-58).
template <typename T>
__global__ void k_apply_c_up(const T *__restrict__ x, T *__restrict__ y, int nu_out, int ld_out, int nd,
                             int ld_in, const int *__restrict__ out_words, const int *__restrict__ in_rank,
                             int bit, int pm)
{
    const long long n = (long long)ld_out * nd;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int u = (int)(i % ld_out);
        const long long d = i / ld_out;
        T v = T(0);
        if (u < nu_out) {
            const unsigned w = (unsigned)out_words[u];
            const bool occ = (w >> bit) & 1u;
            if ((pm == 1) == occ) {
                const int sgn = __popc(w & ((1u << bit) - 1u)) & 1;
                const int j = in_rank[w ^ (1u << bit)];
                const T src = x[d * ld_in + j];
                v = sgn ? -src : src;
            }
        }
        y[i] = v;
    }
}

// spin down: the sign also counts every up-spin bit (bitidx = nsite + iorb - 1),
// i.e. a factor (-1)^(N_up) on top of the down-word parity.
template <typename T>
__global__ void k_apply_c_dn(const T *__restrict__ x, T *__restrict__ y, int nu, int ld, int nd_out,
                             const int *__restrict__ out_words, const int *__restrict__ in_rank,
                             int bit, int pm, int up_parity)
{
    const long long n = (long long)ld * nd_out;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int u = (int)(i % ld);
        const int d = (int)(i / ld);
        const unsigned w = (unsigned)out_words[d];
        const bool occ = (w >> bit) & 1u;
        T v = T(0);
        if (u < nu && (pm == 1) == occ) {
            const int sgn = (__popc(w & ((1u << bit) - 1u)) + up_parity) & 1;
            const int j = in_rank[w ^ (1u << bit)];
            const T src = x[(long long)j * ld + u];
            v = sgn ? -src : src;
        }
        y[i] = v;
    }
}

int apply_c_dev(mo_ed_ctx *ctx, const Sector &in, const Sector &out, int prec, const void *x, void *y,
                int pm, int iorb, int ispin)
{
    const long long n = out.Dpad();
    if (n <= 0) return MO_ED_OK;
    const int T = 256;
    const int g = (int)std::max(1LL, std::min((n + T - 1) / T, (long long)ctx->num_sms * 8));
    const int bit = iorb - 1;
    if (ispin == 1) {
        if (prec == MO_ED_FP32)
            k_apply_c_up<float><<<g, T, 0, ctx->stream>>>((const float *)x, (float *)y, out.up->n, out.ld(),
                                                         out.dn->n, in.ld(), out.up->words, in.up->rank, bit, pm);
        else
            k_apply_c_up<double><<<g, T, 0, ctx->stream>>>((const double *)x, (double *)y, out.up->n, out.ld(),
                                                          out.dn->n, in.ld(), out.up->words, in.up->rank, bit, pm);
    } else {
        const int upar = out.ne_up & 1;
        if (prec == MO_ED_FP32)
            k_apply_c_dn<float><<<g, T, 0, ctx->stream>>>((const float *)x, (float *)y, out.up->n, out.ld(),
                                                         out.dn->n, out.dn->words, in.dn->rank, bit, pm, upar);
        else
            k_apply_c_dn<double><<<g, T, 0, ctx->stream>>>((const double *)x, (double *)y, out.up->n, out.ld(),
                                                          out.dn->n, out.dn->words, in.dn->rank, bit, pm, upar);
    }
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

// ---------------------------------------------------------------------------
// host restatements used by ed_solve: heapsort (func.f90:301-353) and
// boltzmann_factor (ed_solver.F90:193-219) -- O(nev*nsector) scalar work
// ---------------------------------------------------------------------------
static void heapsort_index(int n, const double *arrin, int *indx)
{
    const double *A = arrin - 1;
    int *X = indx - 1;
    if (n == 1) {
        X[1] = 1;
        return;
    }
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
            if (ir == 1) {
                X[1] = indxt;
                return;
            }
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

static void boltzmann(const double *elv, int nev, double beta, double *p)
{
    for (int i = 0; i < nev; ++i) {
        double Z = 0.0, en = elv[i];
        bool zero = false;
        for (int k = 0; k < nev; ++k) {
            if (-beta * (elv[k] - en) > 10.0) {
                zero = true;
                break;
            }
            Z = Z + std::exp(-beta * (elv[k] - en));
        }
        p[i] = zero ? 0.0 : 1.0 / Z;
    }
}

// ---------------------------------------------------------------------------
// continued fraction (ed_green.F90:160-168, 176-184)
// ---------------------------------------------------------------------------
struct CfRec {
    int iorb;        // 0-based
    int np, nn;      // nstep_calc of the particle / hole runs (-1: no run)
    double E, weight;  // eigenvalue, pev*factor
};

__device__ __forceinline__ double2 cdiv(double2 a, double2 b)   // Smith (1962)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, den = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    }
    const double r = b.x / b.y, den = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

// One thread per (iorb, iw); records accumulated in the reference's order.
__global__ void k_green_cf(const CfRec *__restrict__ rec, int nrec, const double *__restrict__ ab,
                           int ld, const double *__restrict__ omega, int nw, int norb,
                           int fcmplx, double *__restrict__ Gr)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nw * norb) return;
    const int iw = t / norb, iorb = t - iw * norb;
    const double w = fcmplx ? (double)(float)omega[iw] : omega[iw];
    double gre = 0.0, gim = 0.0;
    for (int r = 0; r < nrec; ++r) {
        const CfRec R = rec[r];
        if (R.iorb != iorb) continue;
        const double *ap = ab + (size_t)r * 4 * ld, *bp = ap + ld, *an = bp + ld, *bn = an + ld;
        if (R.np >= 0) {
            const double er = fcmplx ? (double)(float)R.E : R.E;
            double2 z = make_double2(er, w);
            double2 g = cdiv(make_double2(bp[R.np], 0.0), make_double2(z.x - ap[R.np], z.y));
            for (int j = R.np - 1; j >= 0; --j)
                g = cdiv(make_double2(bp[j], 0.0), make_double2(z.x - ap[j] - g.x, z.y - g.y));
            gre += R.weight * g.x;
            gim += R.weight * g.y;
        }
        if (R.nn >= 0) {
            const double er = fcmplx ? (double)(float)(-R.E) : -R.E;
            double2 z = make_double2(er, w);
            double2 g = cdiv(make_double2(bn[R.nn], 0.0), make_double2(z.x + an[R.nn], z.y));
            for (int j = R.nn - 1; j >= 0; --j)
                g = cdiv(make_double2(bn[j], 0.0), make_double2(z.x + an[j] - g.x, z.y - g.y));
            gre += R.weight * g.x;
            gim += R.weight * g.y;
        }
    }
    Gr[2 * ((size_t)iw * norb + iorb)] = gre;
    Gr[2 * ((size_t)iw * norb + iorb) + 1] = gim;
}

// ---------------------------------------------------------------------------
// real-frequency spectral function (dos.f90:1-106)
// ---------------------------------------------------------------------------
// One thread per (iorb, w).  z+ = CMPLX(E + w, small), z- = CMPLX(w - E,
// small) (default-REAL rounding with fcmplx), A = -Im(G+ + G-) / pi.  As
// dos_diag assigns A(iorb, :) for every record, the last record of each
// orbital sets it (weighted = 0); weighted = 1 sums pev * factor * A over the
// records instead.  Runs that leave the Fock space (np / nn < 0) add nothing.
__global__ void k_dos(const CfRec *__restrict__ rec, int nrec, const double *__restrict__ ab, int ld,
                      const double *__restrict__ omega, int nw, int norb, double small, int fcmplx, int weighted,
                      double *__restrict__ aff)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nw * norb) return;
    const int iw = t / norb, iorb = t - iw * norb;
    const double pi = 3.14159265358979323846;
    const double w = omega[iw];
    const double sm = fcmplx ? (double)(float)small : small;
    double out = 0.0;
    for (int r = weighted ? 0 : nrec - 1; weighted ? r < nrec : r >= 0; r += weighted ? 1 : -1) {
        const CfRec R = rec[r];
        if (R.iorb != iorb) continue;
        const double *ap = ab + (size_t)r * 4 * ld, *bp = ap + ld, *an = bp + ld, *bn = an + ld;
        double gim = 0.0;
        if (R.np >= 0) {
            const double zr = fcmplx ? (double)(float)(R.E + w) : R.E + w;
            double2 g = cdiv(make_double2(bp[R.np], 0.0), make_double2(zr - ap[R.np], sm));
            for (int j = R.np - 1; j >= 0; --j)
                g = cdiv(make_double2(bp[j], 0.0), make_double2(zr - ap[j] - g.x, sm - g.y));
            gim += g.y;
        }
        if (R.nn >= 0) {
            const double zr = fcmplx ? (double)(float)(w - R.E) : w - R.E;
            double2 g = cdiv(make_double2(bn[R.nn], 0.0), make_double2(zr + an[R.nn], sm));
            for (int j = R.nn - 1; j >= 0; --j)
                g = cdiv(make_double2(bn[j], 0.0), make_double2(zr + an[j] - g.x, sm - g.y));
            gim += g.y;
        }
        const double a = -gim / pi;
        if (!weighted) {
            out = a;
            break;
        }
        out += R.weight * a;
    }
    aff[(size_t)iw * norb + iorb] = out;
}

// ---------------------------------------------------------------------------
// DMFT self-consistency (ed_hamiltonian.F90:29-85, ed_green.F90:187-253)
// ---------------------------------------------------------------------------
// Square-lattice band: Hk(i,i,ik) = -0.5 (cos kx + cos ky), the same for every
// orbital, kx = dq * (i-1) outer, ky = dq * (j-1) inner.
__global__ void k_band(int nk, double dq, double *hk)
{
    const int ik = blockIdx.x * blockDim.x + threadIdx.x;
    if (ik >= nk * nk) return;
    const int i = ik / nk, j = ik - i * nk;
    hk[ik] = -0.5 * (cos(dq * (double)(float)i) + cos(dq * (double)(float)j));
}

// ef = sum_k Hk / float(Nq), summed in k order (one thread, Nq terms)
__global__ void k_band_mean(const double *hk, int nq, double *ef)
{
    double s = 0.0;
    for (int k = 0; k < nq; ++k) s += hk[k];
    ef[0] = s / (double)(float)nq;
}

// ed_delta_new: one warp per (iorb, w_n).  Its lanes sum 1 / ((1/Gr + D_ev +
// mu) - Hk(q)) over strided q, a xor butterfly adds the lanes (every lane
// ends with the same sum, in a fixed order), then Gksum = sum / float(Nq) and
// D_ev <- 1/Gr - 1/Gksum + D_ev.  Complex divisions by Smith's algorithm.
__global__ void k_delta_new(const double *__restrict__ hk, int nq, double rmu, const double *__restrict__ gr,
                            double *__restrict__ dev, double *__restrict__ gksum, int n)
{
    const int wid = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (wid >= n) return;
    const double2 g = make_double2(gr[2 * wid], gr[2 * wid + 1]);
    const double2 d = make_double2(dev[2 * wid], dev[2 * wid + 1]);
    const double2 gi = cdiv(make_double2(1.0, 0.0), g);
    const double br = gi.x + d.x + rmu, bi = gi.y + d.y;
    double sre = 0.0, sim = 0.0;
    for (int q = lane; q < nq; q += 32) {
        const double2 r = cdiv(make_double2(1.0, 0.0), make_double2(br - __ldg(hk + q), bi));
        sre += r.x;
        sim += r.y;
    }
    for (int off = 16; off > 0; off >>= 1) {
        sre += __shfl_xor_sync(0xffffffffu, sre, off);
        sim += __shfl_xor_sync(0xffffffffu, sim, off);
    }
    if (lane == 0) {
        const double fq = (double)(float)nq;
        const double2 gk = make_double2(sre / fq, sim / fq);
        const double2 gki = cdiv(make_double2(1.0, 0.0), gk);
        gksum[2 * wid] = gk.x;
        gksum[2 * wid + 1] = gk.y;
        dev[2 * wid] = gi.x - gki.x + d.x;
        dev[2 * wid + 1] = gi.y - gki.y + d.y;
    }
}

// n_from_gksum: one CTA per orbital, nocc = 2 sum_w Re Gksum / beta + 0.5
__global__ void k_nocc(const double *__restrict__ gksum, int nw, int norb, double beta, double *__restrict__ nocc)
{
    __shared__ double red[256];
    const int iorb = blockIdx.x;
    double s = 0.0;
    for (int iw = threadIdx.x; iw < nw; iw += blockDim.x) s += gksum[2 * ((size_t)iw * norb + iorb)];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) nocc[iorb] = 2.0 * red[0] / beta + 0.5;
}

// ---------------------------------------------------------------------------
// ed_calc_green_ftn
// ---------------------------------------------------------------------------
int calc_green(mo_ed_ctx *ctx, double *Gr)
{
    if (ctx->states.empty()) return fail(ctx, MO_ED_ERR_STATE, "mo_ed_solve has not been run");
    if (ctx->omega.empty()) return fail(ctx, MO_ED_ERR_STATE, "omega grid not set");
    // The recurrence runs in the eigenvectors' precision, or in FP64 with
    // green_fp64 (FP32 eigenvectors are widened before c / c^dagger).
    const int sprec = ctx->states[0].prec;
    const int prec = ctx->opt.green_fp64 ? MO_ED_FP64 : sprec;
    const int nstep = ctx->opt.nstep;
    const int norb = ctx->norb;

    // excitation list in the reference's record order
    struct Exc {
        int iev, ispin, iorb, pm;
        Sector in, out;
        bool ok;
    };
    std::vector<Exc> exc;
    std::vector<GreenRecord> recs;
    for (size_t iev = 0; iev < ctx->states.size(); ++iev) {
        const StateVec &st = ctx->states[iev];
        const int nu = ctx->nup[st.sector], nd = ctx->nelec[st.sector] - nu;
        const bool even = nd == nu;
        Sector in;
        if (int rc = get_sector(ctx, nu, nd, &in)) return rc;
        for (int ispin = 1; ispin <= (even ? 1 : 2); ++ispin)
            for (int iorb = 1; iorb <= norb; ++iorb) {
                GreenRecord g;
                g.iev = (int)iev + 1;
                g.iorb = iorb;
                g.even = even;
                g.val = st.val;
                g.prob = st.prob;
                g.np = g.nn = 0;
                recs.push_back(g);
                for (int pm = 1; pm <= 2; ++pm) {
                    Exc e;
                    e.iev = (int)iev;
                    e.ispin = ispin;
                    e.iorb = iorb;
                    e.pm = pm;
                    e.in = in;
                    const int d = pm == 1 ? 1 : -1;
                    const int tu = nu + (ispin == 1 ? d : 0), td = nd + (ispin == 2 ? d : 0);
                    e.ok = tu >= 0 && tu <= ctx->nsite && td >= 0 && td <= ctx->nsite;
                    if (e.ok)
                        if (int rc = get_sector(ctx, tu, td, &e.out)) return rc;
                    exc.push_back(e);
                }
            }
    }
    // batched reference Lanczos over all valid excitations
    std::vector<double> normsq(exc.size(), 0.0);
    std::vector<int> nsc(exc.size(), -1);
    std::vector<std::vector<double>> A(exc.size()), B(exc.size());
    std::vector<int> valid;
    for (size_t i = 0; i < exc.size(); ++i)
        if (exc[i].ok) valid.push_back((int)i);
    // green_fp64 over FP32 states: each kept eigenvector refined in FP64 once
    std::vector<DevBuf> wide(ctx->states.size());
    ctx->refine_res = 0.0;
    if (sprec != prec) {
        if (prec != MO_ED_FP64) return fail(ctx, MO_ED_ERR_STATE, "eigenvector precision mismatch");
        for (size_t iev = 0; iev < ctx->states.size(); ++iev) {
            const StateVec &st = ctx->states[iev];
            const int nu = ctx->nup[st.sector], nd = ctx->nelec[st.sector] - nu;
            Sector in;
            if (int rc = get_sector(ctx, nu, nd, &in)) return rc;
            double res = 0.0;
            if (int rc = refine_fp64(ctx, in, (const float *)st.vec.p, wide[iev], &res)) return rc;
            ctx->refine_res = std::max(ctx->refine_res, res);
        }
    }
    for (size_t b0 = 0; b0 < valid.size(); b0 += kLzMaxRuns) {
        const size_t b1 = std::min(valid.size(), b0 + kLzMaxRuns);
        std::vector<Sector> secs;
        for (size_t k = b0; k < b1; ++k) secs.push_back(exc[valid[k]].out);
        LzBatch lb;
        if (int rc = lz_setup(ctx, lb, secs, prec, nstep)) return rc;
        for (size_t k = b0; k < b1; ++k) {
            const Exc &e = exc[valid[k]];
            const StateVec &st = ctx->states[e.iev];
            const void *x = st.prec == prec ? st.vec.p : wide[e.iev].p;
            if (int rc = apply_c_dev(ctx, e.in, e.out, prec, x, lz_start_vector(lb, (int)(k - b0)),
                                     e.pm, e.iorb, e.ispin))
                return rc;
        }
        std::vector<std::vector<double>> a, bb;
        std::vector<int> nc;
        if (int rc = lz_run(ctx, lb, a, bb, nc)) return rc;
        // normsq = ||start||^2 (ed_green.F90:157): nrm[0] of each run
        std::vector<double> coef(lb.coef.bytes / sizeof(double));
        MOED_CUDA(ctx, cudaMemcpyAsync(coef.data(), lb.coef.p, lb.coef.bytes, cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t k = b0; k < b1; ++k) {
            const int r = (int)(k - b0), i = valid[k];
            normsq[i] = coef[(size_t)2 * (nstep + 1) * r + (nstep + 1)];
            nsc[i] = nc[r];
            A[i] = a[r];
            B[i] = bb[r];
        }
    }
    // records: ap, bp(0) = normsq, an, bn(0) = 1 - normsq (ed_green.F90:158,174)
    const int ld = nstep + 1;
    std::vector<double> ab(recs.size() * 4 * (size_t)ld, 0.0);
    std::vector<CfRec> cf(recs.size());
    for (size_t r = 0; r < recs.size(); ++r) {
        const Exc &ep = exc[2 * r], &en = exc[2 * r + 1];
        GreenRecord &g = recs[r];
        const double nsq = normsq[2 * r];
        g.ap.assign(ld, 0.0);
        g.bp.assign(ld, 0.0);
        g.an.assign(ld, 0.0);
        g.bn.assign(ld, 0.0);
        if (ep.ok) {
            g.ap = A[2 * r];
            g.bp = B[2 * r];
        }
        if (en.ok) {
            g.an = A[2 * r + 1];
            g.bn = B[2 * r + 1];
        }
        g.bp[0] = nsq;
        g.bn[0] = 1.0 - nsq;
        g.np = ep.ok ? nsc[2 * r] : -1;
        g.nn = en.ok ? nsc[2 * r + 1] : -1;
        const StateVec &st = ctx->states[ep.iev];
        const int nu = ctx->nup[st.sector], nd = ctx->nelec[st.sector] - nu;
        cf[r].iorb = g.iorb - 1;
        cf[r].np = g.np;
        cf[r].nn = g.nn;
        cf[r].E = st.val;
        cf[r].weight = st.prob * (nd == nu ? 1.0 : 0.5);
        std::copy(g.ap.begin(), g.ap.end(), ab.begin() + (r * 4 + 0) * ld);
        std::copy(g.bp.begin(), g.bp.end(), ab.begin() + (r * 4 + 1) * ld);
        std::copy(g.an.begin(), g.an.end(), ab.begin() + (r * 4 + 2) * ld);
        std::copy(g.bn.begin(), g.bn.end(), ab.begin() + (r * 4 + 3) * ld);
    }
    ctx->green = recs;
    const int nw = (int)ctx->omega.size();
    DevBuf drec, dab, dom, dG;
    if (int rc = dev_alloc(ctx, drec, sizeof(CfRec) * std::max<size_t>(1, cf.size()))) return rc;
    if (int rc = dev_alloc(ctx, dab, sizeof(double) * std::max<size_t>(1, ab.size()))) return rc;
    if (int rc = dev_alloc(ctx, dom, sizeof(double) * nw)) return rc;
    if (int rc = dev_alloc(ctx, dG, sizeof(double) * 2 * (size_t)nw * norb)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(drec.p, cf.data(), sizeof(CfRec) * cf.size(), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dab.p, ab.data(), sizeof(double) * ab.size(), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dom.p, ctx->omega.data(), sizeof(double) * nw, cudaMemcpyHostToDevice, ctx->stream));
    const int T = 128;
    k_green_cf<<<(nw * norb + T - 1) / T, T, 0, ctx->stream>>>((const CfRec *)drec.p, (int)cf.size(),
                                                              (const double *)dab.p, ld, (const double *)dom.p,
                                                              nw, norb, ctx->opt.fortran_cmplx, (double *)dG.p);
    MOED_CHECK_LAUNCH(ctx);
    MOED_CUDA(ctx, cudaMemcpyAsync(Gr, dG.p, sizeof(double) * 2 * (size_t)nw * norb, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

}  // namespace moed

using namespace moed;

namespace moed {

// The eigensolves of ed_solve's sector list (ed_solver.F90:44-60): eig_all
// [nsector][nev] and the eigenvectors of each sector.  Sectors are
// independent, and a small sector's thick-restart Lanczos is a chain of
// short dependent launches, so lists of many small sectors are spread over
// host threads, each driving worker contexts of its own (same device, model
// and options; own stream and workspace) so that the chains overlap on the
// GPU.  Each sector's eigensolve is the same computation in either case.
static int solve_sectors(mo_ed_ctx *ctx, int nev, std::vector<double> &eig_all,
                         std::vector<std::vector<DevBuf>> &vecs)
{
    const int nsector = (int)ctx->nelec.size();
    int nthreads = ctx->opt.solve_threads;
    if (nthreads == 0) {
        bool small = nsector >= 8;
        for (int is = 0; is < nsector && small; ++is) {
            const int nu = ctx->nup[is], nd = ctx->nelec[is] - nu;
            small = nu >= 0 && nd >= 0 && nu <= ctx->nsite && nd <= ctx->nsite &&
                    binom(ctx->nsite, nu) * binom(ctx->nsite, nd) < (1LL << 18);
        }
        nthreads = small ? 4 : 1;
    }
    nthreads = std::min(nthreads, nsector);
    if (nthreads <= 1) {
        for (int is = 0; is < nsector; ++is) {
            Sector s;
            if (int rc = get_sector(ctx, ctx->nup[is], ctx->nelec[is] - ctx->nup[is], &s)) return rc;
            std::vector<double> v;
            if (int rc = diag_sector(ctx, s, nev, v, &vecs[is])) return rc;
            for (int i = 0; i < nev; ++i) eig_all[(size_t)is * nev + i] = v[i];
        }
        return MO_ED_OK;
    }
    // worker contexts, kept for the context's lifetime; each takes the
    // current model when it holds an older one
    while ((int)ctx->workers.size() < nthreads) {
        mo_ed_ctx *w = nullptr;
        if (int rc = mo_ed_create(&w, ctx->device, nullptr)) return fail(ctx, rc, "worker context");
        ctx->workers.push_back(w);
        ctx->worker_gen.push_back(-1);
    }
    for (int t = 0; t < nthreads; ++t) {
        if (ctx->worker_gen[t] == ctx->model_gen) continue;
        mo_ed_ctx *w = ctx->workers[t];
        if (int rc = mo_ed_set_model(w, ctx->norb, ctx->nbath, ctx->U, ctx->J, ctx->ek.data(), ctx->vk.data()))
            return fail(ctx, rc, std::string("worker context: ") + w->err);
        ctx->worker_gen[t] = ctx->model_gen;
    }
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::atomic<int> next{0}, failed{0};
    std::vector<int> rcs(nthreads, MO_ED_OK);
    std::vector<long long> l0(nthreads);
    std::vector<int> who(nsector, 0);
    auto work = [&](int t) {
        mo_ed_ctx *w = ctx->workers[t];
        cudaSetDevice(w->device);
        w->opt = ctx->opt;
        for (;;) {
            const int is = next.fetch_add(1);
            if (is >= nsector || failed.load()) break;
            Sector s;
            int rc = get_sector(w, ctx->nup[is], ctx->nelec[is] - ctx->nup[is], &s);
            std::vector<double> v;
            if (!rc) rc = diag_sector(w, s, nev, v, &vecs[is]);
            if (rc) {
                rcs[t] = rc;
                failed.store(1);
                break;
            }
            for (int i = 0; i < nev; ++i) eig_all[(size_t)is * nev + i] = v[i];
            who[is] = t;
        }
        cudaStreamSynchronize(w->stream);
    };
    for (int t = 0; t < nthreads; ++t) l0[t] = ctx->workers[t]->launches;
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    cudaSetDevice(ctx->device);
    for (int t = 0; t < nthreads; ++t) {
        mo_ed_ctx *w = ctx->workers[t];
        ctx->launches += w->launches - l0[t];
        if (rcs[t]) return fail(ctx, rcs[t], w->err);
    }
    // statistics of the last sector, as in one thread
    const mo_ed_ctx *last = ctx->workers[who[nsector - 1]];
    ctx->diag_cycles = last->diag_cycles;
    ctx->diag_matvecs = last->diag_matvecs;
    ctx->diag_res_est = last->diag_res_est;
    ctx->diag_res_true = last->diag_res_true;
    return MO_ED_OK;
}

}  // namespace moed

extern "C" {

int mo_ed_diag(mo_ed_ctx *ctx, int ne_up, int ne_down, int nev, double *eigval, double *eigvec)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (nev < 1 || !eigval) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    std::vector<double> vals;
    std::vector<DevBuf> vecs;
    if (int rc = diag_sector(ctx, s, nev, vals, eigvec ? &vecs : nullptr)) return rc;
    for (int i = 0; i < nev; ++i) eigval[i] = vals[i];
    if (eigvec) {
        const long long D = s.D(), Dp = s.Dpad();
        DevBuf tmp;
        if (ctx->opt.precision == MO_ED_FP32)
            if (int rc = dev_alloc(ctx, tmp, sizeof(double) * Dp)) return rc;
        for (int i = 0; i < nev; ++i) {
            double *dst = eigvec + (size_t)i * D;
            if (i >= (int)vecs.size()) {
                memset(dst, 0, sizeof(double) * D);
                continue;
            }
            const void *src = vecs[i].p;
            if (ctx->opt.precision == MO_ED_FP32) {
                if (int rc = convert_f32_to_f64(ctx, (const float *)vecs[i].p, (double *)tmp.p, Dp)) return rc;
                src = tmp.p;
            }
            if (int rc = download_padded(ctx, s, src, dst, sizeof(double))) return rc;
            MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        }
    }
    return MO_ED_OK;
}

int mo_ed_set_band_structure(mo_ed_ctx *ctx, int nq, double *ef)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    if (nq < 1 || !ef) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    const int nk = (int)std::sqrt((double)nq);
    if (nk * nk != nq) return fail(ctx, MO_ED_ERR_ARG, "Nq is not a square (ed_hamiltonian.F90:50 stops)");
    if (int rc = dev_alloc(ctx, ctx->d_hk, sizeof(double) * ((size_t)nq + 1))) return rc;
    ctx->nq = nq;
    const double pi = 4.0 * std::atan(1.0);
    const double dq = 2.0 * pi / (double)(float)nk;
    double *hk = (double *)ctx->d_hk.p;
    k_band<<<(nq + 255) / 256, 256, 0, ctx->stream>>>(nk, dq, hk);
    MOED_CHECK_LAUNCH(ctx);
    k_band_mean<<<1, 1, 0, ctx->stream>>>(hk, nq, hk + nq);
    MOED_CHECK_LAUNCH(ctx);
    double m = 0.0;
    MOED_CUDA(ctx, cudaMemcpyAsync(&m, hk + nq, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < ctx->norb; ++i) ef[i] = m;
    return MO_ED_OK;
}

int mo_ed_delta_new(mo_ed_ctx *ctx, int nwloc, double rmu, const double *Gr, double *D_ev, double *Gksum)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->have_model || !ctx->d_hk.p) return fail(ctx, MO_ED_ERR_STATE, "model or band structure not set");
    if (nwloc < 1 || !Gr || !D_ev) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    const int n = ctx->norb * nwloc;
    const size_t b = sizeof(double) * 2 * (size_t)n;
    DevBuf dg, dd, dk;
    if (int rc = dev_alloc(ctx, dg, b)) return rc;
    if (int rc = dev_alloc(ctx, dd, b)) return rc;
    if (int rc = dev_alloc(ctx, dk, b)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(dg.p, Gr, b, cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dd.p, D_ev, b, cudaMemcpyHostToDevice, ctx->stream));
    const int T = 256;
    k_delta_new<<<(unsigned)(((long long)n * 32 + T - 1) / T), T, 0, ctx->stream>>>(
        (const double *)ctx->d_hk.p, ctx->nq, rmu, (const double *)dg.p, (double *)dd.p, (double *)dk.p, n);
    MOED_CHECK_LAUNCH(ctx);
    MOED_CUDA(ctx, cudaMemcpyAsync(D_ev, dd.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    if (Gksum) MOED_CUDA(ctx, cudaMemcpyAsync(Gksum, dk.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int mo_ed_n_from_gksum(mo_ed_ctx *ctx, int nw, const double *Gksum, double beta, double *nocc)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    if (nw < 1 || !Gksum || !nocc || !(beta > 0)) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    const size_t b = sizeof(double) * 2 * (size_t)nw * ctx->norb;
    DevBuf dk, dn;
    if (int rc = dev_alloc(ctx, dk, b)) return rc;
    if (int rc = dev_alloc(ctx, dn, sizeof(double) * ctx->norb)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(dk.p, Gksum, b, cudaMemcpyHostToDevice, ctx->stream));
    k_nocc<<<ctx->norb, 256, 0, ctx->stream>>>((const double *)dk.p, nw, ctx->norb, beta, (double *)dn.p);
    MOED_CHECK_LAUNCH(ctx);
    MOED_CUDA(ctx, cudaMemcpyAsync(nocc, dn.p, sizeof(double) * ctx->norb, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int mo_ed_dos(mo_ed_ctx *ctx, int nw, const double *omega_real, double small, int weighted, double *Aff)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->green.empty()) return fail(ctx, MO_ED_ERR_STATE, "mo_ed_calc_green_ftn has not been run");
    if (nw < 1 || !omega_real || !Aff || (weighted != 0 && weighted != 1))
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    const int norb = ctx->norb, ld = ctx->opt.nstep + 1;
    const size_t nrec = ctx->green.size();
    std::vector<CfRec> cf(nrec);
    std::vector<double> ab(nrec * 4 * (size_t)ld, 0.0);
    for (size_t r = 0; r < nrec; ++r) {
        const GreenRecord &g = ctx->green[r];
        cf[r].iorb = g.iorb - 1;
        cf[r].np = g.np;
        cf[r].nn = g.nn;
        cf[r].E = g.val;
        cf[r].weight = g.prob * (g.even ? 1.0 : 0.5);
        const std::vector<double> *src[4] = {&g.ap, &g.bp, &g.an, &g.bn};
        for (int k = 0; k < 4; ++k)
            std::copy(src[k]->begin(), src[k]->begin() + std::min<size_t>(ld, src[k]->size()),
                      ab.begin() + (r * 4 + k) * ld);
    }
    DevBuf drec, dab, dom, da;
    if (int rc = dev_alloc(ctx, drec, sizeof(CfRec) * nrec)) return rc;
    if (int rc = dev_alloc(ctx, dab, sizeof(double) * ab.size())) return rc;
    if (int rc = dev_alloc(ctx, dom, sizeof(double) * nw)) return rc;
    if (int rc = dev_alloc(ctx, da, sizeof(double) * (size_t)nw * norb)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(drec.p, cf.data(), sizeof(CfRec) * nrec, cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dab.p, ab.data(), sizeof(double) * ab.size(), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dom.p, omega_real, sizeof(double) * nw, cudaMemcpyHostToDevice, ctx->stream));
    const int T = 128;
    k_dos<<<(nw * norb + T - 1) / T, T, 0, ctx->stream>>>((const CfRec *)drec.p, (int)nrec, (const double *)dab.p,
                                                          ld, (const double *)dom.p, nw, norb, small,
                                                          ctx->opt.fortran_cmplx, weighted, (double *)da.p);
    MOED_CHECK_LAUNCH(ctx);
    MOED_CUDA(ctx, cudaMemcpyAsync(Aff, da.p, sizeof(double) * (size_t)nw * norb, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int mo_ed_green_stats(mo_ed_ctx *ctx, double *refine_res)
{
    if (!ctx) return MO_ED_ERR_ARG;
    if (refine_res) *refine_res = ctx->refine_res;
    return MO_ED_OK;
}

int mo_ed_diag_stats(mo_ed_ctx *ctx, int *cycles, long long *matvecs, double *res_est, double *res_true)
{
    if (!ctx) return MO_ED_ERR_ARG;
    if (cycles) *cycles = ctx->diag_cycles;
    if (matvecs) *matvecs = ctx->diag_matvecs;
    if (res_est) *res_est = ctx->diag_res_est;
    if (res_true) *res_true = ctx->diag_res_true;
    return MO_ED_OK;
}

int mo_ed_solve(mo_ed_ctx *ctx, int *nev_calc, double *val, double *prob, int *sector, int *level,
                int capacity)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!nev_calc) return fail(ctx, MO_ED_ERR_ARG, "null nev_calc");
    if (ctx->nelec.empty()) return fail(ctx, MO_ED_ERR_STATE, "sectors not set");
    const int nsector = (int)ctx->nelec.size(), nev = ctx->opt.nev;
    std::vector<double> eig_all((size_t)nev * nsector, DBL_MAX);
    std::vector<std::vector<DevBuf>> vecs(nsector);
    ctx->states.clear();
    if (int rc = solve_sectors(ctx, nev, eig_all, vecs)) return rc;
    const int ntot = nev * nsector;
    std::vector<int> ind(ntot);
    std::vector<double> pev(ntot);
    heapsort_index(ntot, eig_all.data(), ind.data());
    boltzmann(eig_all.data(), ntot, ctx->opt.beta, pev.data());
    int nc = 0;
    for (int i = 0; i < nev && i < ntot; ++i)
        if (pev[ind[i] - 1] > 0.001) ++nc;   // PROB_THRESHOLD (ed_solver.F90:14)
    double Z = 0.0;
    for (int i = 0; i < nc; ++i) Z += pev[ind[i] - 1];
    *nev_calc = nc;
    for (int i = 0; i < nc; ++i) {
        const int k = ind[i] - 1;
        StateVec st;
        st.sector = k / nev;
        st.level = k % nev;
        st.val = eig_all[k];
        st.prob = pev[k] / Z;
        st.pev = pev[k];
        st.prec = ctx->opt.precision;
        if (st.level < (int)vecs[st.sector].size()) std::swap(st.vec, vecs[st.sector][st.level]);
        ctx->states.push_back(std::move(st));
        // std::move of DevBuf: ensure ownership transferred
    }
    if (nc > capacity) return fail(ctx, MO_ED_ERR_CAPACITY, "output capacity below nev_calc");
    for (int i = 0; i < nc; ++i) {
        if (val) val[i] = ctx->states[i].val;
        if (prob) prob[i] = ctx->states[i].prob;
        if (sector) sector[i] = ctx->states[i].sector + 1;
        if (level) level[i] = ctx->states[i].level + 1;
    }
    return MO_ED_OK;
}

int mo_ed_calc_green_ftn(mo_ed_ctx *ctx, double *Gr)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!Gr) return fail(ctx, MO_ED_ERR_ARG, "null Gr");
    return calc_green(ctx, Gr);
}

int mo_ed_green_coeffs(mo_ed_ctx *ctx, int *nrec, int *nstep_calc, double *ab, int capacity)
{
    if (!ctx || !nrec) return MO_ED_ERR_ARG;
    const int n = (int)ctx->green.size();
    *nrec = n;
    if (!nstep_calc && !ab) return MO_ED_OK;
    if (capacity < n) return fail(ctx, MO_ED_ERR_CAPACITY, "capacity below record count");
    const int ld = ctx->opt.nstep + 1;
    for (int r = 0; r < n; ++r) {
        const GreenRecord &g = ctx->green[r];
        if (nstep_calc) {
            nstep_calc[2 * r] = g.np;
            nstep_calc[2 * r + 1] = g.nn;
        }
        if (ab) {
            double *o = ab + (size_t)r * 4 * ld;
            for (int j = 0; j < ld; ++j) {
                o[j] = j < (int)g.ap.size() ? g.ap[j] : 0.0;
                o[ld + j] = j < (int)g.bp.size() ? g.bp[j] : 0.0;
                o[2 * ld + j] = j < (int)g.an.size() ? g.an[j] : 0.0;
                o[3 * ld + j] = j < (int)g.bn.size() ? g.bn[j] : 0.0;
            }
        }
    }
    return MO_ED_OK;
}

}  // extern "C"
