// fit.cu -- chi^2 bath fit: FUNC / dfunc as one adjoint kernel, whole
// frprmn fits on the device, calc_dev.
//
// FUNC (func.f90:1-45) and dfunc (func.f90:47-142) for x = [eps(1:nbath),
// V(1,1:nbath), ..., V(norb,1:nbath), ef(1:norb)] (x_to_ev, func.f90:193-216):
//   Delta(a,n) = sum_k V_ak^2 / (i w_n - eps_k) + ef_a
//   r(a,n)     = Delta(a,n) - D_ev(a,n)
//   chi2       = sum_{n,a} |r|^2 / w_n / (norb^2 nw)
//   d/d eps_k  = sum_{a,n} 2 Re[conj(r) V^2 / (i w_n - eps_k)^2] / w_n / (norb^2 nw)
//   d/d V_ak   = sum_n     2 Re[2 conj(r) V / (i w_n - eps_k)]  / w_n / (norb^2 nw)
//   d/d ef_a   = sum_n     2 Re[r] / w_n / (norb^2 nw)
// chi2_sums evaluates the forward residual and its adjoint together over a
// CTA's share of the w_n, one thread per frequency stripe, per-parameter
// partials in shared memory summed in a fixed order.  Like the reference,
// i w_n is formed by CMPLX(0, w_n) -- a single-precision w_n -- when
// fortran_cmplx is set, while the 1/w_n weights use the double w_n.
//
// frprmn / linmin / mnbrak / brent (frprmn.f90) are restated once, with the
// reference's default-REAL constants.  mo_ed_minimization and
// mo_ed_fit_batch run them on the device (k_fit): one thread-block cluster
// per fit, which splits each FUNC / dfunc over its CTAs by w_n; nbatch fits
// in one launch of persistent clusters that share the fits out among
// themselves and take turns on long ones.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include <cooperative_groups.h>
#include <cuda/atomic>

#include "internal.h"

namespace moed {

constexpr int kFitThreads = 128;
// Frprmn::run's return value for a fit that gave up its cluster to a
// waiting fit (not an MO_ED code: k_fit parks such fits and resumes them)
constexpr int kFitSuspended = -1;
constexpr int kMaxX = 60;           // nmax of frprmn.f90:12

__device__ __forceinline__ double2 zdiv(double2 a, double2 b)   // Smith (1962)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, den = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    }
    const double r = b.x / b.y, den = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

// 1/d for d > 0 from an FP32 seed y0 = rcp.approx(d) refined by one
// third-order step of the Newton-Raphson family for the reciprocal,
//   y1 = y0 + y0 (e + e^2),  e = 1 - d y0,
// the truncated series y0 / (1 - e) = y0 (1 + e + e^2 + ...).  d is narrowed
// to FP32 by truncating its significand (relative error < 2^-23) and the seed
// widened back exactly, both with integer operations, so the FP64 pipe sees
// only the three FMAs.  The seed's relative error |e| is below 2^-21, the
// truncation error |e|^3 < 2^-63, and y1 is within one ulp of 1/d.  Outside
// [2^-125, 2^126) (and for d <= 0, non-finite d) it is the IEEE division.
__device__ __forceinline__ double rcp_pos(double d)
{
    const long long b = __double_as_longlong(d);
    const int ex = (int)(b >> 52);                          // biased exponent (sign bit 0)
    if ((unsigned)(ex - 898) > 250u) return 1.0 / d;        // FP32 exponent ex - 896 outside [2, 252]
    const float df = __int_as_float(((ex - 896) << 23) | (int)((b >> 29) & 0x7fffff));
    float yf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(df));
    const int fb = __float_as_int(yf);                      // a normal float: 1/df in (2^-126, 2^125]
    const double y0 = __longlong_as_double(((long long)(((fb >> 23) & 0xff) + 896) << 52) |
                                           ((long long)(fb & 0x7fffff) << 29));
    const double e = fma(-d, y0, 1.0);
    return fma(y0, fma(e, e, e), y0);
}

// fixed-order sum over the CTA of one value per thread (blockDim.x a multiple
// of 32, at most 32 warps): a butterfly within each warp, then the warps' sums
// in order by thread 0.  red: blockDim.x / 32 doubles of shared memory.
__device__ __forceinline__ double cta_sum(double v, double *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    return s;
}

// Shared memory of one chi2_block evaluation (doubles, then ints):
//   per-parameter partials [nx][nt] (rows eps_k, V_ak, ef_a);
//   1/z_k of the thread's current w_n, [nbath][2][nt];
//   kRedSlots doubles for the sums;
//   per orbital a the couplings that enter its sums: V_ak^2 and V_ak
//   [kMaxOrb][kListMax] each, bath level k [kMaxOrb][kListMax] and the count.
// nx <= kMaxX = 60 with norb >= 1 bounds nbath by 29 < kListMax.
constexpr int kRedSlots = 4 * (kMaxX + 1);
constexpr int kListMax = 32;
__host__ __device__ inline size_t chi2_smem_bytes(int nx, int nbath, int nt)
{
    return sizeof(double) * ((size_t)nx * nt + 2 * (size_t)nbath * nt + kRedSlots + 2 * kMaxOrb * kListMax) +
           sizeof(int) * (kMaxOrb * kListMax + kMaxOrb);
}

__device__ __forceinline__ bool finite_bits(double x)
{
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// Sums of the chi^2 terms of one parameter set xb (shared or global memory)
// by the whole CTA (blockDim.x threads, a multiple of 32) over the w_n with
// n = n_first + t + k n_step (thread t; n_step = blockDim.x when one CTA
// takes every w_n).
//  * Per (w_n, bath level) one reciprocal 1/|z_k|^2 gives 1/z_k, kept in
//    shared memory for every orbital's sum and the gradient terms.
//  * Orbital a sums over the bath levels it couples to, listed once per
//    evaluation: a coupling V_ak = 0 with a finite eps_k contributes exactly
//    zero to every sum (a non-finite eps_k is kept for every orbital, so it
//    propagates as in the reference).  The lists keep ascending k, the
//    reference's order of the sum over k.
//  * The 2 and 4 of the gradient formulas and the 1/w_n weight of the
//    residual are applied once per term group.
// Per-thread partials are summed in a fixed order.  out[0] = sum_n,a
// |r|^2 / w_n (thread 0); with grad out[1 + i] = the unscaled sum of
// gradient row i (chi2_scale turns the sums into FUNC / dfunc).  Every
// thread returns after a final barrier (unless final_sync is false: the
// caller's next step is a barrier), so out may be shared memory read by all
// next.
__device__ void chi2_sums(const double *__restrict__ xb, int nx, bool grad, int nw, int n_first, int n_step,
                          int norb, int nbath, const double *__restrict__ omega, const double *__restrict__ dev,
                          int fcmplx, double *sm, double *out, bool final_sync = true)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    double *sz = sm + (size_t)nx * nt;                 // [nbath][2][nt]
    double *red = sz + 2 * (size_t)nbath * nt;         // [kRedSlots]
    double *lv2 = red + kRedSlots;                     // [kMaxOrb][kListMax]
    double *lv = lv2 + kMaxOrb * kListMax;             // [kMaxOrb][kListMax]
    int *lk = (int *)(lv + kMaxOrb * kListMax);        // [kMaxOrb][kListMax]
    int *lcnt = lk + kMaxOrb * kListMax;               // [kMaxOrb]
    const double *eps = xb;                            // eps_k
    const double *V = xb + nbath;                      // V[a*nbath + k]
    const double *ef = xb + nx - norb;                 // ef_a
    if (tid < 32) {
        // warp 0, lane k = bath level k (nbath < 32): per orbital, a ballot
        // of the kept levels and each kept level's place among them
        const int k = tid;
        const bool eps_ok = k < nbath && finite_bits(eps[k]);
        for (int a = 0; a < norb; ++a) {
            const double v = k < nbath ? V[a * nbath + k] : 0.0;
            const bool keep = k < nbath && ((__double_as_longlong(v) << 1) != 0 || !eps_ok);
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int c = __popc(m & ((1u << k) - 1u));
                lk[a * kListMax + c] = k;
                lv[a * kListMax + c] = v;
                lv2[a * kListMax + c] = v * v;
            }
            if (k == 0) lcnt[a] = __popc(m);
        }
    }
    if (grad)
        for (int i = 0; i < nx - norb; ++i) sm[(size_t)i * nt + tid] = 0.0;
    __syncthreads();
    double fsum = 0.0, gef[kMaxOrb];
#pragma unroll
    for (int a = 0; a < kMaxOrb; ++a) gef[a] = 0.0;
    for (int n = n_first + tid; n < nw; n += n_step) {
        const double w = omega[n];
        const double wz = fcmplx ? (double)(float)w : w;
        const double wz2 = wz * wz;
        const double inv_w = rcp_pos(w);
        // 1/z_k, z_k = i wz - eps_k
        for (int k = 0; k < nbath; ++k) {
            const double e = eps[k];
            const double y = rcp_pos(fma(e, e, wz2));
            sz[(size_t)(2 * k) * nt + tid] = -e * y;
            sz[(size_t)(2 * k + 1) * nt + tid] = -wz * y;
        }
        // r(a, n) = sum_k V_ak^2 / z_k + ef_a - D_ev(a, n); chi2 terms |r|^2 / w_n
        double Rr[kMaxOrb], Ri[kMaxOrb];
#pragma unroll
        for (int a = 0; a < kMaxOrb; ++a) {
            Rr[a] = Ri[a] = 0.0;
            if (a < norb) {
                double dre = 0.0, dim = 0.0;
                for (int j = 0; j < lcnt[a]; ++j) {
                    const int k = lk[a * kListMax + j];
                    const double v2 = lv2[a * kListMax + j];
                    dre = fma(v2, sz[(size_t)(2 * k) * nt + tid], dre);
                    dim = fma(v2, sz[(size_t)(2 * k + 1) * nt + tid], dim);
                }
                const size_t di = 2 * ((size_t)n * norb + a);
                const double rr = (dre + ef[a]) - dev[di], ri = dim - dev[di + 1];
                fsum = fma(fma(rr, rr, ri * ri), inv_w, fsum);
                if (grad) {
                    Rr[a] = rr * inv_w;
                    Ri[a] = ri * inv_w;
                    gef[a] += Rr[a];
                }
            }
        }
        if (grad) {
            // Re[conj(r) V^2 / z^2] into the eps_k rows, Re[conj(r) V / z] into
            // the V_ak rows, both weighted by 1 / w_n
#pragma unroll
            for (int a = 0; a < kMaxOrb; ++a) {
                if (a < norb) {
                    const double Ri2 = Ri[a] + Ri[a];
                    for (int j = 0; j < lcnt[a]; ++j) {
                        const int k = lk[a * kListMax + j];
                        const double izr = sz[(size_t)(2 * k) * nt + tid], izi = sz[(size_t)(2 * k + 1) * nt + tid];
                        const double sr = fma(izr, izr, -(izi * izi)), si = izr * izi;   // 1/z^2 = sr + 2i si
                        double &ge = sm[(size_t)k * nt + tid];
                        ge = fma(lv2[a * kListMax + j], fma(Rr[a], sr, Ri2 * si), ge);
                        double &gv = sm[(size_t)(nbath + a * nbath + k) * nt + tid];
                        gv = fma(lv[a * kListMax + j], fma(Rr[a], izr, Ri[a] * izi), gv);
                    }
                }
            }
        }
    }
    if (grad) {
#pragma unroll
        for (int a = 0; a < kMaxOrb; ++a)
            if (a < norb) sm[(size_t)(nx - norb + a) * nt + tid] = gef[a];
    }
    const double f = cta_sum(fsum, red);
    if (tid == 0) out[0] = f;
    if (grad) {
        // rows in four fixed column segments, then the segments in order
        __syncthreads();
        const int seg = nt / 4;
        for (int i = tid; i < 4 * nx; i += nt) {
            const int r = i >> 2, q = i & 3;
            const double *row = sm + (size_t)r * nt + q * seg;
            double s = 0.0;
            for (int t = 0; t < seg; ++t) s += row[t];
            red[i] = s;
        }
        __syncthreads();
        for (int i = tid; i < nx; i += nt)
            out[1 + i] = ((red[4 * i] + red[4 * i + 1]) + red[4 * i + 2]) + red[4 * i + 3];
    }
    if (final_sync) __syncthreads();
}

// FUNC = sum / (norb^2 nw) (func.f90:40-43) from out[0] of chi2_sums over
// every w_n; dfunc_i from out[1 + i]: 2 sum / norb^2 / nw, and 4 sum /
// norb^2 / nw for the V_ak (func.f90:128-140)
__device__ __forceinline__ double chi2_scale_f(double s, int norb, int nw)
{
    return s / (double)(float)(norb * norb * nw);
}
__device__ __forceinline__ double chi2_scale_g(double s, int i, int nx, int norb, int nbath, int nw)
{
    const double c = (i >= nbath && i < nx - norb) ? 4.0 : 2.0;
    return c * s / (double)(float)(norb * norb) / (double)(float)nw;
}

// x: [nreq][nx]; dev: Fortran (norb, nw) interleaved complex; f: [nreq];
// g: [nreq][nx] (written only where want_grad[b] != 0, or all if want_grad null)
__global__ void __launch_bounds__(kFitThreads, 1)
k_chi2(const double *__restrict__ x, int nx, const int *__restrict__ want_grad, int nw, int norb,
       int nbath, const double *__restrict__ omega, const double *__restrict__ dev, int fcmplx,
       double *__restrict__ f, double *__restrict__ g)
{
    extern __shared__ double sm[];          // chi2_smem_bytes(nx, nbath, kFitThreads)
    __shared__ double sums[kMaxX + 1];
    const int b = blockIdx.x;
    const bool grad = g != nullptr && (want_grad ? want_grad[b] != 0 : true);
    chi2_sums(x + (size_t)b * nx, nx, grad, nw, 0, blockDim.x, norb, nbath, omega, dev, fcmplx, sm, sums);
    if (threadIdx.x == 0) f[b] = chi2_scale_f(sums[0], norb, nw);
    if (grad)
        for (int i = threadIdx.x; i < nx; i += blockDim.x)
            g[(size_t)b * nx + i] = chi2_scale_g(sums[1 + i], i, nx, norb, nbath, nw);
}

// calc_dev (ed_green.F90:260-273)
__global__ void k_calc_dev(int norb, int nbath, int nw, const double *omega, const double *ek,
                           const double *vk, const double *ef, int fcmplx, double *dev)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= norb * nw) return;
    const int i = t / norb, a = t - i * norb;
    const double wz = fcmplx ? (double)(float)omega[i] : omega[i];
    double2 d = make_double2(0.0, 0.0);
    for (int k = 0; k < nbath; ++k) {
        const double v = vk[(size_t)k * norb + a];
        const double2 q = zdiv(make_double2(v * v, 0.0), make_double2(0.0 - ek[norb + k], wz));
        d.x += q.x;
        d.y += q.y;
    }
    dev[2 * (size_t)t] = d.x + ef[a];
    dev[2 * (size_t)t + 1] = d.y;
}

// dynamic shared memory of k_chi2 / k_fit for these dimensions and nt threads
static int chi2_smem(mo_ed_ctx *ctx, const void *kernel, int nx, int nbath, int nt, size_t *bytes)
{
    *bytes = chi2_smem_bytes(nx, nbath, nt);
    MOED_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*bytes));
    return MO_ED_OK;
}

int chi2_grad_dev(mo_ed_ctx *ctx, int nbatch, const double *x, int nwloc, int ns, int nxsize,
                  const double *omega, const double *dev, int nbath, int norb, double *f, double *g,
                  int want_grad)
{
    (void)ns;
    if (nbatch <= 0) return MO_ED_OK;
    size_t smem;
    if (int rc = chi2_smem(ctx, (const void *)k_chi2, nxsize, nbath, kFitThreads, &smem)) return rc;
    k_chi2<<<nbatch, kFitThreads, smem, ctx->stream>>>(x, nxsize, nullptr, nwloc, norb, nbath, omega, dev,
                                                       ctx->opt.fortran_cmplx, f, want_grad ? g : nullptr);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

// ---------------------------------------------------------------------------
// device evaluator shared by the host fit drivers
// ---------------------------------------------------------------------------
struct FitProblem {
    int nwloc, ns, nxsize, nbath, norb;
    DevBuf omega, dev;        // device copies
};

static int fit_problem(mo_ed_ctx *ctx, FitProblem &P, const double *omega, const double *D_ev, int nwloc,
                       int ns, int nxsize, int nbath, int norb)
{
    if (!omega || !D_ev || nwloc < 1 || nbath < 0 || norb < 1 || ns != norb + nbath ||
        nxsize != nbath + nbath * norb + norb || nxsize > kMaxX || norb > kMaxOrb)
        return fail(ctx, MO_ED_ERR_ARG, "invalid fit dimensions");
    P.nwloc = nwloc;
    P.ns = ns;
    P.nxsize = nxsize;
    P.nbath = nbath;
    P.norb = norb;
    if (int rc = dev_alloc(ctx, P.omega, sizeof(double) * nwloc)) return rc;
    if (int rc = dev_alloc(ctx, P.dev, sizeof(double) * 2 * (size_t)norb * nwloc)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(P.omega.p, omega, sizeof(double) * nwloc, cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(P.dev.p, D_ev, sizeof(double) * 2 * (size_t)norb * nwloc,
                                   cudaMemcpyHostToDevice, ctx->stream));
    return MO_ED_OK;
}

// Evaluate nreq requests (x host [nreq][nx], want_grad host [nreq]).
struct Evaluator {
    mo_ed_ctx *ctx;
    FitProblem *P;
    DevBuf dx, dw, df, dg;
    size_t cap = 0;
    int eval(int nreq, const double *x, const int *want, double *f, double *g)
    {
        const int nx = P->nxsize;
        if ((size_t)nreq > cap) {
            if (int rc = dev_alloc(ctx, dx, sizeof(double) * nreq * nx)) return rc;
            if (int rc = dev_alloc(ctx, dw, sizeof(int) * nreq)) return rc;
            if (int rc = dev_alloc(ctx, df, sizeof(double) * nreq)) return rc;
            if (int rc = dev_alloc(ctx, dg, sizeof(double) * nreq * nx)) return rc;
            cap = nreq;
        }
        MOED_CUDA(ctx, cudaMemcpyAsync(dx.p, x, sizeof(double) * nreq * nx, cudaMemcpyHostToDevice, ctx->stream));
        MOED_CUDA(ctx, cudaMemcpyAsync(dw.p, want, sizeof(int) * nreq, cudaMemcpyHostToDevice, ctx->stream));
        size_t smem;
        if (int rc = chi2_smem(ctx, (const void *)k_chi2, nx, P->nbath, kFitThreads, &smem)) return rc;
        k_chi2<<<nreq, kFitThreads, smem, ctx->stream>>>((const double *)dx.p, nx, (const int *)dw.p, P->nwloc,
                                                         P->norb, P->nbath, (const double *)P->omega.p,
                                                         (const double *)P->dev.p, ctx->opt.fortran_cmplx,
                                                         (double *)df.p, (double *)dg.p);
        MOED_CHECK_LAUNCH(ctx);
        MOED_CUDA(ctx, cudaMemcpyAsync(f, df.p, sizeof(double) * nreq, cudaMemcpyDeviceToHost, ctx->stream));
        if (g)
            MOED_CUDA(ctx, cudaMemcpyAsync(g, dg.p, sizeof(double) * nreq * nx, cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return MO_ED_OK;
    }
};

// ---------------------------------------------------------------------------
// frprmn.f90 restated; func(x) / dfunc(x, g) / func.line through functors
// ---------------------------------------------------------------------------
template <typename F, typename DF>
struct Frprmn {
    F func;
    DF dfunc;
    int n;
    const double *pcom = nullptr, *xicom = nullptr;

    __host__ __device__ static double fsign(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

    // frprmn.f90:212-234: func at pcom + x xicom (formed by the functor)
    __host__ __device__ double f1dim(double x) { return func.line(pcom, xicom, x); }

    __host__ __device__ void mnbrak(double &ax, double &bx, double &cx, double &fa, double &fb, double &fc)
    {
        const double GOLD = (double)1.618034f, GLIMIT = (double)100.f, TINY = (double)1.e-20f;
        double dum, fu, q, r, u, ulim;
        fa = f1dim(ax);
        fb = f1dim(bx);
        if (fb > fa) {
            dum = ax; ax = bx; bx = dum;
            dum = fb; fb = fa; fa = dum;
        }
        cx = bx + GOLD * (bx - ax);
        fc = f1dim(cx);
        while (fb >= fc) {
            r = (bx - ax) * (fb - fc);
            q = (bx - cx) * (fb - fa);
            u = bx - ((bx - cx) * q - (bx - ax) * r) / (2. * fsign(fmax(fabs(q - r), TINY), q - r));
            ulim = bx + GLIMIT * (cx - bx);
            if ((bx - u) * (u - cx) > 0.) {
                fu = f1dim(u);
                if (fu < fc) {
                    ax = bx; fa = fb; bx = u; fb = fu;
                    return;
                } else if (fu > fb) {
                    cx = u; fc = fu;
                    return;
                }
                u = cx + GOLD * (cx - bx);
                fu = f1dim(u);
            } else if ((cx - u) * (u - ulim) > 0.) {
                fu = f1dim(u);
                if (fu < fc) {
                    bx = cx; cx = u; u = cx + GOLD * (cx - bx);
                    fb = fc; fc = fu;
                    fu = f1dim(u);
                }
            } else if ((u - ulim) * (ulim - cx) >= 0.) {
                u = ulim;
                fu = f1dim(u);
            } else {
                u = cx + GOLD * (cx - bx);
                fu = f1dim(u);
            }
            ax = bx; bx = cx; cx = u;
            fa = fb; fb = fc; fc = fu;
        }
    }

    __host__ __device__ int brent(double ax, double bx, double cx, double tol, double &xmin, double &fret)
    {
        const int ITMAX = 100;
        const double CGOLD = (double).3819660f, ZEPS = (double)1.0e-10f;
        double a, b, d = 0.0, e, etemp, fu, fv, fw, fx, p, q, r, tol1, tol2, u, v, w, x, xm;
        a = fmin(ax, cx);
        b = fmax(ax, cx);
        v = bx; w = v; x = v;
        e = 0.;
        fx = f1dim(x);
        fv = fx; fw = fx;
        for (int iter = 1; iter <= ITMAX; ++iter) {
            xm = 0.5 * (a + b);
            tol1 = tol * fabs(x) + ZEPS;
            tol2 = 2. * tol1;
            if (fabs(x - xm) <= (tol2 - .5 * (b - a))) {
                xmin = x;
                fret = fx;
                return 0;
            }
            bool golden = true;
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
                    golden = false;
                }
            }
            if (golden) {
                e = (x >= xm) ? a - x : b - x;
                d = CGOLD * e;
            }
            u = (fabs(d) >= tol1) ? x + d : x + fsign(tol1, d);
            fu = f1dim(u);
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
        xmin = x;
        fret = fx;
        return MO_ED_ERR_FIT;
    }

    __host__ __device__ int linmin(double *p, double *xi, double &fret)
    {
        const double TOL = (double)1.e-8f;
        double pc[kMaxX], xc[kMaxX], ax, xx, bx, fa, fx, fb, xmin = 0.0;
        for (int j = 0; j < n; ++j) {
            pc[j] = p[j];
            xc[j] = xi[j];
        }
        pcom = pc;
        xicom = xc;
        ax = 0.;
        xx = 1.;
        mnbrak(ax, xx, bx, fa, fx, fb);
        int rc = brent(ax, xx, bx, TOL, xmin, fret);
        for (int j = 0; j < n; ++j) {
            xi[j] = xmin * xi[j];
            p[j] = p[j] + xi[j];
        }
        return rc;
    }

    // CG state at the top of an iteration: g, h (xi = h there), fp and the
    // iterations done.  A suspended fit is p plus this state; resumed from
    // it, the fit takes the same steps as one run without a break.
    double g[kMaxX], h[kMaxX], fp = 0.0;
    int its_done = 0;

    // resume: g, h, fp, its_done hold a suspended fit's state.  quantum > 0:
    // every quantum iterations of this call, ask func.yield() whether other
    // fits are waiting; if so, return kFitSuspended (*iter = its_done).
    __host__ __device__ int run(double *p, double ftol, int &iter, double &fret, bool resume = false,
                                int quantum = 0)
    {
        const int itmax = 20000;
        const double eps = 1.e-10;
        double xi[kMaxX], dgg, gam, gg;
        if (resume) {
            for (int j = 0; j < n; ++j) xi[j] = h[j];
        } else {
            its_done = 0;
            fp = func(p);
            dfunc(p, xi);
            for (int j = 0; j < n; ++j) {
                g[j] = -xi[j];
                h[j] = g[j];
                xi[j] = h[j];
            }
        }
        const int its0 = its_done + 1;
        for (int its = its0; its <= itmax; ++its) {
            if (quantum > 0 && its > its0 && (its - its0) % quantum == 0 && func.yield()) {
                iter = its_done;
                fret = fp;
                return kFitSuspended;
            }
            iter = its;
            if (int rc = linmin(p, xi, fret)) return rc;
            if (2. * fabs(fret - fp) <= ftol * (fabs(fret) + fabs(fp) + eps)) return 0;
            fp = fret;
            dfunc(p, xi);
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
            its_done = its;
        }
        return MO_ED_ERR_FIT;
    }
};

// ---------------------------------------------------------------------------
// fits on the device: a cluster of C CTAs (C = 1 .. 8) runs one fit.  Warp 0
// of every CTA executes the same frprmn steps, each lane on its own copy of
// the scalars and vectors; the other warps of the CTA wait for its commands
// (evaluate, look for waiting fits, done) and join each evaluation, so the
// line search's scalar FP64 work runs once per CTA, not once per warp.  Each
// FUNC / dfunc is split over the
// cluster by w_n: CTA r of the cluster sums the terms of the w_n with
// n = r nt + t + k C nt (chi2_sums), writes its sums into its slot, and after
// one cluster barrier every CTA adds the C slots (read through distributed
// shared memory) in rank order.  All CTAs so see bit-identical values and
// take the same path, one cluster barrier per evaluation.  The slots are
// double-buffered: a CTA rewrites a slot two evaluations later, after the
// next barrier, which no CTA passes before every CTA has read it.  No host
// round trip per evaluation.
// ---------------------------------------------------------------------------
// One fit on one SM is bound by the latency of its FP64 dependency chains
// (GB300 has about 2 FP64 lanes per SM and clock), so a fit over nw >= 256
// w_n is spread over a cluster of up to kFitMaxCluster SMs of kFitThreads
// threads, about one w_n per thread.  Smaller grids run on one CTA of
// kFitCta threads where the partial sums fit in shared memory.
constexpr int kFitCta = 256;
constexpr int kFitMaxCluster = 8;
constexpr size_t kFitSmemMax = 220 * 1024;

namespace cg = cooperative_groups;

// Scheduler words of one k_fit launch (global memory, zeroed before it):
// q[kQFresh] fits handed out from the batch, q[kQParked] fits parked,
// q[kQSusp] suspensions, q[kQGaveUp] picks that gave up (an internal error);
// flag[b] = 1 while fit b is parked, its[b] its iterations done.
constexpr int kQFresh = 0, kQParked = 1, kQSusp = 2, kQGaveUp = 3, kQWords = 4;
constexpr int kCmdFunc = 0, kCmdGrad = 1, kCmdYield = 2, kCmdDone = 3;

__device__ __forceinline__ int ld_relaxed(int *a)
{
    return cuda::atomic_ref<int, cuda::thread_scope_device>(*a).load(cuda::memory_order_relaxed);
}

struct DevChi2 {
    int nx, nw, norb, nbath, fcmplx;
    const double *omega, *dev;
    double *sm, *sx, *sres, *slots;   // slots: [2][kMaxX + 1] of this CTA
    int rank, ncta, par;
    int *q, nbatch;                   // scheduler words
    int *bcast;                       // [2] in this CTA's shared memory
    int *s_cmd;                       // warp 0's command to the CTA
    // every thread of every CTA of the cluster passes
    __device__ void sync_all()
    {
        if (ncta > 1)
            cg::this_cluster().sync();
        else
            __syncthreads();
    }
    // rank 0's thread 0 hands a, b to every CTA of the cluster (read them
    // after the next sync_all)
    __device__ void publish(int a, int b)
    {
        if (ncta > 1) {
            cg::cluster_group cl = cg::this_cluster();
            for (int r = 0; r < ncta; ++r) {
                int *t = cl.map_shared_rank(bcast, r);
                t[0] = a;
                t[1] = b;
            }
        } else {
            bcast[0] = a;
            bcast[1] = b;
        }
    }
    // Commands of warp 0 (which runs frprmn) to the other warps of its CTA,
    // which wait in serve(); each starts with a CTA barrier
    __device__ void command(int cmd)
    {
        if (threadIdx.x == 0) *s_cmd = cmd;
        __syncthreads();
    }
    // whether fits wait for a cluster: batch fits not yet started or parked
    // ones.  One thread looks, the cluster follows its answer.
    __device__ bool yield_body()
    {
        if (rank == 0 && threadIdx.x == 0)
            publish(ld_relaxed(&q[kQFresh]) < nbatch || ld_relaxed(&q[kQParked]) > 0, 0);
        sync_all();
        const bool w = bcast[0] != 0;
        sync_all();   // bcast is written again at the next decision
        return w;
    }
    // chi^2 sums at the point sx by every thread of the CTA, reduced over the
    // cluster and scaled into sres
    __device__ void eval_body(bool grad)
    {
        const int nt = blockDim.x;
        double *mine = slots + par * (kMaxX + 1);
        // with a cluster, its barrier right after the sums stands for their final CTA barrier
        chi2_sums(sx, nx, grad, nw, rank * nt, ncta * nt, norb, nbath, omega, dev, fcmplx, sm, mine, ncta == 1);
        const int nout = grad ? nx + 1 : 1;
        if (ncta == 1) {
            for (int i = threadIdx.x; i < nout; i += nt)
                sres[i] = i ? chi2_scale_g(mine[i], i - 1, nx, norb, nbath, nw) : chi2_scale_f(mine[0], norb, nw);
        } else {
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();
            for (int i = threadIdx.x; i < nout; i += nt) {
                double s = 0.0;
                for (int r = 0; r < ncta; ++r) s += cl.map_shared_rank(mine, r)[i];
                sres[i] = i ? chi2_scale_g(s, i - 1, nx, norb, nbath, nw) : chi2_scale_f(s, norb, nw);
            }
        }
        par ^= 1;
        __syncthreads();   // sres is complete
    }
    // warps 1 .. of the CTA: run the commands of warp 0 until kCmdDone
    __device__ void serve()
    {
        for (;;) {
            __syncthreads();
            const int cmd = *s_cmd;
            if (cmd == kCmdFunc || cmd == kCmdGrad)
                eval_body(cmd == kCmdGrad);
            else if (cmd == kCmdYield)
                yield_body();
            else
                return;
        }
    }
    // warp 0 only, from here on.  sx and sres are rewritten only after the
    // barrier of the next command, which the other warps reach once done.
    __device__ bool yield()
    {
        command(kCmdYield);
        return yield_body();
    }
    // chi^2 (and the gradient into g) at the point sx, already in shared memory
    __device__ double eval_sx(double *g)
    {
        command(g ? kCmdGrad : kCmdFunc);
        eval_body(g != nullptr);
        if (g)
            for (int j = 0; j < nx; ++j) g[j] = sres[1 + j];
        return sres[0];
    }
    __device__ double eval(const double *x, double *g)
    {
        for (int j = threadIdx.x; j < nx; j += 32) sx[j] = x[j];
        return eval_sx(g);
    }
    // f1dim's point p + t xi, each element formed once, by one lane
    __device__ double line(const double *p, const double *xi, double t)
    {
        for (int j = threadIdx.x; j < nx; j += 32) sx[j] = p[j] + t * xi[j];
        return eval_sx(nullptr);
    }
};
struct DevFunc {
    DevChi2 *c;
    __device__ double operator()(const double *x) const { return c->eval(x, nullptr); }
    __device__ double line(const double *p, const double *xi, double t) const { return c->line(p, xi, t); }
    __device__ bool yield() const { return c->yield(); }
};
struct DevDFunc {
    DevChi2 *c;
    __device__ void operator()(const double *x, double *g) const { c->eval(x, g); }
};

// A parked fit, taken by one cluster: the one with the fewest iterations
// done (the waiting fits share the clusters about equally, so the long
// fits of a batch progress from the start instead of starting last).
// Called by one thread; returns -1 when no fit is parked.  A fit is parked
// only by a cluster that picks right after parking it, so a fit that this
// pick misses is taken by that cluster: no parked fit is left behind when
// the clusters leave.  Bounded: a failed claim means another cluster took
// that fit; after 4 nbatch + 4 failed claims the pick gives up (q[kQGaveUp]
// counts it, and the host reports the fits left unfinished).
__device__ int take_parked(int *q, int *flag, int *its, int nbatch)
{
    for (int attempt = 0; attempt < 4 * nbatch + 4; ++attempt) {
        int best = -1, fewest = INT_MAX;
        for (int j = 0; j < nbatch; ++j)
            if (ld_relaxed(&flag[j]) == 1) {
                const int d = ld_relaxed(&its[j]);
                if (d < fewest) {
                    fewest = d;
                    best = j;
                }
            }
        if (best < 0) return -1;
        if (atomicCAS(&flag[best], 1, 0) == 1) {
            atomicSub(&q[kQParked], 1);
            __threadfence();   // the parked state is read after this
            return best;
        }
    }
    atomicAdd(&q[kQGaveUp], 1);
    return -1;
}

// grid: persistent clusters of ncta CTAs (ncta = 1: one CTA each).  A
// cluster takes batch fits in order (q[kQFresh]); every `quantum` CG
// iterations a running fit yields its cluster if fits are waiting, and is
// parked: p in X, g, h, fp in state[b][2 nx + 1], its iterations in its[b].
// When the batch is handed out, clusters resume parked fits.  A resumed fit
// continues from its state, so every fit takes the same steps as when run
// alone.  Rank 0's thread 0 makes each decision and hands it to the
// cluster.  NT threads per CTA, MINB CTAs per SM (the shared memory of the
// chi^2 partials allows two kFitThreads-thread CTAs per SM for C5's
// 51 parameters).
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
k_fit(double *__restrict__ X, int nbatch, int nx, int nw, int norb, int nbath, const double *__restrict__ omega,
      const double *__restrict__ dev, int fcmplx, double ftol, int ncta, int quantum, int *q, int *flag, int *its,
      double *state, double *fret, int *iter, int *status)
{
    extern __shared__ double sm[];   // chi2_smem_bytes(nx, nbath, blockDim.x)
    __shared__ double sx[kMaxX], sres[kMaxX + 1], slots[2 * (kMaxX + 1)];
    __shared__ int bcast[2], s_cmd;
    const int rank = blockIdx.x % ncta;
    const bool lead = rank == 0 && threadIdx.x == 0;
    const size_t sw = 2 * (size_t)nx + 1;
    DevChi2 c{nx, nw, norb, nbath, fcmplx, omega, dev, sm, sx, sres, slots, rank, ncta, 0, q, nbatch, bcast, &s_cmd};
    Frprmn<DevFunc, DevDFunc> fr{DevFunc{&c}, DevDFunc{&c}, nx};
    double p[kMaxX];
    c.sync_all();   // every CTA of the cluster runs before its shared memory is written remotely
    for (;;) {
        if (lead) {
            int b = atomicAdd(&q[kQFresh], 1), resume = 0;
            if (b >= nbatch) {
                b = take_parked(q, flag, its, nbatch);
                resume = 1;
            }
            c.publish(b, resume);
        }
        c.sync_all();
        const int b = bcast[0];
        const bool resume = bcast[1] != 0;
        c.sync_all();   // bcast is written again by yield()
        if (b < 0) break;
        if (threadIdx.x >= 32) {
            c.serve();   // the chi^2 evaluations of warp 0's fit
            continue;
        }
        // L2 loads: a parked fit's words were written by another SM
        for (int j = 0; j < nx; ++j) p[j] = __ldcg(&X[(size_t)b * nx + j]);
        if (resume) {
            const double *st = state + (size_t)b * sw;
            for (int j = 0; j < nx; ++j) {
                fr.g[j] = __ldcg(&st[j]);
                fr.h[j] = __ldcg(&st[nx + j]);
            }
            fr.fp = __ldcg(&st[2 * nx]);
            fr.its_done = __ldcg(&its[b]);
        }
        int it = 0;
        double f = 0.0;
        const int rc = fr.run(p, ftol, it, f, resume, quantum);
        c.command(kCmdDone);
        if (lead) {
            for (int j = 0; j < nx; ++j) X[(size_t)b * nx + j] = p[j];
            if (rc == kFitSuspended) {
                double *st = state + (size_t)b * sw;
                for (int j = 0; j < nx; ++j) {
                    st[j] = fr.g[j];
                    st[nx + j] = fr.h[j];
                }
                st[2 * nx] = fr.fp;
                its[b] = fr.its_done;
                __threadfence();   // the state is visible before the flag
                atomicExch(&flag[b], 1);
                atomicAdd(&q[kQParked], 1);
                atomicAdd(&q[kQSusp], 1);
            } else {
                fret[b] = f;
                iter[b] = it;
                status[b] = rc;
            }
        }
    }
    // no CTA leaves while another may still read its slots
    if (ncta > 1) cg::this_cluster().sync();
}

// CG iterations between two looks for waiting fits (mo_ed_options.fit_quantum
// = 0): short against a long fit (20000 iterations at most), long against a
// look (two cluster barriers)
constexpr int kFitQuantum = 256;

// nbatch fits of host parameter sets x[nbatch][nxsize], in place
static int fit_on_device(mo_ed_ctx *ctx, FitProblem &P, int nbatch, double *x, double ftol, double *fret, int *iter,
                         int *status)
{
    const int nx = P.nxsize;
    const size_t sw = 2 * (size_t)nx + 1;
    DevBuf dx, df, di, ds, dq, dst;
    if (int rc = dev_alloc(ctx, dx, sizeof(double) * (size_t)nbatch * nx)) return rc;
    if (int rc = dev_alloc(ctx, df, sizeof(double) * nbatch)) return rc;
    if (int rc = dev_alloc(ctx, di, sizeof(int) * nbatch)) return rc;
    if (int rc = dev_alloc(ctx, ds, sizeof(int) * nbatch)) return rc;
    if (int rc = dev_alloc(ctx, dq, sizeof(int) * (kQWords + 2 * (size_t)nbatch))) return rc;
    if (int rc = dev_alloc(ctx, dst, sizeof(double) * (size_t)nbatch * sw)) return rc;
    int *q = (int *)dq.p, *flag = q + kQWords, *its = flag + nbatch;
    MOED_CUDA(ctx, cudaMemcpyAsync(dx.p, x, sizeof(double) * (size_t)nbatch * nx, cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemsetAsync(dq.p, 0, dq.bytes, ctx->stream));
    // a status the kernel never wrote reads kFitSuspended (all bits set)
    MOED_CUDA(ctx, cudaMemsetAsync(ds.p, 0xff, ds.bytes, ctx->stream));
    // a cluster of ncta CTAs of kFitThreads per fit for nw >= 256 (about one
    // w_n per thread); else one CTA of kFitCta threads where the partial sums
    // fit in shared memory, or of kFitThreads
    int ncta = 1, nt = kFitThreads;
    while (ncta < kFitMaxCluster && P.nwloc >= 2 * ncta * kFitThreads) ncta *= 2;
    if (P.nwloc < 2 * kFitThreads && chi2_smem_bytes(nx, P.nbath, kFitCta) <= kFitSmemMax) nt = kFitCta;
    size_t smem;
    auto kern = nt == kFitCta ? k_fit<kFitCta, 1> : k_fit<kFitThreads, 2>;
    if (int rc = chi2_smem(ctx, (const void *)kern, nx, P.nbath, nt, &smem)) return rc;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    cfg.gridDim = dim3((unsigned)(nbatch * ncta));
    cfg.blockDim = dim3((unsigned)nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)ncta;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // persistent clusters: as many as fit on the GPU at once, at most nbatch
    // (more would only start when others leave, and find less work)
    int nclu = nbatch, resident = 0;
    if (cudaOccupancyMaxActiveClusters(&resident, kern, &cfg) == cudaSuccess && resident > 0)
        nclu = std::min(nbatch, resident);
    else
        (void)cudaGetLastError();
    cfg.gridDim = dim3((unsigned)(nclu * ncta));
    MOED_CUDA(ctx, cudaLaunchKernelEx(&cfg, kern, (double *)dx.p, nbatch, nx, P.nwloc, P.norb, P.nbath,
                                      (const double *)P.omega.p, (const double *)P.dev.p, ctx->opt.fortran_cmplx,
                                      ftol, ncta, ctx->opt.fit_quantum > 0 ? ctx->opt.fit_quantum : kFitQuantum, q,
                                      flag, its, (double *)dst.p, (double *)df.p,
                                      (int *)di.p, (int *)ds.p));
    MOED_CHECK_LAUNCH(ctx);
    int qh[kQWords];
    MOED_CUDA(ctx, cudaMemcpyAsync(x, dx.p, sizeof(double) * (size_t)nbatch * nx, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(fret, df.p, sizeof(double) * nbatch, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(iter, di.p, sizeof(int) * nbatch, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(status, ds.p, sizeof(int) * nbatch, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(qh, dq.p, sizeof(qh), cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->fit_suspensions = qh[kQSusp];
    ctx->fit_clusters = nclu;
    for (int b = 0; b < nbatch; ++b)
        if (status[b] == kFitSuspended)
            return fail(ctx, MO_ED_ERR_CUDA, "k_fit: a fit was left unfinished by the cluster scheduler");
    return MO_ED_OK;
}

}  // namespace moed

using namespace moed;

extern "C" {

int mo_ed_func(mo_ed_ctx *ctx, const double *x, int ns, int nwloc, int nxsize, const double *omega,
               const double *D_ev, int nbath, int norb, double *f)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!x || !f) return fail(ctx, MO_ED_ERR_ARG, "null argument");
    FitProblem P;
    if (int rc = fit_problem(ctx, P, omega, D_ev, nwloc, ns, nxsize, nbath, norb)) return rc;
    Evaluator ev{ctx, &P};
    int want = 0;
    return ev.eval(1, x, &want, f, nullptr);
}

int mo_ed_dfunc(mo_ed_ctx *ctx, const double *x, double *p, int nwloc, int ns, int nxsize,
                const double *omega, const double *D_ev, int nbath, int norb)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!x || !p) return fail(ctx, MO_ED_ERR_ARG, "null argument");
    FitProblem P;
    if (int rc = fit_problem(ctx, P, omega, D_ev, nwloc, ns, nxsize, nbath, norb)) return rc;
    Evaluator ev{ctx, &P};
    int want = 1;
    double f;
    return ev.eval(1, x, &want, &f, p);
}

int mo_ed_chi2_grad_dev(mo_ed_ctx *ctx, int nbatch, const double *x, int nwloc, int ns, int nxsize,
                        const double *omega, const double *D_ev, int nbath, int norb, double *f,
                        double *g)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!x || !f || !omega || !D_ev || nbatch < 0 || nxsize > kMaxX || norb < 1 || norb > kMaxOrb ||
        nxsize != nbath + nbath * norb + norb || ns != norb + nbath)
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    return chi2_grad_dev(ctx, nbatch, x, nwloc, ns, nxsize, omega, D_ev, nbath, norb, f, g, g != nullptr);
}

int mo_ed_minimization(mo_ed_ctx *ctx, double *x, int nwloc, int ns, int nxsize, const double *omega,
                       const double *D_ev, int nbath, int norb, double *fret, int *iter)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!x || !fret || !iter) return fail(ctx, MO_ED_ERR_ARG, "null argument");
    FitProblem P;
    if (int rc = fit_problem(ctx, P, omega, D_ev, nwloc, ns, nxsize, nbath, norb)) return rc;
    int status = 0;
    if (int rc = fit_on_device(ctx, P, 1, x, 1.0e-7, fret, iter, &status)) return rc;   // FTOL (func.f90:155)
    if (status) return fail(ctx, status, "frprmn: iteration limit exceeded");
    return MO_ED_OK;
}

int mo_ed_fit_batch(mo_ed_ctx *ctx, int nbatch, double *x, int nwloc, int ns, int nxsize,
                    const double *omega, const double *D_ev, int nbath, int norb, double ftol,
                    double *fret, int *iter, int *status)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (nbatch < 1 || !x || !fret || !iter || !status || !(ftol > 0))
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    FitProblem P;
    if (int rc = fit_problem(ctx, P, omega, D_ev, nwloc, ns, nxsize, nbath, norb)) return rc;
    return fit_on_device(ctx, P, nbatch, x, ftol, fret, iter, status);
}

int mo_ed_fit_stats(mo_ed_ctx *ctx, long long *suspensions, int *clusters)
{
    if (!ctx) return MO_ED_ERR_ARG;
    if (suspensions) *suspensions = ctx->fit_suspensions;
    if (clusters) *clusters = ctx->fit_clusters;
    return MO_ED_OK;
}

int mo_ed_calc_dev(mo_ed_ctx *ctx, int norb, int nsite, int nwloc, const double *omega, const double *ek,
                   const double *vk, const double *ef, double *D_ev)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int nbath = nsite - norb;
    if (norb < 1 || nbath < 0 || nwloc < 1 || !omega || !ek || !ef || !D_ev || (nbath > 0 && !vk))
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    DevBuf dom, dek, dvk, def, ddev;
    if (int rc = dev_alloc(ctx, dom, sizeof(double) * nwloc)) return rc;
    if (int rc = dev_alloc(ctx, dek, sizeof(double) * nsite)) return rc;
    if (int rc = dev_alloc(ctx, dvk, sizeof(double) * std::max(1, norb * nbath))) return rc;
    if (int rc = dev_alloc(ctx, def, sizeof(double) * norb)) return rc;
    if (int rc = dev_alloc(ctx, ddev, sizeof(double) * 2 * (size_t)norb * nwloc)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(dom.p, omega, sizeof(double) * nwloc, cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dek.p, ek, sizeof(double) * nsite, cudaMemcpyHostToDevice, ctx->stream));
    if (nbath > 0)
        MOED_CUDA(ctx, cudaMemcpyAsync(dvk.p, vk, sizeof(double) * norb * nbath, cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(def.p, ef, sizeof(double) * norb, cudaMemcpyHostToDevice, ctx->stream));
    const int T = 128;
    k_calc_dev<<<(norb * nwloc + T - 1) / T, T, 0, ctx->stream>>>(norb, nbath, nwloc, (const double *)dom.p,
                                                                  (const double *)dek.p, (const double *)dvk.p,
                                                                  (const double *)def.p, ctx->opt.fortran_cmplx,
                                                                  (double *)ddev.p);
    MOED_CHECK_LAUNCH(ctx);
    MOED_CUDA(ctx, cudaMemcpyAsync(D_ev, ddev.p, sizeof(double) * 2 * (size_t)norb * nwloc, cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

}  // extern "C"
