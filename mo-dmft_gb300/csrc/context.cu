// context.cu -- context lifecycle, configuration and the C-ABI entry points
// for the basis, H*v and apply_c.
#include <cmath>
#include <cstring>

#include "internal.h"

namespace moed {

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

int fail(mo_ed_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(mo_ed_ctx *ctx, cudaError_t e, const char *what)
{
    int code = (e == cudaErrorMemoryAllocation) ? MO_ED_ERR_NOMEM : MO_ED_ERR_CUDA;
    return fail(ctx, code, std::string(what) + ": " + cudaGetErrorString(e));
}

int dev_alloc(mo_ed_ctx *ctx, DevBuf &b, size_t bytes)
{
    b.release();
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        return cuda_fail(ctx, e, "cudaMalloc");
    }
    b.bytes = bytes;
    return MO_ED_OK;
}

int ensure(mo_ed_ctx *ctx, DevBuf &b, size_t bytes)
{
    if (b.p && b.bytes >= bytes) return MO_ED_OK;
    return dev_alloc(ctx, b, bytes);
}

int upload_padded(mo_ed_ctx *ctx, const Sector &s, const void *host, void *dev, size_t es)
{
    const size_t nu = s.up->n, ld = s.ld(), nd = s.dn->n;
    if (ld > nu)
        MOED_CUDA(ctx, cudaMemset2DAsync((char *)dev + nu * es, ld * es, 0, (ld - nu) * es, nd, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpy2DAsync(dev, ld * es, host, nu * es, nu * es, nd, cudaMemcpyHostToDevice,
                                     ctx->stream));
    return MO_ED_OK;
}

int download_padded(mo_ed_ctx *ctx, const Sector &s, const void *dev, void *host, size_t es)
{
    const size_t nu = s.up->n, ld = s.ld(), nd = s.dn->n;
    MOED_CUDA(ctx, cudaMemcpy2DAsync(host, nu * es, dev, ld * es, nu * es, nd, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    return MO_ED_OK;
}

}  // namespace moed

using namespace moed;

#define CTX_CHECK(ctx)                  \
    do {                                \
        if (!(ctx)) return MO_ED_ERR_ARG; \
        cudaSetDevice((ctx)->device);   \
    } while (0)

extern "C" {

const char *mo_ed_version(void) { return "mo_ed 0.1 (sm_103a)"; }

int mo_ed_default_options(mo_ed_options *o)
{
    if (!o) return MO_ED_ERR_ARG;
    memset(o, 0, sizeof(*o));
    o->nstep = 50;
    o->nev = 30;
    o->beta = 100.0;
    o->precision = MO_ED_FP32;
    o->fortran_cmplx = 1;
    o->gs_ncv = 0;
    o->gs_maxcycles = 200;
    o->gs_tol = 0.0;
    o->green_reorth = 0;
    return MO_ED_OK;
}

int mo_ed_create(mo_ed_ctx **out, int device, void *stream)
{
    if (!out) return MO_ED_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return MO_ED_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return MO_ED_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return MO_ED_ERR_CUDA;
    mo_ed_ctx *ctx = new mo_ed_ctx;
    ctx->device = device;
    mo_ed_default_options(&ctx->opt);
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return MO_ED_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    // commit the no-allocation region now, while the host's memory pool (if
    // any) has not taken the device yet; a failure here is reported by the
    // no-allocation call itself
    if (noalloc_prepare(ctx) != MO_ED_OK) ctx->err.clear();
    *out = ctx;
    return MO_ED_OK;
}

int mo_ed_destroy(mo_ed_ctx *ctx)
{
    if (!ctx) return MO_ED_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (mo_ed_ctx *w : ctx->workers) mo_ed_destroy(w);
    ctx->workers.clear();
    ctx->species.clear();
    ctx->states.clear();
    if (ctx->d_mdl) cudaFree(ctx->d_mdl);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MO_ED_OK;
}

const char *mo_ed_last_error(const mo_ed_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long mo_ed_kernel_launches(const mo_ed_ctx *ctx) { return ctx ? ctx->launches : 0; }

int mo_ed_set_options(mo_ed_ctx *ctx, const mo_ed_options *o)
{
    CTX_CHECK(ctx);
    if (!o) return fail(ctx, MO_ED_ERR_ARG, "null options");
    if (o->nstep < 1 || o->nev < 1 || !(o->beta > 0) ||
        (o->precision != MO_ED_FP32 && o->precision != MO_ED_FP64) || o->gs_ncv < 0 ||
        o->gs_maxcycles < 1 || o->gs_tol < 0 || (o->green_fp64 != 0 && o->green_fp64 != 1) ||
        o->solve_threads < 0 || o->solve_threads > 64 || o->fit_quantum < 0)
        return fail(ctx, MO_ED_ERR_ARG, "invalid options");
    if (o->green_reorth != 0)
        return fail(ctx, MO_ED_ERR_ARG, "green_reorth = 1 is not available: the Green's-function "
                                        "recurrence is the reference's, without reorthogonalisation");
    ctx->opt = *o;
    return MO_ED_OK;
}

long long mo_ed_icom(int n, int m) { return binom(n, m); }

int mo_ed_set_model(mo_ed_ctx *ctx, int norb, int nbath, double U, double Jex, const double *ek,
                    const double *vk)
{
    CTX_CHECK(ctx);
    if (norb < 1 || norb > kMaxOrb || nbath < 0 || norb + nbath > kMaxSite || !ek ||
        (nbath > 0 && !vk))
        return fail(ctx, MO_ED_ERR_ARG, "invalid model dimensions (norb 1..5, nsite <= 15)");
    const int nsite = norb + nbath;
    if (!std::isfinite(U) || !std::isfinite(Jex))
        return fail(ctx, MO_ED_ERR_ARG, "non-finite U or J");
    for (int i = 0; i < nsite; ++i)
        if (!std::isfinite(ek[i])) return fail(ctx, MO_ED_ERR_ARG, "non-finite ek");
    for (int i = 0; i < norb * nbath; ++i)
        if (!std::isfinite(vk[i])) return fail(ctx, MO_ED_ERR_ARG, "non-finite vk");
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->norb = norb;
    ctx->nbath = nbath;
    ctx->nsite = nsite;
    ctx->U = U;
    ctx->J = Jex;
    ctx->ek.assign(ek, ek + nsite);
    ctx->vk.assign(vk, vk + (size_t)norb * nbath);
    ctx->states.clear();
    ++ctx->model_gen;   // worker contexts take the new model at their next use
    ctx->green.clear();
    ctx->have_model = false;
    if (int rc = build_model(ctx)) return rc;
    ctx->have_model = true;
    return MO_ED_OK;
}

int mo_ed_set_sectors(mo_ed_ctx *ctx, int nsector, const int *nelec, const int *nup)
{
    CTX_CHECK(ctx);
    if (nsector < 1 || !nelec || !nup) return fail(ctx, MO_ED_ERR_ARG, "invalid sector list");
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    for (int i = 0; i < nsector; ++i) {
        int nd = nelec[i] - nup[i];
        if (nup[i] < 0 || nup[i] > ctx->nsite || nd < 0 || nd > ctx->nsite)
            return fail(ctx, MO_ED_ERR_SECTOR, "sector " + std::to_string(i + 1) + " out of range");
    }
    ctx->nelec.assign(nelec, nelec + nsector);
    ctx->nup.assign(nup, nup + nsector);
    ctx->states.clear();
    return MO_ED_OK;
}

int mo_ed_set_omega(mo_ed_ctx *ctx, int nw, const double *omega)
{
    CTX_CHECK(ctx);
    if (nw < 1 || !omega) return fail(ctx, MO_ED_ERR_ARG, "invalid omega grid");
    for (int i = 0; i < nw; ++i)
        if (!std::isfinite(omega[i])) return fail(ctx, MO_ED_ERR_ARG, "non-finite omega");
    ctx->omega.assign(omega, omega + nw);
    return MO_ED_OK;
}

int mo_ed_sector_dims(mo_ed_ctx *ctx, int ne_up, int ne_down, int *nup, int *ndown, long long *ntot)
{
    CTX_CHECK(ctx);
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    if (ne_up < 0 || ne_up > ctx->nsite || ne_down < 0 || ne_down > ctx->nsite)
        return fail(ctx, MO_ED_ERR_SECTOR, "sector out of range");
    long long a = binom(ctx->nsite, ne_up), b = binom(ctx->nsite, ne_down);
    if (nup) *nup = (int)a;
    if (ndown) *ndown = (int)b;
    if (ntot) *ntot = a * b;
    return MO_ED_OK;
}

int mo_ed_vector_layout(mo_ed_ctx *ctx, int ne_up, int ne_down, int *ld, long long *nelem)
{
    CTX_CHECK(ctx);
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    if (ld) *ld = s.ld();
    if (nelem) *nelem = s.Dpad();
    return MO_ED_OK;
}

int mo_ed_generate_basis(mo_ed_ctx *ctx, int ne_up, int ne_down, int *up, int *down, int *idx_up,
                         int *idx_down)
{
    CTX_CHECK(ctx);
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    const size_t nw = (size_t)1 << ctx->nsite;
    if (up)
        MOED_CUDA(ctx, cudaMemcpyAsync(up, s.up->words, sizeof(int) * s.up->n,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    if (down)
        MOED_CUDA(ctx, cudaMemcpyAsync(down, s.dn->words, sizeof(int) * s.dn->n,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    if (idx_up)
        MOED_CUDA(ctx, cudaMemcpyAsync(idx_up, s.up->rank, sizeof(int) * nw,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    if (idx_down)
        MOED_CUDA(ctx, cudaMemcpyAsync(idx_down, s.dn->rank, sizeof(int) * nw,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // device ranks are 0-based with -1 outside; the reference's tables are 1-based
    if (idx_up)
        for (size_t i = 0; i < nw; ++i) idx_up[i] += 1;
    if (idx_down)
        for (size_t i = 0; i < nw; ++i) idx_down[i] += 1;
    return MO_ED_OK;
}

int mo_ed_basis_get(mo_ed_ctx *ctx, int ne_up, int ne_down, long long n, const long long *idx,
                    unsigned int *state)
{
    CTX_CHECK(ctx);
    if (n < 0 || (n > 0 && (!idx || !state))) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    for (long long i = 0; i < n; ++i)
        if (idx[i] < 1 || idx[i] > s.D()) return fail(ctx, MO_ED_ERR_ARG, "row index out of range");
    if (n == 0) return MO_ED_OK;
    DevBuf di, ds;
    if (int rc = dev_alloc(ctx, di, sizeof(long long) * n)) return rc;
    if (int rc = dev_alloc(ctx, ds, sizeof(unsigned) * n)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(di.p, idx, sizeof(long long) * n, cudaMemcpyHostToDevice,
                                   ctx->stream));
    if (int rc = basis_get_dev(ctx, s, n, (const long long *)di.p, (unsigned *)ds.p)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(state, ds.p, sizeof(unsigned) * n, cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int mo_ed_basis_idx(mo_ed_ctx *ctx, int ne_up, int ne_down, long long n, const unsigned int *state,
                    long long *idx)
{
    CTX_CHECK(ctx);
    if (n < 0 || (n > 0 && (!idx || !state))) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    if (n == 0) return MO_ED_OK;
    DevBuf di, ds;
    if (int rc = dev_alloc(ctx, di, sizeof(long long) * n)) return rc;
    if (int rc = dev_alloc(ctx, ds, sizeof(unsigned) * n)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(ds.p, state, sizeof(unsigned) * n, cudaMemcpyHostToDevice,
                                   ctx->stream));
    if (int rc = basis_idx_dev(ctx, s, n, (const unsigned *)ds.p, (long long *)di.p)) return rc;
    MOED_CUDA(ctx, cudaMemcpyAsync(idx, di.p, sizeof(long long) * n, cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

static int multiply_host(mo_ed_ctx *ctx, int ne_up, int ne_down, const void *A, void *B, size_t es,
                         int kind)
{
    CTX_CHECK(ctx);
    if (!A || !B) return fail(ctx, MO_ED_ERR_ARG, "null vector");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    const size_t bytes = es * (size_t)s.Dpad();
    if (int rc = ensure(ctx, ctx->scratch_a, bytes)) return rc;
    if (int rc = ensure(ctx, ctx->scratch_b, bytes)) return rc;
    if (int rc = upload_padded(ctx, s, A, ctx->scratch_a.p, es)) return rc;
    if (int rc = hv_single(ctx, s, kind, ctx->scratch_a.p, ctx->scratch_b.p)) return rc;
    if (int rc = download_padded(ctx, s, ctx->scratch_b.p, B, es)) return rc;
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int mo_ed_multiply_h(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *A, double *B)
{
    return multiply_host(ctx, ne_up, ne_down, A, B, sizeof(double), HV_F64);
}

int mo_ed_multiply_h_f32(mo_ed_ctx *ctx, int ne_up, int ne_down, const float *A, float *B)
{
    return multiply_host(ctx, ne_up, ne_down, A, B, sizeof(float), HV_F32);
}

int mo_ed_multiply_h_dev(mo_ed_ctx *ctx, int ne_up, int ne_down, int dtype, const void *dA, void *dB)
{
    CTX_CHECK(ctx);
    if (!dA || !dB || (dtype != MO_ED_FP32 && dtype != MO_ED_FP64))
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    return hv_single(ctx, s, dtype == MO_ED_FP32 ? HV_F32 : HV_F64, dA, dB);
}

int mo_ed_multiply_h_mixed_dev(mo_ed_ctx *ctx, int ne_up, int ne_down, const float *dA, double *dB)
{
    CTX_CHECK(ctx);
    if (!dA || !dB) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    return hv_single(ctx, s, HV_MIXED, dA, dB);
}

int mo_ed_hv_tuning(mo_ed_ctx *ctx, int ne_up, int ne_down, int dtype, int capacity, int *nvariant,
                    int *shape, float *ms, int *chosen)
{
    CTX_CHECK(ctx);
    if (!nvariant || !chosen || (dtype != MO_ED_FP32 && dtype != MO_ED_FP64))
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    return hv_tuning(ctx, s, dtype == MO_ED_FP32 ? HV_F32 : HV_F64, capacity, nvariant, shape, ms, chosen);
}

int mo_ed_hv_set_variant(mo_ed_ctx *ctx, int ne_up, int ne_down, int dtype, int variant)
{
    CTX_CHECK(ctx);
    if (dtype != MO_ED_FP32 && dtype != MO_ED_FP64) return fail(ctx, MO_ED_ERR_ARG, "bad dtype");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    return hv_set_variant(ctx, s, dtype == MO_ED_FP32 ? HV_F32 : HV_F64, variant);
}

int mo_ed_apply_c(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *vec, int pm, int iorb,
                  int ispin, double *vec_out, long long capacity, long long *ntot_out)
{
    CTX_CHECK(ctx);
    if (!vec || (pm != 1 && pm != 2) || (ispin != 1 && ispin != 2))
        return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    if (iorb < 1 || iorb > ctx->nsite) return fail(ctx, MO_ED_ERR_ARG, "orbital out of range");
    Sector in, out;
    if (int rc = get_sector(ctx, ne_up, ne_down, &in)) return rc;
    int d = (pm == 1) ? 1 : -1;
    int nu = ne_up + (ispin == 1 ? d : 0), nd = ne_down + (ispin == 2 ? d : 0);
    if (int rc = get_sector(ctx, nu, nd, &out)) return rc;
    if (ntot_out) *ntot_out = out.D();
    if (!vec_out || capacity < out.D())
        return fail(ctx, MO_ED_ERR_CAPACITY, "vec_out capacity below target dimension");
    const size_t bin = sizeof(double) * in.Dpad(), bout = sizeof(double) * out.Dpad();
    if (int rc = ensure(ctx, ctx->scratch_a, bin)) return rc;
    if (int rc = ensure(ctx, ctx->scratch_b, bout)) return rc;
    if (int rc = upload_padded(ctx, in, vec, ctx->scratch_a.p, sizeof(double))) return rc;
    if (int rc = apply_c_dev(ctx, in, out, MO_ED_FP64, ctx->scratch_a.p, ctx->scratch_b.p, pm, iorb,
                             ispin))
        return rc;
    if (int rc = download_padded(ctx, out, ctx->scratch_b.p, vec_out, sizeof(double))) return rc;
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int mo_ed_lanczos_iteration(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *vec,
                            int *nstep_calc, double *a, double *b)
{
    CTX_CHECK(ctx);
    if (!vec || !nstep_calc || !a || !b) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = get_sector(ctx, ne_up, ne_down, &s)) return rc;
    return lanczos_reference(ctx, s, vec, ctx->opt.nstep, nstep_calc, a, b);
}

int mo_ed_ev_to_x(const double *ek, const double *vk, const double *ef, int ns, int nbath,
                  int nxsize, double *x)
{
    // func.f90:165-191
    if (!ek || !ef || !x || nbath < 0 || ns <= nbath) return MO_ED_ERR_ARG;
    const int norb = ns - nbath;
    if (nxsize != nbath + nbath * norb + norb || (nbath > 0 && !vk)) return MO_ED_ERR_ARG;
    for (int i = 1; i <= nbath; ++i) x[i - 1] = ek[norb + i - 1];
    for (int iorb = 1; iorb <= norb; ++iorb) {
        int iinit = nbath + 1 + (iorb - 1) * nbath, ifina = nbath + iorb * nbath;
        for (int k = iinit; k <= ifina; ++k) x[k - 1] = vk[(size_t)(k - iinit) * norb + (iorb - 1)];
    }
    for (int i = 1; i <= norb; ++i) x[nxsize - norb + i - 1] = ef[i - 1];
    return MO_ED_OK;
}

int mo_ed_x_to_ev(const double *x, int nxsize, int ns, int nbath, int norb, double *ef, double *ek,
                  double *vk)
{
    // func.f90:193-216
    if (!x || !ef || !ek || nbath < 0 || norb < 1 || ns != norb + nbath ||
        nxsize != nbath + nbath * norb + norb || (nbath > 0 && !vk))
        return MO_ED_ERR_ARG;
    for (int i = 1; i <= norb; ++i) {
        ek[i - 1] = x[nxsize - norb + i - 1];
        ef[i - 1] = ek[i - 1];
    }
    for (int i = norb + 1; i <= norb + nbath; ++i) ek[i - 1] = x[i - norb - 1];
    for (int iorb = 1; iorb <= norb; ++iorb) {
        int ia = (iorb - 1) * nbath;
        for (int i = norb + 1; i <= ns; ++i)
            vk[(size_t)(i - norb - 1) * norb + (iorb - 1)] = x[i + nbath + ia - norb - 1];
    }
    return MO_ED_OK;
}

}  // extern "C"
