// krylov.cu -- Lanczos on the device.
//
//  * lz_* : the reference three-term recurrence (ed_lanczos.F90:14-68) as
//    batched kernels: update -> H*v (fused alpha partials) -> finalize, so
//    that every excitation vector of the Green's function advances in the
//    same three launches per step and no host round trip occurs.
//  * diag_sector : replaces the PARPACK 'SA' solve of diag()
//    (ed_solver.F90:107-191) by a thick-restart Lanczos with full
//    reorthogonalisation (classical Gram-Schmidt, two passes), an FP64
//    projected matrix and an FP64 parallel-Jacobi eigensolve in one CTA;
//    eigenvalues are returned as FP64 Rayleigh quotients of the Ritz
//    vectors (FP64-accumulated H*v for FP32 vectors).
// All reductions are per-block partials summed in a fixed order (run-to-run
// deterministic).  Per-element work of FP32 vectors stays in FP32; FP64 is
// used once per 4-8 elements in the partial sums.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "krylov.cuh"
#include "symeig.h"

namespace moed {

constexpr int kVecThreads = 256;

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}
__device__ __forceinline__ float warp_sum(float v)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

// block-wide sum, result valid in thread 0
__device__ double block_sum(double v, double *sred)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sred[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sred[w];
    return t;
}

template <typename TX, typename TY>
__global__ void k_dot_part(const TX *__restrict__ x, const TY *__restrict__ y, long long n,
                           double *part)
{
    __shared__ double sred[32];
    double acc = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    // products and sums in FP64 (an FP32 x FP32 product is exact in FP64)
    for (; i + 3 * stride < n; i += 4 * stride) {
        acc += (double)x[i] * (double)y[i] + (double)x[i + stride] * (double)y[i + stride] +
               (double)x[i + 2 * stride] * (double)y[i + 2 * stride] +
               (double)x[i + 3 * stride] * (double)y[i + 3 * stride];
    }
    for (; i < n; i += stride) acc += (double)x[i] * (double)y[i];
    double t = block_sum(acc, sred);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_sum_parts(const double *part, int n, double *out)
{
    __shared__ double sred[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
    double t = block_sum(acc, sred);
    if (threadIdx.x == 0) *out = t;
}

static int dot_grid(mo_ed_ctx *ctx, long long n)
{
    long long g = (n + kVecThreads * 4 - 1) / (kVecThreads * 4);
    return (int)std::max(1LL, std::min(g, (long long)ctx->num_sms * 4));
}

int dot_dev(mo_ed_ctx *ctx, int prec_x, const void *x, int prec_y, const void *y, long long n,
            double *d_out)
{
    const int g = dot_grid(ctx, n);
    if (int rc = ensure(ctx, ctx->scratch_part, sizeof(double) * g)) return rc;
    double *part = (double *)ctx->scratch_part.p;
    if (prec_x == MO_ED_FP32 && prec_y == MO_ED_FP32)
        k_dot_part<float, float><<<g, kVecThreads, 0, ctx->stream>>>((const float *)x, (const float *)y, n, part);
    else if (prec_x == MO_ED_FP32)
        k_dot_part<float, double><<<g, kVecThreads, 0, ctx->stream>>>((const float *)x, (const double *)y, n, part);
    else if (prec_y == MO_ED_FP32)
        k_dot_part<double, float><<<g, kVecThreads, 0, ctx->stream>>>((const double *)x, (const float *)y, n, part);
    else
        k_dot_part<double, double><<<g, kVecThreads, 0, ctx->stream>>>((const double *)x, (const double *)y, n, part);
    MOED_CHECK_LAUNCH(ctx);
    k_sum_parts<<<1, kVecThreads, 0, ctx->stream>>>(part, g, d_out);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

template <typename TI, typename TO>
__global__ void k_convert(const TI *__restrict__ in, TO *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = (TO)in[i];
}

int convert_f64_to_f32(mo_ed_ctx *ctx, const double *in, float *out, long long n)
{
    if (n <= 0) return MO_ED_OK;
    k_convert<double, float><<<dot_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(in, out, n);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

int convert_f32_to_f64(mo_ed_ctx *ctx, const float *in, double *out, long long n)
{
    if (n <= 0) return MO_ED_OK;
    k_convert<float, double><<<dot_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(in, out, n);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

// 16-byte vector access to 4 consecutive elements (vectors are padded to a
// multiple of 32 elements and 256-byte aligned)
template <typename T>
__device__ __forceinline__ void vload4(const T *p, T (&r)[4])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        r[0] = a.x;
        r[1] = a.y;
        r[2] = a.z;
        r[3] = a.w;
    } else {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
        const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
        r[0] = a.x;
        r[1] = a.y;
        r[2] = b.x;
        r[3] = b.y;
    }
}

template <typename T>
__device__ __forceinline__ void vstore4(T *p, const T (&r)[4])
{
    if constexpr (sizeof(T) == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(r[0], r[1], r[2], r[3]);
    } else {
        reinterpret_cast<double2 *>(p)[0] = make_double2(r[0], r[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(r[2], r[3]);
    }
}

// ---------------------------------------------------------------------------
// reference recurrence, batched
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_run_upd(const LzBatchDev &b, int item)
{
    int r = 0;
    while (r + 1 < b.nrun && item >= b.run[r + 1].upd_item0) ++r;
    return r;
}

// step j = 0: partial sums of ||u_0||^2
template <typename T>
__global__ void k_lz_norm0(const __grid_constant__ LzBatchDev b)
{
    __shared__ double sred[32];
    for (int item = blockIdx.x; item < b.total_items; item += gridDim.x) {
        const int r = find_run_upd(b, item);
        const LzRunDev &R = b.run[r];
        const int it = item - R.upd_item0;
        const long long i0 = (long long)it * kVecChunk, i1 = min(R.D, i0 + kVecChunk);
        const T *u = (const T *)R.u[0];
        double acc = 0.0;
        for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) acc += (double)u[i] * (double)u[i];
        double t = block_sum(acc, sred);
        if (threadIdx.x == 0) R.upd_part[it] = t;
    }
}

// step j >= 1: u_j = s (w - a_{j-1} u_{j-1}) - c u_{j-2},  s = 1/sqrt(b_{j-1}),
// c = sqrt(b_{j-1}/b_{j-2}) -- ed_lanczos.F90:38 (j = 1) and :54 (j >= 2)
// with the reference's normalized vectors written as scaled stored ones.
// 4 consecutive elements per thread (16-byte accesses; run lengths are
// multiples of 32 elements).
template <typename T>
__global__ void k_lz_update(const __grid_constant__ LzBatchDev b, int j)
{
    __shared__ double sred[32];
    for (int item = blockIdx.x; item < b.total_items; item += gridDim.x) {
        const int r = find_run_upd(b, item);
        const LzRunDev &R = b.run[r];
        if (*R.active == 0) continue;
        const int it = item - R.upd_item0;
        const long long i0 = (long long)it * kVecChunk, i1 = min(R.D, i0 + kVecChunk);
        const double nb1 = R.nrm[j - 1];
        const T s = (T)(1.0 / sqrt(nb1));
        const T a = (T)R.a[j - 1];
        const T c = (j >= 2) ? (T)sqrt(nb1 / R.nrm[j - 2]) : T(0);
        const T *w = (const T *)R.w;
        const T *uc = (const T *)R.u[(j - 1) % 3];
        const T *up = (const T *)R.u[(j + 1) % 3];   // (j-2) mod 3
        T *un = (T *)R.u[j % 3];
        // ||u_j||^2: partials of 4 squares in T, added to the FP64 sum every
        // 8 iterations (per-element FP64 work would bound the kernel on GB300)
        double acc = 0.0;
        T sacc = T(0);
        int cnt = 0;
        for (long long i = i0 + 4 * threadIdx.x; i < i1; i += 4 * blockDim.x) {
            T wv[4], cv[4], pv[4], v[4];
            vload4(w + i, wv);
            vload4(uc + i, cv);
            if (j >= 2) {
                vload4(up + i, pv);
            } else {
                pv[0] = pv[1] = pv[2] = pv[3] = T(0);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e)
                v[e] = (j >= 2) ? s * (wv[e] - a * cv[e]) - c * pv[e] : s * (wv[e] - a * cv[e]);
            sacc += (v[0] * v[0] + v[1] * v[1]) + (v[2] * v[2] + v[3] * v[3]);
            if (++cnt == 8) {
                acc += (double)sacc;
                sacc = T(0);
                cnt = 0;
            }
            vstore4(un + i, v);
        }
        acc += (double)sacc;
        double t = block_sum(acc, sred);
        if (threadIdx.x == 0) R.upd_part[it] = t;
    }
}

// nrm_j and a_j from the partials; the reference's stop test b(j) < 1.e-12
// (a default-REAL literal, ed_lanczos.F90:62) -- applied from j = 1 on.
__global__ void k_lz_finalize(const __grid_constant__ LzBatchDev b, int j, int nstep)
{
    __shared__ double sred[32];
    const LzRunDev &R = b.run[blockIdx.x];
    if (*R.active == 0) return;
    double acc = 0.0;
    for (int i = threadIdx.x; i < R.upd_nitems; i += blockDim.x) acc += R.upd_part[i];
    const double nrm = block_sum(acc, sred);
    acc = 0.0;
    for (int i = threadIdx.x; i < R.hv_nitems; i += blockDim.x) acc += R.hv_part[i];
    const double dot = block_sum(acc, sred);
    if (threadIdx.x == 0) {
        R.nrm[j] = nrm;
        if (j == 0 && nrm == 0.0) {        // zero start vector: no contribution
            R.a[0] = 0.0;
            *R.nstep_calc = 0;
            *R.active = 0;
            return;
        }
        R.a[j] = dot / nrm;
        const double tiny = (double)1.e-12f;
        if (j >= 1 && nrm < tiny) {
            *R.nstep_calc = j;
            *R.active = 0;
        } else if (j == nstep) {
            *R.nstep_calc = nstep;
            *R.active = 0;
        }
    }
}

void *lz_start_vector(LzBatch &b, int r) { return b.vecs[4 * r].p; }

int lz_setup(mo_ed_ctx *ctx, LzBatch &b, const std::vector<Sector> &secs, int prec, int nstep)
{
    const int nrun = (int)secs.size();
    if (nrun > kLzMaxRuns) return fail(ctx, MO_ED_ERR_ARG, "too many Lanczos runs in one batch");
    b.prec = prec;
    b.nstep = nstep;
    b.sec = secs;
    b.vecs.clear();
    b.vecs.resize(4 * nrun);
    const size_t es = prec == MO_ED_FP32 ? sizeof(float) : sizeof(double);
    for (int r = 0; r < nrun; ++r)
        for (int k = 0; k < 4; ++k)
            if (int rc = dev_alloc(ctx, b.vecs[4 * r + k], es * (size_t)secs[r].Dpad())) return rc;
    if (int rc = dev_alloc(ctx, b.coef, sizeof(double) * 2 * (nstep + 1) * nrun)) return rc;
    if (int rc = dev_alloc(ctx, b.flags, sizeof(int) * 2 * nrun)) return rc;
    MOED_CUDA(ctx, cudaMemsetAsync(b.coef.p, 0, b.coef.bytes, ctx->stream));
    std::vector<int> fl(2 * nrun);
    for (int r = 0; r < nrun; ++r) {
        fl[2 * r] = 1;
        fl[2 * r + 1] = 0;
    }
    MOED_CUDA(ctx, cudaMemcpyAsync(b.flags.p, fl.data(), sizeof(int) * 2 * nrun,
                                   cudaMemcpyHostToDevice, ctx->stream));
    b.upd_item0.resize(nrun);
    b.upd_nitems.resize(nrun);
    b.hv_item0.resize(nrun);
    b.hv_nitems.resize(nrun);
    b.upd_total = b.hv_total = 0;
    const int kind = prec == MO_ED_FP32 ? HV_F32 : HV_F64;
    // one tile shape for the whole batch: the one tuned for its largest sector
    int big = 0;
    for (int r = 1; r < nrun; ++r)
        if (secs[r].D() > secs[big].D()) big = r;
    if (int rc = hv_prepare(ctx, secs[big], kind, &b.hv_variant, &b.hv_rows)) return rc;
    for (int r = 0; r < nrun; ++r) {
        if (int rc = hv_prepare_rows(ctx, secs[r], kind, b.hv_variant)) return rc;
        b.upd_item0[r] = b.upd_total;
        b.upd_nitems[r] = (int)((secs[r].Dpad() + kVecChunk - 1) / kVecChunk);
        b.upd_total += b.upd_nitems[r];
        b.hv_item0[r] = b.hv_total;
        b.hv_nitems[r] = secs[r].dn->nitems.at(b.hv_rows);
        b.hv_total += b.hv_nitems[r];
    }
    if (int rc = dev_alloc(ctx, b.upd_part, sizeof(double) * std::max(1, b.upd_total))) return rc;
    if (int rc = dev_alloc(ctx, b.hv_part, sizeof(double) * std::max(1, b.hv_total))) return rc;
    return MO_ED_OK;
}

static void lz_fill_dev(LzBatch &b, LzBatchDev &d)
{
    const int nrun = (int)b.sec.size();
    memset(&d, 0, sizeof(d));
    d.nrun = nrun;
    d.total_items = b.upd_total;
    double *coef = (double *)b.coef.p;
    int *fl = (int *)b.flags.p;
    for (int r = 0; r < nrun; ++r) {
        LzRunDev &R = d.run[r];
        for (int k = 0; k < 3; ++k) R.u[k] = b.vecs[4 * r + k].p;
        R.w = b.vecs[4 * r + 3].p;
        R.D = b.sec[r].Dpad();
        R.upd_item0 = b.upd_item0[r];
        R.upd_nitems = b.upd_nitems[r];
        R.hv_item0 = b.hv_item0[r];
        R.hv_nitems = b.hv_nitems[r];
        R.a = coef + (size_t)2 * (b.nstep + 1) * r;
        R.nrm = R.a + (b.nstep + 1);
        R.active = fl + 2 * r;
        R.nstep_calc = fl + 2 * r + 1;
        R.upd_part = (double *)b.upd_part.p + b.upd_item0[r];
        R.hv_part = (double *)b.hv_part.p + b.hv_item0[r];
    }
}

template <typename T>
static int lz_enqueue(mo_ed_ctx *ctx, LzBatch &b, LzBatchDev &d)
{
    const int nrun = d.nrun;
    const int kind = sizeof(T) == 4 ? HV_F32 : HV_F64;
    std::vector<HvJobT<T>> jobs[3];
    for (int k = 0; k < 3; ++k) {
        jobs[k].resize(nrun);
        for (int r = 0; r < nrun; ++r) {
            hv_fill_job<T>(ctx, b.sec[r], b.hv_rows, d.run[r].u[k], d.run[r].w, jobs[k][r]);
            jobs[k][r].dot_partial = d.run[r].hv_part;
            jobs[k][r].active = d.run[r].active;
        }
    }
    const int gv = std::max(1, std::min(d.total_items, ctx->num_sms * 8));
    for (int j = 0; j <= b.nstep; ++j) {
        if (j == 0) {
            k_lz_norm0<T><<<gv, kVecThreads, 0, ctx->stream>>>(d);
        } else {
            k_lz_update<T><<<gv, kVecThreads, 0, ctx->stream>>>(d, j);
        }
        MOED_CHECK_LAUNCH(ctx);
        int rc = (sizeof(T) == 4)
                     ? hv_launch_f32(ctx, b.hv_variant, (const HvJobT<float> *)jobs[j % 3].data(), nrun)
                     : hv_launch_f64(ctx, HV_F64, b.hv_variant, (const HvJobT<double> *)jobs[j % 3].data(), nrun);
        if (rc) return rc;
        k_lz_finalize<<<nrun, kVecThreads, 0, ctx->stream>>>(d, j, b.nstep);
        MOED_CHECK_LAUNCH(ctx);
    }
    return MO_ED_OK;
}

// All nstep+1 steps of a batch (3 launches per step, no host round trip:
// runs stop on the device through their active flags).  With `graph` the
// launches are captured once into a CUDA graph and replayed as one launch;
// a stream that is already being captured gets the plain launches.
template <typename T>
static int lz_steps(mo_ed_ctx *ctx, LzBatch &b, LzBatchDev &d, bool graph)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    MOED_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cs));
    if (!graph || cs != cudaStreamCaptureStatusNone) return lz_enqueue<T>(ctx, b, d);
    MOED_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = lz_enqueue<T>(ctx, b, d);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    cudaGraphExec_t x = nullptr;
    if (rc == MO_ED_OK && e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
    if (g) cudaGraphDestroy(g);
    if (rc != MO_ED_OK || e != cudaSuccess) {
        // a capture the runtime refused: the same launches, issued directly
        cudaGetLastError();
        if (x) cudaGraphExecDestroy(x);
        return lz_enqueue<T>(ctx, b, d);
    }
    e = cudaGraphLaunch(x, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaGraphExecDestroy(x);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphLaunch");
    return MO_ED_OK;
}

int lz_run(mo_ed_ctx *ctx, LzBatch &b, std::vector<std::vector<double>> &a,
           std::vector<std::vector<double>> &bb, std::vector<int> &nstep_calc)
{
    LzBatchDev d;
    lz_fill_dev(b, d);
    const int nrun = d.nrun;
    int rc = (b.prec == MO_ED_FP32) ? lz_steps<float>(ctx, b, d, true) : lz_steps<double>(ctx, b, d, true);
    if (rc) return rc;
    std::vector<double> coef((size_t)2 * (b.nstep + 1) * nrun);
    std::vector<int> fl(2 * nrun);
    MOED_CUDA(ctx, cudaMemcpyAsync(coef.data(), b.coef.p, sizeof(double) * coef.size(),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(fl.data(), b.flags.p, sizeof(int) * fl.size(),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    a.assign(nrun, std::vector<double>(b.nstep + 1, 0.0));
    bb.assign(nrun, std::vector<double>(b.nstep + 1, 0.0));
    nstep_calc.assign(nrun, 0);
    for (int r = 0; r < nrun; ++r) {
        const double *ar = coef.data() + (size_t)2 * (b.nstep + 1) * r;
        const double *nr = ar + (b.nstep + 1);
        nstep_calc[r] = fl[2 * r + 1];
        for (int j = 0; j <= b.nstep; ++j) {
            a[r][j] = ar[j];
            bb[r][j] = (j == 0) ? 0.0 : nr[j];
        }
    }
    return MO_ED_OK;
}

int lanczos_reference(mo_ed_ctx *ctx, const Sector &s, const double *h_vec, int nstep,
                      int *nstep_calc, double *a, double *b)
{
    LzBatch lb;
    const int prec = ctx->opt.precision;
    if (int rc = lz_setup(ctx, lb, {s}, prec, nstep)) return rc;
    const long long Dp = s.Dpad();
    if (prec == MO_ED_FP32) {
        if (int rc = ensure(ctx, ctx->scratch_a, sizeof(double) * Dp)) return rc;
        if (int rc = upload_padded(ctx, s, h_vec, ctx->scratch_a.p, sizeof(double))) return rc;
        if (int rc = convert_f64_to_f32(ctx, (const double *)ctx->scratch_a.p,
                                        (float *)lz_start_vector(lb, 0), Dp))
            return rc;
    } else {
        if (int rc = upload_padded(ctx, s, h_vec, lz_start_vector(lb, 0), sizeof(double))) return rc;
    }
    std::vector<std::vector<double>> A, B;
    std::vector<int> nc;
    if (int rc = lz_run(ctx, lb, A, B, nc)) return rc;
    *nstep_calc = nc[0];
    for (int j = 0; j <= nstep; ++j) {
        a[j] = A[0][j];
        b[j] = B[0][j];
    }
    return MO_ED_OK;
}

// The same recurrence inside a caller-provided device region.  Layout, each
// part starting on a 256-byte boundary: a and nrm [nstep+1] each, the two
// flags, the update and H*v partial sums, u_0, u_1 u_2 (adjacent; for FP32
// runs they first hold the FP64 start vector before its conversion) and w.
namespace {
struct LzRegion {
    size_t coef, flags, upd, hv, u0, u12, w, end;
};

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

LzRegion lz_region(const Sector &s, int prec, int nstep, int hv_rows)
{
    const size_t es = prec == MO_ED_FP32 ? sizeof(float) : sizeof(double);
    const size_t Dp = (size_t)s.Dpad();
    const size_t upd_n = (Dp + kVecChunk - 1) / kVecChunk;
    const size_t hv_n = (size_t)std::max(1, s.dn->nitems.at(hv_rows));
    LzRegion r;
    r.coef = 0;
    r.flags = up256(r.coef + sizeof(double) * 2 * (size_t)(nstep + 1));
    r.upd = up256(r.flags + sizeof(int) * 2);
    r.hv = up256(r.upd + sizeof(double) * upd_n);
    r.u0 = up256(r.hv + sizeof(double) * hv_n);
    r.u12 = up256(r.u0 + es * Dp);
    r.w = up256(r.u12 + std::max(2 * es * Dp, prec == MO_ED_FP32 ? sizeof(double) * Dp : 0));
    r.end = up256(r.w + es * Dp);
    return r;
}

// a = nrm = 0, active = 1, nstep_calc = 0 (the region keeps an earlier call's contents)
__global__ void k_lz_reset(const __grid_constant__ LzBatchDev b, int nstep)
{
    const LzRunDev &R = b.run[blockIdx.x];
    for (int j = threadIdx.x; j <= nstep; j += blockDim.x) {
        R.a[j] = 0.0;
        R.nrm[j] = 0.0;
    }
    if (threadIdx.x == 0) {
        *R.active = 1;
        *R.nstep_calc = 0;
    }
}
}  // namespace

// Load the kernel only the region path uses (lazy loading would otherwise
// load it, and may take device memory, on the first no-allocation call).
int lanczos_region_preload(mo_ed_ctx *ctx)
{
    cudaFuncAttributes a;
    MOED_CUDA(ctx, cudaFuncGetAttributes(&a, k_lz_reset));
    return MO_ED_OK;
}

size_t lanczos_region_bytes(const Sector &s, int prec, int nstep, int hv_rows)
{
    return lz_region(s, prec, nstep, hv_rows).end;
}

int lanczos_reference_in(mo_ed_ctx *ctx, const Sector &s, const double *h_vec, int nstep,
                         int *nstep_calc, double *a, double *b, void *scratch, size_t cap)
{
    const int prec = ctx->opt.precision;
    const int kind = prec == MO_ED_FP32 ? HV_F32 : HV_F64;
    LzBatch lb;
    lb.prec = prec;
    lb.nstep = nstep;
    lb.sec = {s};
    if (int rc = hv_lookup(ctx, s, kind, &lb.hv_variant, &lb.hv_rows)) return rc;
    const LzRegion g = lz_region(s, prec, nstep, lb.hv_rows);
    if (g.end > cap || ((size_t)scratch & 255)) return fail(ctx, MO_ED_ERR_CAPACITY, "Lanczos region too small");
    char *base = (char *)scratch;
    const size_t es = prec == MO_ED_FP32 ? sizeof(float) : sizeof(double);
    const long long Dp = s.Dpad();

    LzBatchDev d;
    memset(&d, 0, sizeof(d));
    d.nrun = 1;
    LzRunDev &R = d.run[0];
    R.u[0] = base + g.u0;
    R.u[1] = base + g.u12;
    R.u[2] = base + g.u12 + es * (size_t)Dp;
    R.w = base + g.w;
    R.D = Dp;
    R.upd_item0 = 0;
    R.upd_nitems = (int)((Dp + kVecChunk - 1) / kVecChunk);
    R.hv_item0 = 0;
    R.hv_nitems = s.dn->nitems.at(lb.hv_rows);
    R.a = (double *)(base + g.coef);
    R.nrm = R.a + (nstep + 1);
    R.active = (int *)(base + g.flags);
    R.nstep_calc = R.active + 1;
    R.upd_part = (double *)(base + g.upd);
    R.hv_part = (double *)(base + g.hv);
    d.total_items = R.upd_nitems;

    k_lz_reset<<<1, kVecThreads, 0, ctx->stream>>>(d, nstep);
    MOED_CHECK_LAUNCH(ctx);
    if (prec == MO_ED_FP32) {
        double *stage = (double *)(base + g.u12);
        if (int rc = upload_padded(ctx, s, h_vec, stage, sizeof(double))) return rc;
        if (int rc = convert_f64_to_f32(ctx, stage, (float *)R.u[0], Dp)) return rc;
        if (int rc = lz_steps<float>(ctx, lb, d, false)) return rc;
    } else {
        if (int rc = upload_padded(ctx, s, h_vec, R.u[0], sizeof(double))) return rc;
        if (int rc = lz_steps<double>(ctx, lb, d, false)) return rc;
    }
    MOED_CUDA(ctx, cudaMemcpyAsync(a, R.a, sizeof(double) * (nstep + 1), cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(b, R.nrm, sizeof(double) * (nstep + 1), cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(nstep_calc, R.nstep_calc, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    b[0] = 0.0;
    return MO_ED_OK;
}

// ---------------------------------------------------------------------------
// thick-restart Lanczos with full reorthogonalisation (diag replacement)
// ---------------------------------------------------------------------------
constexpr int kMaxNcv = 200;
constexpr int kJacobiSmem = 80;   // k_jacobi keeps A and V in shared memory up to this order
constexpr size_t kTrlPoolBytes = (size_t)64 << 20;   // largest pooled Krylov vector

template <typename T>
struct VPtrs {
    const T *p[kMaxNcv + 1];
};

template <typename T>
struct alignas(16) V4Raw {
    T v[4];
};

// part[b][l] = block b's share of V_l . w for l < nv.  Threads walk 4
// consecutive elements at a time (16-byte loads), w once per pass, and keep
// one accumulator per vector: up to kDotPass vectors per pass over w.
// Products are summed in the vector precision over 8 quads (32 elements),
// then in FP64; block sums in FP64 in a fixed order.
constexpr int kDotPass = 24;

template <typename T>
__global__ void __launch_bounds__(kVecThreads)
k_multidot(const __grid_constant__ VPtrs<T> V, int nv, const T *__restrict__ w, long long D,
           double *part)
{
    __shared__ double sred[kVecThreads / 32][kDotPass];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int l0 = 0; l0 < nv; l0 += kDotPass) {
        const int np = min(kDotPass, nv - l0);
        double acc[kDotPass];
        T sacc[kDotPass];
#pragma unroll
        for (int l = 0; l < kDotPass; ++l) {
            acc[l] = 0.0;
            sacc[l] = T(0);
        }
        int cnt = 0;
        bool flushed = false;
        for (long long i = 4 * (blockIdx.x * (long long)blockDim.x + threadIdx.x); i < D;
             i += 4 * (long long)gridDim.x * blockDim.x) {
            T x[4];
            vload4(w + i, x);
#pragma unroll
            for (int l = 0; l < kDotPass; ++l) {
                if (l < np) {
                    T a[4];
                    vload4(V.p[l0 + l] + i, a);
                    sacc[l] += a[0] * x[0] + a[1] * x[1] + a[2] * x[2] + a[3] * x[3];
                }
            }
            if (++cnt == 8) {
#pragma unroll
                for (int l = 0; l < kDotPass; ++l) {
                    acc[l] += (double)sacc[l];
                    sacc[l] = T(0);
                }
                cnt = 0;
                flushed = true;
            }
        }
        // The warp's partials of the np live columns.  When no lane has moved
        // a partial to FP64 yet (at most 8 iterations per thread: small
        // sectors), an FP32 vector's partials are summed in FP32 and widened
        // once: FP64 shuffle trees of every column would bound the kernel on
        // GB300's FP64 rate.
        const bool wide = sizeof(T) == 8 || __any_sync(0xffffffffu, flushed);
#pragma unroll
        for (int l = 0; l < kDotPass; ++l) {
            if (l < np) {
                const double v = wide ? warp_sum(acc[l] + (double)sacc[l]) : (double)warp_sum(sacc[l]);
                if (lane == 0) sred[wid][l] = v;
            }
        }
        __syncthreads();
        for (int l = threadIdx.x; l < np; l += blockDim.x) {
            double t = 0.0;
            for (int q = 0; q < kVecThreads / 32; ++q) t += sred[q][l];
            part[(size_t)blockIdx.x * nv + l0 + l] = t;
        }
        __syncthreads();
    }
}

// out[l] = sum_b part[b][l]  (fixed order)
__global__ void k_reduce_cols(const double *part, int G, int nv, double *out)
{
    for (int l = threadIdx.x; l < nv; l += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < G; ++b) s += part[(size_t)b * nv + l];
        out[l] = s;
    }
}

// part[b][l] = block b's share of V_l . w with FP64 products and sums (an
// FP32 x FP32 product is exact in FP64): the Gram and projected matrices of
// the final Rayleigh-Ritz step.
template <typename TV, typename TW>
__global__ void __launch_bounds__(kVecThreads)
k_multidot_exact(const __grid_constant__ VPtrs<TV> V, int nv, const TW *__restrict__ w, long long D,
                 double *part)
{
    __shared__ double sred[kVecThreads / 32][kDotPass];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int l0 = 0; l0 < nv; l0 += kDotPass) {
        const int np = min(kDotPass, nv - l0);
        double acc[kDotPass];
#pragma unroll
        for (int l = 0; l < kDotPass; ++l) acc[l] = 0.0;
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < D;
             i += (long long)gridDim.x * blockDim.x) {
            const double x = (double)w[i];
#pragma unroll
            for (int l = 0; l < kDotPass; ++l)
                if (l < np) acc[l] += (double)V.p[l0 + l][i] * x;
        }
#pragma unroll
        for (int l = 0; l < kDotPass; ++l) {
            const double v = warp_sum(acc[l]);
            if (lane == 0) sred[wid][l] = v;
        }
        __syncthreads();
        for (int l = threadIdx.x; l < np; l += blockDim.x) {
            double t = 0.0;
            for (int q = 0; q < kVecThreads / 32; ++q) t += sred[q][l];
            part[(size_t)blockIdx.x * nv + l0 + l] = t;
        }
        __syncthreads();
    }
}

// w -= sum_l V_l h_l ; optional partial of ||w||^2.  4 consecutive elements
// per thread, 4 vectors' loads in flight.
template <typename T>
__global__ void __launch_bounds__(kVecThreads)
k_multiaxpy(const __grid_constant__ VPtrs<T> V, int nv, const double *__restrict__ part, int Gm, T *w,
            long long D, double *norm_part)
{
    __shared__ T sh[kMaxNcv + 4];
    __shared__ double sred[32];
    // h_l = sum_b part[b][l] in block order, the sum k_multidot's partials
    // stand for (each block forms it; no separate reduction launch)
    for (int l = threadIdx.x; l < nv + 4; l += blockDim.x) {
        double h = 0.0;
        if (l < nv)
            for (int b = 0; b < Gm; ++b) h += part[(size_t)b * nv + l];
        sh[l] = (T)h;
    }
    __syncthreads();
    // ||w||^2: partials of 4 squares in T, added in FP64 every 8 iterations
    double acc = 0.0;
    T sacc = T(0);
    int cnt = 0;
    for (long long i = 4 * (blockIdx.x * (long long)blockDim.x + threadIdx.x); i < D;
         i += 4 * (long long)gridDim.x * blockDim.x) {
        T s[4] = {T(0), T(0), T(0), T(0)};
        for (int l = 0; l < nv; l += 4) {
            T a[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (l + q < nv) vload4(V.p[l + q] + i, a[q]);
                else a[q][0] = a[q][1] = a[q][2] = a[q][3] = T(0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int e = 0; e < 4; ++e) s[e] += a[q][e] * sh[l + q];
        }
        T x[4];
        vload4(w + i, x);
#pragma unroll
        for (int e = 0; e < 4; ++e) x[e] -= s[e];
        sacc += (x[0] * x[0] + x[1] * x[1]) + (x[2] * x[2] + x[3] * x[3]);
        if (++cnt == 8) {
            acc += (double)sacc;
            sacc = T(0);
            cnt = 0;
        }
        vstore4(w + i, x);
    }
    acc += (double)sacc;
    if (norm_part) {
        double t = block_sum(acc, sred);
        if (threadIdx.x == 0) norm_part[blockIdx.x] = t;
    }
}

// column j of the projected matrix, beta, 1/beta
// p1, p2: the two CGS passes' coefficients as [Gm][nv] partials (Gm = 1:
// already reduced); column j of the projected matrix is h1 + h2 with
// h = sum_b p[b][l] in block order
__global__ void k_cgs_finish(const double *p1, const double *p2, int Gm, int nv, const double *norm_part,
                             int G, double *Hcol, double *beta_out)
{
    __shared__ double sred[32];
    for (int l = threadIdx.x; l < nv; l += blockDim.x) {
        double h1 = 0.0, h2 = 0.0;
        for (int b = 0; b < Gm; ++b) {
            h1 += p1[(size_t)b * nv + l];
            h2 += p2[(size_t)b * nv + l];
        }
        Hcol[l] = h1 + h2;
    }
    double acc = 0.0;
    for (int i = threadIdx.x; i < G; i += blockDim.x) acc += norm_part[i];
    double t = block_sum(acc, sred);
    if (threadIdx.x == 0) {
        double beta = sqrt(t);
        Hcol[nv] = beta;
        beta_out[0] = beta;
        beta_out[1] = beta > 0 ? 1.0 / beta : 0.0;
    }
}

template <typename T>
__global__ void k_scale_copy(const T *__restrict__ in, T *__restrict__ out, long long n,
                             const double *scale)
{
    const T s = (T)*scale;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i] * s;
}

// partial sums of ||y - theta x||^2 (x of type T, y FP64)
template <typename T>
__global__ void k_resid_part(const T *__restrict__ x, const double *__restrict__ y, const double *theta,
                             long long n, double *part)
{
    __shared__ double sred[32];
    const double th = *theta;
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double r = y[i] - th * (double)x[i];
        acc += r * r;
    }
    double t = block_sum(acc, sred);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// deterministic pseudo-random start vector in [-1, 1) (zero in the row pads)
template <typename T>
__global__ void k_random(T *x, long long n, int ld, int nu, unsigned long long seed)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        if ((int)(i % ld) >= nu) {
            x[i] = T(0);
            continue;
        }
        unsigned long long z = (unsigned long long)i + seed * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        x[i] = (T)((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
    }
}

// X_c = sum_l V_l Y[l][c] for c in [c0, c0+KC).  Accumulated in the vector
// precision (FP32 vectors: FP32; GB300 runs FP64 at a small fraction of the
// FP32 rate), coefficients from shared memory, 4 vectors' loads in flight.
template <typename T, int KC>
__global__ void __launch_bounds__(kVecThreads)
k_rotate(const __grid_constant__ VPtrs<T> V, int nv, const double *__restrict__ Y, int ldy, int c0,
         int nc, const __grid_constant__ VPtrs<T> X, long long D)
{
    __shared__ __align__(16) T sy[(kMaxNcv + 4) * KC];
    for (int idx = threadIdx.x; idx < (nv + 4) * KC; idx += blockDim.x) {
        int l = idx / KC, c = idx - l * KC;
        sy[idx] = (c < nc && l < nv) ? (T)Y[(size_t)(c0 + c) * ldy + l] : T(0);
    }
    __syncthreads();
    // 4 consecutive elements per thread (16-byte accesses; D is a multiple
    // of 32 and the vectors are 256-byte aligned)
    for (long long i = 4 * (blockIdx.x * (long long)blockDim.x + threadIdx.x); i < D;
         i += 4 * (long long)gridDim.x * blockDim.x) {
        T acc[KC][4];
#pragma unroll
        for (int c = 0; c < KC; ++c)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[c][e] = T(0);
        for (int l = 0; l < nv; l += 4) {
            T v[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (l + q < nv) vload4(V.p[l + q] + i, v[q]);
                else v[q][0] = v[q][1] = v[q][2] = v[q][3] = T(0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int c = 0; c < KC; ++c) {
                    const T y = sy[(l + q) * KC + c];
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[c][e] += v[q][e] * y;
                }
        }
#pragma unroll
        for (int c = 0; c < KC; ++c)
            if (c < nc) vstore4(const_cast<T *>(X.p[c]) + i, acc[c]);
    }
}

// FP64 parallel (round-robin) two-sided Jacobi on the symmetrized projected
// matrix.  M[i][j] (i <= j) = kept-block diag(theta) for j < kk, else the
// computed column j (Hp[j*ldh + i]).  One CTA.  Outputs ascending eigenvalues
// and the matching eigenvectors (column-major m x m).
__global__ void k_jacobi(const double *__restrict__ Hp, int ldh, int m, int kk,
                         const double *__restrict__ theta, double *Ag, double *Vg, double *evals,
                         double *evecs, int max_sweeps)
{
    __shared__ double s_c[kMaxNcv / 2 + 1], s_s[kMaxNcv / 2 + 1];
    __shared__ int s_p[kMaxNcv / 2 + 1], s_q[kMaxNcv / 2 + 1];
    extern __shared__ double s_work[];
    const int n = m + (m & 1);
    const int half = n / 2;
    // working matrices in shared memory when the launch provides room (n <= kJacobiSmem)
    double *A = n <= kJacobiSmem ? s_work : Ag;
    double *V = n <= kJacobiSmem ? s_work + (size_t)n * n : Vg;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        const int i = idx % n, j = idx / n;
        double v;
        if (i >= m || j >= m) {
            v = 0.0;
        } else {
            const int r = min(i, j), c = max(i, j);
            if (c < kk) v = (r == c) ? theta[r] : 0.0;
            else v = Hp[(size_t)c * ldh + r];
        }
        A[idx] = v;
        V[idx] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    // Off-diagonal entries below the rounding level of the matrix, 4e-16
    // ||A||_F, are left alone: rotations keep regenerating entries of that
    // size, so a smaller threshold never lets a sweep rotate nothing.  An
    // entry delta left there moves the eigenvalues by delta^2 / gap.
    __shared__ double s_red[32], s_thr;
    {
        double acc = 0.0;
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) acc += A[idx] * A[idx];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
            s_thr = 4e-16 * sqrt(t);
        }
        __syncthreads();
    }
    const double thr = s_thr;
    __shared__ int s_rot;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        // threshold Jacobi: a sweep that rotates nothing ends the iteration
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        for (int rnd = 0; rnd < n - 1; ++rnd) {
            for (int k = threadIdx.x; k < half; k += blockDim.x) {
                int p, q;
                if (k == 0) {
                    p = 0;
                    q = (rnd % (n - 1)) + 1;
                } else {
                    p = ((rnd + k) % (n - 1)) + 1;
                    q = ((rnd - k + (n - 1)) % (n - 1)) + 1;
                }
                const double apq = A[(size_t)q * n + p];
                const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                double c = 1.0, s = 0.0;
                if (fabs(apq) > fmax(1e-17 * sqrt(fabs(app) * fabs(aqq)), thr) + 1e-300) {
                    atomicAdd(&s_rot, 1);
                    const double tau = (aqq - app) / (2.0 * apq);
                    const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                    c = 1.0 / sqrt(1.0 + t * t);
                    s = t * c;
                }
                s_p[k] = p;
                s_q[k] = q;
                s_c[k] = c;
                s_s[k] = s;
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < half * n; idx += blockDim.x) {   // A <- A J
                const int k = idx / n, r = idx - k * n;
                const int p = s_p[k], q = s_q[k];
                const double c = s_c[k], s = s_s[k];
                const double arp = A[(size_t)p * n + r], arq = A[(size_t)q * n + r];
                A[(size_t)p * n + r] = c * arp - s * arq;
                A[(size_t)q * n + r] = s * arp + c * arq;
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < half * n; idx += blockDim.x) {   // A <- J^T A
                const int k = idx / n, col = idx - k * n;
                const int p = s_p[k], q = s_q[k];
                const double c = s_c[k], s = s_s[k];
                const double apc = A[(size_t)col * n + p], aqc = A[(size_t)col * n + q];
                A[(size_t)col * n + p] = c * apc - s * aqc;
                A[(size_t)col * n + q] = s * apc + c * aqc;
            }
            for (int idx = threadIdx.x; idx < half * n; idx += blockDim.x) {   // V <- V J
                const int k = idx / n, r = idx - k * n;
                const int p = s_p[k], q = s_q[k];
                const double c = s_c[k], s = s_s[k];
                const double vrp = V[(size_t)p * n + r], vrq = V[(size_t)q * n + r];
                V[(size_t)p * n + r] = c * vrp - s * vrq;
                V[(size_t)q * n + r] = s * vrp + c * vrq;
            }
            __syncthreads();
        }
        if (s_rot == 0) break;
        __syncthreads();
    }
    // sort ascending (pad index, if any, excluded)
    __shared__ int order[kMaxNcv + 1];
    if (threadIdx.x == 0) {
        for (int i = 0; i < m; ++i) order[i] = i;
        for (int i = 1; i < m; ++i) {
            int t = order[i];
            double v = A[(size_t)t * n + t];
            int k = i - 1;
            while (k >= 0 && A[(size_t)order[k] * n + order[k]] > v) {
                order[k + 1] = order[k];
                --k;
            }
            order[k + 1] = t;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) evals[i] = A[(size_t)order[i] * n + order[i]];
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int r = idx % m, c = idx / m;
        evecs[idx] = V[(size_t)order[c] * n + r];
    }
}

// dynamic shared memory of a k_jacobi launch of order m
static size_t jacobi_smem(int m)
{
    const int n = m + (m & 1);
    return n <= kJacobiSmem ? 2 * sizeof(double) * (size_t)n * n : 0;
}

// Generalized symmetric problem P c = lambda S c (k x k, column-major, upper
// triangles of P and S filled): S = L L^T (Cholesky), A = L^-1 P L^-T.  One
// thread; k is the number of Ritz vectors.  flag = 1 if S is not positive.
__global__ void k_gen_eig_prep(const double *P, const double *S, int k, double *A, double *L, double *flag)
{
    flag[0] = 0.0;
    for (int j = 0; j < k; ++j)
        for (int i = 0; i < k; ++i) L[(size_t)j * k + i] = 0.0;
    for (int j = 0; j < k; ++j) {
        double d = S[(size_t)j * k + j];
        for (int t = 0; t < j; ++t) d -= L[(size_t)t * k + j] * L[(size_t)t * k + j];
        if (!(d > 0.0)) {
            flag[0] = 1.0;
            return;
        }
        const double ljj = sqrt(d);
        L[(size_t)j * k + j] = ljj;
        for (int i = j + 1; i < k; ++i) {
            double v = S[(size_t)i * k + j];   // S(j,i), upper triangle
            for (int t = 0; t < j; ++t) v -= L[(size_t)t * k + i] * L[(size_t)t * k + j];
            L[(size_t)j * k + i] = v / ljj;
        }
    }
    // B = L^-1 Psym (column by column), then A = L^-1 B^T
    for (int c = 0; c < k; ++c) {
        for (int i = 0; i < k; ++i) {
            const double pic = 0.5 * (P[(size_t)c * k + i] + P[(size_t)i * k + c]);
            double v = pic;
            for (int t = 0; t < i; ++t) v -= L[(size_t)t * k + i] * A[(size_t)c * k + t];
            A[(size_t)c * k + i] = v / L[(size_t)i * k + i];
        }
    }
    // A currently holds B = L^-1 Psym; form L^-1 B^T in place via a copy
    for (int r = 0; r < k; ++r)
        for (int c = r + 1; c < k; ++c) {
            const double t = A[(size_t)c * k + r];
            A[(size_t)c * k + r] = A[(size_t)r * k + c];
            A[(size_t)r * k + c] = t;
        }
    for (int c = 0; c < k; ++c) {
        for (int i = 0; i < k; ++i) {
            double v = A[(size_t)c * k + i];
            for (int t = 0; t < i; ++t) v -= L[(size_t)t * k + i] * A[(size_t)c * k + t];
            A[(size_t)c * k + i] = v / L[(size_t)i * k + i];
        }
    }
    for (int r = 0; r < k; ++r)   // symmetrize
        for (int c = r + 1; c < k; ++c) {
            const double v = 0.5 * (A[(size_t)c * k + r] + A[(size_t)r * k + c]);
            A[(size_t)c * k + r] = v;
            A[(size_t)r * k + c] = v;
        }
}

// C = L^-T W (back substitution per column)
__global__ void k_gen_eig_post(const double *L, const double *W, int k, double *C)
{
    for (int c = 0; c < k; ++c)
        for (int i = k - 1; i >= 0; --i) {
            double v = W[(size_t)c * k + i];
            for (int t = i + 1; t < k; ++t) v -= L[(size_t)i * k + t] * C[(size_t)c * k + t];
            C[(size_t)c * k + i] = v / L[(size_t)i * k + i];
        }
}

template <typename T>
static VPtrs<T> make_ptrs(const std::vector<DevBuf *> &v, int n)
{
    VPtrs<T> p;
    memset(&p, 0, sizeof(p));
    for (int i = 0; i < n; ++i) p.p[i] = (const T *)v[i]->p;
    return p;
}

// blocks of k_multidot over a vector of D elements
static int multidot_grid(const mo_ed_ctx *ctx, long long D)
{
    return (int)std::max(1LL, std::min((D / 4 + kVecThreads - 1) / kVecThreads, (long long)ctx->num_sms * 4));
}

// part: two passes' partials of ortho_pass_stride(ctx) doubles each, then
// the two passes' reduced coefficients (kMaxNcv + 2 each)
static long long ortho_pass_stride(const mo_ed_ctx *ctx) { return (long long)(kMaxNcv + 2) * ctx->num_sms * 4; }
static size_t ortho_part_doubles(const mo_ed_ctx *ctx) { return 2 * (size_t)ortho_pass_stride(ctx) + 2 * (kMaxNcv + 2); }
// up to this many multi-dot blocks every multi-axpy block adds the partials
// itself; beyond, one extra launch reduces them (each of the multi-axpy's
// blocks redoing Gm x nv FP64 additions would cost more than the launch)
constexpr int kFuseReduceBlocks = 32;

// Where the coefficients of the two CGS passes of an orthogonalize call are:
// [Gm][nv] partials, Gm = 1 once reduced.
struct OrthoCoef {
    const double *p[2];
    int Gm;
};

// classical Gram-Schmidt, twice: w -= V (V^T w).  Each pass is a multi-dot
// into per-block partials and a multi-axpy, which for small grids adds the
// partials itself; pass 1 leaves the partials of ||w||^2 in norm_part.
template <typename T>
static int orthogonalize(mo_ed_ctx *ctx, const std::vector<DevBuf *> &basis, int nv, T *w,
                         long long D, double *part, double *norm_part, int G, OrthoCoef *coef = nullptr)
{
    VPtrs<T> P = make_ptrs<T>(basis, nv);
    const int Gm = multidot_grid(ctx, D);
    const bool fuse = Gm <= kFuseReduceBlocks;
    for (int pass = 0; pass < 2; ++pass) {
        double *pp = part + pass * ortho_pass_stride(ctx);
        double *hp = part + 2 * ortho_pass_stride(ctx) + pass * (kMaxNcv + 2);
        k_multidot<T><<<Gm, kVecThreads, 0, ctx->stream>>>(P, nv, w, D, pp);
        MOED_CHECK_LAUNCH(ctx);
        if (!fuse) {
            k_reduce_cols<<<1, 256, 0, ctx->stream>>>(pp, Gm, nv, hp);
            MOED_CHECK_LAUNCH(ctx);
        }
        k_multiaxpy<T><<<G, kVecThreads, 0, ctx->stream>>>(P, nv, fuse ? pp : hp, fuse ? Gm : 1, w, D,
                                                           pass == 1 ? norm_part : nullptr);
        MOED_CHECK_LAUNCH(ctx);
        if (coef) coef->p[pass] = fuse ? pp : hp;
    }
    if (coef) coef->Gm = fuse ? Gm : 1;
    return MO_ED_OK;
}

template <typename T>
static int trl_solve(mo_ed_ctx *ctx, const Sector &s, int nev, std::vector<double> &vals,
                     std::vector<DevBuf> *vecs)
{
    const long long D = s.D();          // dimension
    const long long Dp = s.Dpad();      // device elements (row pads are zero)
    const int prec = sizeof(T) == 4 ? MO_ED_FP32 : MO_ED_FP64;
    const int kind = sizeof(T) == 4 ? HV_F32 : HV_F64;
    const int nwant = (int)std::min<long long>(nev, D);
    int ncv = ctx->opt.gs_ncv > 0 ? ctx->opt.gs_ncv : std::max(2 * nwant + 10, 40);
    ncv = (int)std::min<long long>(std::min(ncv, kMaxNcv - 1), D);
    if (ncv < nwant) return fail(ctx, MO_ED_ERR_ARG, "gs_ncv smaller than nev");
    int kkeep = std::min(ncv - 1, nwant + (ncv - nwant) / 2);
    if (kkeep < nwant) kkeep = nwant;
    // Residual tolerance relative to ||H||.  FP32 vectors carry a noise floor
    // near eps_32*||H||; the stagnation test below accepts Ritz pairs that
    // stop improving there.
    const double tol = ctx->opt.gs_tol > 0 ? ctx->opt.gs_tol : (prec == MO_ED_FP32 ? 1e-7 : 1e-11);
    std::vector<double> res_hist;
    const size_t vb = sizeof(T) * (size_t)Dp;

    // Krylov vectors: sectors up to kTrlPoolBytes per vector reuse buffers kept
    // in the context (many small sectors: no allocation per sector)
    std::vector<DevBuf> local;
    std::vector<DevBuf> &store = vb <= kTrlPoolBytes ? ctx->trl_pool : local;
    if (store.size() < (size_t)(ncv + 2 + kkeep)) store.resize(ncv + 2 + kkeep);
    for (int i = 0; i < ncv + 2 + kkeep; ++i)
        if (int rc = ensure(ctx, store[i], vb)) return rc;
    std::vector<DevBuf *> V(ncv + 1);
    for (int i = 0; i <= ncv; ++i) V[i] = &store[i];
    DevBuf *W = &store[ncv + 1];
    std::vector<DevBuf *> spare(kkeep);
    for (int i = 0; i < kkeep; ++i) spare[i] = &store[ncv + 2 + i];

    const int G = (int)std::max(1LL, std::min((Dp + kVecThreads - 1) / kVecThreads, (long long)ctx->num_sms * 4));
    const int n2 = ncv + 2;
    std::vector<DevBuf> &sm = ctx->trl_small;   // projected-problem workspace, kept in the context
    if (sm.size() < 12) sm.resize(12);
    DevBuf &dHp = sm[0], &dh1 = sm[1], &dh2 = sm[2], &dpart = sm[3], &dnorm = sm[4], &dbeta = sm[5];
    DevBuf &devecs = sm[9], &dsc = sm[11];
    if (int rc = ensure(ctx, dHp, sizeof(double) * (size_t)n2 * n2)) return rc;
    if (int rc = ensure(ctx, dh1, sizeof(double) * n2)) return rc;
    if (int rc = ensure(ctx, dh2, sizeof(double) * n2)) return rc;
    if (int rc = ensure(ctx, dpart, sizeof(double) * ortho_part_doubles(ctx))) return rc;
    if (int rc = ensure(ctx, dnorm, sizeof(double) * G)) return rc;
    if (int rc = ensure(ctx, dbeta, sizeof(double) * 2)) return rc;
    if (int rc = ensure(ctx, devecs, sizeof(double) * (size_t)n2 * n2)) return rc;
    if (int rc = ensure(ctx, dsc, sizeof(double) * 4)) return rc;
    MOED_CUDA(ctx, cudaMemsetAsync(dHp.p, 0, dHp.bytes, ctx->stream));
    double *Hp = (double *)dHp.p;
    const int ldh = n2;

    long long matvecs = 0;
    auto hv = [&](const void *x, void *y) -> int {
        ++matvecs;
        return hv_single(ctx, s, kind, x, y);
    };
    auto normalize_into = [&](T *src, DevBuf *dst) -> int {
        // dst = src / ||src||
        if (int rc = dot_dev(ctx, prec, src, prec, src, Dp, (double *)dsc.p)) return rc;
        double nrm2;
        MOED_CUDA(ctx, cudaMemcpyAsync(&nrm2, dsc.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        double inv = nrm2 > 0 ? 1.0 / std::sqrt(nrm2) : 0.0;
        MOED_CUDA(ctx, cudaMemcpyAsync((double *)dsc.p + 1, &inv, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        k_scale_copy<T><<<G, kVecThreads, 0, ctx->stream>>>(src, (T *)dst->p, Dp, (double *)dsc.p + 1);
        MOED_CHECK_LAUNCH(ctx);
        return MO_ED_OK;
    };

    // start vector
    unsigned long long seed = 0x5eedULL + 977ULL * (unsigned)s.ne_up + 131ULL * (unsigned)s.ne_down;
    k_random<T><<<G, kVecThreads, 0, ctx->stream>>>((T *)W->p, Dp, s.ld(), s.up->n, seed);
    MOED_CHECK_LAUNCH(ctx);
    if (int rc = normalize_into((T *)W->p, V[0])) return rc;

    int k = 0;           // kept Ritz vectors at the front of V
    int m = ncv;
    std::vector<double> theta(n2), ylast(n2), evecs_h;
    bool done = false;
    int cycle = 0;
    double anorm = 0.0;
    for (; cycle < ctx->opt.gs_maxcycles && !done; ++cycle) {
        m = ncv;
        // The steps of a cycle run without a host round trip; the diagonal and
        // the betas are read once at the end of the cycle.  A step whose beta
        // falls below the breakdown threshold ends the cycle there (its Krylov
        // space is invariant; later steps of the cycle are discarded).
        for (int j = k; j < ncv; ++j) {
            if (int rc = hv(V[j]->p, W->p)) return rc;
            const bool last = j + 1 >= D;   // Krylov space is the whole sector
            OrthoCoef oc;
            if (int rc = orthogonalize<T>(ctx, V, j + 1, (T *)W->p, Dp, (double *)dpart.p, (double *)dnorm.p, G, &oc))
                return rc;
            k_cgs_finish<<<1, 256, 0, ctx->stream>>>(oc.p[0], oc.p[1], oc.Gm, j + 1, (const double *)dnorm.p, G,
                                                     Hp + (size_t)j * ldh, (double *)dbeta.p);
            MOED_CHECK_LAUNCH(ctx);
            if (!last) {
                k_scale_copy<T><<<G, kVecThreads, 0, ctx->stream>>>((const T *)W->p, (T *)V[j + 1]->p, Dp,
                                                                    (double *)dbeta.p + 1);
                MOED_CHECK_LAUNCH(ctx);
            }
            if (last) {
                m = j + 1;
                break;
            }
        }
        bool broke = false;
        std::vector<double> hc((size_t)ldh * m);
        {
            MOED_CUDA(ctx, cudaMemcpyAsync(hc.data(), Hp, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost, ctx->stream));
            MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int j = k; j < m; ++j) {
                const double diag = hc[(size_t)j * ldh + j], beta = hc[(size_t)j * ldh + j + 1];
                anorm = std::max(anorm, std::fabs(diag) + beta);
                if (j + 1 >= D) break;
                const double bd = (prec == MO_ED_FP32 ? 1e-5 : 1e-12) * std::max(anorm, 1.0);
                if (beta <= bd) {
                    m = j + 1;
                    broke = true;
                    break;
                }
            }
        }
        // Rayleigh-Ritz on span V[0..m-1], on the host as PARPACK does: the
        // projected matrix is diag(theta) on the kept block and the columns
        // of Hp after it (its entries are on the host already)
        evecs_h.resize((size_t)m * m);
        {
            std::vector<double> Am((size_t)m * m);
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < m; ++j) {
                    const int r = std::min(i, j), c = std::max(i, j);
                    Am[(size_t)i * m + j] = c < k ? (r == c ? theta[r] : 0.0) : hc[(size_t)c * ldh + r];
                }
            if (!sym_eig(m, Am, theta.data(), evecs_h.data()))
                return fail(ctx, MO_ED_ERR_NOCONV, "projected eigenproblem did not converge");
            MOED_CUDA(ctx, cudaMemcpyAsync(devecs.p, evecs_h.data(), sizeof(double) * (size_t)m * m,
                                           cudaMemcpyHostToDevice, ctx->stream));
        }
        const double beta_m = m < D ? hc[(size_t)(m - 1) * ldh + m] : 0.0;
        int nconv = 0;
        double maxres = 0.0;
        for (int i = 0; i < std::min(nwant, m); ++i) {
            double res = std::fabs(beta_m * evecs_h[(size_t)i * m + (m - 1)]);
            maxres = std::max(maxres, res);
            if (res <= tol * std::max(anorm, 1.0) && nconv == i) ++nconv;
        }
        res_hist.push_back(maxres);
        ctx->diag_res_est = maxres;
        const size_t h = res_hist.size();
        const bool stalled = prec == MO_ED_FP32 && h >= 6 && maxres <= 1e-6 * std::max(anorm, 1.0) &&
                             maxres > 0.9 * res_hist[h - 6];
        if (nconv >= nwant || m >= D || stalled) {
            done = true;
            break;
        }
        // thick restart: keep kkeep lowest Ritz vectors, then the residual vector
        // after a breakdown every Ritz vector of the invariant subspace is kept
        const int kk = broke ? std::min(kkeep, m) : std::min(kkeep, m - 1);
        VPtrs<T> P = make_ptrs<T>(V, m);
        for (int c0 = 0; c0 < kk; c0 += 8) {
            const int nc = std::min(8, kk - c0);
            std::vector<DevBuf *> outs(spare.begin() + c0, spare.begin() + c0 + nc);
            VPtrs<T> X = make_ptrs<T>(outs, nc);
            k_rotate<T, 8><<<G, kVecThreads, 0, ctx->stream>>>(P, m, (const double *)devecs.p, m, c0, nc, X, Dp);
            MOED_CHECK_LAUNCH(ctx);
        }
        for (int i = 0; i < kk; ++i) std::swap(V[i], spare[i]);
        if (broke) {
            // invariant subspace: continue from a fresh random direction
            k_random<T><<<G, kVecThreads, 0, ctx->stream>>>((T *)W->p, Dp, s.ld(), s.up->n,
                                                            seed + 7919ULL * (cycle + 1) * kMaxNcv);
            MOED_CHECK_LAUNCH(ctx);
            if (int rc = orthogonalize<T>(ctx, V, kk, (T *)W->p, Dp, (double *)dpart.p, (double *)dnorm.p, G))
                return rc;
            if (int rc = normalize_into((T *)W->p, V[kk])) return rc;
        } else {
            std::swap(V[kk], V[m]);
        }
        k = kk;
        MOED_CUDA(ctx, cudaMemsetAsync(dHp.p, 0, dHp.bytes, ctx->stream));
    }
    if (!done) return fail(ctx, MO_ED_ERR_NOCONV, "eigensolver did not converge");

    // Ritz vectors, then an FP64-accurate Rayleigh-Ritz on their span:
    // P = X^T H X with H applied in FP64 accumulation, S = X^T X (X in the
    // vector precision), P c = lambda S c.  Eigenvalues of a cluster of
    // near-degenerate states are then accurate to ~res^2 / (gap to the rest
    // of the spectrum), whatever the mixing inside the cluster.
    vals.assign(nev, DBL_MAX);
    const int nout = nwant;
    // X, HX, HX2 and the small arrays come from the context's pool for sectors
    // up to kTrlPoolBytes per FP64 vector; the refined vectors X2 are returned
    const size_t vb64 = sizeof(double) * (size_t)Dp;
    std::vector<DevBuf> rr_local;
    std::vector<DevBuf> &rp = vb64 <= kTrlPoolBytes ? ctx->rr_pool : rr_local;
    if (rp.size() < (size_t)(3 * nout + 2)) rp.resize(3 * nout + 2);
    DevBuf *X = &rp[0], *HX = &rp[nout], *HX2 = &rp[2 * nout];
    for (int i = 0; i < nout; ++i) {
        if (int rc = ensure(ctx, X[i], vb)) return rc;
        if (int rc = ensure(ctx, HX[i], vb64)) return rc;
        if (int rc = ensure(ctx, HX2[i], vb64)) return rc;
    }
    {
        VPtrs<T> P = make_ptrs<T>(V, m);
        for (int c0 = 0; c0 < nout; c0 += 8) {
            const int nc = std::min(8, nout - c0);
            std::vector<DevBuf *> outs;
            for (int c = 0; c < nc; ++c) outs.push_back(&X[c0 + c]);
            VPtrs<T> Xp = make_ptrs<T>(outs, nc);
            k_rotate<T, 8><<<G, kVecThreads, 0, ctx->stream>>>(P, m, (const double *)devecs.p, m, c0, nc, Xp, Dp);
            MOED_CHECK_LAUNCH(ctx);
        }
    }
    const int hk = prec == MO_ED_FP32 ? HV_MIXED : HV_F64;
    for (int i = 0; i < nout; ++i) {
        if (int rc = hv_single(ctx, s, hk, X[i].p, HX[i].p)) return rc;
        ++matvecs;
    }
    DevBuf &dPS = rp[3 * nout], &dRR = rp[3 * nout + 1];
    if (int rc = ensure(ctx, dPS, sizeof(double) * 2 * (size_t)nout * nout)) return rc;
    const size_t k2 = (size_t)nout * nout, kp2 = (size_t)(nout + 1) * (nout + 1);
    if (int rc = ensure(ctx, dRR, sizeof(double) * (4 * k2 + 2 * kp2 + nout + 4))) return rc;
    double *dP = (double *)dPS.p, *dS = dP + (size_t)nout * nout;
    {   // P[i][j] = X_i . H X_j, S[i][j] = X_i . X_j: one exact multi-dot per column
        std::vector<DevBuf *> xin(nout);
        for (int i = 0; i < nout; ++i) xin[i] = &X[i];
        VPtrs<T> Px = make_ptrs<T>(xin, nout);
        const int Gd = (int)std::max(1LL, std::min((Dp + kVecThreads - 1) / kVecThreads, (long long)ctx->num_sms * 4));
        for (int j = 0; j < nout; ++j) {
            k_multidot_exact<T, double><<<Gd, kVecThreads, 0, ctx->stream>>>(Px, nout, (const double *)HX[j].p, Dp,
                                                                              (double *)dpart.p);
            MOED_CHECK_LAUNCH(ctx);
            k_reduce_cols<<<1, 256, 0, ctx->stream>>>((const double *)dpart.p, Gd, nout, dP + (size_t)j * nout);
            MOED_CHECK_LAUNCH(ctx);
            k_multidot_exact<T, T><<<Gd, kVecThreads, 0, ctx->stream>>>(Px, nout, (const T *)X[j].p, Dp,
                                                                         (double *)dpart.p);
            MOED_CHECK_LAUNCH(ctx);
            k_reduce_cols<<<1, 256, 0, ctx->stream>>>((const double *)dpart.p, Gd, nout, dS + (size_t)j * nout);
            MOED_CHECK_LAUNCH(ctx);
        }
    }
    double *rr = (double *)dRR.p;
    double *dGA = rr, *dL = dGA + k2, *dW = dL + k2, *dC = dW + k2;
    double *dJa = dC + k2, *dJv = dJa + kp2;          // Jacobi work (n x n, n = k rounded up to even)
    double *dEv = dJv + kp2, *dFlag = dEv + nout;
    k_gen_eig_prep<<<1, 1, 0, ctx->stream>>>(dP, dS, nout, dGA, dL, dFlag);
    MOED_CHECK_LAUNCH(ctx);
    MOED_CUDA(ctx, cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)jacobi_smem(kJacobiSmem)));
    k_jacobi<<<1, 256, jacobi_smem(nout), ctx->stream>>>(dGA, nout, nout, 0, dEv, dJa, dJv, dEv, dW, 60);
    MOED_CHECK_LAUNCH(ctx);
    k_gen_eig_post<<<1, 1, 0, ctx->stream>>>(dL, dW, nout, dC);
    MOED_CHECK_LAUNCH(ctx);
    std::vector<double> ev(nout);
    double flag = 0.0;
    MOED_CUDA(ctx, cudaMemcpyAsync(ev.data(), dEv, sizeof(double) * nout, cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(&flag, dFlag, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (flag != 0.0) return fail(ctx, MO_ED_ERR_NOCONV, "Ritz vectors numerically dependent");
    // refined vectors X C and their images (H X) C
    std::vector<DevBuf> X2(nout);
    for (auto &b : X2)
        if (int rc = dev_alloc(ctx, b, vb)) return rc;
    {
        std::vector<DevBuf *> xin, hin;
        for (int i = 0; i < nout; ++i) {
            xin.push_back(&X[i]);
            hin.push_back(&HX[i]);
        }
        VPtrs<T> Px = make_ptrs<T>(xin, nout);
        VPtrs<double> Ph = make_ptrs<double>(hin, nout);
        for (int c0 = 0; c0 < nout; c0 += 8) {
            const int nc = std::min(8, nout - c0);
            std::vector<DevBuf *> ox, oh;
            for (int c = 0; c < nc; ++c) {
                ox.push_back(&X2[c0 + c]);
                oh.push_back(&HX2[c0 + c]);
            }
            VPtrs<T> Ox = make_ptrs<T>(ox, nc);
            VPtrs<double> Oh = make_ptrs<double>(oh, nc);
            k_rotate<T, 8><<<G, kVecThreads, 0, ctx->stream>>>(Px, nout, dC, nout, c0, nc, Ox, Dp);
            MOED_CHECK_LAUNCH(ctx);
            k_rotate<double, 8><<<G, kVecThreads, 0, ctx->stream>>>(Ph, nout, dC, nout, c0, nc, Oh, Dp);
            MOED_CHECK_LAUNCH(ctx);
        }
    }
    double res_true = 0.0;
    for (int i = 0; i < nout; ++i) {
        vals[i] = ev[i];
        // true residual ||H x - E x|| / ||x|| in FP64
        double th = ev[i];
        MOED_CUDA(ctx, cudaMemcpyAsync((double *)dsc.p + 2, &th, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        k_resid_part<T><<<G, kVecThreads, 0, ctx->stream>>>((const T *)X2[i].p, (const double *)HX2[i].p,
                                                            (const double *)dsc.p + 2, Dp, (double *)dnorm.p);
        MOED_CHECK_LAUNCH(ctx);
        k_sum_parts<<<1, kVecThreads, 0, ctx->stream>>>((const double *)dnorm.p, G, (double *)dsc.p + 3);
        MOED_CHECK_LAUNCH(ctx);
        if (int rc = dot_dev(ctx, prec, X2[i].p, prec, X2[i].p, Dp, (double *)dsc.p + 1)) return rc;
        double rr2[3];
        MOED_CUDA(ctx, cudaMemcpyAsync(rr2, (double *)dsc.p + 1, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        res_true = std::max(res_true, std::sqrt(rr2[2] / rr2[0]));
    }
    ctx->diag_cycles = cycle + 1;
    ctx->diag_matvecs = matvecs;
    ctx->diag_res_true = res_true;
    if (vecs) {
        vecs->clear();
        vecs->resize(nout);
        for (int i = 0; i < nout; ++i) std::swap((*vecs)[i], X2[i]);
    }
    return MO_ED_OK;
}

// FP64 refinement of an FP32 eigenvector x (Dpad elements of sector s).
// The FP32 eigensolve leaves a residual near eps_32 * ||H|| in x, spread over
// the whole spectrum.  A Lanczos run of kRefineSteps FP64 steps from x (full
// CGS2 reorthogonalisation) and a Rayleigh-Ritz on its Krylov space damp every
// component away from the eigenvalue; the Ritz vector with the largest weight
// on x is the refined vector.  Rounds repeat from it until the Ritz residual
// is below 1e-9 * ||H|| or kRefineRounds have run: G(i w_n) inherits the
// vector's error to first order, and a residual 1e-9 * ||H|| leaves it near
// 1e-8 relative.  out receives the FP64 vector; res the last Ritz residual.
int refine_fp64(mo_ed_ctx *ctx, const Sector &s, const float *x, DevBuf &out, double *res)
{
    constexpr int kRefineSteps = 16, kRefineRounds = 3;
    const long long D = s.D(), Dp = s.Dpad();
    const int m0 = (int)std::min<long long>(kRefineSteps, D);
    const size_t vb = sizeof(double) * (size_t)Dp;
    std::vector<DevBuf> buf(m0 + 1);
    for (auto &b : buf)
        if (int rc = dev_alloc(ctx, b, vb)) return rc;
    std::vector<DevBuf *> V(m0);
    for (int i = 0; i < m0; ++i) V[i] = &buf[i];
    DevBuf *W = &buf[m0];
    const int G = (int)std::max(1LL, std::min((Dp + kVecThreads - 1) / kVecThreads, (long long)ctx->num_sms * 4));
    const int n2 = m0 + 2, ldh = n2;
    DevBuf dHp, dh1, dh2, dpart, dnorm, dbeta, devecs, dsc;
    if (int rc = dev_alloc(ctx, dHp, sizeof(double) * (size_t)n2 * n2)) return rc;
    if (int rc = dev_alloc(ctx, dh1, sizeof(double) * n2)) return rc;
    if (int rc = dev_alloc(ctx, dh2, sizeof(double) * n2)) return rc;
    if (int rc = dev_alloc(ctx, dpart, sizeof(double) * ortho_part_doubles(ctx))) return rc;
    if (int rc = dev_alloc(ctx, dnorm, sizeof(double) * G)) return rc;
    if (int rc = dev_alloc(ctx, dbeta, sizeof(double) * 2)) return rc;
    if (int rc = dev_alloc(ctx, devecs, sizeof(double) * (size_t)n2 * n2)) return rc;
    if (int rc = dev_alloc(ctx, dsc, sizeof(double) * 2)) return rc;
    if (int rc = dev_alloc(ctx, out, vb)) return rc;
    if (int rc = convert_f32_to_f64(ctx, x, (double *)out.p, Dp)) return rc;
    double *Hp = (double *)dHp.p;
    *res = -1.0;
    for (int round = 0; round < kRefineRounds; ++round) {
        // V[0] = out / ||out||
        if (int rc = dot_dev(ctx, MO_ED_FP64, out.p, MO_ED_FP64, out.p, Dp, (double *)dsc.p)) return rc;
        double nrm2 = 0.0;
        MOED_CUDA(ctx, cudaMemcpyAsync(&nrm2, dsc.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (!(nrm2 > 0)) return fail(ctx, MO_ED_ERR_NOCONV, "zero eigenvector in FP64 refinement");
        const double inv = 1.0 / std::sqrt(nrm2);
        MOED_CUDA(ctx, cudaMemcpyAsync((double *)dsc.p + 1, &inv, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        k_scale_copy<double><<<G, kVecThreads, 0, ctx->stream>>>((const double *)out.p, (double *)V[0]->p, Dp,
                                                                 (double *)dsc.p + 1);
        MOED_CHECK_LAUNCH(ctx);
        MOED_CUDA(ctx, cudaMemsetAsync(dHp.p, 0, dHp.bytes, ctx->stream));
        // the steps run without a host round trip; a breakdown is found
        // afterwards and ends the Krylov space there (later steps are discarded)
        for (int j = 0; j < m0; ++j) {
            if (int rc = hv_single(ctx, s, HV_F64, V[j]->p, W->p)) return rc;
            OrthoCoef oc;
            if (int rc = orthogonalize<double>(ctx, V, j + 1, (double *)W->p, Dp, (double *)dpart.p,
                                               (double *)dnorm.p, G, &oc))
                return rc;
            k_cgs_finish<<<1, 256, 0, ctx->stream>>>(oc.p[0], oc.p[1], oc.Gm, j + 1, (const double *)dnorm.p, G,
                                                     Hp + (size_t)j * ldh, (double *)dbeta.p);
            MOED_CHECK_LAUNCH(ctx);
            if (j + 1 < m0) {
                k_scale_copy<double><<<G, kVecThreads, 0, ctx->stream>>>((const double *)W->p, (double *)V[j + 1]->p,
                                                                         Dp, (double *)dbeta.p + 1);
                MOED_CHECK_LAUNCH(ctx);
            }
        }
        std::vector<double> hc((size_t)ldh * m0);
        MOED_CUDA(ctx, cudaMemcpyAsync(hc.data(), Hp, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int m = m0;
        double anorm = 0.0, beta_m = 0.0;
        for (int j = 0; j < m0; ++j) {
            const double diag = hc[(size_t)j * ldh + j], beta = hc[(size_t)j * ldh + j + 1];
            anorm = std::max(anorm, std::fabs(diag) + beta);
            beta_m = beta;
            if (j + 1 >= D || beta <= 1e-12 * std::max(anorm, 1.0)) {
                m = j + 1;
                beta_m = 0.0;   // invariant subspace: its Ritz pairs are exact
                break;
            }
        }
        // the projected tridiagonal problem on the host (symeig.h)
        std::vector<double> Am((size_t)m * m), w(m), ev((size_t)m * m);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) Am[(size_t)i * m + j] = hc[(size_t)std::max(i, j) * ldh + std::min(i, j)];
        if (!sym_eig(m, Am, w.data(), ev.data()))
            return fail(ctx, MO_ED_ERR_NOCONV, "projected eigenproblem did not converge");
        MOED_CUDA(ctx, cudaMemcpyAsync(devecs.p, ev.data(), sizeof(double) * ev.size(), cudaMemcpyHostToDevice,
                                       ctx->stream));
        int best = 0;
        for (int i = 1; i < m; ++i)
            if (std::fabs(ev[(size_t)i * m]) > std::fabs(ev[(size_t)best * m])) best = i;
        *res = std::fabs(beta_m * ev[(size_t)best * m + (m - 1)]);
        VPtrs<double> P = make_ptrs<double>(V, m);
        std::vector<DevBuf *> o(1, &out);
        VPtrs<double> X = make_ptrs<double>(o, 1);
        k_rotate<double, 8><<<G, kVecThreads, 0, ctx->stream>>>(P, m, (const double *)devecs.p, m, best, 1, X, Dp);
        MOED_CHECK_LAUNCH(ctx);
        if (*res <= 1e-9 * std::max(anorm, 1.0)) break;
    }
    return MO_ED_OK;
}

int diag_sector(mo_ed_ctx *ctx, const Sector &s, int nev, std::vector<double> &vals,
                std::vector<DevBuf> *vecs)
{
    if (ctx->opt.precision == MO_ED_FP32) return trl_solve<float>(ctx, s, nev, vals, vecs);
    return trl_solve<double>(ctx, s, nev, vals, vecs);
}

}  // namespace moed
