// hv.cu -- matrix-free Kanamori H*v on a (Nup, Ndn) sector.
//
// Replaces multiply_H (ed_hamiltonian.F90:88-191).  For output row index
// (d, u) (down rank d, up rank u, element X[d][u]) the reference sums
//   diagonal   onsite + dens_dens                      (:112-141)
//   hybridisation  V c+_o c_k and V c+_k c_o, both spins (:146-161)
//   spin-flip  -J c+_{i up} c_{i dn} c+_{j dn} c_{j up}  (:163-174)
//   pair hop   -J c+_{i up} c+_{i dn} c_{j up} c_{j dn}  (:176-187)
// gathering A at the state each operator maps row (d, u) to.  Here:
//   * diagonal = Dup[u] + Ddn[d] + Cross[imp(u)][imp(d)] (tables.cu);
//   * up-spin hops read X[d][u'] for the <= hw precomputed (u', +-V) of u;
//   * down-spin hops read whole rows X[d'][*] -- coalesced AXPYs;
//   * spin-flip / pair-hop factor into an up-spin transfer T_{i<-j}(u) and a
//     down-spin transfer (T_{j<-i}(d) resp. T_{i<-j}(d)) with coefficient
//     +J t_up t_dn (the reordering of the four operators gives -1 which
//     cancels the -J), both transfers staying inside their bath group.
// A work item is R consecutive rows of one job; a CTA sweeps all columns u of
// the item, loading the up-hop entries of u once for the R rows.  The kernel
// walks a batch of jobs (vectors of possibly different sectors) so that all
// excitation vectors of a Lanczos step share one launch.  Optionally each
// item writes sum_{its rows} x*y (FP64) for the Lanczos alpha.
#include <algorithm>

#include "internal.h"

namespace moed {

constexpr int kHvThreads = 256;
constexpr int kMaxJobs = 24;

template <typename TA>
struct HvBatch {
    int njobs, total_items;
    HvJobT<TA> job[kMaxJobs];
};

template <typename TX, typename TA, typename TY, int R>
__global__ void __launch_bounds__(kHvThreads)
k_hv(const __grid_constant__ HvBatch<TA> batch, const ModelDev *__restrict__ mdl)
{
    __shared__ int s_t4[kMaxPair * kMaxImp];
    __shared__ TA s_cross[kMaxImp * kMaxImp];
    __shared__ int s_d[R], s_id[R], s_dcnt[R];
    __shared__ TA s_ddiag[R];
    __shared__ int s_dtgt[R][kMaxHop];
    __shared__ TA s_dval[R][kMaxHop];
    __shared__ unsigned s_sfmask[R], s_phmask[R];
    __shared__ int s_sfoff[R][kMaxPair], s_phoff[R][kMaxPair];
    __shared__ TA s_sfc[R][kMaxPair], s_phc[R][kMaxPair];
    __shared__ double s_red[kHvThreads / 32];

    const int tid = threadIdx.x;
    const int npair = mdl->npair, nimp = mdl->nimp, impmask = nimp - 1;
    for (int i = tid; i < npair * nimp; i += kHvThreads) s_t4[i] = mdl->t4[i];
    for (int i = tid; i < nimp * nimp; i += kHvThreads) s_cross[i] = (TA)mdl->cross[i];
    const TA Jc = (TA)mdl->J;

    for (int item = blockIdx.x; item < batch.total_items; item += gridDim.x) {
        int j = 0;
        while (j + 1 < batch.njobs && item >= batch.job[j + 1].item0) ++j;
        const HvJobT<TA> &jb = batch.job[j];
        if (jb.active && *jb.active == 0) continue;
        const int it = item - jb.item0;
        const int d0 = it * R;
        const int nr = min(R, jb.nd - d0);
        const int nu = jb.nu, nd = jb.nd;
        const TX *__restrict__ x = (const TX *)jb.x;
        TY *__restrict__ y = (TY *)jb.y;

        __syncthreads();  // previous item finished with the row tables
        if (tid < R) {
            int r = tid;
            if (r < nr) {
                int d = d0 + r;
                s_d[r] = d;
                s_id[r] = jb.dn_words[d] & impmask;
                s_ddiag[r] = jb.dn_diag[d];
                s_dcnt[r] = jb.dn_cnt[d];
            } else {
                s_d[r] = d0;
                s_id[r] = 0;
                s_ddiag[r] = TA(0);
                s_dcnt[r] = 0;
            }
            s_sfmask[r] = 0u;
            s_phmask[r] = 0u;
        }
        __syncthreads();
        for (int i = tid; i < R * jb.dn_maxcnt; i += kHvThreads) {
            int r = i / jb.dn_maxcnt, s = i - r * jb.dn_maxcnt;
            if (r < nr && s < s_dcnt[r]) {
                s_dtgt[r][s] = jb.dn_tgt[(size_t)s * nd + s_d[r]];
                s_dval[r][s] = jb.dn_val[(size_t)s * nd + s_d[r]];
            }
        }
        if (tid < R * npair) {
            int r = tid / npair, p = tid - r * npair;
            if (r < nr) {
                // spin-flip: down transfer j <- i, i.e. table of the reversed pair
                int esf = s_t4[mdl->pair_rev[p] * nimp + s_id[r]];
                int eph = s_t4[p * nimp + s_id[r]];
                if (esf < 0) {
                    s_sfoff[r][p] = (int)(short)(esf & 0xffff);
                    s_sfc[r][p] = (esf & 0x40000000) ? -Jc : Jc;
                    atomicOr(&s_sfmask[r], 1u << p);
                }
                if (eph < 0) {
                    s_phoff[r][p] = (int)(short)(eph & 0xffff);
                    s_phc[r][p] = (eph & 0x40000000) ? -Jc : Jc;
                    atomicOr(&s_phmask[r], 1u << p);
                }
            }
        }
        __syncthreads();

        double dacc = 0.0;
        for (int u = tid; u < nu; u += kHvThreads) {
            const int iu = jb.up_words[u] & impmask;
            const TA ud = jb.up_diag[u];
            TA acc[R];
            TX xs[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r < nr) {
                    xs[r] = __ldg(x + (size_t)s_d[r] * nu + u);
                    acc[r] = (ud + s_ddiag[r] + s_cross[iu * nimp + s_id[r]]) * (TA)xs[r];
                } else {
                    xs[r] = TX(0);
                    acc[r] = TA(0);
                }
            }
            // up-spin hybridisation: in-row gathers
            const int cnt = jb.up_cnt[u];
            for (int s = 0; s < cnt; ++s) {
                const int t = __ldg(jb.up_tgt + (size_t)s * nu + u);
                const TA v = __ldg(jb.up_val + (size_t)s * nu + u);
#pragma unroll
                for (int r = 0; r < R; ++r)
                    if (r < nr) acc[r] += v * (TA)__ldg(x + (size_t)s_d[r] * nu + t);
            }
            // down-spin hybridisation: row AXPYs
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r < nr) {
                    const int c = s_dcnt[r];
                    for (int s = 0; s < c; ++s)
                        acc[r] += s_dval[r][s] * (TA)__ldg(x + (size_t)s_dtgt[r][s] * nu + u);
                }
            }
            // spin-flip and pair hopping
            for (int p = 0; p < npair; ++p) {
                const int e = s_t4[p * nimp + iu];
                if (e < 0) {
                    const int uu = u + (int)(short)(e & 0xffff);
                    const bool neg = (e & 0x40000000) != 0;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        if (r < nr) {
                            if ((s_sfmask[r] >> p) & 1u) {
                                TA c = neg ? -s_sfc[r][p] : s_sfc[r][p];
                                acc[r] += c * (TA)__ldg(x + (size_t)(s_d[r] + s_sfoff[r][p]) * nu + uu);
                            }
                            if ((s_phmask[r] >> p) & 1u) {
                                TA c = neg ? -s_phc[r][p] : s_phc[r][p];
                                acc[r] += c * (TA)__ldg(x + (size_t)(s_d[r] + s_phoff[r][p]) * nu + uu);
                            }
                        }
                    }
                }
            }
            TA part = TA(0);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r < nr) {
                    TY o = (TY)acc[r];
                    y[(size_t)s_d[r] * nu + u] = o;
                    part += (TA)xs[r] * (TA)o;
                }
            }
            dacc += (double)part;
        }
        if (jb.dot_partial) {
            for (int off = 16; off > 0; off >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, off);
            if ((tid & 31) == 0) s_red[tid >> 5] = dacc;
            __syncthreads();
            if (tid == 0) {
                double t = 0.0;
                for (int w = 0; w < kHvThreads / 32; ++w) t += s_red[w];
                jb.dot_partial[it] = t;
            }
        }
    }
}

int hv_rows_per_item(int kind) { return kind == HV_F32 ? 4 : 2; }

template <typename TA>
void hv_fill_job(const mo_ed_ctx *ctx, const Sector &s, int kind, const void *x, void *y,
                 HvJobT<TA> &j)
{
    (void)ctx;
    const bool f32 = sizeof(TA) == 4;
    j.x = x;
    j.y = y;
    j.dot_partial = nullptr;
    j.active = nullptr;
    j.nu = s.up->n;
    j.nd = s.dn->n;
    const int R = hv_rows_per_item(kind);
    j.nitems = (j.nd + R - 1) / R;
    j.item0 = 0;
    j.up_words = s.up->words;
    j.up_cnt = s.up->hop_cnt;
    j.up_tgt = s.up->hop_tgt;
    j.up_val = f32 ? (const TA *)s.up->hop_val_f : (const TA *)s.up->hop_val_d;
    j.up_diag = f32 ? (const TA *)s.up->diag_f : (const TA *)s.up->diag_d;
    j.dn_words = s.dn->words;
    j.dn_cnt = s.dn->hop_cnt;
    j.dn_tgt = s.dn->hop_tgt;
    j.dn_val = f32 ? (const TA *)s.dn->hop_val_f : (const TA *)s.dn->hop_val_d;
    j.dn_diag = f32 ? (const TA *)s.dn->diag_f : (const TA *)s.dn->diag_d;
    j.up_hw = s.up->hw;
    j.dn_hw = s.dn->hw;
    j.dn_maxcnt = s.dn->max_cnt;
    j.pad = 0;
}
template void hv_fill_job<float>(const mo_ed_ctx *, const Sector &, int, const void *, void *,
                                 HvJobT<float> &);
template void hv_fill_job<double>(const mo_ed_ctx *, const Sector &, int, const void *, void *,
                                  HvJobT<double> &);

template <typename TX, typename TA, typename TY, int R>
static int launch_batch(mo_ed_ctx *ctx, const HvBatch<TA> &b)
{
    if (b.total_items <= 0) return MO_ED_OK;
    int grid = std::min(b.total_items, ctx->num_sms * 8);
    k_hv<TX, TA, TY, R><<<grid, kHvThreads, 0, ctx->stream>>>(b, ctx->d_mdl);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

template <typename TA>
static int launch_kind(mo_ed_ctx *ctx, int kind, const HvBatch<TA> &b)
{
    if constexpr (sizeof(TA) == 4) {
        (void)kind;
        return launch_batch<float, float, float, 4>(ctx, b);
    } else {
        if (kind == HV_F64) return launch_batch<double, double, double, 2>(ctx, b);
        return launch_batch<float, double, double, 2>(ctx, b);
    }
}

template <typename TA>
static int hv_run_jobs(mo_ed_ctx *ctx, int kind, const HvJobT<TA> *jobs, int njobs)
{
    HvBatch<TA> b;
    b.njobs = 0;
    b.total_items = 0;
    for (int i = 0; i < njobs; ++i) {
        if (b.njobs == kMaxJobs) {
            if (int rc = launch_kind<TA>(ctx, kind, b)) return rc;
            b.njobs = 0;
            b.total_items = 0;
        }
        b.job[b.njobs] = jobs[i];
        b.job[b.njobs].item0 = b.total_items;
        b.total_items += jobs[i].nitems;
        b.njobs++;
    }
    if (b.njobs == 0) return MO_ED_OK;
    return launch_kind<TA>(ctx, kind, b);
}

int hv_launch_f32(mo_ed_ctx *ctx, const HvJobT<float> *jobs, int njobs)
{
    return hv_run_jobs<float>(ctx, HV_F32, jobs, njobs);
}
int hv_launch_f64(mo_ed_ctx *ctx, int kind, const HvJobT<double> *jobs, int njobs)
{
    return hv_run_jobs<double>(ctx, kind, jobs, njobs);
}

int hv_single(mo_ed_ctx *ctx, const Sector &s, int kind, const void *x, void *y)
{
    if (kind == HV_F32) {
        HvJobT<float> j;
        hv_fill_job<float>(ctx, s, kind, x, y, j);
        return hv_launch_f32(ctx, &j, 1);
    }
    HvJobT<double> j;
    hv_fill_job<double>(ctx, s, kind, x, y, j);
    return hv_launch_f64(ctx, kind, &j, 1);
}

}  // namespace moed
