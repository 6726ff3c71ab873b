// hv.cu -- matrix-free Kanamori H*v on a (Nup, Ndn) sector.
//
// Replaces multiply_H (ed_hamiltonian.F90:88-191).  For output element
// (d, u) (down rank d, up rank u, X[d][u]) the reference sums
//   diagonal       onsite + dens_dens                      (:112-141)
//   hybridisation  V c+_o c_k and V c+_k c_o, both spins     (:146-161)
//   spin-flip      -J c+_{i up} c_{i dn} c+_{j dn} c_{j up}  (:163-174)
//   pair hop       -J c+_{i up} c+_{i dn} c_{j up} c_{j dn}  (:176-187)
// gathering A at the state each operator maps row (d, u) to.  Here:
//   * diagonal = Dup[u] + Ddn[d] + Cross[imp(u)][imp(d)] (tables.cu);
//   * up-spin hops gather X[d][u'] for the precomputed moves (u', +-V) of u;
//   * down-spin hops are whole-row AXPYs from rows d';
//   * spin-flip / pair hop factor into an up-spin transfer T_{i<-j}(u) and a
//     down-spin transfer (T_{j<-i}(d) for spin-flip, T_{i<-j}(d) for pair
//     hopping) with coefficient +J t_up t_dn: reordering the four operators
//     of ed_operators.F90:183-213 / 236-266 gives a factor -1 that cancels
//     the -J.  Both transfers stay inside a bath group (rank offsets that
//     depend only on the impurity bits).
//
// Work decomposition.  An item is up to R rows made of whole down-spin bath
// groups, so the partner rows of spin-flip / pair hopping are in the item.
// Items are ordered by the bath occupations of the conserved subsystems, so
// the down-spin neighbours of the rows in flight stay L2-resident.  A CTA
// stages its rows in shared memory transposed, S[u][r]: one shared load of
// S[u'] serves the up-spin move u -> u' for all rows of the item, and the
// partner rows are shared-memory reads too.  Each thread owns 4 consecutive
// columns: 16-byte aligned global loads for the down-spin row AXPYs and
// 16-byte stores of y (rows are padded to a 128-byte stride); its column
// moves come from a chunk-major table, one contiguous block per slot.  The
// kernel walks a batch of jobs (vectors of possibly different sectors) so that
// all excitation vectors of a Lanczos step share one launch; optionally each
// item writes the FP64 partial of x*y for the Lanczos alpha.
#include <algorithm>

#include "internal.h"

namespace moed {

constexpr int kMaxJobs = 24;

template <typename TA>
struct HvBatch {
    int njobs, total_items;
    HvJobT<TA> job[kMaxJobs];
};

template <typename T>
struct alignas(16) Vec4 {
    T v[4];
};

template <typename T, int R>
struct alignas(8) RowVec {
    T v[R];
};

// Spin-flip / pair-hop terms of one (row, column impurity pattern) pair: at
// most 2 for up to three orbitals.  Term t reads the staged partner row
// src[t] at column u + du[t] with coefficient c[t] (+-J with both transfer
// signs folded in).
template <typename TA>
struct alignas(16) Quad {
    int cnt;
    signed char du[2];
    unsigned char src[2];
    TA c[2];
};

template <typename T>
__device__ __forceinline__ Vec4<T> ldg4(const T *p)
{
    Vec4<T> r;
    if constexpr (sizeof(T) == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        r.v[0] = a.x;
        r.v[1] = a.y;
        r.v[2] = a.z;
        r.v[3] = a.w;
    } else {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
        const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
        r.v[0] = a.x;
        r.v[1] = a.y;
        r.v[2] = b.x;
        r.v[3] = b.y;
    }
    return r;
}

__device__ __forceinline__ int4 ldg_i4(const int *p) { return __ldg(reinterpret_cast<const int4 *>(p)); }

template <typename T>
__device__ __forceinline__ void stg4(T *p, const T (&v)[4])
{
    if constexpr (sizeof(T) == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    }
}

// the 4 moves of slot s of one 4-column chunk
template <typename TA>
__device__ __forceinline__ void ld_moves(const HopEnt<TA> *p, HopEnt<TA> (&e)[4])
{
    if constexpr (sizeof(TA) == 4) {
        const int4 a = __ldg(reinterpret_cast<const int4 *>(p));
        const int4 b = __ldg(reinterpret_cast<const int4 *>(p) + 1);
        e[0].t = a.x;
        e[0].v = __int_as_float(a.y);
        e[1].t = a.z;
        e[1].v = __int_as_float(a.w);
        e[2].t = b.x;
        e[2].v = __int_as_float(b.y);
        e[3].t = b.z;
        e[3].v = __int_as_float(b.w);
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int4 a = __ldg(reinterpret_cast<const int4 *>(p + k));
            e[k].t = a.x;
            e[k].v = __hiloint2double(a.w, a.z);
        }
    }
}

template <typename TX, typename TA, typename TY, int R, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
k_hv(const __grid_constant__ HvBatch<TA> batch, const ModelDev *__restrict__ mdl)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int npair = mdl->npair, nimp = mdl->nimp;
    int ldmax = 0;
    for (int i = 0; i < batch.njobs; ++i) ldmax = max(ldmax, batch.job[i].ld);
    // dynamic shared memory: staged rows transposed, S[u] = row values of
    // column u; then the interspecies diagonal and the 4-operator table
    RowVec<TX, R> *S = reinterpret_cast<RowVec<TX, R> *>(smem_raw);
    TA *s_cross = reinterpret_cast<TA *>(smem_raw + ((sizeof(RowVec<TX, R>) * (size_t)ldmax + 15) & ~(size_t)15));
    int *s_t4 = reinterpret_cast<int *>(s_cross + nimp * nimp);

    __shared__ unsigned s_pmask[kMaxImp];
    __shared__ RowVec<TA, R> s_crossT[kMaxImp];   // per item: cross[iu][id_r] for the R rows
    __shared__ int s_d[R], s_id[R], s_dcnt[R];
    __shared__ TA s_ddiag[R];
    __shared__ int s_dtgt[R][kMaxHop];
    __shared__ TA s_dval[R][kMaxHop];
    // per (row, pair): spin-flip / pair-hop partner as an item slot (>= 0) or
    // as -(1 + global row) when the partner row is not staged, and the
    // coefficient +-J; s_sfm[r] / s_phm[r]: pairs valid for row r
    __shared__ unsigned s_sfm[R], s_phm[R];
    __shared__ unsigned s_rowmask[kMaxPair];   // generic path: bit r spin-flip, bit 16+r pair hop
    __shared__ unsigned s_itemmask;
    __shared__ Quad<TA> s_q[R * kMaxImp];      // fast path table
    __shared__ int s_slow;                     // 1: an item needs the generic path
    __shared__ int s_sfsrc[R][kMaxPair], s_phsrc[R][kMaxPair];
    __shared__ TA s_sfc[R][kMaxPair], s_phc[R][kMaxPair];
    __shared__ double s_red[NT / 32];

    const int tid = threadIdx.x;
    for (int i = tid; i < npair * nimp; i += NT) s_t4[i] = mdl->t4[i];
    for (int i = tid; i < nimp; i += NT) s_pmask[i] = mdl->pairmask[i];
    for (int i = tid; i < nimp * nimp; i += NT) s_cross[i] = (TA)mdl->cross[i];
    const TA Jc = (TA)mdl->J;

    for (int item = blockIdx.x; item < batch.total_items; item += gridDim.x) {
        int j = 0;
        while (j + 1 < batch.njobs && item >= batch.job[j + 1].item0) ++j;
        const HvJobT<TA> &jb = batch.job[j];
        if (jb.active && *jb.active == 0) continue;
        const int it = item - jb.item0;
        const int nd = jb.nd, ld = jb.ld, nchunk = ld >> 2;
        const TX *__restrict__ x = (const TX *)jb.x;
        TY *__restrict__ y = (TY *)jb.y;

        __syncthreads();  // the previous item is done with S and the row tables
        if (tid < R) {
            const int r = tid;
            const int d = jb.items[it * R + r];
            if (d >= 0) {
                const int inf = jb.dn_info[d];
                s_d[r] = d;
                s_id[r] = (inf >> 8) & 0xff;
                s_dcnt[r] = inf & 0xff;
                s_ddiag[r] = jb.dn_diag[d];
            } else {
                s_d[r] = -1;
                s_id[r] = 0;
                s_dcnt[r] = 0;
                s_ddiag[r] = TA(0);
            }
            s_sfm[r] = 0u;
            s_phm[r] = 0u;
        }
        for (int p = tid; p < kMaxPair; p += NT) s_rowmask[p] = 0u;
        if (tid == 0) {
            s_itemmask = 0u;
            s_slow = 0;
        }
        __syncthreads();
        for (int i = tid; i < nimp * R; i += NT) {
            const int iu = i / R, r = i - iu * R;
            s_crossT[iu].v[r] = s_cross[iu * nimp + s_id[r]];
        }
        for (int i = tid; i < R * jb.dn_maxcnt; i += NT) {
            const int r = i / jb.dn_maxcnt, s = i - r * jb.dn_maxcnt;
            if (s < s_dcnt[r]) {
                s_dtgt[r][s] = jb.dn_tgt[(size_t)s * nd + s_d[r]];
                s_dval[r][s] = jb.dn_val[(size_t)s * nd + s_d[r]];
            }
        }
        if (tid < R * npair) {
            const int r = tid / npair, p = tid - r * npair;
            if (s_d[r] >= 0) {
                const int esf = s_t4[mdl->pair_rev[p] * nimp + s_id[r]];   // spin-flip: T_{j<-i}(d)
                const int eph = s_t4[p * nimp + s_id[r]];                  // pair hop:  T_{i<-j}(d)
                if (esf < 0) {
                    const int off = (int)(short)(esf & 0xffff), dp = s_d[r] + off, rp = r + off;
                    const bool local = rp >= 0 && rp < R && s_d[rp] == dp;
                    s_sfsrc[r][p] = local ? rp : -(1 + dp);
                    s_sfc[r][p] = (esf & 0x40000000) ? -Jc : Jc;
                    atomicOr(&s_sfm[r], 1u << p);
                    atomicOr(&s_rowmask[p], 1u << r);
                    atomicOr(&s_itemmask, 1u << p);
                    if (!local) s_slow = 1;
                }
                if (eph < 0) {
                    const int off = (int)(short)(eph & 0xffff), dp = s_d[r] + off, rp = r + off;
                    const bool local = rp >= 0 && rp < R && s_d[rp] == dp;
                    s_phsrc[r][p] = local ? rp : -(1 + dp);
                    s_phc[r][p] = (eph & 0x40000000) ? -Jc : Jc;
                    atomicOr(&s_phm[r], 1u << p);
                    atomicOr(&s_rowmask[p], 1u << (16 + r));
                    atomicOr(&s_itemmask, 1u << p);
                    if (!local) s_slow = 1;
                }
            }
        }
        __syncthreads();
        // fast-path table: terms of every (row, column impurity pattern)
        for (int i = tid; i < R * nimp; i += NT) {
            const int r = i / nimp, iu = i - r * nimp;
            Quad<TA> q;
            q.cnt = 0;
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                q.du[t] = 0;
                q.src[t] = 0;
                q.c[t] = TA(0);
            }
            if (s_d[r] >= 0) {
                for (int p = 0; p < npair; ++p) {
                    const int e = s_t4[p * nimp + iu];
                    if (e >= 0) continue;
                    const int du = (int)(short)(e & 0xffff);
                    const TA tu = (e & 0x40000000) ? TA(-1) : TA(1);
                    if ((s_sfm[r] >> p) & 1u) {
                        if (q.cnt == 2) s_slow = 1;
                        else {
                            q.du[q.cnt] = (signed char)du;
                            q.src[q.cnt] = (unsigned char)max(s_sfsrc[r][p], 0);
                            q.c[q.cnt] = tu * s_sfc[r][p];
                            ++q.cnt;
                        }
                    }
                    if ((s_phm[r] >> p) & 1u) {
                        if (q.cnt == 2) s_slow = 1;
                        else {
                            q.du[q.cnt] = (signed char)du;
                            q.src[q.cnt] = (unsigned char)max(s_phsrc[r][p], 0);
                            q.c[q.cnt] = tu * s_phc[r][p];
                            ++q.cnt;
                        }
                    }
                }
            }
            s_q[i] = q;
        }
        // stage the rows, transposed (pad rows staged as zeros)
        for (int c = tid; c < nchunk; c += NT) {
            Vec4<TX> v[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int d = jb.items[it * R + r];
                if (d >= 0) {
                    v[r] = ldg4(x + (size_t)d * ld + 4 * c);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) v[r].v[k] = TX(0);
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                RowVec<TX, R> t;
#pragma unroll
                for (int r = 0; r < R; ++r) t.v[r] = v[r].v[k];
                S[4 * c + k] = t;
            }
        }
        __syncthreads();

        // item-uniform row data in registers
        TA ddiag[R];
        bool live[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ddiag[r] = s_ddiag[r];
            live[r] = s_d[r] >= 0;
        }
        const bool slow = s_slow != 0;
        const bool want_dot = jb.dot_partial != nullptr;
        const unsigned imask = s_itemmask;
        double dacc = 0.0;
        int4 nx_inf = tid < nchunk ? ldg_i4(jb.up_info + 4 * tid) : make_int4(0, 0, 0, 0);
        Vec4<TA> nx_ud = tid < nchunk ? ldg4(jb.up_diag + 4 * tid) : Vec4<TA>{};
        for (int c = tid; c < nchunk; c += NT) {
            const int u0 = 4 * c;
            const int4 inf4 = nx_inf;
            const Vec4<TA> ud = nx_ud;
            if (c + NT < nchunk) {   // prefetch the next chunk's column data
                nx_inf = ldg_i4(jb.up_info + u0 + 4 * NT);
                nx_ud = ldg4(jb.up_diag + u0 + 4 * NT);
            }
            const int inf[4] = {inf4.x, inf4.y, inf4.z, inf4.w};
            TA acc[4][R];
            int cnt[4], iu[4];
            int maxc = 0;
            // diagonal
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                iu[k] = (inf[k] >> 8) & 0xff;
                cnt[k] = inf[k] & 0xff;
                maxc = max(maxc, cnt[k]);
                const RowVec<TX, R> sx = S[u0 + k];
                const RowVec<TA, R> cr = s_crossT[iu[k]];
#pragma unroll
                for (int r = 0; r < R; ++r) acc[k][r] = (ud.v[k] + ddiag[r] + cr.v[r]) * (TA)sx.v[r];
            }
            // up-spin hybridisation: shared-memory gathers, all rows at once
            // The moves of SB slots are loaded together so that their L2
            // latencies overlap; a gather is issued only for a column's own
            // moves (no shared-memory traffic for padded slots).
            constexpr int SB = R > 4 ? 2 : 4;
            const HopEnt<TA> *tab = jb.up_tab + (size_t)c * jb.up_hw * 4;
            for (int s0 = 0; s0 < maxc; s0 += SB) {
                HopEnt<TA> e[SB][4];
#pragma unroll
                for (int t = 0; t < SB; ++t) {
                    if (s0 + t < maxc) ld_moves<TA>(tab + (size_t)(s0 + t) * 4, e[t]);
                }
#pragma unroll
                for (int t = 0; t < SB; ++t) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (s0 + t < cnt[k]) {
                            const RowVec<TX, R> g = S[e[t][k].t];
#pragma unroll
                            for (int r = 0; r < R; ++r) acc[k][r] += e[t][k].v * (TA)g.v[r];
                        }
                    }
                }
            }
            // down-spin hybridisation: row AXPYs (16-byte loads)
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int n = s_dcnt[r];
#pragma unroll 4
                for (int s = 0; s < n; ++s) {
                    const TA v = s_dval[r][s];
                    const Vec4<TX> g = ldg4(x + (size_t)s_dtgt[r][s] * ld + u0);
#pragma unroll
                    for (int k = 0; k < 4; ++k) acc[k][r] += v * (TA)g.v[k];
                }
            }
            // spin-flip and pair hopping (partner rows are in the stage)
            if (!slow) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const Quad<TA> q = s_q[r * nimp + iu[k]];
#pragma unroll
                        for (int t = 0; t < 2; ++t)
                            if (t < q.cnt)
                                acc[k][r] += q.c[t] * (TA)reinterpret_cast<const TX *>(&S[u0 + k + q.du[t]])[q.src[t]];
                    }
                }
            } else {
                // generic: pairs valid for this column and for some row of the item
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    unsigned pm = s_pmask[iu[k]] & imask;
                    while (pm) {
                        const int p = __ffs(pm) - 1;
                        pm &= pm - 1;
                        const int e = s_t4[p * nimp + iu[k]];
                        const int uu = u0 + k + (int)(short)(e & 0xffff);
                        const bool neg = (e & 0x40000000) != 0;
                        const unsigned rm = s_rowmask[p];
                        const TX *su = reinterpret_cast<const TX *>(&S[uu]);
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            if ((rm >> r) & 1u) {
                                const int src = s_sfsrc[r][p];
                                const TX xv = src >= 0 ? su[src] : __ldg(x + (size_t)(-1 - src) * ld + uu);
                                const TA cf = neg ? -s_sfc[r][p] : s_sfc[r][p];
                                acc[k][r] += cf * (TA)xv;
                            }
                            if ((rm >> (16 + r)) & 1u) {
                                const int src = s_phsrc[r][p];
                                const TX xv = src >= 0 ? su[src] : __ldg(x + (size_t)(-1 - src) * ld + uu);
                                const TA cf = neg ? -s_phc[r][p] : s_phc[r][p];
                                acc[k][r] += cf * (TA)xv;
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (live[r]) {
                    TY o[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) o[k] = (TY)acc[k][r];
                    stg4(y + (size_t)s_d[r] * ld + u0, o);
                }
            }
            if (want_dot) {   // x (re-read from the stage) . y of this chunk
                TA part = TA(0);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const RowVec<TX, R> sx = S[u0 + k];
#pragma unroll
                    for (int r = 0; r < R; ++r) part += (TA)sx.v[r] * (TA)(TY)acc[k][r];
                }
                dacc += (double)part;
            }
        }
        if (jb.dot_partial) {
            for (int off = 16; off > 0; off >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, off);
            if ((tid & 31) == 0) s_red[tid >> 5] = dacc;
            __syncthreads();
            if (tid == 0) {
                double t = 0.0;
                for (int w = 0; w < NT / 32; ++w) t += s_red[w];
                jb.dot_partial[it] = t;
            }
        }
    }
}

template <typename TX, typename TA, int R>
static size_t dyn_smem_bytes(int ld, const ModelDev &m)
{
    return ((sizeof(RowVec<TX, R>) * (size_t)ld + 15) & ~(size_t)15) + sizeof(TA) * (size_t)m.nimp * m.nimp +
           sizeof(int) * (size_t)m.npair * m.nimp;
}

// ---------------------------------------------------------------------------
// tile-shape variants and the autotuner
// ---------------------------------------------------------------------------
// A variant fixes the rows per item R, the CTA size NT and the CTAs per SM the
// register budget is cut for (MINB).  All variants compute every element with
// the same sequence of operations, so their outputs are bit-identical; only
// the speed differs.  The first H*v of a (kind, Nup, Ndn) shape times each
// variant on that sector (scratch vectors, CUDA events on the context stream)
// and keeps the fastest.
struct HvVariant {
    int R, NT, MINB;
};
static const HvVariant kVarF32[] = {{3, 512, 2}, {4, 256, 2}, {6, 512, 1}, {3, 256, 3}, {8, 512, 1}};
static const HvVariant kVarF64[] = {{2, 256, 2}, {3, 256, 1}, {2, 512, 1}};
static const int kNVarF32 = sizeof(kVarF32) / sizeof(kVarF32[0]);
static const int kNVarF64 = sizeof(kVarF64) / sizeof(kVarF64[0]);

static const HvVariant &variant(int kind, int v) { return kind == HV_F32 ? kVarF32[v] : kVarF64[v]; }
static int nvariants(int kind) { return kind == HV_F32 ? kNVarF32 : kNVarF64; }

static long long shape_key(int kind, const Sector &s) { return ((long long)kind << 32) | (s.ne_up << 16) | s.ne_down; }

template <typename TA>
void hv_fill_job(const mo_ed_ctx *ctx, const Sector &s, int R, const void *x, void *y, HvJobT<TA> &j)
{
    const bool f32 = sizeof(TA) == 4;
    (void)ctx;
    j.x = x;
    j.y = y;
    j.dot_partial = nullptr;
    j.active = nullptr;
    j.nu = s.up->n;
    j.nd = s.dn->n;
    j.ld = s.ld();
    auto it = s.dn->items.find(R);
    j.items = it != s.dn->items.end() ? it->second : nullptr;
    j.nitems = it != s.dn->items.end() ? s.dn->nitems.at(R) : 0;
    j.item0 = 0;
    j.up_info = s.up->info;
    j.up_tab = f32 ? (const HopEnt<TA> *)s.up->tab_f : (const HopEnt<TA> *)s.up->tab_d;
    j.up_diag = f32 ? (const TA *)s.up->diag_f : (const TA *)s.up->diag_d;
    j.up_hw = s.up->hw;
    j.up_maxcnt = s.up->max_cnt;
    j.dn_info = s.dn->info;
    j.dn_tgt = s.dn->hop_tgt;
    j.dn_val = f32 ? (const TA *)s.dn->hop_val_f : (const TA *)s.dn->hop_val_d;
    j.dn_diag = f32 ? (const TA *)s.dn->diag_f : (const TA *)s.dn->diag_d;
    j.dn_maxcnt = s.dn->max_cnt;
    j.pad = 0;
}
template void hv_fill_job<float>(const mo_ed_ctx *, const Sector &, int, const void *, void *, HvJobT<float> &);
template void hv_fill_job<double>(const mo_ed_ctx *, const Sector &, int, const void *, void *, HvJobT<double> &);

template <typename TX, typename TA, typename TY, int R, int NT, int MINB>
static int launch_batch(mo_ed_ctx *ctx, const HvBatch<TA> &b)
{
    if (b.total_items <= 0) return MO_ED_OK;
    int ldmax = 0;
    for (int i = 0; i < b.njobs; ++i) {
        ldmax = std::max(ldmax, b.job[i].ld);
        if (!b.job[i].items) return fail(ctx, MO_ED_ERR_STATE, "H*v item table missing");
    }
    const size_t smem = dyn_smem_bytes<TX, TA, R>(ldmax, ctx->mdl);
    auto kern = k_hv<TX, TA, TY, R, NT, MINB>;
    MOED_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MOED_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int per_sm = 0;
    MOED_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem));
    if (per_sm < 1) return fail(ctx, MO_ED_ERR_ARG, "sector rows too long for the shared-memory stage");
    const int grid = std::min(b.total_items, ctx->num_sms * per_sm);
    kern<<<grid, NT, smem, ctx->stream>>>(b, ctx->d_mdl);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

template <typename TA>
static int launch_variant(mo_ed_ctx *ctx, int kind, int v, const HvBatch<TA> &b)
{
    if constexpr (sizeof(TA) == 4) {
        (void)kind;
        switch (v) {
        case 0: return launch_batch<float, float, float, 3, 512, 2>(ctx, b);
        case 1: return launch_batch<float, float, float, 4, 256, 2>(ctx, b);
        case 2: return launch_batch<float, float, float, 6, 512, 1>(ctx, b);
        case 3: return launch_batch<float, float, float, 3, 256, 3>(ctx, b);
        default: return launch_batch<float, float, float, 8, 512, 1>(ctx, b);
        }
    } else if (kind == HV_F64) {
        switch (v) {
        case 0: return launch_batch<double, double, double, 2, 256, 2>(ctx, b);
        case 1: return launch_batch<double, double, double, 3, 256, 1>(ctx, b);
        default: return launch_batch<double, double, double, 2, 512, 1>(ctx, b);
        }
    } else {
        switch (v) {
        case 0: return launch_batch<float, double, double, 2, 256, 2>(ctx, b);
        case 1: return launch_batch<float, double, double, 3, 256, 1>(ctx, b);
        default: return launch_batch<float, double, double, 2, 512, 1>(ctx, b);
        }
    }
}

template <typename TA>
static int hv_run_jobs(mo_ed_ctx *ctx, int kind, int v, const HvJobT<TA> *jobs, int njobs)
{
    HvBatch<TA> b;
    b.njobs = 0;
    b.total_items = 0;
    for (int i = 0; i < njobs; ++i) {
        if (b.njobs == kMaxJobs) {
            if (int rc = launch_variant<TA>(ctx, kind, v, b)) return rc;
            b.njobs = 0;
            b.total_items = 0;
        }
        b.job[b.njobs] = jobs[i];
        b.job[b.njobs].item0 = b.total_items;
        b.total_items += jobs[i].nitems;
        b.njobs++;
    }
    if (b.njobs == 0) return MO_ED_OK;
    return launch_variant<TA>(ctx, kind, v, b);
}

int hv_launch_f32(mo_ed_ctx *ctx, int v, const HvJobT<float> *jobs, int njobs)
{
    return hv_run_jobs<float>(ctx, HV_F32, v, jobs, njobs);
}
int hv_launch_f64(mo_ed_ctx *ctx, int kind, int v, const HvJobT<double> *jobs, int njobs)
{
    return hv_run_jobs<double>(ctx, kind, v, jobs, njobs);
}

static int launch_one(mo_ed_ctx *ctx, const Sector &s, int kind, int v, const void *x, void *y)
{
    const int R = variant(kind, v).R;
    if (kind == HV_F32) {
        HvJobT<float> j;
        hv_fill_job<float>(ctx, s, R, x, y, j);
        return hv_launch_f32(ctx, v, &j, 1);
    }
    HvJobT<double> j;
    hv_fill_job<double>(ctx, s, R, x, y, j);
    return hv_launch_f64(ctx, kind, v, &j, 1);
}

// Time every variant once on sector s and keep the fastest.
static int tune(mo_ed_ctx *ctx, const Sector &s, int kind, int *best)
{
    const size_t ex = kind == HV_F64 ? sizeof(double) : sizeof(float);
    const size_t ey = kind == HV_F32 ? sizeof(float) : sizeof(double);
    DevBuf dx, dy;
    if (int rc = dev_alloc(ctx, dx, ex * (size_t)s.Dpad())) return rc;
    if (int rc = dev_alloc(ctx, dy, ey * (size_t)s.Dpad())) return rc;
    MOED_CUDA(ctx, cudaMemsetAsync(dx.p, 0, dx.bytes, ctx->stream));
    cudaEvent_t e0, e1;
    MOED_CUDA(ctx, cudaEventCreate(&e0));
    MOED_CUDA(ctx, cudaEventCreate(&e1));
    float tbest = 1e30f;
    *best = -1;
    std::vector<float> &times = ctx->hv_times[shape_key(kind, s)];
    times.assign(nvariants(kind), -1.0f);
    for (int v = 0; v < nvariants(kind); ++v) {
        const int *items;
        int n;
        if (int rc = species_items(ctx, s.dn, variant(kind, v).R, &items, &n)) return rc;
        if (launch_one(ctx, s, kind, v, dx.p, dy.p) != MO_ED_OK) {   // variant does not fit this sector
            cudaGetLastError();
            continue;
        }
        float tv = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            MOED_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
            if (int rc = launch_one(ctx, s, kind, v, dx.p, dy.p)) return rc;
            MOED_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
            MOED_CUDA(ctx, cudaEventSynchronize(e1));
            float ms = 0.f;
            MOED_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
            tv = std::min(tv, ms);
        }
        times[v] = tv;
        if (tv < tbest) {
            tbest = tv;
            *best = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (*best < 0) return fail(ctx, MO_ED_ERR_ARG, "no H*v tile shape fits this sector");
    ctx->err.clear();
    return MO_ED_OK;
}

int hv_prepare(mo_ed_ctx *ctx, const Sector &s, int kind, int *v_out, int *R_out)
{
    const long long key = shape_key(kind, s);
    auto it = ctx->hv_choice.find(key);
    int v;
    if (it != ctx->hv_choice.end()) {
        v = it->second;
    } else {
        if (int rc = tune(ctx, s, kind, &v)) return rc;
        ctx->hv_choice[key] = v;
    }
    const int *items;
    int n;
    if (int rc = species_items(ctx, s.dn, variant(kind, v).R, &items, &n)) return rc;
    if (v_out) *v_out = v;
    if (R_out) *R_out = variant(kind, v).R;
    return MO_ED_OK;
}

int hv_tuning(mo_ed_ctx *ctx, const Sector &s, int kind, int cap, int *nvar, int *shape, float *ms, int *chosen)
{
    int v;
    if (int rc = hv_prepare(ctx, s, kind, &v, nullptr)) return rc;
    const std::vector<float> &t = ctx->hv_times[shape_key(kind, s)];
    *nvar = nvariants(kind);
    *chosen = v;
    for (int i = 0; i < *nvar && i < cap; ++i) {
        const HvVariant &h = variant(kind, i);
        if (shape) {
            shape[3 * i] = h.R;
            shape[3 * i + 1] = h.NT;
            shape[3 * i + 2] = h.MINB;
        }
        if (ms) ms[i] = i < (int)t.size() ? t[i] : -1.0f;
    }
    return MO_ED_OK;
}

int hv_prepare_rows(mo_ed_ctx *ctx, const Sector &s, int R)
{
    const int *items;
    int n;
    return species_items(ctx, s.dn, R, &items, &n);
}

int hv_lookup(mo_ed_ctx *ctx, const Sector &s, int kind, int *v_out, int *R_out)
{
    auto it = ctx->hv_choice.find(shape_key(kind, s));
    if (it == ctx->hv_choice.end())
        return fail(ctx, MO_ED_ERR_STATE, "H*v tile shape of this sector not chosen yet");
    const int R = variant(kind, it->second).R;
    if (s.dn->items.find(R) == s.dn->items.end())
        return fail(ctx, MO_ED_ERR_STATE, "H*v item table of this sector not built yet");
    if (v_out) *v_out = it->second;
    if (R_out) *R_out = R;
    return MO_ED_OK;
}

int hv_single(mo_ed_ctx *ctx, const Sector &s, int kind, const void *x, void *y)
{
    int v;
    if (int rc = hv_prepare(ctx, s, kind, &v, nullptr)) return rc;
    return launch_one(ctx, s, kind, v, x, y);
}

}  // namespace moed
