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
// Work decomposition (both kernels).  An item is up to R rows made of whole
// down-spin bath groups, so the partner rows of spin-flip / pair hopping are
// in the item.  Items are ordered by the bath occupations of the conserved
// subsystems, so the down-spin neighbours of the rows in flight stay
// L2-resident.  A kernel walks a batch of jobs (vectors of possibly different
// sectors) so that all excitation vectors of a Lanczos step share one launch;
// optionally each item writes the FP64 partial of x*y for the Lanczos alpha.
//
// k_hv (first design): a CTA stages its rows in shared memory transposed,
// S[u][r], by blocking loads; one shared load of S[u'] serves the up-spin move
// u -> u' for all rows of the item.  Each thread owns 4 consecutive columns:
// 16-byte global loads for the down-spin row AXPYs and 16-byte stores of y
// (rows are padded to a 128-byte stride); its column moves come from a
// chunk-major table, one contiguous block per slot.
//
// k_hv_async (below): double-buffered asynchronous stage, conflict-free
// scheduled up-spin gathers, precomputed item descriptors.
//
// Split (below): k_hv_down computes the down-spin hybridisation over
// down-spin blocks x column slices from shared memory, or k_hv_down_rows as
// row AXPYs from L2; then k_hv_async<SPLIT> adds the other terms.  The
// autotuner picks among all of them per (precision, sector).
#include <algorithm>
#include <climits>
#include <map>
#include <mutex>
#include <tuple>

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
// staged variant (k_hv_async)
// ---------------------------------------------------------------------------
// The same sum per element, organised for latency hiding and few instructions:
//   * stage layout [tile][r][32]: column u of staged row r sits at
//     ((u >> 5) * R + r) * 32 + (u & 31).  The R values of a column are 32
//     elements apart, so one address serves every row (immediate offsets),
//     and column u is in bank u mod 32 for every row;
//   * the rows of the next item and its descriptor (the row data k_hv
//     computes per item: row indices, down-spin moves, interspecies diagonal,
//     spin-flip / pair-hop terms; built once by k_item_desc) are copied
//     (cp.async, 16 bytes per thread, L2 only) into the second of two stage
//     buffers while the current item is computed: two barriers per item;
//   * warp w owns chunks c = w + NW * (kHvCh * i + q) (32 columns each, one
//     column per lane), so every global load and store of a warp covers one
//     128-byte line and the kHvCh chunks of an iteration share their address
//     arithmetic (immediate offsets);
//   * up-spin moves follow the conflict-free schedule (species_sched): the
//     entries hold the stage offset of the target, one bank-conflict-free
//     shared load per staged row and slot, no predication;
//   * down-spin row AXPYs: one row offset per move serves the kHvCh chunks.
constexpr int kHvCh = 4;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all_but_newest() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

template <typename TA>
__device__ __forceinline__ int hv_find_job(const HvBatch<TA> &b, int item)
{
    int j = 0;
    while (j + 1 < b.njobs && item >= b.job[j + 1].item0) ++j;
    return j;
}

// next item of this CTA at or after `from` (stride gridDim.x) whose job is active
template <typename TA>
__device__ __forceinline__ int hv_next_item(const HvBatch<TA> &b, int from)
{
    for (int item = from; item < b.total_items; item += gridDim.x) {
        const HvJobT<TA> &jb = b.job[hv_find_job(b, item)];
        if (!jb.active || *jb.active != 0) return item;
    }
    return -1;
}

// Item descriptor: the per-item row data of k_hv (row indices, impurity
// patterns, down-spin moves, interspecies diagonal of the rows, spin-flip /
// pair-hop terms), computed once per (down species, R, precision) by
// k_item_desc and staged next to the rows.  Offsets are in 4-byte words.
struct DescGeom {
    int words, dm, nimp, npair;
    int o_d, o_id, o_dcnt, o_flags, o_ddiag, o_dtgt, o_dval, o_cross, o_quad;
    int o_sfsrc, o_phsrc, o_sfc, o_phc, o_rowmask;
};

template <typename TA, int R>
static DescGeom desc_geom(int dm, const ModelDev &m)
{
    const int ts = sizeof(TA) / 4;
    auto al = [](int w, int a) { return (w + a - 1) / a * a; };
    DescGeom g;
    g.dm = std::max(dm, 1);
    g.nimp = m.nimp;
    g.npair = std::max(m.npair, 1);
    int w = 0;
    g.o_d = w;       w += R;
    g.o_id = w;      w += R;
    g.o_dcnt = w;    w += R;
    g.o_flags = w;   w += 2;            // slow, item pair mask
    w = al(w, 2);
    g.o_ddiag = w;   w += R * ts;
    g.o_dtgt = w;    w += R * g.dm;
    w = al(w, 2);
    g.o_dval = w;    w += R * g.dm * ts;
    g.o_cross = w;   w += g.nimp * R * ts;
    w = al(w, 4);
    g.o_quad = w;    w += R * g.nimp * (int)(sizeof(Quad<TA>) / 4);
    g.o_sfsrc = w;   w += R * g.npair;
    g.o_phsrc = w;   w += R * g.npair;
    w = al(w, 2);
    g.o_sfc = w;     w += R * g.npair * ts;
    g.o_phc = w;     w += R * g.npair * ts;
    g.o_rowmask = w; w += g.npair;
    g.words = al(w, 4);
    return g;
}

// one thread per item: the row data the k_hv setup computes per item
template <typename TA, int R>
__global__ void k_item_desc(int nitems, const int *__restrict__ items, const int *__restrict__ dn_info,
                            const TA *__restrict__ dn_diag, const int *__restrict__ dn_tgt,
                            const TA *__restrict__ dn_val, int nd, const ModelDev *__restrict__ mdl, DescGeom g,
                            unsigned *__restrict__ out)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nitems) return;
    unsigned *rec = out + (size_t)it * g.words;
    for (int i = 0; i < g.words; ++i) rec[i] = 0u;
    int *od = (int *)(rec + g.o_d), *oid = (int *)(rec + g.o_id), *ocnt = (int *)(rec + g.o_dcnt);
    int *oflags = (int *)(rec + g.o_flags);
    TA *oddiag = (TA *)(rec + g.o_ddiag);
    int *odtgt = (int *)(rec + g.o_dtgt);
    TA *odval = (TA *)(rec + g.o_dval);
    TA *ocross = (TA *)(rec + g.o_cross);
    Quad<TA> *oquad = (Quad<TA> *)(rec + g.o_quad);
    int *osfsrc = (int *)(rec + g.o_sfsrc), *ophsrc = (int *)(rec + g.o_phsrc);
    TA *osfc = (TA *)(rec + g.o_sfc), *ophc = (TA *)(rec + g.o_phc);
    unsigned *orowmask = rec + g.o_rowmask;
    const int nimp = mdl->nimp, npair = mdl->npair;
    const TA Jc = (TA)mdl->J;
    int d[R], id[R];
    unsigned sfm[R], phm[R];
    int slow = 0;
    unsigned itemmask = 0u;
    for (int r = 0; r < R; ++r) {
        d[r] = items[it * R + r];
        id[r] = 0;
        sfm[r] = phm[r] = 0u;
        int cnt = 0;
        TA dg = TA(0);
        if (d[r] >= 0) {
            const int inf = dn_info[d[r]];
            id[r] = (inf >> 8) & 0xff;
            cnt = inf & 0xff;
            dg = dn_diag[d[r]];
            for (int s = 0; s < cnt; ++s) {
                odtgt[r * g.dm + s] = dn_tgt[(size_t)s * nd + d[r]];
                odval[r * g.dm + s] = dn_val[(size_t)s * nd + d[r]];
            }
        }
        od[r] = d[r];
        oid[r] = id[r];
        ocnt[r] = cnt;
        oddiag[r] = dg;
    }
    for (int iu = 0; iu < nimp; ++iu)
        for (int r = 0; r < R; ++r) ocross[iu * R + r] = (TA)mdl->cross[iu * nimp + id[r]];
    for (int r = 0; r < R; ++r) {
        if (d[r] < 0) continue;
        for (int p = 0; p < npair; ++p) {
            const int esf = mdl->t4[mdl->pair_rev[p] * nimp + id[r]];   // spin-flip: T_{j<-i}(d)
            const int eph = mdl->t4[p * nimp + id[r]];                  // pair hop:  T_{i<-j}(d)
            if (esf < 0) {
                const int off = (int)(short)(esf & 0xffff), dp = d[r] + off, rp = r + off;
                const bool local = rp >= 0 && rp < R && d[rp] == dp;
                osfsrc[r * g.npair + p] = local ? rp : -(1 + dp);
                osfc[r * g.npair + p] = (esf & 0x40000000) ? -Jc : Jc;
                sfm[r] |= 1u << p;
                orowmask[p] |= 1u << r;
                itemmask |= 1u << p;
                if (!local) slow = 1;
            }
            if (eph < 0) {
                const int off = (int)(short)(eph & 0xffff), dp = d[r] + off, rp = r + off;
                const bool local = rp >= 0 && rp < R && d[rp] == dp;
                ophsrc[r * g.npair + p] = local ? rp : -(1 + dp);
                ophc[r * g.npair + p] = (eph & 0x40000000) ? -Jc : Jc;
                phm[r] |= 1u << p;
                orowmask[p] |= 1u << (16 + r);
                itemmask |= 1u << p;
                if (!local) slow = 1;
            }
        }
    }
    for (int r = 0; r < R; ++r)
        for (int iu = 0; iu < nimp; ++iu) {
            Quad<TA> q;
            q.cnt = 0;
            for (int t = 0; t < 2; ++t) {
                q.du[t] = 0;
                q.src[t] = 0;
                q.c[t] = TA(0);
            }
            if (d[r] >= 0) {
                for (int p = 0; p < npair; ++p) {
                    const int e = mdl->t4[p * nimp + iu];
                    if (e >= 0) continue;
                    const int du = (int)(short)(e & 0xffff);
                    const TA tu = (e & 0x40000000) ? TA(-1) : TA(1);
                    if ((sfm[r] >> p) & 1u) {
                        if (q.cnt == 2) slow = 1;
                        else {
                            q.du[q.cnt] = (signed char)du;
                            q.src[q.cnt] = (unsigned char)max(osfsrc[r * g.npair + p], 0);
                            q.c[q.cnt] = tu * osfc[r * g.npair + p];
                            ++q.cnt;
                        }
                    }
                    if ((phm[r] >> p) & 1u) {
                        if (q.cnt == 2) slow = 1;
                        else {
                            q.du[q.cnt] = (signed char)du;
                            q.src[q.cnt] = (unsigned char)max(ophsrc[r * g.npair + p], 0);
                            q.c[q.cnt] = tu * ophc[r * g.npair + p];
                            ++q.cnt;
                        }
                    }
                }
            }
            oquad[r * nimp + iu] = q;
        }
    oflags[0] = slow;
    oflags[1] = (int)itemmask;
}

// all threads: copy the rows and the descriptor of `item` into a stage
// buffer and its descriptor buffer, and commit the group
template <typename TX, typename TA, int R, int NT>
__device__ __forceinline__ void hv_stage_item(const HvBatch<TA> &b, int item, TX *stage, unsigned *desc,
                                              int dwords)
{
    const HvJobT<TA> &jb = b.job[hv_find_job(b, item)];
    const int it = item - jb.item0;
    const int ld = jb.ld;
    constexpr int EPV = 16 / sizeof(TX);   // elements per 16-byte copy
    const int nv = ld / EPV;
    const TX *x = (const TX *)jb.x;
    const unsigned *src_desc = jb.desc + (size_t)it * dwords;
    for (int q = threadIdx.x; q < dwords / 4; q += NT) cp_async16(desc + 4 * q, src_desc + 4 * q);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int d = jb.items[it * R + r];
        if (d < 0) continue;
        const TX *src = x + (size_t)d * ld;
        for (int q = threadIdx.x; q < nv; q += NT) {
            const int u = q * EPV;
            cp_async16(stage + ((u >> 5) * R + r) * 32 + (u & 31), src + u);
        }
    }
    cp_async_commit();
}

// SPLIT: k_hv_down has already written the down-spin hybridisation into y;
// this kernel adds the other terms to it instead of computing the row AXPYs.
template <typename TX, typename TA, typename TY, int R, int NT, int MINB, bool SPLIT>
__global__ void __launch_bounds__(NT, MINB)
k_hv_async(const __grid_constant__ HvBatch<TA> batch, const ModelDev *__restrict__ mdl, const DescGeom g)
{
    extern __shared__ __align__(16) unsigned char smem_async[];
    const int nimp = mdl->nimp;
    int ldmax = 0;
    for (int i = 0; i < batch.njobs; ++i) ldmax = max(ldmax, batch.job[i].ld);
    const int stage_elems = R * ldmax;
    TX *stage0 = reinterpret_cast<TX *>(smem_async);
    TX *stage1 = stage0 + stage_elems;
    unsigned *desc0 = reinterpret_cast<unsigned *>(smem_async + ((2 * (size_t)stage_elems * sizeof(TX) + 15) & ~(size_t)15));
    unsigned *desc1 = desc0 + g.words;
    int *s_t4 = reinterpret_cast<int *>(desc1 + g.words);
    __shared__ unsigned s_pmask[kMaxImp];
    __shared__ double s_red[NT / 32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
    for (int i = tid; i < mdl->npair * nimp; i += NT) s_t4[i] = mdl->t4[i];
    for (int i = tid; i < nimp; i += NT) s_pmask[i] = mdl->pairmask[i];
    __syncthreads();

    int cur = hv_next_item(batch, (int)blockIdx.x);
    if (cur >= 0) hv_stage_item<TX, TA, R, NT>(batch, cur, stage0, desc0, g.words);
    int k = 0;
    while (cur >= 0) {
        const int buf = k & 1;
        const int nxt = hv_next_item(batch, cur + (int)gridDim.x);
        // buffers (k+1)&1 were released by the barrier that ended item k-1;
        // one commit group per iteration either way
        if (nxt >= 0) hv_stage_item<TX, TA, R, NT>(batch, nxt, buf ? stage0 : stage1, buf ? desc0 : desc1, g.words);
        else cp_async_commit();

        const HvJobT<TA> &jb = batch.job[hv_find_job(batch, cur)];
        const int it = cur - jb.item0;
        const int ld = jb.ld, nch = ld >> 5;
        const TX *__restrict__ x = (const TX *)jb.x;
        TY *__restrict__ y = (TY *)jb.y;
        cp_async_wait_all_but_newest();   // this thread's copies of the current item
        __syncthreads();                  // everyone's
        const TX *S = buf ? stage1 : stage0;
        const unsigned *dsc = buf ? desc1 : desc0;
        const int *s_d = (const int *)(dsc + g.o_d);
        const int *s_dcnt = (const int *)(dsc + g.o_dcnt);
        const int *s_dtgt = (const int *)(dsc + g.o_dtgt);
        const TA *s_dval = (const TA *)(dsc + g.o_dval);
        const TA *s_crossT = (const TA *)(dsc + g.o_cross);
        const Quad<TA> *s_q = (const Quad<TA> *)(dsc + g.o_quad);
        const int *s_sfsrc = (const int *)(dsc + g.o_sfsrc), *s_phsrc = (const int *)(dsc + g.o_phsrc);
        const TA *s_sfc = (const TA *)(dsc + g.o_sfc), *s_phc = (const TA *)(dsc + g.o_phc);
        const unsigned *s_rowmask = dsc + g.o_rowmask;
        const bool slow = ((const int *)(dsc + g.o_flags))[0] != 0;
        const unsigned imask = (unsigned)((const int *)(dsc + g.o_flags))[1];
        const int dm = g.dm, npr = g.npair;

        TA ddiag[R];
        bool live[R];
        int dcnt[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ddiag[r] = ((const TA *)(dsc + g.o_ddiag))[r];
            live[r] = s_d[r] >= 0;
            dcnt[r] = s_dcnt[r];
        }
        const bool want_dot = jb.dot_partial != nullptr;
        double dacc = 0.0;
        constexpr int SB = 4;
        constexpr int DB = 2;
        for (int cb = warp; cb < nch; cb += NW * kHvCh) {
            // chunks cb + NW*q, q < kHvCh; column of this lane in chunk q: ub + 32*NW*q
            const int ub = 32 * cb + lane;
            bool has[kHvCh];
            int iu[kHvCh];
            int2 h[kHvCh];
            TA acc[kHvCh][R];
#pragma unroll
            for (int q = 0; q < kHvCh; ++q) {
                has[q] = cb + NW * q < nch;
                h[q] = has[q] ? __ldg(jb.up_sched_hdr + cb + NW * q) : make_int2(0, 0);
            }
            // the first DB down-spin moves of every row (SPLIT: the down-spin
            // part already in y): loads in flight early
            TX gd[R][DB][kHvCh];
            TY yp[R][kHvCh];
            if constexpr (SPLIT) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const TY *yr = y + (size_t)(live[r] ? s_d[r] : 0) * ld + ub;
#pragma unroll
                    for (int q = 0; q < kHvCh; ++q) yp[r][q] = (live[r] && has[q]) ? yr[32 * NW * q] : TY(0);
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int t = 0; t < DB; ++t) {
                        const bool mv = t < dcnt[r];
                        const TX *xr = x + (size_t)s_dtgt[r * dm + (mv ? t : 0)] * ld + ub;
#pragma unroll
                        for (int q = 0; q < kHvCh; ++q)
                            gd[r][t][q] = (mv && has[q]) ? __ldg(xr + 32 * NW * q) : TX(0);
                    }
            }
            // first SB schedule entries of every chunk
            HopEnt<TA> e0[kHvCh][SB];
#pragma unroll
            for (int q = 0; q < kHvCh; ++q)
#pragma unroll
                for (int t = 0; t < SB; ++t)
                    e0[q][t] = (t < h[q].y) ? jb.up_sched[h[q].x + 32 * t + lane] : HopEnt<TA>{};
            // diagonal
#pragma unroll
            for (int q = 0; q < kHvCh; ++q) {
                const int u = ub + 32 * NW * q;
                int inf = 0;
                TA ud = TA(0);
                if (has[q]) {
                    inf = __ldg(jb.up_info + u);
                    ud = __ldg(jb.up_diag + u);
                }
                iu[q] = (inf >> 8) & 0xff;
#pragma unroll
                for (int r = 0; r < R; ++r) acc[q][r] = TA(0);
                if (has[q]) {
                    const TX *so = S + ((u >> 5) * R) * 32 + (u & 31);
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        acc[q][r] = (ud + ddiag[r] + s_crossT[iu[q] * R + r]) * (TA)so[32 * r];
                }
            }
            // up-spin hybridisation: scheduled conflict-free gathers
#pragma unroll
            for (int q = 0; q < kHvCh; ++q) {
                const int ns = h[q].y;
                const HopEnt<TA> *tab = jb.up_sched + h[q].x + lane;
                HopEnt<TA> e[SB];
#pragma unroll
                for (int t = 0; t < SB; ++t) e[t] = e0[q][t];
                for (int s0 = 0; s0 < ns; s0 += SB) {
                    HopEnt<TA> f[SB];
#pragma unroll
                    for (int t = 0; t < SB; ++t) f[t] = (s0 + SB + t < ns) ? tab[32 * (s0 + SB + t)] : HopEnt<TA>{};
#pragma unroll
                    for (int t = 0; t < SB; ++t) {
                        if (s0 + t < ns) {
                            const TX *st = S + e[t].t;
#pragma unroll
                            for (int r = 0; r < R; ++r) acc[q][r] += e[t].v * (TA)st[32 * r];
                        }
                    }
#pragma unroll
                    for (int t = 0; t < SB; ++t) e[t] = f[t];
                }
            }
            // spin-flip and pair hopping (partner rows staged)
#pragma unroll
            for (int q = 0; q < kHvCh; ++q) {
                if (!has[q]) continue;
                const int u = ub + 32 * NW * q;
                if (!slow) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const Quad<TA> qd = s_q[r * nimp + iu[q]];
                        if (qd.cnt > 0) {
#pragma unroll
                            for (int t = 0; t < 2; ++t) {
                                if (t < qd.cnt) {
                                    const int w = u + qd.du[t];
                                    acc[q][r] += qd.c[t] * (TA)S[((w >> 5) * R + qd.src[t]) * 32 + (w & 31)];
                                }
                            }
                        }
                    }
                } else {
                    unsigned pm = s_pmask[iu[q]] & imask;
                    while (pm) {
                        const int p = __ffs(pm) - 1;
                        pm &= pm - 1;
                        const int e = s_t4[p * nimp + iu[q]];
                        const int w = u + (int)(short)(e & 0xffff);
                        const bool neg = (e & 0x40000000) != 0;
                        const unsigned rm = s_rowmask[p];
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            if ((rm >> r) & 1u) {
                                const int src = s_sfsrc[r * npr + p];
                                const TX xv = src >= 0 ? S[((w >> 5) * R + src) * 32 + (w & 31)]
                                                       : __ldg(x + (size_t)(-1 - src) * ld + w);
                                const TA cf = neg ? -s_sfc[r * npr + p] : s_sfc[r * npr + p];
                                acc[q][r] += cf * (TA)xv;
                            }
                            if ((rm >> (16 + r)) & 1u) {
                                const int src = s_phsrc[r * npr + p];
                                const TX xv = src >= 0 ? S[((w >> 5) * R + src) * 32 + (w & 31)]
                                                       : __ldg(x + (size_t)(-1 - src) * ld + w);
                                const TA cf = neg ? -s_phc[r * npr + p] : s_phc[r * npr + p];
                                acc[q][r] += cf * (TA)xv;
                            }
                        }
                    }
                }
            }
            // down-spin hybridisation: the early loads, then the remaining moves
            if constexpr (SPLIT) {
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int q = 0; q < kHvCh; ++q) acc[q][r] += (TA)yp[r][q];
            } else {
#pragma unroll
            for (int r = 0; r < R; ++r) {
#pragma unroll
                for (int t = 0; t < DB; ++t) {
                    if (t < dcnt[r]) {
                        const TA v = s_dval[r * dm + t];
#pragma unroll
                        for (int q = 0; q < kHvCh; ++q) acc[q][r] += v * (TA)gd[r][t][q];
                    }
                }
                for (int t0 = DB; t0 < dcnt[r]; t0 += DB) {
                    TX g2[DB][kHvCh];
#pragma unroll
                    for (int t = 0; t < DB; ++t) {
                        const bool mv = t0 + t < dcnt[r];
                        const TX *xr = x + (size_t)s_dtgt[r * dm + (mv ? t0 + t : t0)] * ld + ub;
#pragma unroll
                        for (int q = 0; q < kHvCh; ++q) g2[t][q] = (mv && has[q]) ? __ldg(xr + 32 * NW * q) : TX(0);
                    }
#pragma unroll
                    for (int t = 0; t < DB; ++t) {
                        if (t0 + t < dcnt[r]) {
                            const TA v = s_dval[r * dm + t0 + t];
#pragma unroll
                            for (int q = 0; q < kHvCh; ++q) acc[q][r] += v * (TA)g2[t][q];
                        }
                    }
                }
            }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (!live[r]) continue;
                TY *yr = y + (size_t)s_d[r] * ld + ub;
#pragma unroll
                for (int q = 0; q < kHvCh; ++q)
                    if (has[q]) yr[32 * NW * q] = (TY)acc[q][r];
            }
            if (want_dot) {
                TA part = TA(0);
#pragma unroll
                for (int q = 0; q < kHvCh; ++q) {
                    if (!has[q]) continue;
                    const int u = ub + 32 * NW * q;
                    const TX *so = S + ((u >> 5) * R) * 32 + (u & 31);
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        if (live[r]) part += (TA)so[32 * r] * (TA)(TY)acc[q][r];
                }
                dacc += (double)part;
            }
        }
        if (want_dot) {
            for (int off = 16; off > 0; off >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, off);
            if (lane == 0) s_red[warp] = dacc;
        }
        __syncthreads();   // item done: its buffers are free
        if (want_dot && tid == 0) {
            double t = 0.0;
            for (int w = 0; w < NW; ++w) t += s_red[w];
            jb.dot_partial[it] = t;
        }
        cur = nxt;
        ++k;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// ---------------------------------------------------------------------------
// k_hv_down: the down-spin hybridisation of the split H*v,
//   y[d][u] = sum over moves (d -> d', t) of t * x[d'][u],
// for every row d, written (not accumulated) into y; k_hv_async<SPLIT> then
// adds the other terms.  The rows of a down-spin block (equal electron counts
// in every conserved subsystem) are closed under the moves, so a chunk = one
// block x a range of columns is independent of all others.  A CTA stages the
// block's move list once ({target index within the block, signed coupling})
// and then walks the chunk's column slices, staged by cp.async and double-
// buffered when two slices fit.  A slice is kb groups of WB bytes (one 64- or
// 128-byte line segment) of every row of the block, kb as large as the buffer
// allows, so small blocks take wide slices.  Every element of x is read from
// memory once per H*v and the moves read shared memory only.  CTAs take
// contiguous chunk ranges, so consecutive chunks usually share the block and
// its move list.
// ---------------------------------------------------------------------------
template <typename TA>
__device__ __forceinline__ int hv_tile_job(const HvBatch<TA> &b, int tile)
{
    int j = 0;
    while (j + 1 < b.njobs && tile >= b.job[j + 1].tile0) ++j;
    return j;
}

struct DownLayout {        // shared-memory layout of k_hv_down, in bytes
    int ptr, rows, mv, x0, x1;
};

// stage columns [col, col + kw * W) of the block's rows: row i at buf + i * kw * W
template <typename TX, int NT, int WB>
__device__ __forceinline__ void hv_down_slice(const TX *__restrict__ x, const int *s_rows, int nr, int ld,
                                              int col, int kw, TX *buf)
{
    constexpr int CPG = WB / 16;                // 16-byte copies per group of a row
    constexpr int EPV = 16 / (int)sizeof(TX);
    const int cpr = kw * CPG;
    for (int q = threadIdx.x; q < nr * cpr; q += NT) {
        const int i = q / cpr, c = q - i * cpr;
        cp_async16(buf + (size_t)i * cpr * EPV + c * EPV, x + (size_t)s_rows[i] * ld + col + c * EPV);
    }
}

template <typename TX, typename TA, typename TY, int NT, int WB>
__global__ void __launch_bounds__(NT, 1)
k_hv_down(const __grid_constant__ HvBatch<TA> batch, int total, const DownLayout L, int cap_rows, int dbuf)
{
    extern __shared__ __align__(16) unsigned char smem_down[];
    constexpr int W = WB / (int)sizeof(TX);   // columns per group (one WB-byte segment of a row)
    constexpr int RPW = 32 / W;               // groups per warp pass
    constexpr int NW = NT / 32;
    int *s_ptr = reinterpret_cast<int *>(smem_down + L.ptr);
    int *s_rows = reinterpret_cast<int *>(smem_down + L.rows);
    HopEnt<TA> *s_mv = reinterpret_cast<HopEnt<TA> *>(smem_down + L.mv);
    TX *const xb0 = reinterpret_cast<TX *>(smem_down + L.x0);
    TX *const xb1 = reinterpret_cast<TX *>(smem_down + L.x1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int sub = lane / W, c = lane - sub * W;
    const int c_begin = (int)((long long)total * blockIdx.x / gridDim.x);
    const int c_end = (int)((long long)total * (blockIdx.x + 1) / gridDim.x);
    int have_job = -1, have_blk = -1;
    for (int ch = c_begin; ch < c_end; ++ch) {
        const int jid = hv_tile_job(batch, ch);
        const HvJobT<TA> &jb = batch.job[jid];
        if (jb.active && *jb.active == 0) continue;
        const int lc = ch - jb.tile0;
        // block of this chunk: last b with chunks[b].x <= lc
        int lo = 0, hi = jb.dblk_n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&jb.dblk_chunks[mid].x) <= lc) lo = mid;
            else hi = mid - 1;
        }
        const int blk = lo;
        const int2 cinfo = jb.dblk_chunks[blk];
        const int ld = jb.ld;
        const int col0 = (lc - cinfo.x) * cinfo.y * 32;
        const int col1 = min(ld, col0 + cinfo.y * 32);
        const int p0 = __ldg(jb.dblk_off + blk), nr = __ldg(jb.dblk_off + blk + 1) - p0;
        const TX *x = (const TX *)jb.x;
        TY *y = (TY *)jb.y;
        __syncthreads();   // the previous chunk is done with shared memory
        if (jid != have_job || blk != have_blk) {
            const int m0 = __ldg(jb.dblk_ptr + p0), nm = __ldg(jb.dblk_ptr + p0 + nr) - m0;
            for (int i = tid; i <= nr; i += NT) s_ptr[i] = __ldg(jb.dblk_ptr + p0 + i) - m0;
            for (int i = tid; i < nr; i += NT) s_rows[i] = __ldg(jb.dblk_rows + p0 + i);
            for (int i = tid; i < nm; i += NT) s_mv[i] = jb.dblk_mv[m0 + i];
            have_job = jid;
            have_blk = blk;
            __syncthreads();
        }
        // a slice = kb groups of W columns of every row (small blocks: wide slices)
        const int ngr = (col1 - col0) / W;
        const int kb = max(1, min(cap_rows / nr, ngr));
        const int ns = (ngr + kb - 1) / kb;
        hv_down_slice<TX, NT, WB>(x, s_rows, nr, ld, col0, min(kb, ngr), xb0);
        cp_async_commit();
        for (int sl = 0; sl < ns; ++sl) {
            const TX *S = (dbuf && (sl & 1)) ? xb1 : xb0;
            const int kw = min(kb, ngr - sl * kb);   // groups in this slice
            if (dbuf && sl + 1 < ns) {
                hv_down_slice<TX, NT, WB>(x, s_rows, nr, ld, col0 + (sl + 1) * kb * W, min(kb, ngr - (sl + 1) * kb),
                                          (sl & 1) ? xb0 : xb1);
                cp_async_commit();
                cp_async_wait_all_but_newest();
            } else {
                asm volatile("cp.async.wait_all;" ::: "memory");
            }
            __syncthreads();
            const int ws = kw * W;               // row stride of the staged slice
            TY *ys = y + col0 + sl * kb * W + c;
            if (kw == 1) {
                // one group per row (large blocks): 4 moves in flight
                for (int i = warp * RPW + sub; i < nr; i += NW * RPW) {
                    const int b1 = s_ptr[i], e1 = s_ptr[i + 1];
                    const TX *Sc = S + c;
                    TA a = TA(0);
                    int e = b1;
                    for (; e + 4 <= e1; e += 4) {
                        const HopEnt<TA> m0 = s_mv[e], m1 = s_mv[e + 1], m2 = s_mv[e + 2], m3 = s_mv[e + 3];
                        const TX x0 = Sc[m0.t * W], x1 = Sc[m1.t * W], x2 = Sc[m2.t * W], x3 = Sc[m3.t * W];
                        a += m0.v * (TA)x0;
                        a += m1.v * (TA)x1;
                        a += m2.v * (TA)x2;
                        a += m3.v * (TA)x3;
                    }
                    for (; e < e1; ++e) {
                        const HopEnt<TA> m = s_mv[e];
                        a += m.v * (TA)Sc[m.t * W];
                    }
                    ys[(size_t)s_rows[i] * ld] = (TY)a;
                }
            } else {
                // several groups per row (small blocks, wide slices): each move
                // serves up to KQ groups
                constexpr int KQ = 4;
                const int npass = (kw + KQ - 1) / KQ;
                for (int it = warp * RPW + sub; it < nr * npass; it += NW * RPW) {
                    const int i = it / npass, g0 = (it - i * npass) * KQ;
                    const int b1 = s_ptr[i], e1 = s_ptr[i + 1];
                    const TX *Sc = S + g0 * W + c;
                    TA a[KQ];
#pragma unroll
                    for (int q = 0; q < KQ; ++q) a[q] = TA(0);
                    for (int e = b1; e < e1; ++e) {
                        const HopEnt<TA> m = s_mv[e];
                        const TX *Sm = Sc + m.t * ws;
#pragma unroll
                        for (int q = 0; q < KQ; ++q)
                            if (g0 + q < kw) a[q] += m.v * (TA)Sm[q * W];
                    }
                    TY *yr = ys + (size_t)s_rows[i] * ld + g0 * W;
#pragma unroll
                    for (int q = 0; q < KQ; ++q)
                        if (g0 + q < kw) yr[q * W] = (TY)a[q];
                }
            }
            __syncthreads();   // slice done: its buffer is free
            if (!dbuf && sl + 1 < ns) {
                hv_down_slice<TX, NT, WB>(x, s_rows, nr, ld, col0 + (sl + 1) * kb * W, min(kb, ngr - (sl + 1) * kb),
                                          xb0);
                cp_async_commit();
            }
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// ---------------------------------------------------------------------------
// k_hv_down_rows: the same down-spin term as k_hv_down, as row AXPYs,
//   y[d][c] = sum over moves (d -> d', t) of t * x[d'][c],
// straight from the species' per-row move tables (dn_info / dn_tgt /
// dn_val), with no staging.  A tile is one row d times 4 NT CPT columns,
// each thread CPT chunks of four consecutive columns, 4 NT apart (16-byte
// loads and stores; rows are padded to a multiple of 32 elements).  The
// row's move targets and couplings are staged in shared memory first, one
// per thread, so the x loads of all its moves can be in flight at once.
// Tiles run
// column-tile-major: the CTAs in flight share one column tile of x (C4 with
// CPT = 2: 6,435 rows x 1,024 columns, 26 MB), which stays in L2 while each
// source segment is read by the rows that move to it, so x comes from memory
// about once per H*v.
// ---------------------------------------------------------------------------
// The host guarantees dn_maxcnt <= NT (launch_batch_rows).
template <typename TX, typename TA, typename TY, int NT, int CPT>
__global__ void __launch_bounds__(NT)
k_hv_down_rows(const __grid_constant__ HvBatch<TA> batch, int total)
{
    __shared__ int s_tgt[NT];
    __shared__ TA s_val[NT];
    for (int t = blockIdx.x; t < total; t += gridDim.x) {   // t is uniform over the CTA
        const int jid = hv_tile_job(batch, t);
        const HvJobT<TA> &jb = batch.job[jid];
        if (jb.active && *jb.active == 0) continue;
        const int lt = t - jb.tile0;
        const int ct = lt / jb.nd, d = lt - ct * jb.nd;
        const int cnt = min(__ldg(&jb.dn_info[d]) & 0xff, NT);
        __syncthreads();   // the previous tile is done with s_tgt / s_val
        if ((int)threadIdx.x < cnt) {
            s_tgt[threadIdx.x] = __ldg(&jb.dn_tgt[(size_t)threadIdx.x * jb.nd + d]);
            s_val[threadIdx.x] = __ldg(&jb.dn_val[(size_t)threadIdx.x * jb.nd + d]);
        }
        __syncthreads();
        const int c0 = ct * 4 * NT * CPT + 4 * (int)threadIdx.x;
        if (c0 >= jb.ld) continue;   // ld is a multiple of 4: a chunk at c < ld ends before ld
        const TX *x = (const TX *)jb.x;
        TA a[CPT][4];
#pragma unroll
        for (int k = 0; k < CPT; ++k)
#pragma unroll
            for (int q = 0; q < 4; ++q) a[k][q] = TA(0);
#pragma unroll 4
        for (int h = 0; h < cnt; ++h) {
            const TA v = s_val[h];
            const TX *xr = x + (size_t)s_tgt[h] * jb.ld;
#pragma unroll
            for (int k = 0; k < CPT; ++k)
                if (k == 0 || c0 + k * 4 * NT < jb.ld) {   // chunk 0 is in range (checked above)
                    const Vec4<TX> xv = ldg4(xr + c0 + k * 4 * NT);
#pragma unroll
                    for (int q = 0; q < 4; ++q) a[k][q] += v * (TA)xv.v[q];
                }
        }
        TY *yr = (TY *)jb.y + (size_t)d * jb.ld;
#pragma unroll
        for (int k = 0; k < CPT; ++k)
            if (k == 0 || c0 + k * 4 * NT < jb.ld) {
                TY o[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) o[q] = (TY)a[k][q];
                stg4(yr + c0 + k * 4 * NT, o);
            }
    }
}

template <typename TX, typename TA, int R>
static size_t dyn_smem_bytes_async(int ld, const ModelDev &m, const DescGeom &g)
{
    return ((2 * (size_t)R * ld * sizeof(TX) + 15) & ~(size_t)15) + sizeof(unsigned) * 2 * (size_t)g.words +
           sizeof(int) * (size_t)m.npair * m.nimp;
}

// ---------------------------------------------------------------------------
// tile-shape variants and the autotuner
// ---------------------------------------------------------------------------
// A variant fixes the kernel (k_hv or k_hv_async), the rows per item R, the CTA
// size NT and the CTAs per SM the register budget is cut for (MINB).  The
// k_hv variants compute every element with the same sequence of operations
// (bit-identical outputs); k_hv_async adds the up-spin terms in the order of
// the gather schedule, so FP32 outputs of the two kernels agree to rounding.
// The first H*v of a (kind, Nup, Ndn) shape times each variant on that sector
// (scratch vectors, CUDA events on the context stream) and keeps the fastest.
struct HvVariant {
    int R, NT, MINB;
    // 0: k_hv; 1: k_hv_async (double-buffered asynchronous stage);
    // 2 / 3: split, k_hv_down on 128- / 64-byte row slices + k_hv_async<SPLIT>;
    // 4: split, k_hv_down_rows (row AXPYs from L2) + k_hv_async<SPLIT>
    int staged;
};
static const HvVariant kVarF32[] = {{3, 512, 2, 0}, {4, 256, 2, 0}, {6, 512, 1, 0}, {3, 256, 3, 0},
                                    {8, 512, 1, 0}, {4, 512, 1, 1}, {3, 512, 1, 1}, {2, 512, 2, 1},
                                    {2, 256, 2, 1}, {3, 512, 1, 2}, {4, 512, 1, 2}, {3, 512, 1, 3},
                                    {3, 512, 1, 4}, {4, 512, 1, 4}, {4, 512, 1, 4}};
static const HvVariant kVarF64[] = {{2, 256, 2, 0}, {3, 256, 1, 0}, {2, 512, 1, 0}, {2, 512, 1, 1},
                                    {4, 512, 1, 1}, {2, 512, 1, 2}, {2, 512, 1, 3}, {2, 512, 1, 4}};
static const int kNVarF32 = sizeof(kVarF32) / sizeof(kVarF32[0]);
static const int kNVarF64 = sizeof(kVarF64) / sizeof(kVarF64[0]);

static const HvVariant &variant(int kind, int v) { return kind == HV_F32 ? kVarF32[v] : kVarF64[v]; }
static int nvariants(int kind) { return kind == HV_F32 ? kNVarF32 : kNVarF64; }

constexpr long long kTuneMinElems = 1ll << 18;   // smaller sectors take variant 0 untimed

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
    j.up_sched_hdr = s.up->sched_hdr;
    j.up_sched_ent = s.up->sched_ent;
    {
        auto dsc = s.dn->desc.find(R * 2 + (f32 ? 0 : 1));
        j.desc = dsc != s.dn->desc.end() ? dsc->second : nullptr;
    }
    j.dblk_off = s.dn->dblk_off;
    j.dblk_rows = s.dn->dblk_rows;
    j.dblk_ptr = s.dn->dblk_ptr;
    j.dblk_mv = f32 ? (const HopEnt<TA> *)s.dn->dblk_mv_f : (const HopEnt<TA> *)s.dn->dblk_mv_d;
    {
        auto ch = s.dn->dblk_chunks.find(s.ld());
        j.dblk_chunks = ch != s.dn->dblk_chunks.end() ? ch->second : nullptr;
        j.ntiles = ch != s.dn->dblk_chunks.end() ? s.dn->dblk_nchunks.at(s.ld()) : 0;
    }
    j.dblk_n = s.dn->dblk_n;
    j.dblk_max = s.dn->dblk_max;
    j.dblk_mvmax = s.dn->dblk_mvmax;
    j.tile0 = 0;
    if (f32) {
        auto sf = s.up->sched_rf.find(R);
        j.up_sched = sf != s.up->sched_rf.end() ? (const HopEnt<TA> *)sf->second : nullptr;
    } else {
        auto sd = s.up->sched_rd.find(R);
        j.up_sched = sd != s.up->sched_rd.end() ? (const HopEnt<TA> *)sd->second : nullptr;
    }
}
template void hv_fill_job<float>(const mo_ed_ctx *, const Sector &, int, const void *, void *, HvJobT<float> &);
template void hv_fill_job<double>(const mo_ed_ctx *, const Sector &, int, const void *, void *, HvJobT<double> &);

// Makes kernel k launchable with smem bytes of dynamic shared memory (and the
// full carveout) and returns its resident CTAs per SM at nt threads.  The
// runtime calls cost more than the launch of a small sector's H*v, so they
// are made once per (device, kernel): the shared-memory limit only ever
// rises, and the occupancy is kept per (device, kernel, size, threads).
// Process-wide, under a lock, so contexts on one device agree.
static std::mutex g_kfit_mu;
static std::map<std::pair<int, const void *>, size_t> g_kfit_smem;
static std::map<std::tuple<int, const void *, size_t, int>, int> g_kfit_occ;

template <typename K>
static int kernel_fit(mo_ed_ctx *ctx, K k, int nt, size_t smem, int *per_sm)
{
    std::lock_guard<std::mutex> lock(g_kfit_mu);
    const void *kp = (const void *)k;
    auto ins = g_kfit_smem.emplace(std::make_pair(ctx->device, kp), (size_t)0);
    size_t &set = ins.first->second;
    if (ins.second)
        MOED_CUDA(ctx, cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    if (smem > set) {
        MOED_CUDA(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        set = smem;
    }
    const auto key = std::make_tuple(ctx->device, kp, smem, nt);
    auto it = g_kfit_occ.find(key);
    if (it == g_kfit_occ.end()) {
        int n = 0;
        MOED_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, nt, smem));
        it = g_kfit_occ.emplace(key, n).first;
    }
    *per_sm = it->second;
    return MO_ED_OK;
}

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
    int per_sm = 0;
    if (int rc = kernel_fit(ctx, kern, NT, smem, &per_sm)) return rc;
    if (per_sm < 1) return fail(ctx, MO_ED_ERR_ARG, "sector rows too long for the shared-memory stage");
    const int grid = std::min(b.total_items, ctx->num_sms * per_sm);
    kern<<<grid, NT, smem, ctx->stream>>>(b, ctx->d_mdl);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

template <typename TX, typename TA, typename TY, int R, int NT, int MINB = 1, bool SPLIT = false>
static int launch_batch_async(mo_ed_ctx *ctx, const HvBatch<TA> &b)
{
    if (b.total_items <= 0) return MO_ED_OK;
    int ldmax = 0;
    for (int i = 0; i < b.njobs; ++i) {
        ldmax = std::max(ldmax, b.job[i].ld);
        if (!b.job[i].items || !b.job[i].up_sched_hdr || !b.job[i].up_sched || !b.job[i].desc)
            return fail(ctx, MO_ED_ERR_STATE, "H*v tables missing");
    }
    const DescGeom g = desc_geom<TA, R>(ctx->mdl.ncpl, ctx->mdl);
    const size_t smem = dyn_smem_bytes_async<TX, TA, R>(ldmax, ctx->mdl, g);
    auto kern = k_hv_async<TX, TA, TY, R, NT, MINB, SPLIT>;
    int per_sm = 0;
    if (int rc = kernel_fit(ctx, kern, NT, smem, &per_sm)) return rc;
    if (per_sm < 1) return fail(ctx, MO_ED_ERR_ARG, "sector rows too long for the shared-memory stage");
    const int grid = std::min(b.total_items, ctx->num_sms * per_sm);
    kern<<<grid, NT, smem, ctx->stream>>>(b, ctx->d_mdl, g);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

constexpr int kDownNT = 1024;
constexpr size_t kDownSmemMax = 220 * 1024;   // dynamic shared memory of one k_hv_down CTA

static size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// shared-memory layout of k_hv_down for blocks of up to `rows` rows and `mv`
// moves and slices of wb bytes per row; nbuf = 1 or 2 slice buffers
static DownLayout down_layout(int rows, int mv, size_t wb, int nbuf, size_t ent_bytes, size_t *total)
{
    DownLayout L;
    size_t o = 0;
    L.ptr = (int)o;
    o = align16(o + sizeof(int) * ((size_t)rows + 1));
    L.rows = (int)o;
    o = align16(o + sizeof(int) * (size_t)rows);
    L.mv = (int)o;
    o = align16(o + ent_bytes * (size_t)std::max(mv, 1));
    L.x0 = (int)o;
    o += (size_t)rows * wb;
    L.x1 = (int)o;
    if (nbuf == 2) o += (size_t)rows * wb;
    *total = o;
    return L;
}

// Split H*v: k_hv_down writes the down-spin hybridisation into y, then
// k_hv_async<SPLIT> adds the other terms (both on the context stream).
template <typename TX, typename TA, typename TY, int R, int NT, int MINB, int WB>
static int launch_batch_split(mo_ed_ctx *ctx, const HvBatch<TA> &b0)
{
    if (b0.total_items <= 0) return MO_ED_OK;
    HvBatch<TA> b = b0;
    int tiles = 0, maxrows = 0, maxmv = 0;
    for (int i = 0; i < b.njobs; ++i) {
        HvJobT<TA> &j = b.job[i];
        if (!j.dblk_ptr || !j.dblk_chunks || j.dblk_n < 1 || j.ld % 32 != 0)
            return fail(ctx, MO_ED_ERR_STATE, "H*v down-spin block tables missing");
        j.tile0 = tiles;
        tiles += j.ntiles;
        maxrows = std::max(maxrows, j.dblk_max);
        maxmv = std::max(maxmv, j.dblk_mvmax);
    }
    size_t smem = 0;
    int dbuf = 1;
    DownLayout L = down_layout(maxrows, maxmv, WB, 2, sizeof(HopEnt<TA>), &smem);
    if (smem > kDownSmemMax) {
        dbuf = 0;
        L = down_layout(maxrows, maxmv, WB, 1, sizeof(HopEnt<TA>), &smem);
    }
    if (smem > kDownSmemMax) return fail(ctx, MO_ED_ERR_ARG, "down-spin blocks too large for the split H*v");
    auto kd = k_hv_down<TX, TA, TY, kDownNT, WB>;
    int per_sm = 0;
    if (int rc = kernel_fit(ctx, kd, kDownNT, smem, &per_sm)) return rc;
    if (per_sm < 1) return fail(ctx, MO_ED_ERR_ARG, "down-spin blocks too large for the split H*v");
    const int grid = std::min(tiles, ctx->num_sms * per_sm);
    kd<<<grid, kDownNT, smem, ctx->stream>>>(b, tiles, L, maxrows, dbuf);
    MOED_CHECK_LAUNCH(ctx);
    return launch_batch_async<TX, TA, TY, R, NT, MINB, true>(ctx, b);
}

// Split H*v with the row-AXPY down pass: k_hv_down_rows writes the
// down-spin hybridisation into y, then k_hv_async<SPLIT> adds the rest.
constexpr int kRowsNT = 128;   // 512 CPT columns per tile
template <typename TX, typename TA, typename TY, int R, int NT, int MINB, int CPT = 2>
static int launch_batch_rows(mo_ed_ctx *ctx, const HvBatch<TA> &b0)
{
    if (b0.total_items <= 0) return MO_ED_OK;
    HvBatch<TA> b = b0;
    long long tiles = 0;
    for (int i = 0; i < b.njobs; ++i) {
        HvJobT<TA> &j = b.job[i];
        if (!j.dn_info || !j.dn_tgt || !j.dn_val || j.ld % 4 != 0)
            return fail(ctx, MO_ED_ERR_STATE, "H*v down-spin move tables missing");
        if (j.dn_maxcnt > kRowsNT) return fail(ctx, MO_ED_ERR_ARG, "more down-spin moves per row than the row-AXPY CTA stages");
        j.tile0 = (int)tiles;
        j.ntiles = j.nd * ((j.ld + 4 * kRowsNT * CPT - 1) / (4 * kRowsNT * CPT));
        tiles += j.ntiles;
    }
    if (tiles > INT_MAX) return fail(ctx, MO_ED_ERR_ARG, "too many row tiles for the row-AXPY H*v");
    auto kd = k_hv_down_rows<TX, TA, TY, kRowsNT, CPT>;
    int per_sm = 0;
    if (int rc = kernel_fit(ctx, kd, kRowsNT, 0, &per_sm)) return rc;
    const int grid = (int)std::min<long long>(tiles, (long long)ctx->num_sms * std::max(per_sm, 1));
    if (grid > 0) {
        kd<<<grid, kRowsNT, 0, ctx->stream>>>(b, (int)tiles);
        MOED_CHECK_LAUNCH(ctx);
    }
    return launch_batch_async<TX, TA, TY, R, NT, MINB, true>(ctx, b);
}

// Whether the split kernel fits every down-spin block of the model (any
// electron count: at most dblk_bound rows and dblk_mv_bound moves).
static bool split_fits(const mo_ed_ctx *ctx, size_t wb, size_t ent_bytes)
{
    size_t smem = 0;
    down_layout(ctx->dblk_bound, ctx->dblk_mv_bound, wb, 1, ent_bytes, &smem);
    return smem <= kDownSmemMax;
}

template <typename TA, int R>
static int build_desc_r(mo_ed_ctx *ctx, Species *dn, unsigned **out)
{
    const DescGeom g = desc_geom<TA, R>(ctx->mdl.ncpl, ctx->mdl);
    const int n = dn->nitems.at(R);
    unsigned *p = nullptr;
    MOED_CUDA(ctx, cudaMalloc(&p, sizeof(unsigned) * (size_t)g.words * std::max(n, 1)));
    *out = p;
    const bool f32 = sizeof(TA) == 4;
    k_item_desc<TA, R><<<(n + 127) / 128, 128, 0, ctx->stream>>>(
        n, dn->items.at(R), dn->info, f32 ? (const TA *)dn->diag_f : (const TA *)dn->diag_d, dn->hop_tgt,
        f32 ? (const TA *)dn->hop_val_f : (const TA *)dn->hop_val_d, dn->n, ctx->d_mdl, g, p);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

// item descriptors of the down species for R rows per item (k_hv_async)
static int species_desc(mo_ed_ctx *ctx, Species *dn, int R, bool f32)
{
    const int key = R * 2 + (f32 ? 0 : 1);
    if (dn->desc.count(key)) return MO_ED_OK;
    unsigned *p = nullptr;
    int rc;
    switch (R) {
    case 2: rc = f32 ? build_desc_r<float, 2>(ctx, dn, &p) : build_desc_r<double, 2>(ctx, dn, &p); break;
    case 3: rc = f32 ? build_desc_r<float, 3>(ctx, dn, &p) : build_desc_r<double, 3>(ctx, dn, &p); break;
    case 4: rc = f32 ? build_desc_r<float, 4>(ctx, dn, &p) : build_desc_r<double, 4>(ctx, dn, &p); break;
    default: return fail(ctx, MO_ED_ERR_ARG, "no item descriptors for this rows-per-item");
    }
    if (p) dn->desc[key] = p;
    return rc;
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
        case 4: return launch_batch<float, float, float, 8, 512, 1>(ctx, b);
        case 5: return launch_batch_async<float, float, float, 4, 512>(ctx, b);
        case 6: return launch_batch_async<float, float, float, 3, 512>(ctx, b);
        case 7: return launch_batch_async<float, float, float, 2, 512, 2>(ctx, b);
        case 8: return launch_batch_async<float, float, float, 2, 256, 2>(ctx, b);
        case 9: return launch_batch_split<float, float, float, 3, 512, 1, 128>(ctx, b);
        case 10: return launch_batch_split<float, float, float, 4, 512, 1, 128>(ctx, b);
        case 11: return launch_batch_split<float, float, float, 3, 512, 1, 64>(ctx, b);
        case 12: return launch_batch_rows<float, float, float, 3, 512, 1>(ctx, b);
        case 13: return launch_batch_rows<float, float, float, 4, 512, 1>(ctx, b);
        default: return launch_batch_rows<float, float, float, 4, 512, 1, 4>(ctx, b);   // 2,048-column tiles
        }
    } else if (kind == HV_F64) {
        switch (v) {
        case 0: return launch_batch<double, double, double, 2, 256, 2>(ctx, b);
        case 1: return launch_batch<double, double, double, 3, 256, 1>(ctx, b);
        case 2: return launch_batch<double, double, double, 2, 512, 1>(ctx, b);
        case 3: return launch_batch_async<double, double, double, 2, 512>(ctx, b);
        case 4: return launch_batch_async<double, double, double, 4, 512>(ctx, b);
        case 5: return launch_batch_split<double, double, double, 2, 512, 1, 128>(ctx, b);
        case 6: return launch_batch_split<double, double, double, 2, 512, 1, 64>(ctx, b);
        default: return launch_batch_rows<double, double, double, 2, 512, 1>(ctx, b);
        }
    } else {
        switch (v) {
        case 0: return launch_batch<float, double, double, 2, 256, 2>(ctx, b);
        case 1: return launch_batch<float, double, double, 3, 256, 1>(ctx, b);
        case 2: return launch_batch<float, double, double, 2, 512, 1>(ctx, b);
        case 3: return launch_batch_async<float, double, double, 2, 512>(ctx, b);
        case 4: return launch_batch_async<float, double, double, 4, 512>(ctx, b);
        case 5: return launch_batch_split<float, double, double, 2, 512, 1, 128>(ctx, b);
        case 6: return launch_batch_split<float, double, double, 2, 512, 1, 64>(ctx, b);
        default: return launch_batch_rows<float, double, double, 2, 512, 1>(ctx, b);
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

// tables variant v of `kind` reads for sector s: the item table of its R,
// and for the staged kernel the up-spin schedule and the item descriptors
static int prepare_variant(mo_ed_ctx *ctx, const Sector &s, int kind, int v)
{
    const HvVariant &h = variant(kind, v);
    const int *items;
    int n;
    if (int rc = species_items(ctx, s.dn, h.R, &items, &n)) return rc;
    if (!h.staged) return MO_ED_OK;
    if (h.staged == 2 || h.staged == 3) {
        // the split kernel stages whole down-spin blocks: the largest block of
        // the model (any electron count) must fit one CTA's shared memory
        const size_t wb = h.staged == 2 ? 128 : 64;
        if (!split_fits(ctx, wb, kind == HV_F32 ? sizeof(HopEnt<float>) : sizeof(HopEnt<double>)))
            return fail(ctx, MO_ED_ERR_ARG, "down-spin blocks too large for the split H*v");
        if (int rc = species_dblocks(ctx, s.dn, s.ld())) return rc;
    }
    if (int rc = species_sched(ctx, s.up, h.R)) return rc;
    return species_desc(ctx, s.dn, h.R, kind == HV_F32);
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
        if (int rc = prepare_variant(ctx, s, kind, v)) {
            if (rc == MO_ED_ERR_ARG) continue;   // variant not applicable to this model
            return rc;
        }
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
    } else if (s.Dpad() < kTuneMinElems) {
        v = 0;   // small sector: timing the variants would cost more than it saves
        ctx->hv_choice[key] = v;
        ctx->hv_times[key].assign(nvariants(kind), -1.0f);
    } else {
        if (int rc = tune(ctx, s, kind, &v)) return rc;
        ctx->hv_choice[key] = v;
    }
    if (int rc = prepare_variant(ctx, s, kind, v)) return rc;
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
            shape[4 * i] = h.R;
            shape[4 * i + 1] = h.NT;
            shape[4 * i + 2] = h.MINB;
            shape[4 * i + 3] = h.staged;
        }
        if (ms) ms[i] = i < (int)t.size() ? t[i] : -1.0f;
    }
    return MO_ED_OK;
}

int hv_prepare_rows(mo_ed_ctx *ctx, const Sector &s, int kind, int v)
{
    return prepare_variant(ctx, s, kind, v);
}

int hv_lookup(mo_ed_ctx *ctx, const Sector &s, int kind, int *v_out, int *R_out)
{
    auto it = ctx->hv_choice.find(shape_key(kind, s));
    if (it == ctx->hv_choice.end())
        return fail(ctx, MO_ED_ERR_STATE, "H*v tile shape of this sector not chosen yet");
    const HvVariant &h = variant(kind, it->second);
    const int R = h.R;
    bool ready = s.dn->items.count(R) != 0;
    if (h.staged)
        ready = ready && s.up->sched_rf.count(R) && s.dn->desc.count(R * 2 + (kind == HV_F32 ? 0 : 1));
    if (h.staged == 2 || h.staged == 3)
        ready = ready && s.dn->dblk_ptr != nullptr && s.dn->dblk_chunks.count(s.ld());
    if (!ready) return fail(ctx, MO_ED_ERR_STATE, "H*v item table of this sector not built yet");
    if (v_out) *v_out = it->second;
    if (R_out) *R_out = R;
    return MO_ED_OK;
}

int hv_set_variant(mo_ed_ctx *ctx, const Sector &s, int kind, int v)
{
    if (v < 0 || v >= nvariants(kind)) return fail(ctx, MO_ED_ERR_ARG, "H*v variant out of range");
    if (int rc = prepare_variant(ctx, s, kind, v)) return rc;
    ctx->hv_choice[shape_key(kind, s)] = v;
    return MO_ED_OK;
}

int hv_single(mo_ed_ctx *ctx, const Sector &s, int kind, const void *x, void *y)
{
    int v;
    if (int rc = hv_prepare(ctx, s, kind, &v, nullptr)) return rc;
    return launch_one(ctx, s, kind, v, x, y);
}

}  // namespace moed
