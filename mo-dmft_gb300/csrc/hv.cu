// hv.cu -- matrix-free Kanamori H*v on a (Nup, Ndn) sector.
//
// Replaces multiply_H (ed_hamiltonian.F90:88-191).  For output element
// (d, u) (down rank d, up rank u) the reference sums
//   diagonal       onsite + dens_dens                      (:112-141)
//   hybridisation  V c+_o c_k and V c+_k c_o, both spins     (:146-161)
//   spin-flip      -J c+_{i up} c_{i dn} c+_{j dn} c_{j up}  (:163-174)
//   pair hop       -J c+_{i up} c+_{i dn} c_{j up} c_{j dn}  (:176-187)
// gathering A at the state each operator maps row (d, u) to.  Here:
//   * diagonal = Dup[u] + Ddn[d] + Cross[imp(u)][imp(d)];
//   * up-spin hops move inside the up block of u (conserved subsystem
//     counts), i.e. inside one contiguous column range of a row;
//   * down-spin hops are row AXPYs from rows d' of the same down block;
//   * spin-flip / pair hop factor into an up-spin transfer T_{i<-j}(u) and a
//     down-spin transfer (T_{j<-i}(d) for spin-flip, T_{i<-j}(d) for pair
//     hopping) with coefficient +J t_up t_dn: reordering the four operators
//     of ed_operators.F90:183-213 / 236-266 gives a factor -1 that cancels
//     the -J.
//
// Work decomposition.  A tile is one row set of the down species (rows of a
// down block with equal local states in its leading subsystems, so the moves
// of the trailing subsystems stay inside the set) times one whole up block.
// One persistent kernel walks the tiles of a batch of jobs (vectors of
// possibly different sectors).  Per tile:
//   * one warp issues a cp.async.bulk copy per row segment (the block's
//     columns of one row) into a shared-memory stage, completing on an
//     mbarrier; the next tile's copies run while the current tile computes
//     (two stages);
//   * a thread owns 4 consecutive columns (a quad) of up to RG rows; a warp
//     covers 32 quads of one row group, or for narrow blocks several row
//     groups of fewer quads;
//   * up-spin moves read the stage through the block's gather schedule
//     (edge-coloured so the 32 lanes of a slot hit 32 banks), one schedule
//     entry serving all RG rows;
//   * down-spin moves inside the set read the stage (16-byte loads of the
//     quad), the others read the neighbour row from global memory (L2: the
//     tiles of one block pair run together), as do spin-flip / pair hopping;
//   * optionally the FP64 sum of x*y (the Lanczos alpha) is accumulated per
//     CTA and job.
// HBM traffic is one read of x and one write of y; the CTAs also zero the
// row tails past the last block (pads).
#include <algorithm>

#include "internal.h"

namespace moed {

constexpr int kMaxJobs = 24;
constexpr long long kTuneMinElems = 1 << 18;

template <typename TA>
struct HvBatch {
    int njobs, total;
    int *err;
    HvJobT<TA> job[kMaxJobs];
};

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier and bulk global->shared copies
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(unsigned long long *b, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned long long *b, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *b)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(b))
                 : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// 4-element loads and stores
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void lds4(const T *p, T (&v)[4])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        v[3] = a.w;
    } else {
        const double2 a = reinterpret_cast<const double2 *>(p)[0];
        const double2 b = reinterpret_cast<const double2 *>(p)[1];
        v[0] = a.x;
        v[1] = a.y;
        v[2] = b.x;
        v[3] = b.y;
    }
}

template <typename T>
__device__ __forceinline__ void ldcg4(const T *p, T (&v)[4])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = __ldcg(reinterpret_cast<const float4 *>(p));
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        v[3] = a.w;
    } else {
        const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
        const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
        v[0] = a.x;
        v[1] = a.y;
        v[2] = b.x;
        v[3] = b.y;
    }
}

template <typename T>
__device__ __forceinline__ void ldg4(const T *p, T (&v)[4])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        v[3] = a.w;
    } else {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
        const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
        v[0] = a.x;
        v[1] = a.y;
        v[2] = b.x;
        v[3] = b.y;
    }
}

template <typename T, typename TA>
__device__ __forceinline__ void stg4(T *p, const TA (&v)[4])
{
    if constexpr (sizeof(T) == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
    } else {
        reinterpret_cast<double2 *>(p)[0] = make_double2((double)v[0], (double)v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2((double)v[2], (double)v[3]);
    }
}

// Shared-memory row pitch of a tile with W4 columns: W4 rounded up to 16 (mod
// 32), so that two half-warps reading two consecutive rows at 16 distinct
// (mod 16) columns hit 32 different banks.  Tiles of 64..1024 columns (the
// fast path) all use the fixed pitch kPit, which turns the row offsets of a
// thread into immediates.
constexpr int kPit = 1040;
constexpr int kFastMinW4 = 64, kFastMaxW4 = 1024;
constexpr int kSeg = 4;           // consecutive tiles per CTA turn
constexpr int kNBuf = 2;
constexpr int kMaxCW = 32;        // consumer warps at most (dot-product slots)

__host__ __device__ inline int tile_pitch(int W4)
{
    return (W4 >= kFastMinW4 && W4 <= kFastMaxW4) ? kPit : W4 + ((48 - (W4 & 31)) & 31);
}

struct TileDesc {             // one per stage buffer, written by the producer warp
    int job, g, W4, col0, hdr0, pitch, on, flags;   // flags: 1 schedule staged, 2 partner columns staged
};

struct StageSizes {           // bytes per stage buffer of each region; consumer warps
    int stage, meta, up4, s16, ncw;
};

template <typename TA>
struct SmemLayout {
    size_t stage, meta, up4, s16, desc, cf, cross, dot, bar, total;
};

template <typename TA>
__host__ __device__ inline SmemLayout<TA> smem_layout(const StageSizes &Z, int nimp)
{
    SmemLayout<TA> L;
    size_t o = 0;
    L.stage = o;
    o += (size_t)kNBuf * Z.stage;
    L.meta = o;
    o += (size_t)kNBuf * Z.meta;
    L.up4 = o;
    o += (size_t)kNBuf * Z.up4;
    L.s16 = o;
    o += (size_t)kNBuf * Z.s16;
    L.desc = o;
    o += kNBuf * sizeof(TileDesc);
    L.cf = o;
    o += ((size_t)kMaxCoef * sizeof(TA) + 15) & ~(size_t)15;
    L.cross = o;
    o += ((size_t)nimp * nimp * sizeof(TA) + 15) & ~(size_t)15;
    L.dot = o;
    o += sizeof(double) * kMaxJobs * Z.ncw;
    L.bar = o;
    o += 2 * kNBuf * sizeof(unsigned long long);
    L.total = o;
    return L;
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *b, unsigned bytes)
{
    asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

// Wait for a phase; false when the wait ran out (about 2 s): the error word
// is set and the caller leaves its loop.
__device__ __forceinline__ bool bar_wait(unsigned long long *bar, unsigned parity, int *err)
{
    int spins = 0;
    unsigned long long t0 = 0;
    while (!mbar_try(bar, parity)) {
        ++spins;
        if (spins == 32) {
            t0 = global_ns();
        } else if (spins > 32 && (spins & 31) == 0 && global_ns() - t0 > 2000000000ull) {
            if (err) atomicExch(err, 1);
            return false;
        }
    }
    return true;
}

template <typename TA>
__device__ __forceinline__ int find_job(const HvBatch<TA> &B, int t)
{
    int j = 0;
    while (j + 1 < B.njobs && t >= B.job[j + 1].tile0) ++j;
    return j;
}

// Quads per warp row (log2) and row slots of a tile: the fast path covers 32
// quads (two 16-quad schedule chunks, one per half-warp) of the same rows, so
// the per-row loops are warp-uniform; other tiles use 16 quads x 2 rows, or
// spread narrower tiles over more rows.
__host__ __device__ inline int tile_lqw(int nq, bool fast)
{
    if (fast) return 5;
    if (nq >= 16) return 4;
    int l = 0;
    while ((1 << l) < nq) ++l;
    return l;
}

// One warp task: a chunk of quads times a batch of rows of the tile in
// stage S (pitch P; FAST: P == kPit and two half-warps per row pair).
template <bool FAST, typename TX, typename TA, typename TY, int RG>
__device__ __forceinline__ double hv_task_body(const HvJobT<TA> &jb, const TileDesc &D, const TX *__restrict__ S,
                                          const unsigned char *__restrict__ meta,
                                          const unsigned *__restrict__ up4s, const unsigned char *__restrict__ s16,
                                          const TA *__restrict__ s_cf, const TA *__restrict__ s_cross, int nimp,
                                          TA Jc, int task, int lane, bool want_dot)
{
    const int W4 = D.W4, nq = W4 >> 2, g = D.g, ld = jb.ld;
    const int P = FAST ? kPit : D.pitch;
    const int lqw = tile_lqw(nq, FAST);
    const int qw = 1 << lqw, rs = 32 >> lqw;
    const int nch = (nq + qw - 1) >> lqw;
    const int ch = task % nch, rb = task / nch;
    const int ql = lane & (qw - 1), slot = lane >> lqw;
    // schedule chunk (16 quads) and lane within it
    const int sch = FAST ? 2 * ch + (lane >> 4) : ch, sql = FAST ? (lane & 15) : ql;
    const int q = (ch << lqw) + ql;
    const bool act = q < nq;
    const int c = act ? 4 * q : 0;
    const int rbase = rb * rs * RG + slot;
    const int4 *info = reinterpret_cast<const int4 *>(meta + 16);
    const double *dgv = reinterpret_cast<const double *>(meta + 16 + 16 * (size_t)g);
    const int4 mh = *reinterpret_cast<const int4 *>(meta);
    const unsigned *mv = reinterpret_cast<const unsigned *>(meta + mh.y);
    const unsigned *q4 = reinterpret_cast<const unsigned *>(meta + mh.z);
    const TX *__restrict__ x = (const TX *)jb.x;
    TY *__restrict__ y = (TY *)jb.y;

    // column tables of the quad (consumed after the up-spin moves, so their
    // latency overlaps them)
    TA dup[4];
    ldg4<TA>(jb.up_diag + D.col0 + c, dup);
    const unsigned imq = __ldg(reinterpret_cast<const unsigned *>(jb.up_imp + D.col0 + c));
    // rows r_i = rbase + rs*i; row pointers at offsets roff[i] from Sb
    // (FAST: compile-time offsets; invalid rows read inside the stage and
    // are not stored)
    const TX *Sb = S + (size_t)rbase * P;
    int roff[RG];
    unsigned vmask = 0;
    TA acc[RG][4];
#pragma unroll
    for (int i = 0; i < RG; ++i) {
        const int r = rbase + rs * i;
        const bool ok = act && r < g;
        vmask |= ok ? 1u << i : 0u;
        roff[i] = FAST ? i * kPit : ((ok ? r : 0) - rbase) * P;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) acc[i][kk] = TA(0);
    }
    // first open-move loads of row 0, issued before the up-spin moves so that
    // their L2 latency overlaps them; row i+1's are issued once row i's are
    // consumed
    constexpr int OPB = sizeof(TA) == 8 ? 2 : 4;
    const TX *xc = x + D.col0 + c;
    TX ov[OPB][4];
    auto issue_open = [&](int i, TX (&o)[OPB][4]) {
        const int r = rbase + rs * i;
        const bool ok = (vmask >> i) & 1u;
        const int4 inf = info[ok ? r : 0];
        const int nin = (inf.x >> 8) & 0xff, nopen = ok ? (inf.x >> 16) & 0xff : 0;
        const unsigned *m1 = mv + inf.y + nin;
#pragma unroll
        for (int t = 0; t < OPB; ++t) {
            if (t < nopen) {
                ldcg4<TX>(xc + (size_t)(m1[t] & 0xffffu) * ld, o[t]);
            } else {
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) o[t][kk] = TX(0);
            }
        }
    };
    issue_open(0, ov);
    // up-spin moves: one schedule entry per slot serves every row
    if (FAST && (D.flags & 1)) {
        // 16-bit schedule staged in shared memory
        const int nch16 = (nq + 15) >> 4;
        const unsigned *sh = reinterpret_cast<const unsigned *>(s16);
        const unsigned short *se = reinterpret_cast<const unsigned short *>(s16 + 16 * (size_t)nch16);
        const bool live = sch < nch16;
        // one column of the quad at a time on acc[.][0]; the columns rotate
        // after each, so the loop body exists once
#pragma unroll 1
        for (int kk = 0; kk < 4; ++kk) {
            const unsigned hw = live ? sh[sch * 4 + kk] : 0u;
            const int ns = hw & 255;
            const unsigned short *E = se + (hw >> 8) + sql;
            for (int sl = 0; sl < ns; sl += 4) {
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    if (sl + t < ns) {
                        const unsigned e = E[16 * (sl + t)];
                        const TA cf = s_cf[e >> 10];
                        const TX *col = Sb + (e & 1023u);
#pragma unroll
                        for (int i = 0; i < RG; ++i) acc[i][0] += cf * (TA)col[roff[i]];
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < RG; ++i) {
                const TA a0 = acc[i][0];
                acc[i][0] = acc[i][1];
                acc[i][1] = acc[i][2];
                acc[i][2] = acc[i][3];
                acc[i][3] = a0;
            }
        }
    } else {
        const int nch16 = (nq + 15) >> 4;
        const bool live = sch < nch16;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int2 h = live ? __ldg(jb.sched_hdr + D.hdr0 + sch * 4 + kk) : make_int2(0, 0);
            const unsigned *E = jb.sched_ent + h.x + sql;
            for (int sl = 0; sl < h.y; sl += 8) {
                unsigned e[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) e[t] = sl + t < h.y ? __ldg(E + 16 * (sl + t)) : 0u;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    if (sl + t < h.y) {
                        const TA cf = s_cf[e[t] >> 16];
                        const TX *col = Sb + (e[t] & 0xffffu);
#pragma unroll
                        for (int i = 0; i < RG; ++i) acc[i][kk] += cf * (TA)col[roff[i]];
                    }
                }
            }
        }
    }
    // diagonal, down-spin moves, 4-operator terms, store
    int iu[4];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) iu[kk] = (imq >> (8 * kk)) & 0xff;
    double dsum = 0.0;
    // rows in a runtime loop on acc[0], rotating acc after each row (register
    // moves), so the per-row code exists once in the kernel
#pragma unroll 1
    for (int i = 0; i < RG; ++i) {
        const bool ok = (vmask >> i) & 1u;
        const int r = rbase + rs * i;
        const int4 inf = info[ok ? r : 0];
        const int nin = (inf.x >> 8) & 0xff, nopen = (inf.x >> 16) & 0xff, n4 = (inf.x >> 24) & 0xff;
        const unsigned *m0 = mv + inf.y;
        const unsigned *m1 = m0 + nin;
        TA a[4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) a[kk] = acc[0][kk];
        // the prefetched open moves of this row
        if (ok) {
#pragma unroll
            for (int t = 0; t < OPB; ++t)
                if (t < nopen) {
                    const TA cf = s_cf[m1[t] >> 16];
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) a[kk] += cf * (TA)ov[t][kk];
                }
        }
        if (i + 1 < RG) issue_open(i + 1, ov);
        if (ok) {
            const TX *xrow = S + (size_t)r * P + c;
            {
                const TA ddn = (TA)dgv[r];
                const int id = inf.x & 0xff;
                TX xs[4];
                lds4<TX>(xrow, xs);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) a[kk] += (dup[kk] + ddn + s_cross[iu[kk] * nimp + id]) * (TA)xs[kk];
            }
            for (int m = 0; m < nin; ++m) {
                const unsigned e = m0[m];
                const TA cf = s_cf[e >> 16];
                TX v[4];
                lds4<TX>(S + (size_t)(e & 0xffffu) * P + c, v);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) a[kk] += cf * (TA)v[kk];
            }
            for (int m = OPB; m < nopen; ++m) {
                TX v[4];
                ldcg4<TX>(xc + (size_t)(m1[m] & 0xffffu) * ld, v);
                const TA cf = s_cf[m1[m] >> 16];
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) a[kk] += cf * (TA)v[kk];
            }
            for (int mm = 0; mm < n4; ++mm) {
                const unsigned e = q4[inf.z + mm];
                const int p = (e >> 16) & 31;
                const uint4 u4 = (D.flags & 2)
                                     ? *reinterpret_cast<const uint4 *>(up4s + (size_t)p * W4 + c)
                                     : __ldg(reinterpret_cast<const uint4 *>(jb.up4 + (size_t)p * ld + D.col0 + c));
                const unsigned ue[4] = {u4.x, u4.y, u4.z, u4.w};
                const TX *xr = x + (size_t)(e & 0xffffu) * ld;
                TX v[4];
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) v[kk] = (ue[kk] >> 31) ? __ldg(xr + (ue[kk] & 0xffffu)) : TX(0);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const bool neg = ((ue[kk] >> 30) ^ (e >> 22)) & 1u;
                    a[kk] += (neg ? -Jc : Jc) * (TA)v[kk];
                }
            }
            stg4<TY, TA>(y + (size_t)inf.w * ld + D.col0 + c, a);
            if (want_dot) {
                TX xs[4];
                lds4<TX>(xrow, xs);
                TA part = TA(0);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) part += (TA)xs[kk] * a[kk];
                dsum += (double)part;
            }
        }
        // rotate: the next row's accumulators move to acc[0]
#pragma unroll
        for (int j2 = 0; j2 + 1 < RG; ++j2)
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) acc[j2][kk] = acc[j2 + 1][kk];
    }
    return dsum;
}

// The fast path inlined into the consumer loop; the other tiles (narrow or
// very wide blocks) through an out-of-line call, to keep the hot loop small.
template <bool FAST, typename TX, typename TA, typename TY, int RG>
__device__ __forceinline__ double hv_task(const HvJobT<TA> &jb, const TileDesc &D, const TX *__restrict__ S,
                                          const unsigned char *__restrict__ meta,
                                          const unsigned *__restrict__ up4s, const unsigned char *__restrict__ s16,
                                          const TA *__restrict__ s_cf, const TA *__restrict__ s_cross, int nimp,
                                          TA Jc, int task, int lane, bool want_dot)
{
    return hv_task_body<FAST, TX, TA, TY, RG>(jb, D, S, meta, up4s, s16, s_cf, s_cross, nimp, Jc, task, lane,
                                              want_dot);
}

template <typename TX, typename TA, typename TY, int RG>
__device__ __noinline__ double hv_task_generic(const HvJobT<TA> &jb, const TileDesc &D, const TX *__restrict__ S,
                                               const unsigned char *__restrict__ meta,
                                               const unsigned *__restrict__ up4s,
                                               const unsigned char *__restrict__ s16, const TA *__restrict__ s_cf,
                                               const TA *__restrict__ s_cross, int nimp, TA Jc, int task, int lane,
                                               bool want_dot)
{
    return hv_task_body<false, TX, TA, TY, RG>(jb, D, S, meta, up4s, s16, s_cf, s_cross, nimp, Jc, task, lane,
                                               want_dot);
}

__host__ __device__ inline int tile_ntasks(int g, int W4, int pitch, int RG)
{
    const int nq = W4 >> 2;
    const int lqw = tile_lqw(nq, pitch == kPit);
    const int qw = 1 << lqw, rs = 32 >> lqw;
    const int nch = (nq + qw - 1) >> lqw;
    const int rpt = rs * RG;
    return nch * ((g + rpt - 1) / rpt);
}

// Persistent H*v over a batch of jobs.  Warp 0 produces (bulk copies of the
// next tiles' row segments and metadata blobs), warps 1..NCW consume; each
// consumer warp walks one stream of tasks across tile boundaries, so a tile
// with fewer tasks than warps leaves no warp idle.  Tiles run in turns of
// kSeg consecutive tiles per CTA, round-robin over the grid, so the tiles in
// flight over the GPU stay close in the (L2-ordered) tile list.
template <typename TX, typename TA, typename TY, int RG, int NCW, int MINB>
__global__ void __launch_bounds__(32 * (NCW + 1), MINB)
k_hvt(const __grid_constant__ HvBatch<TA> B, const ModelDev *__restrict__ mdl, const StageSizes Z)
{
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NT = 32 * (NCW + 1);
    static_assert(NCW <= kMaxCW, "too many consumer warps");
    const int nimp = mdl->nimp, npair = mdl->npair;
    const SmemLayout<TA> L = smem_layout<TA>(Z, nimp);
    TA *s_cf = reinterpret_cast<TA *>(smem + L.cf);
    TA *s_cross = reinterpret_cast<TA *>(smem + L.cross);
    double *s_dot = reinterpret_cast<double *>(smem + L.dot);
    TileDesc *s_desc = reinterpret_cast<TileDesc *>(smem + L.desc);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(smem + L.bar);
    unsigned long long *empty = full + kNBuf;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int i = tid; i < kMaxCoef; i += NT) {
        TA v = TA(0);
        if (i > 0 && (i - 1) / 2 < mdl->ncpl) {
            const double cv = mdl->cval[(i - 1) >> 1];
            v = (TA)(((i - 1) & 1) ? -cv : cv);
        }
        s_cf[i] = v;
    }
    for (int i = tid; i < nimp * nimp; i += NT) s_cross[i] = (TA)mdl->cross[i];
    // x.y partials: one slot per (job, consumer warp), each written by its
    // warp only and summed in a fixed order, so the result is reproducible
    for (int i = tid; i < kMaxJobs * NCW; i += NT) s_dot[i] = 0.0;
    if (tid == 0) {
        for (int b = 0; b < kNBuf; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], NCW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const TA Jc = (TA)mdl->J;
    const bool four = mdl->J != 0.0 && npair > 0;
    // this CTA's tiles: turns of kSeg consecutive tiles, round-robin over the grid
    auto next_tile = [&](int t) {
        const int t1 = min(B.total, (t / kSeg + 1) * kSeg);
        return t + 1 < t1 ? t + 1 : (t / kSeg + (int)gridDim.x) * kSeg;
    };
    const int tfirst = blockIdx.x * kSeg;

    if (warp == 0) {
        // ---- producer ----
        const void *c_sp[kNBuf];
        int c_ub[kNBuf];
        for (int b = 0; b < kNBuf; ++b) {
            c_sp[b] = nullptr;
            c_ub[b] = -1;
        }
        auto load_tile = [&](int t, int *j, HvTile *T, int *rr) {
            *j = find_job(B, t);
            const HvJobT<TA> &jb = B.job[*j];
            const int4 *tp = reinterpret_cast<const int4 *>(jb.tiles + (t - jb.tile0));
            const int4 a = __ldg(tp), b2 = __ldg(tp + 1), c2 = __ldg(tp + 2);
            *T = HvTile{a.x, a.y, a.z, a.w, b2.x, b2.y, b2.z, b2.w, c2.x, c2.y, c2.z, c2.w};
            *rr = lane < T->rows ? __ldg(jb.rs_row + T->rs0 + lane) : 0;
        };
        int k = 0, t = tfirst, j = 0, rr = 0;
        HvTile T;
        if (t < B.total) load_tile(t, &j, &T, &rr);
        while (t < B.total) {
            // prefetch the next tile's descriptor and row ranks
            const int tn = next_tile(t);
            int jn = 0, rrn = 0;
            HvTile Tn;
            if (tn < B.total) load_tile(tn, &jn, &Tn, &rrn);
            const int buf = k & 1;
            if (k >= kNBuf && !bar_wait(&empty[buf], (unsigned)((k >> 1) - 1) & 1u, B.err)) break;
            const HvJobT<TA> &jb = B.job[j];
            const bool on = !jb.active || *jb.active != 0;
            const int pitch = tile_pitch(T.W4);
            const unsigned rowb = (unsigned)T.W4 * (unsigned)sizeof(TX);
            const bool s16_ok = pitch == kPit && T.s16_bytes > 0 && T.s16_bytes <= Z.s16;
            const bool up4_ok = four && npair * T.W4 * 4 <= Z.up4;
            const bool fresh = c_sp[buf] != (const void *)jb.up4 || c_ub[buf] != T.ub;
            const bool copy_up = on && (s16_ok || up4_ok) && fresh;
            unsigned bytes = 0;
            if (on) {
                bytes = (unsigned)T.blob_bytes + (unsigned)T.rows * rowb;
                if (copy_up) bytes += (s16_ok ? (unsigned)T.s16_bytes : 0u) + (up4_ok ? (unsigned)(npair * T.W4 * 4) : 0u);
            }
            if (lane == 0) {
                s_desc[buf] = TileDesc{j, T.rows, T.W4, T.col0, T.hdr0, pitch, on ? 1 : 0,
                                       (s16_ok ? 1 : 0) | (up4_ok ? 2 : 0)};
                mbar_expect_tx(&full[buf], bytes);
            }
            __syncwarp();
            if (on) {
                if (lane == 0)
                    bulk_g2s(smem + L.meta + (size_t)buf * Z.meta, jb.blob + (size_t)T.blob16 * 16,
                             (unsigned)T.blob_bytes, &full[buf]);
                if (copy_up) {
                    if (s16_ok && lane == 31)
                        bulk_g2s(smem + L.s16 + (size_t)buf * Z.s16, jb.sched16 + (size_t)T.s16_off * 16,
                                 (unsigned)T.s16_bytes, &full[buf]);
                    if (up4_ok)
                        for (int p = lane; p < npair; p += 32)
                            bulk_g2s(smem + L.up4 + (size_t)buf * Z.up4 + (size_t)p * T.W4 * 4,
                                     jb.up4 + (size_t)p * jb.ld + T.col0, (unsigned)T.W4 * 4u, &full[buf]);
                    c_sp[buf] = (const void *)jb.up4;
                    c_ub[buf] = T.ub;
                }
                unsigned char *st = smem + L.stage + (size_t)buf * Z.stage;
                const TX *x = (const TX *)jb.x + T.col0;
                for (int r = lane; r < T.rows; r += 32) {
                    const int d = r < 32 ? rr : __ldg(jb.rs_row + T.rs0 + r);
                    bulk_g2s(st + (size_t)r * pitch * sizeof(TX), x + (size_t)d * jb.ld, rowb, &full[buf]);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&full[buf]);
            t = tn;
            j = jn;
            T = Tn;
            rr = rrn;
            ++k;
        }
    } else {
        // ---- consumers ----
        const int cw = warp - 1;
        int k = 0, tk = cw, cur = -1;
        double dsum = 0.0;
        for (int t = tfirst; t < B.total; t = next_tile(t), ++k) {
            const int buf = k & 1;
            if (!bar_wait(&full[buf], (unsigned)(k >> 1) & 1u, B.err)) break;
            const TileDesc D = s_desc[buf];
            const int nt = D.on ? tile_ntasks(D.g, D.W4, D.pitch, RG) : 0;
            if (nt > tk && D.job != cur) {
                if (cur >= 0 && B.job[cur].dot_partial) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
                    if (lane == 0) s_dot[cur * NCW + cw] += dsum;
                }
                dsum = 0.0;
                cur = D.job;
            }
            const HvJobT<TA> &jb = B.job[D.job];
            const TX *S = reinterpret_cast<const TX *>(smem + L.stage + (size_t)buf * Z.stage);
            const unsigned char *meta = smem + L.meta + (size_t)buf * Z.meta;
            const unsigned *up4s = reinterpret_cast<const unsigned *>(smem + L.up4 + (size_t)buf * Z.up4);
            const unsigned char *s16 = smem + L.s16 + (size_t)buf * Z.s16;
            const bool want_dot = jb.dot_partial != nullptr;
            for (; tk < nt; tk += NCW) {
                if (D.pitch == kPit)
                    dsum += hv_task<true, TX, TA, TY, RG>(jb, D, S, meta, up4s, s16, s_cf, s_cross, nimp, Jc, tk,
                                                          lane, want_dot);
                else
                    dsum += hv_task_generic<TX, TA, TY, RG>(jb, D, S, meta, up4s, s16, s_cf, s_cross, nimp, Jc, tk,
                                                            lane, want_dot);
            }
            tk -= nt;
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[buf]);
        }
        if (cur >= 0 && B.job[cur].dot_partial) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
            if (lane == 0) s_dot[cur * NCW + cw] += dsum;
        }
        // the row tails past the last block are pads: zero them
        for (int j = 0; j < B.njobs; ++j) {
            const HvJobT<TA> &jb = B.job[j];
            if (jb.active && *jb.active == 0) continue;
            const int tail = jb.ld - jb.ncol;
            if (tail <= 0) continue;
            TY *y = (TY *)jb.y + jb.ncol;
            const long long n = (long long)jb.nrow * tail;
            for (long long i = ((long long)blockIdx.x * NCW + cw) * 32 + lane; i < n;
                 i += (long long)gridDim.x * NCW * 32) {
                const long long d = i / tail;
                y[d * jb.ld + (i - d * tail)] = TY(0);
            }
        }
    }
    __syncthreads();
    for (int j = tid; j < B.njobs; j += NT)
        if (B.job[j].dot_partial) {
            double v = 0.0;
            for (int w = 0; w < NCW; ++w) v += s_dot[j * NCW + w];
            B.job[j].dot_partial[blockIdx.x] = v;
        }
}

// ---------------------------------------------------------------------------
// host side: variants, tile lists, launch, autotuner
// ---------------------------------------------------------------------------
struct HvVariant {
    int RG;      // rows per thread and task
    int NCW;     // consumer warps (plus one producer warp)
    int MINB;    // CTAs per SM
    int TR;      // fast-path stage rows (a multiple of RG)
    int meta_kb; // metadata blob budget per stage
    int up4_kb;  // staged spin-flip / pair-hop partner columns per stage (0: read from L2)
    int s16_kb;  // staged 16-bit gather schedule per stage (0: read from L2)
};

// FP32 (TX = float): 10 stage rows of pitch 1040 hold the 10-row fibres of the
// largest block pairs of the 3-orbital x 4-bath ground sector.
static const HvVariant kVarF32[] = {{5, 15, 1, 10, 12, 24, 28}, {2, 31, 1, 12, 10, 20, 24},
                                    {3, 15, 1, 12, 10, 20, 24}, {3, 23, 1, 12, 10, 20, 24}};
// FP64 and FP32 -> FP64 (TA = double)
static const HvVariant kVarF64[] = {{3, 15, 1, 6, 8, 20, 28}, {5, 15, 1, 10, 8, 0, 0}, {3, 7, 2, 6, 4, 0, 0}};
static const int kNVarF32 = sizeof(kVarF32) / sizeof(kVarF32[0]);
static const int kNVarF64 = sizeof(kVarF64) / sizeof(kVarF64[0]);

static const HvVariant &variant(int kind, int v) { return kind == HV_F32 ? kVarF32[v] : kVarF64[v]; }
static int nvariants(int kind) { return kind == HV_F32 ? kNVarF32 : kNVarF64; }
static size_t x_size(int kind) { return kind == HV_F64 ? sizeof(double) : sizeof(float); }
static StageSizes sizes_of(int kind, int v)
{
    const HvVariant &h = variant(kind, v);
    return StageSizes{h.TR * kPit * (int)x_size(kind), h.meta_kb * 1024, h.up4_kb * 1024, h.s16_kb * 1024, h.NCW};
}
static long long shape_key(int kind, const Sector &s) { return ((long long)kind << 32) | (s.ne_up << 16) | s.ne_down; }
static long long tile_key(const Sector &s, int kind, int v)
{
    const HvVariant &h = variant(kind, v);
    const long long sel = (((long long)x_size(kind) * 64 + h.TR) * 256 + h.meta_kb) * 64 + h.RG;
    return (sel << 32) | ((long long)s.ne_up << 16) | s.ne_down;
}

// Tiles of a sector: for every (down block, up block) pair the row sets of
// the first level whose sets fit the stage (fast path: at most TR rows;
// others: rows x pitch elements) and whose metadata blob fits its budget.
// Tiles are ordered by the total electron count per subsystem (spin-flip
// keeps it, so its partner tiles run together), then by block pair, so the
// neighbour rows that moves between row sets read are recent in L2.
int hv_tile_list(mo_ed_ctx *ctx, const Sector &s, int kind, int v, const HvTile **tiles, int *ntiles)
{
    const long long key = tile_key(s, kind, v);
    auto it = ctx->hv_tiles.find(key);
    if (it == ctx->hv_tiles.end()) {
        const Species &dn = *s.dn, &up = *s.up;
        const int nsub = dn.nsub;
        const HvVariant &hv = variant(kind, v);
        const StageSizes Z = sizes_of(kind, v);
        const long long sbytes = Z.stage, mbytes = Z.meta;
        const long long es = (long long)x_size(kind);
        struct Ent {
            long long orbit;
            int bd, bu;
            HvTile tile;
        };
        std::vector<Ent> ents;
        for (int bd = 0; bd < (int)dn.h_dblk.size(); ++bd) {
            const DownBlock &db = dn.h_dblk[bd];
            for (int bu = 0; bu < (int)up.h_ublk.size(); ++bu) {
                const UpBlock &ub = up.h_ublk[bu];
                const int pitch = tile_pitch(ub.W4);
                const bool fast = pitch == kPit;
                int lev = -1;
                for (int j = 0; j <= nsub; ++j) {
                    const bool rows_ok = fast ? db.rs_rows[j] <= hv.TR : db.rs_rows[j] * (long long)pitch * es <= sbytes;
                    if (rows_ok && db.blob_max[j] <= mbytes) {
                        lev = j;
                        break;
                    }
                }
                if (lev < 0) return fail(ctx, MO_ED_ERR_ARG, "an up-spin block is wider than the H*v stage");
                long long orbit = 0;
                for (int k = 0; k < nsub; ++k) orbit = orbit * 64 + db.cnt[k] + up.h_ublk_cnt[(size_t)bu * kMaxSub + k];
                for (int q = 0; q < db.nset[lev]; ++q) {
                    const int set = db.rs0[lev] + q;
                    const int2 r = dn.h_rs[set], b = dn.h_rs_blob[set];
                    ents.push_back({orbit, bd, bu,
                                    HvTile{r.x, r.y, b.x, b.y, ub.col0, ub.W4, ub.hdr0, ub.s16_off, ub.s16_bytes, bu, 0, 0}});
                }
            }
        }
        std::stable_sort(ents.begin(), ents.end(), [](const Ent &a, const Ent &b) {
            if (a.orbit != b.orbit) return a.orbit < b.orbit;
            if (a.bd != b.bd) return a.bd < b.bd;
            return a.bu < b.bu;
        });
        std::vector<HvTile> h(ents.size());
        for (size_t i = 0; i < ents.size(); ++i) h[i] = ents[i].tile;
        DevBuf d;
        if (int rc = dev_alloc(ctx, d, sizeof(HvTile) * std::max<size_t>(1, h.size()))) return rc;
        MOED_CUDA(ctx, cudaMemcpyAsync(d.p, h.data(), sizeof(HvTile) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        it = ctx->hv_tiles.emplace(key, std::make_pair(std::move(d), (int)h.size())).first;
    }
    *tiles = (const HvTile *)it->second.first.p;
    *ntiles = it->second.second;
    return MO_ED_OK;
}

static int ensure_err(mo_ed_ctx *ctx)
{
    if (ctx->d_err.p) return MO_ED_OK;
    if (int rc = dev_alloc(ctx, ctx->d_err, sizeof(int))) return rc;
    MOED_CUDA(ctx, cudaMemsetAsync(ctx->d_err.p, 0, sizeof(int), ctx->stream));
    return MO_ED_OK;
}

template <typename TA>
void hv_fill_job(const mo_ed_ctx *ctx, const Sector &s, int kind, int v, const void *x, void *y, HvJobT<TA> &j)
{
    memset(&j, 0, sizeof(j));
    j.x = x;
    j.y = y;
    j.ld = s.ld();
    j.ncol = s.up->ncol;
    j.nrow = s.dn->n;
    auto it = ctx->hv_tiles.find(tile_key(s, kind, v));
    if (it != ctx->hv_tiles.end()) {
        j.tiles = (const HvTile *)it->second.first.p;
        j.ntiles = it->second.second;
    }
    const Species &up = *s.up, &dn = *s.dn;
    j.ublk = up.ublk;
    j.sched_hdr = up.sched_hdr;
    j.sched_ent = up.sched_ent;
    j.sched16 = up.sched16;
    j.up_imp = up.up_imp;
    j.up4 = up.up4;
    j.rs = dn.rs;
    j.rs_row = dn.rs_row;
    j.rs_blob = dn.rs_blob;
    j.blob = dn.blob;
    if constexpr (sizeof(TA) == 4)
        j.up_diag = up.up_diag_f;
    else
        j.up_diag = up.up_diag_d;
}
template void hv_fill_job<float>(const mo_ed_ctx *, const Sector &, int, int, const void *, void *, HvJobT<float> &);
template void hv_fill_job<double>(const mo_ed_ctx *, const Sector &, int, int, const void *, void *, HvJobT<double> &);

template <typename TX, typename TA, typename TY, int RG, int NCW, int MINB>
static int launch_batch(mo_ed_ctx *ctx, const StageSizes &Z, const HvBatch<TA> &b)
{
    const SmemLayout<TA> L = smem_layout<TA>(Z, ctx->mdl.nimp);
    auto kern = k_hvt<TX, TA, TY, RG, NCW, MINB>;
    int optin = 0;
    MOED_CUDA(ctx, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    if ((size_t)optin < L.total) return fail(ctx, MO_ED_ERR_ARG, "H*v variant needs more shared memory than a CTA has");
    static size_t attr_set = 0;   // per instantiation
    if (attr_set < L.total) {
        MOED_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
        attr_set = L.total;
    }
    const int grid = ctx->num_sms * MINB;
    kern<<<grid, 32 * (NCW + 1), L.total, ctx->stream>>>(b, ctx->d_mdl, Z);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

template <typename TA>
static int launch_variant(mo_ed_ctx *ctx, int kind, int v, const HvBatch<TA> &b)
{
    const StageSizes Z = sizes_of(kind, v);
    if constexpr (sizeof(TA) == 4) {
        (void)kind;
        switch (v) {
        case 0: return launch_batch<float, float, float, 5, 15, 1>(ctx, Z, b);
        case 1: return launch_batch<float, float, float, 2, 31, 1>(ctx, Z, b);
        case 2: return launch_batch<float, float, float, 3, 15, 1>(ctx, Z, b);
        default: return launch_batch<float, float, float, 3, 23, 1>(ctx, Z, b);
        }
    } else if (kind == HV_F64) {
        switch (v) {
        case 0: return launch_batch<double, double, double, 3, 15, 1>(ctx, Z, b);
        case 1: return launch_batch<double, double, double, 5, 15, 1>(ctx, Z, b);
        default: return launch_batch<double, double, double, 3, 7, 2>(ctx, Z, b);
        }
    } else {
        switch (v) {
        case 0: return launch_batch<float, double, double, 3, 15, 1>(ctx, Z, b);
        case 1: return launch_batch<float, double, double, 5, 15, 1>(ctx, Z, b);
        default: return launch_batch<float, double, double, 3, 7, 2>(ctx, Z, b);
        }
    }
}

static int nparts_of(const mo_ed_ctx *ctx, int kind, int v) { return ctx->num_sms * variant(kind, v).MINB; }

template <typename TA>
static int hv_run_jobs(mo_ed_ctx *ctx, int kind, int v, const HvJobT<TA> *jobs, int njobs)
{
    if (int rc = ensure_err(ctx)) return rc;
    HvBatch<TA> b;
    memset(&b, 0, sizeof(b));
    b.err = (int *)ctx->d_err.p;
    for (int i = 0; i < njobs; ++i) {
        if (!jobs[i].tiles) return fail(ctx, MO_ED_ERR_STATE, "H*v tile list of a job not built");
        if (b.njobs == kMaxJobs) {
            if (int rc = launch_variant<TA>(ctx, kind, v, b)) return rc;
            b.njobs = 0;
            b.total = 0;
        }
        b.job[b.njobs] = jobs[i];
        b.job[b.njobs].tile0 = b.total;
        b.total += jobs[i].ntiles;
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
    if (kind == HV_F32) {
        HvJobT<float> j;
        hv_fill_job<float>(ctx, s, kind, v, x, y, j);
        return hv_launch_f32(ctx, v, &j, 1);
    }
    HvJobT<double> j;
    hv_fill_job<double>(ctx, s, kind, v, x, y, j);
    return hv_launch_f64(ctx, kind, v, &j, 1);
}

static int prepare_variant(mo_ed_ctx *ctx, const Sector &s, int kind, int v)
{
    const HvTile *t;
    int n;
    return hv_tile_list(ctx, s, kind, v, &t, &n);
}

// Time every variant on sector s and keep the fastest.
static int tune(mo_ed_ctx *ctx, const Sector &s, int kind, int *best)
{
    const size_t ex = x_size(kind);
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
            if (rc == MO_ED_ERR_ARG) continue;   // a block does not fit this variant's stage
            return rc;
        }
        if (launch_one(ctx, s, kind, v, dx.p, dy.p) != MO_ED_OK) {
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
    int herr = 0;
    MOED_CUDA(ctx, cudaMemcpy(&herr, ctx->d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return fail(ctx, MO_ED_ERR_CUDA, "H*v stage wait timed out");
    ctx->err.clear();
    return MO_ED_OK;
}

int hv_prepare(mo_ed_ctx *ctx, const Sector &s, int kind, int *v_out, int *nparts)
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
    if (int rc = ensure_err(ctx)) return rc;
    if (int rc = prepare_variant(ctx, s, kind, v)) return rc;
    if (v_out) *v_out = v;
    if (nparts) *nparts = nparts_of(ctx, kind, v);
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
            shape[4 * i] = h.RG;
            shape[4 * i + 1] = 32 * (h.NCW + 1);
            shape[4 * i + 2] = h.MINB;
            shape[4 * i + 3] = h.TR;
        }
        if (ms) ms[i] = i < (int)t.size() ? t[i] : -1.0f;
    }
    return MO_ED_OK;
}

int hv_prepare_rows(mo_ed_ctx *ctx, const Sector &s, int kind, int v) { return prepare_variant(ctx, s, kind, v); }

int hv_lookup(mo_ed_ctx *ctx, const Sector &s, int kind, int *v_out, int *nparts)
{
    auto it = ctx->hv_choice.find(shape_key(kind, s));
    if (it == ctx->hv_choice.end())
        return fail(ctx, MO_ED_ERR_STATE, "H*v tile shape of this sector not chosen yet");
    if (!ctx->hv_tiles.count(tile_key(s, kind, it->second)) || !ctx->d_err.p)
        return fail(ctx, MO_ED_ERR_STATE, "H*v tile list of this sector not built yet");
    if (v_out) *v_out = it->second;
    if (nparts) *nparts = nparts_of(ctx, kind, it->second);
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
