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

template <typename TA>
struct SmemLayout {
    size_t cf, cross, dot, bar, total;
};

template <typename TA>
__host__ __device__ inline SmemLayout<TA> smem_layout(int stage_bytes, int nimp)
{
    SmemLayout<TA> L;
    size_t o = 2 * (size_t)stage_bytes;
    L.cf = o;
    o += ((size_t)kMaxCoef * sizeof(TA) + 15) & ~(size_t)15;
    L.cross = o;
    o += ((size_t)nimp * nimp * sizeof(TA) + 15) & ~(size_t)15;
    L.dot = o;
    o += sizeof(double) * kMaxJobs;
    L.bar = o;
    o += 2 * sizeof(unsigned long long);
    L.total = o;
    return L;
}

// Wait for a stage; false when the wait ran out (about 2 s): the error word
// is set and the caller returns.
__device__ __forceinline__ bool stage_wait(unsigned long long *bar, unsigned parity, int *err)
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

// Issue the row copies of tile t into stage buffer `dst` (called by one warp).
template <typename TX, typename TA>
__device__ __forceinline__ void issue_tile(const HvBatch<TA> &B, int t, unsigned char *dst, unsigned long long *bar,
                                           int lane)
{
    const HvJobT<TA> &jb = B.job[find_job(B, t)];
    const HvTile tl = jb.tiles[t - jb.tile0];
    const int2 rsr = __ldg(jb.rs + tl.rs);
    const UpBlock ub = jb.ublk[tl.ub];
    const bool on = !jb.active || *jb.active != 0;
    const unsigned rowb = (unsigned)ub.W4 * (unsigned)sizeof(TX);
    if (lane == 0) mbar_arrive_tx(bar, on ? (unsigned)rsr.y * rowb : 0u);
    __syncwarp();
    if (!on) return;
    const TX *x = (const TX *)jb.x + ub.col0;
    for (int r = lane; r < rsr.y; r += 32) {
        const int d = __ldg(jb.rs_row + rsr.x + r);
        bulk_g2s(dst + (size_t)r * rowb, x + (size_t)d * jb.ld, rowb, bar);
    }
}

template <typename TX, typename TA, typename TY, int NT, int RG, int MINB>
__global__ void __launch_bounds__(NT, MINB)
k_hvt(const __grid_constant__ HvBatch<TA> B, const ModelDev *__restrict__ mdl, int stage_bytes)
{
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NW = NT / 32;
    const int nimp = mdl->nimp;
    const SmemLayout<TA> L = smem_layout<TA>(stage_bytes, nimp);
    TA *s_cf = reinterpret_cast<TA *>(smem + L.cf);
    TA *s_cross = reinterpret_cast<TA *>(smem + L.cross);
    double *s_dot = reinterpret_cast<double *>(smem + L.dot);
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + L.bar);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int i = tid; i < kMaxCoef; i += NT) {
        TA v = TA(0);
        if (i > 0 && (i - 1) / 2 < mdl->ncpl) {
            const double c = mdl->cval[(i - 1) >> 1];
            v = (TA)(((i - 1) & 1) ? -c : c);
        }
        s_cf[i] = v;
    }
    for (int i = tid; i < nimp * nimp; i += NT) s_cross[i] = (TA)mdl->cross[i];
    for (int i = tid; i < kMaxJobs; i += NT) s_dot[i] = 0.0;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const TA Jc = (TA)mdl->J;

    int t = blockIdx.x;
    if (warp == 0 && t < B.total) issue_tile<TX, TA>(B, t, smem, &bar[0], lane);
    for (int k = 0; t < B.total; t += gridDim.x, ++k) {
        const int buf = k & 1;
        if (warp == 0 && t + (int)gridDim.x < B.total)
            issue_tile<TX, TA>(B, t + gridDim.x, smem + (size_t)(buf ^ 1) * stage_bytes, &bar[buf ^ 1], lane);
        if (!stage_wait(&bar[buf], (unsigned)(k >> 1) & 1u, B.err)) return;

        const int jid = find_job(B, t);
        const HvJobT<TA> &jb = B.job[jid];
        if (!jb.active || *jb.active != 0) {
            const HvTile tl = jb.tiles[t - jb.tile0];
            const int2 rsr = __ldg(jb.rs + tl.rs);
            const UpBlock ub = jb.ublk[tl.ub];
            const int g = rsr.y, W4 = ub.W4, nq = W4 >> 2, ld = jb.ld;
            const TX *S = reinterpret_cast<const TX *>(smem + (size_t)buf * stage_bytes);
            const TX *__restrict__ x = (const TX *)jb.x;
            TY *__restrict__ y = (TY *)jb.y;
            const int lqw = nq >= 32 ? 5 : (nq <= 1 ? 0 : 32 - __clz(nq - 1));
            const int qw = 1 << lqw, rs = 32 >> lqw;
            const int nch = (nq + qw - 1) >> lqw;
            const int rpt = rs * RG;
            const int nrb = (g + rpt - 1) / rpt;
            const bool want_dot = jb.dot_partial != nullptr;
            double dsum = 0.0;
            for (int task = warp; task < nch * nrb; task += NW) {
                const int ch = task % nch, rb = task / nch;
                const int ql = lane & (qw - 1), slot = lane >> lqw;
                const int q = (ch << lqw) + ql;
                const bool act = q < nq;
                const int c = act ? 4 * q : 0;
                const int rbase = rb * rpt + slot;
                // column data of the quad
                TA dup[4];
                int iu[4];
                {
                    TA tmp[4];
                    ldg4<TA>(jb.up_diag + ub.col0 + c, tmp);
                    const unsigned im = __ldg(reinterpret_cast<const unsigned *>(jb.up_imp + ub.col0 + c));
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        dup[kk] = tmp[kk];
                        iu[kk] = (im >> (8 * kk)) & 0xff;
                    }
                }
                // rows: r_i = rbase + rs*i; invalid rows read row 0 and are not stored
                unsigned vmask = 0;
                int roff[RG];
                TA acc[RG][4];
#pragma unroll
                for (int i = 0; i < RG; ++i) {
                    const int r = rbase + rs * i;
                    const bool ok = act && r < g;
                    vmask |= ok ? 1u << i : 0u;
                    const int rr = ok ? r : 0;
                    roff[i] = rr * W4;
                    const int id = ok ? __ldg(&jb.rs_info[rsr.x + rr].x) & 0xff : 0;
                    const TA ddn = ok ? jb.rs_diag[rsr.x + rr] : TA(0);
                    TX xs[4];
                    lds4<TX>(S + roff[i] + c, xs);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        acc[i][kk] = (dup[kk] + ddn + s_cross[iu[kk] * nimp + id]) * (TA)xs[kk];
                }
                // up-spin moves: one schedule entry per slot serves every row
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const int2 h = __ldg(jb.sched_hdr + ub.hdr0 + ch * 4 + kk);
                    const unsigned *E = jb.sched_ent + h.x + ql;
#pragma unroll 2
                    for (int sl = 0; sl < h.y; ++sl) {
                        const unsigned e = __ldg(E + 32 * sl);
                        const TA cf = s_cf[e >> 16];
                        const TX *col = S + (e & 0xffffu);
#pragma unroll
                        for (int i = 0; i < RG; ++i) acc[i][kk] += cf * (TA)col[roff[i]];
                    }
                }
                // down-spin moves, 4-operator terms, store
#pragma unroll
                for (int i = 0; i < RG; ++i) {
                    if (!((vmask >> i) & 1u)) continue;
                    const int rec = rsr.x + rbase + rs * i;
                    const int4 info = __ldg(jb.rs_info + rec);
                    const int nin = (info.x >> 8) & 0xff, nopen = (info.x >> 16) & 0xff;
                    const unsigned *mv = jb.rs_mv + info.y;
                    for (int m = 0; m < nin; ++m) {
                        const unsigned e = __ldg(mv + m);
                        const TA cf = s_cf[e >> 16];
                        TX v[4];
                        lds4<TX>(S + (int)(e & 0xffffu) * W4 + c, v);
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) acc[i][kk] += cf * (TA)v[kk];
                    }
                    const TX *xc = x + ub.col0 + c;
#pragma unroll 4
                    for (int m = 0; m < nopen; ++m) {
                        const unsigned e = __ldg(mv + nin + m);
                        const TA cf = s_cf[e >> 16];
                        TX v[4];
                        ldcg4<TX>(xc + (size_t)(e & 0xffffu) * ld, v);
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) acc[i][kk] += cf * (TA)v[kk];
                    }
                    const int n4 = (info.x >> 24) & 0xff;
                    for (int m = 0; m < n4; ++m) {
                        const unsigned e = __ldg(jb.rs_q4 + info.z + m);
                        const int p = (e >> 16) & 31;
                        const uint4 u4 = __ldg(reinterpret_cast<const uint4 *>(jb.up4 + (size_t)p * ld + ub.col0 + c));
                        const unsigned ue[4] = {u4.x, u4.y, u4.z, u4.w};
                        const TX *xr = x + (size_t)(e & 0xffffu) * ld;
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            if (ue[kk] >> 31) {
                                const bool neg = ((ue[kk] >> 30) ^ (e >> 22)) & 1u;
                                const TA v = (TA)__ldcg(xr + (ue[kk] & 0xffffu));
                                acc[i][kk] += neg ? -Jc * v : Jc * v;
                            }
                        }
                    }
                    const int d = __ldg(jb.rs_row + rec);
                    stg4<TY, TA>(y + (size_t)d * ld + ub.col0 + c, acc[i]);
                    if (want_dot) {
                        TX xs[4];
                        lds4<TX>(S + roff[i] + c, xs);
                        TA part = TA(0);
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) part += (TA)xs[kk] * acc[i][kk];
                        dsum += (double)part;
                    }
                }
            }
            if (want_dot) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
                if (lane == 0 && dsum != 0.0) atomicAdd(&s_dot[jid], dsum);
            }
        }
        __syncthreads();   // stage `buf` is free for the copies issued next iteration
    }
    // the row tails past the last block are pads: zero them (rows strided over the grid)
    for (int j = 0; j < B.njobs; ++j) {
        const HvJobT<TA> &jb = B.job[j];
        if (jb.active && *jb.active == 0) continue;
        const int tail = jb.ld - jb.ncol;
        if (tail <= 0) continue;
        TY *y = (TY *)jb.y + jb.ncol;
        for (long long i = (long long)blockIdx.x * NT + tid; i < (long long)jb.nrow * tail;
             i += (long long)gridDim.x * NT) {
            const long long d = i / tail;
            y[d * jb.ld + (i - d * tail)] = TY(0);
        }
    }
    __syncthreads();
    for (int j = tid; j < B.njobs; j += NT)
        if (B.job[j].dot_partial) B.job[j].dot_partial[blockIdx.x] = s_dot[j];
}

// ---------------------------------------------------------------------------
// host side: variants, tile lists, launch, autotuner
// ---------------------------------------------------------------------------
struct HvVariant {
    int RG, NT, MINB, stage_kb;
};

// FP32 (TX = float): a 48 KB stage holds the 10 x 1000 tile of the largest
// block pair of the 3-orbital x 4-bath ground sector
static const HvVariant kVarF32[] = {{5, 256, 2, 48}, {10, 256, 2, 48}, {4, 256, 2, 48}, {8, 256, 2, 48}};
// FP64 and FP32 -> FP64 (TA = double)
static const HvVariant kVarF64[] = {{5, 512, 1, 96}, {2, 512, 1, 96}, {4, 256, 2, 48}};
static const int kNVarF32 = sizeof(kVarF32) / sizeof(kVarF32[0]);
static const int kNVarF64 = sizeof(kVarF64) / sizeof(kVarF64[0]);

static const HvVariant &variant(int kind, int v) { return kind == HV_F32 ? kVarF32[v] : kVarF64[v]; }
static int nvariants(int kind) { return kind == HV_F32 ? kNVarF32 : kNVarF64; }
static size_t x_size(int kind) { return kind == HV_F64 ? sizeof(double) : sizeof(float); }
static int stage_elems(int kind, int v) { return (int)((size_t)variant(kind, v).stage_kb * 1024 / x_size(kind)); }
static long long shape_key(int kind, const Sector &s) { return ((long long)kind << 32) | (s.ne_up << 16) | s.ne_down; }
static long long tile_key(const Sector &s, int elems)
{
    return ((long long)elems << 32) | ((long long)s.ne_up << 16) | s.ne_down;
}

// Tiles of a sector: for every (down block, up block) pair the row sets of
// the first level whose sets fit the stage with the block's columns.  Tiles
// are ordered by the total electron count per subsystem (spin-flip keeps it,
// so its partner tiles run together), then by block pair, so the neighbour
// rows that moves between row sets read are recent in L2.
int hv_tile_list(mo_ed_ctx *ctx, const Sector &s, int elems, const HvTile **tiles, int *ntiles)
{
    const long long key = tile_key(s, elems);
    auto it = ctx->hv_tiles.find(key);
    if (it == ctx->hv_tiles.end()) {
        const Species &dn = *s.dn, &up = *s.up;
        const int nsub = dn.nsub;
        struct Ent {
            long long orbit;
            int bd, bu, t;
            HvTile tile;
        };
        std::vector<Ent> v;
        for (int bd = 0; bd < (int)dn.h_dblk.size(); ++bd) {
            const DownBlock &db = dn.h_dblk[bd];
            for (int bu = 0; bu < (int)up.h_ublk.size(); ++bu) {
                const UpBlock &ub = up.h_ublk[bu];
                int lev = -1;
                for (int j = 0; j <= nsub; ++j)
                    if ((long long)db.rs_rows[j] * ub.W4 <= elems) {
                        lev = j;
                        break;
                    }
                if (lev < 0) return fail(ctx, MO_ED_ERR_ARG, "an up-spin block is wider than the H*v stage");
                long long orbit = 0;
                for (int k = 0; k < nsub; ++k) orbit = orbit * 64 + db.cnt[k] + up.h_ublk_cnt[(size_t)bu * kMaxSub + k];
                for (int q = 0; q < db.nset[lev]; ++q) v.push_back({orbit, bd, bu, q, HvTile{db.rs0[lev] + q, bu}});
            }
        }
        std::stable_sort(v.begin(), v.end(), [](const Ent &a, const Ent &b) {
            if (a.orbit != b.orbit) return a.orbit < b.orbit;
            if (a.bd != b.bd) return a.bd < b.bd;
            return a.bu < b.bu;
        });
        std::vector<HvTile> h(v.size());
        for (size_t i = 0; i < v.size(); ++i) h[i] = v[i].tile;
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
    auto it = ctx->hv_tiles.find(tile_key(s, stage_elems(kind, v)));
    if (it != ctx->hv_tiles.end()) {
        j.tiles = (const HvTile *)it->second.first.p;
        j.ntiles = it->second.second;
    }
    const Species &up = *s.up, &dn = *s.dn;
    j.ublk = up.ublk;
    j.sched_hdr = up.sched_hdr;
    j.sched_ent = up.sched_ent;
    j.up_imp = up.up_imp;
    j.up4 = up.up4;
    j.rs = dn.rs;
    j.rs_row = dn.rs_row;
    j.rs_info = dn.rs_info;
    j.rs_mv = dn.rs_mv;
    j.rs_q4 = dn.rs_q4;
    if constexpr (sizeof(TA) == 4) {
        j.up_diag = up.up_diag_f;
        j.rs_diag = dn.rs_diag_f;
    } else {
        j.up_diag = up.up_diag_d;
        j.rs_diag = dn.rs_diag_d;
    }
}
template void hv_fill_job<float>(const mo_ed_ctx *, const Sector &, int, int, const void *, void *, HvJobT<float> &);
template void hv_fill_job<double>(const mo_ed_ctx *, const Sector &, int, int, const void *, void *, HvJobT<double> &);

template <typename TX, typename TA, typename TY, int NT, int RG, int MINB>
static int launch_batch(mo_ed_ctx *ctx, int stage_bytes, const HvBatch<TA> &b)
{
    const SmemLayout<TA> L = smem_layout<TA>(stage_bytes, ctx->mdl.nimp);
    auto kern = k_hvt<TX, TA, TY, NT, RG, MINB>;
    static size_t attr_set = 0;   // per instantiation
    if (attr_set < L.total) {
        MOED_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
        attr_set = L.total;
    }
    const int grid = ctx->num_sms * MINB;
    kern<<<grid, NT, L.total, ctx->stream>>>(b, ctx->d_mdl, stage_bytes);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

template <typename TA>
static int launch_variant(mo_ed_ctx *ctx, int kind, int v, const HvBatch<TA> &b)
{
    const int sb = variant(kind, v).stage_kb * 1024;
    if constexpr (sizeof(TA) == 4) {
        (void)kind;
        switch (v) {
        case 0: return launch_batch<float, float, float, 256, 5, 2>(ctx, sb, b);
        case 1: return launch_batch<float, float, float, 256, 10, 2>(ctx, sb, b);
        case 2: return launch_batch<float, float, float, 256, 4, 2>(ctx, sb, b);
        default: return launch_batch<float, float, float, 256, 8, 2>(ctx, sb, b);
        }
    } else if (kind == HV_F64) {
        switch (v) {
        case 0: return launch_batch<double, double, double, 512, 5, 1>(ctx, sb, b);
        case 1: return launch_batch<double, double, double, 512, 2, 1>(ctx, sb, b);
        default: return launch_batch<double, double, double, 256, 4, 2>(ctx, sb, b);
        }
    } else {
        switch (v) {
        case 0: return launch_batch<float, double, double, 512, 5, 1>(ctx, sb, b);
        case 1: return launch_batch<float, double, double, 512, 2, 1>(ctx, sb, b);
        default: return launch_batch<float, double, double, 256, 4, 2>(ctx, sb, b);
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
    return hv_tile_list(ctx, s, stage_elems(kind, v), &t, &n);
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
            shape[4 * i + 1] = h.NT;
            shape[4 * i + 2] = h.MINB;
            shape[4 * i + 3] = h.stage_kb;
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
    if (!ctx->hv_tiles.count(tile_key(s, stage_elems(kind, it->second))) || !ctx->d_err.p)
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
