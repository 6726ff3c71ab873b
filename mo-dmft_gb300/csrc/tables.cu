// tables.cu -- sector basis and operator tables, built on the device.
//
// Replaces generate_basis / ed_basis_get / ed_basis_idx (ed_basis.F90:35-139)
// and the per-row operator bit loops of ed_operators.F90:63-348.
//
// The reference enumerates all words in [minrange, maxrange] and keeps those
// with popcount N in ascending integer order (ed_basis.F90:69-105).  Ascending
// order of N-subsets of bit positions is colexicographic order, so the
// 0-based rank of a word with set bits p_1 < ... < p_N is sum_i C(p_i, i)
// (combinatorial number system) and a rank is unranked greedily from the top
// bit.  Both directions are one thread per element here.
#include <algorithm>
#include <cstring>

#include "internal.h"

namespace moed {

__constant__ int c_binom[kMaxSite + 1][kMaxSite + 2];

long long binom(int n, int k)
{
    if (k < 0 || n < 0 || k > n) return 0;
    long long r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

static int upload_binom(mo_ed_ctx *ctx)
{
    static int h[kMaxSite + 1][kMaxSite + 2];
    for (int n = 0; n <= kMaxSite; ++n)
        for (int k = 0; k <= kMaxSite + 1; ++k) h[n][k] = (int)binom(n, k);
    MOED_CUDA(ctx, cudaMemcpyToSymbolAsync(c_binom, h, sizeof(h), 0, cudaMemcpyHostToDevice,
                                           ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

Species::~Species()
{
    cudaFree(words);
    cudaFree(rank);
    cudaFree(hop_cnt);
    cudaFree(hop_tgt);
    cudaFree(hop_val_d);
    cudaFree(hop_val_f);
    cudaFree(info);
    cudaFree(diag_d);
    cudaFree(diag_f);
    cudaFree(tab_f);
    cudaFree(tab_d);
    cudaFree(sched_hdr);
    cudaFree(sched_ent);
    for (auto &kv : sched_rf) cudaFree(kv.second);
    for (auto &kv : sched_rd) cudaFree(kv.second);
    for (auto &kv : items) cudaFree(kv.second);
    for (auto &kv : desc) cudaFree(kv.second);
    cudaFree(dblk_off);
    cudaFree(dblk_rows);
    cudaFree(dblk_ptr);
    cudaFree(dblk_mv_f);
    cudaFree(dblk_mv_d);
    for (auto &kv : dblk_chunks) cudaFree(kv.second);
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ int parity_below(unsigned w, int bit)
{
    return __popc(w & ((1u << bit) - 1u)) & 1;
}

// colex unrank: rank r -> word with N bits among nsite
__global__ void k_unrank(int nsite, int N, int n, int *words)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int k = N, rem = r;
    unsigned w = 0;
    for (int p = nsite - 1; p >= 0 && k > 0; --p) {
        int c = c_binom[p][k];
        if (rem >= c) {
            w |= 1u << p;
            rem -= c;
            --k;
        }
    }
    words[r] = (int)w;
}

// colex rank over all 2^nsite words (-1 outside the species)
__global__ void k_rank(int nsite, int N, int *rank)
{
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= (1 << nsite)) return;
    if (__popc(w) != N) {
        rank[w] = -1;
        return;
    }
    int r = 0, i = 1;
    for (int p = 0; p < nsite; ++p)
        if ((w >> p) & 1) r += c_binom[p][i++];
    rank[w] = r;
}

struct CplList {
    int n;
    int orb[kMaxHop];   // impurity bit (0-based orbital)
    int bath[kMaxHop];  // bath bit (norb + ibath - 1)
    double val[kMaxHop];
};

// Hybridisation moves of one species word, compacted, in the reference's loop
// order (iorb outer, ibath inner; hybridization1 then hybridization2,
// ed_hamiltonian.F90:146-161).  Signs: product of the destruction / creation
// signs (parity of occupied bits below the target bit), ed_operators.F90:292-348.
// For the down species the reference also counts all up-spin bits below; that
// parity appears once in each of the two operators and cancels.
__global__ void k_hops(int n, int n_pad, int impmask, CplList cpl, const int *words, const int *rank,
                       int *cnt, int *tgt, double *vd, float *vf, int *info, int *max_cnt)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_pad) return;
    if (r >= n) {             // pad columns: no moves, impurity bits 0
        info[r] = 0;
        return;
    }
    unsigned w = (unsigned)words[r];
    int c = 0;
    for (int i = 0; i < cpl.n; ++i) {
        int o = cpl.orb[i], k = cpl.bath[i];
        int ob = (w >> o) & 1, kb = (w >> k) & 1;
        int src, dst;
        if (kb && !ob) {          // hybridization1: c_k then c+_o
            src = k;
            dst = o;
        } else if (ob && !kb) {   // hybridization2: c_o then c+_k
            src = o;
            dst = k;
        } else {
            continue;
        }
        int s1 = parity_below(w, src);
        unsigned w1 = w & ~(1u << src);
        int s2 = parity_below(w1, dst);
        unsigned w2 = w1 | (1u << dst);
        const int neg = (s1 ^ s2) & 1;
        double v = cpl.val[i] * (neg ? -1.0 : 1.0);
        const int t = rank[w2];
        tgt[(size_t)c * n + r] = t;
        vd[(size_t)c * n + r] = v;
        vf[(size_t)c * n + r] = (float)v;
        ++c;
    }
    for (int i = c; i < cpl.n; ++i) {
        tgt[(size_t)i * n + r] = r;   // padding: harmless in-range target
        vd[(size_t)i * n + r] = 0.0;
        vf[(size_t)i * n + r] = 0.0f;
    }
    cnt[r] = c;
    info[r] = c | ((int)(w & (unsigned)impmask) << 8);
    atomicMax(max_cnt, c);
}

// Chunk-major column move tables: entry (c, s, k) = move s of column 4c+k.
// Slots beyond a column's count (and pad columns) hold (own rank, 0).
__global__ void k_chunk_tables(int n, int n_pad, int hw, const int *cnt, const int *tgt, const double *vd,
                               HopEnt<float> *tf, HopEnt<double> *td)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)n_pad * hw) return;
    const int u = (int)(i % n_pad), s = (int)(i / n_pad);
    const size_t o = ((size_t)(u >> 2) * hw + s) * 4 + (u & 3);
    int t = u < n ? u : 0;
    double v = 0.0;
    if (u < n && s < cnt[u]) {
        t = tgt[(size_t)s * n + u];
        v = vd[(size_t)s * n + u];
    }
    tf[o].t = t;
    tf[o].v = (float)v;
    td[o].t = t;
    td[o].pad = 0;
    td[o].v = v;
}

// Species part of the diagonal: sum_site ek(site) n_site (onsite,
// ed_operators.F90:68-84) + (U-3J) sum_{i<j} n_i n_j over impurity orbitals
// (same-spin dens_dens, ed_operators.F90:157-159).
__global__ void k_species_diag(int n, int n_pad, int nsite, int norb, const int *words, const double *ek,
                               double Usame, double *dd, float *df)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_pad) return;
    if (r >= n) {
        dd[r] = 0.0;
        df[r] = 0.0f;
        return;
    }
    unsigned w = (unsigned)words[r];
    double s = 0.0;
    for (int i = 0; i < nsite; ++i)
        if ((w >> i) & 1) s += ek[i];
    for (int i = 0; i < norb; ++i)
        for (int j = i + 1; j < norb; ++j)
            if (((w >> i) & 1) && ((w >> j) & 1)) s += Usame;
    dd[r] = s;
    df[r] = (float)s;
}

__global__ void k_basis_get(long long n, const long long *idx, unsigned *state, const int *up,
                            const int *dn, int nu, int nsite)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    long long i = idx[t] - 1;
    long long iu = i % nu, id = i / nu;
    state[t] = (unsigned)up[iu] + (1u << nsite) * (unsigned)dn[id];
}

__global__ void k_basis_idx(long long n, const unsigned *state, long long *idx, const int *rank_up,
                            const int *rank_dn, int nu, int nsite)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    unsigned s = state[t];
    unsigned su = s & ((1u << nsite) - 1u), sd = s >> nsite;
    int ru = (sd >> nsite) ? -1 : rank_up[su];
    int rd = (sd >> nsite) ? -1 : rank_dn[sd];
    idx[t] = (ru < 0 || rd < 0) ? 0 : (long long)rd * nu + ru + 1;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int imp_pos(int I, int norb)
{
    // rank of impurity pattern I among norb-bit patterns of equal popcount
    int pc = __builtin_popcount(I), pos = 0;
    for (int J = 0; J < I; ++J)
        if (__builtin_popcount(J) == pc) ++pos;
    (void)norb;
    return pos;
}

int build_model(mo_ed_ctx *ctx)
{
    ModelDev &m = ctx->mdl;
    memset(&m, 0, sizeof(m));
    const int norb = ctx->norb, nbath = ctx->nbath;
    m.norb = norb;
    m.nbath = nbath;
    m.nsite = norb + nbath;
    m.nimp = 1 << norb;
    m.npair = norb * (norb - 1);
    m.U = ctx->U;
    m.J = ctx->J;

    // nonzero couplings in the reference loop order (iorb outer, ibath inner)
    ctx->cpl_orb.clear();
    ctx->cpl_bath.clear();
    ctx->cpl_val.clear();
    for (int io = 0; io < norb; ++io)
        for (int ib = 0; ib < nbath; ++ib) {
            double v = ctx->vk[(size_t)ib * norb + io];
            if (v != 0.0) {
                ctx->cpl_orb.push_back(io);
                ctx->cpl_bath.push_back(norb + ib);
                ctx->cpl_val.push_back(v);
            }
        }
    m.ncpl = (int)ctx->cpl_val.size();
    if (m.ncpl > kMaxHop) return fail(ctx, MO_ED_ERR_ARG, "too many nonzero couplings");

    // ordered pairs (i,j), i != j, in the reference's (iorb, jorb) loop order
    int pidx[kMaxOrb][kMaxOrb];
    int p = 0;
    for (int i = 0; i < norb; ++i)
        for (int j = 0; j < norb; ++j)
            if (i != j) pidx[i][j] = p++;
    for (int i = 0; i < norb; ++i)
        for (int j = 0; j < norb; ++j)
            if (i != j) {
                int pp = pidx[i][j];
                m.pair_rev[pp] = pidx[j][i];
                for (int I = 0; I < m.nimp; ++I) {
                    int e = 0;
                    if (((I >> j) & 1) && !((I >> i) & 1)) {
                        int s1 = __builtin_popcount(I & ((1 << j) - 1)) & 1;
                        int I1 = I & ~(1 << j);
                        int s2 = __builtin_popcount(I1 & ((1 << i) - 1)) & 1;
                        int I2 = I1 | (1 << i);
                        int delta = imp_pos(I2, norb) - imp_pos(I, norb);
                        e = (int)(0x80000000u | ((s1 ^ s2) ? 0x40000000u : 0u) | (unsigned)(delta & 0xffff));
                    }
                    m.t4[pp * m.nimp + I] = e;
                }
            }
    // interspecies diagonal: U n_i^up n_i^dn (ed_operators.F90:148-156) and
    // (U-2J) n_i^sigma n_j^-sigma, i != j (ed_operators.F90:160-162)
    for (int Iu = 0; Iu < m.nimp; ++Iu)
        for (int Id = 0; Id < m.nimp; ++Id) {
            double s = 0.0;
            for (int i = 0; i < norb; ++i)
                if (((Iu >> i) & 1) && ((Id >> i) & 1)) s += ctx->U;
            for (int i = 0; i < norb; ++i)
                for (int j = 0; j < norb; ++j)
                    if (i != j && ((Iu >> i) & 1) && ((Id >> j) & 1)) s += ctx->U - 2 * ctx->J;
            m.cross[Iu * m.nimp + Id] = s;
        }
    for (int I = 0; I < m.nimp; ++I) {
        unsigned mask = 0;
        for (int pp = 0; pp < m.npair; ++pp)
            if (m.t4[pp * m.nimp + I] < 0) mask |= 1u << pp;
        m.pairmask[I] = mask;
    }
    for (int i = 0; i < m.ncpl; ++i) m.cval[i] = ctx->cpl_val[i];
    // conserved subsystems: connected components of the orbital / bath-level
    // coupling graph (union-find).  Hybridisation moves keep the electron
    // count of each subsystem, so rows sorted by those counts form blocks
    // closed under down-spin moves.
    {
        std::vector<int> par(m.nsite);
        for (int i = 0; i < m.nsite; ++i) par[i] = i;
        auto find = [&](int a) {
            while (par[a] != a) a = par[a] = par[par[a]];
            return a;
        };
        for (int i = 0; i < m.ncpl; ++i) par[find(ctx->cpl_orb[i])] = find(ctx->cpl_bath[i]);
        std::vector<int> id(m.nsite, -1);
        ctx->site_subsys.assign(m.nsite, 0);
        int nsub = 0;
        for (int i = 0; i < m.nsite; ++i) {
            const int r = find(i);
            if (id[r] < 0) id[r] = nsub++;
            ctx->site_subsys[i] = id[r];
        }
        // largest down-spin block and most hybridisation moves in one block,
        // over every electron count (all 2^nsite words, nsite <= 15)
        std::map<unsigned long long, std::pair<long long, long long>> blk;
        for (unsigned w = 0; w < (1u << m.nsite); ++w) {
            unsigned long long key = (unsigned long long)__builtin_popcount(w);
            for (int sub = 0; sub < nsub; ++sub) {
                int c = 0;
                for (int i = 0; i < m.nsite; ++i)
                    if (((w >> i) & 1) && ctx->site_subsys[i] == sub) ++c;
                key = key * 32 + (unsigned)c;
            }
            int mv = 0;
            for (int i = 0; i < m.ncpl; ++i)
                mv += (int)(((w >> ctx->cpl_orb[i]) & 1) != ((w >> ctx->cpl_bath[i]) & 1));
            auto &e = blk[key];
            e.first += 1;
            e.second += mv;
        }
        ctx->dblk_bound = 0;
        ctx->dblk_mv_bound = 0;
        for (const auto &kv : blk) {
            ctx->dblk_bound = (int)std::max<long long>(ctx->dblk_bound, kv.second.first);
            ctx->dblk_mv_bound = (int)std::max<long long>(ctx->dblk_mv_bound, kv.second.second);
        }
    }
    if (!ctx->d_mdl) MOED_CUDA(ctx, cudaMalloc(&ctx->d_mdl, sizeof(ModelDev)));
    MOED_CUDA(ctx, cudaMemcpyAsync(ctx->d_mdl, &m, sizeof(m), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // species tables and tile-shape choices belong to the model
    ctx->hv_choice.clear();
    ctx->hv_times.clear();
    ctx->species.clear();
    return upload_binom(ctx);
}

// Row items of a species for R rows per item.  Words sharing their bath bits
// (a bath group) are consecutive ranks; spin-flip / pair hopping map a row
// into its own group, so whole groups are kept in one item when they fit.
// Groups are ordered by the bath-electron counts of the conserved subsystems
// (down-spin moves change those counts by one), then packed greedily.
int species_items(mo_ed_ctx *ctx, Species *sp, int R, const int **items, int *nitems)
{
    auto it = sp->items.find(R);
    if (it != sp->items.end()) {
        *items = it->second;
        *nitems = sp->nitems[R];
        return MO_ED_OK;
    }
    const int nsite = sp->nsite, N = sp->N, norb = ctx->norb;
    int nsub = 0;
    for (int v : ctx->site_subsys) nsub = std::max(nsub, v + 1);
    struct Group {
        unsigned long long key;
        int first, size;
    };
    std::vector<Group> groups;
    int r = 0;
    unsigned prev = ~0u;
    for (unsigned w = 0; w < (1u << nsite); ++w) {
        if (__builtin_popcount(w) != N) continue;
        const unsigned bath = w >> norb;
        if (groups.empty() || bath != prev) {
            unsigned long long k = 0;
            for (int sub = 0; sub < nsub; ++sub) {
                int c = 0;
                for (int i = norb; i < nsite; ++i)
                    if (((w >> i) & 1) && ctx->site_subsys[i] == sub) ++c;
                k = k * 16 + (unsigned)c;
            }
            groups.push_back({k, r, 0});
            prev = bath;
        }
        groups.back().size++;
        ++r;
    }
    std::stable_sort(groups.begin(), groups.end(),
                     [](const Group &a, const Group &b) { return a.key < b.key; });
    std::vector<int> tab;
    int fill = R;
    for (const Group &g : groups) {
        for (int off = 0; off < g.size; off += R) {       // a group larger than R is split
            const int len = std::min(R, g.size - off);
            if (fill + len > R) {
                tab.insert(tab.end(), R, -1);
                fill = 0;
            }
            for (int i = 0; i < len; ++i) tab[tab.size() - R + fill + i] = g.first + off + i;
            fill += len;
        }
    }
    const int n_items = (int)(tab.size() / R);
    int *d = nullptr;
    MOED_CUDA(ctx, cudaMalloc(&d, sizeof(int) * std::max<size_t>(1, tab.size())));
    MOED_CUDA(ctx, cudaMemcpyAsync(d, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    sp->items[R] = d;
    sp->nitems[R] = n_items;
    *items = d;
    *nitems = n_items;
    return MO_ED_OK;
}

// Down-spin blocks of a species for the split H*v.  Rows (words, rank order)
// are keyed by their electron count in every conserved subsystem; a
// hybridisation move stays inside its subsystem, so every block is closed
// under the moves and a block times a column range is an independent chunk.
// Moves are copied from the species' move tables with their targets rewritten
// as indices within the block.  Chunks: a block's columns are cut into ranges of about
// kChunkElems elements (whole 32-column units), so the chunks of a sector do
// similar work whatever the block sizes.
int species_dblocks(mo_ed_ctx *ctx, Species *sp, int ld)
{
    constexpr long long kChunkElems = 1 << 16;
    if (!sp->dblk_ptr) {
        // a build that failed part way left some tables: start over
        cudaFree(sp->dblk_off);
        cudaFree(sp->dblk_rows);
        cudaFree(sp->dblk_mv_f);
        cudaFree(sp->dblk_mv_d);
        sp->dblk_off = sp->dblk_rows = nullptr;
        sp->dblk_mv_f = nullptr;
        sp->dblk_mv_d = nullptr;
        const int n = sp->n, hw = sp->hw, nsite = sp->nsite, N = sp->N;
        int nsub = 0;
        for (int v : ctx->site_subsys) nsub = std::max(nsub, v + 1);
        std::vector<int> cnt(n), tgt((size_t)hw * n);
        std::vector<double> val((size_t)hw * n);
        MOED_CUDA(ctx, cudaMemcpyAsync(cnt.data(), sp->hop_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaMemcpyAsync(tgt.data(), sp->hop_tgt, sizeof(int) * tgt.size(), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MOED_CUDA(ctx, cudaMemcpyAsync(val.data(), sp->hop_val_d, sizeof(double) * val.size(),
                                       cudaMemcpyDeviceToHost, ctx->stream));
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        // block key of every rank (words in increasing numeric order = rank order)
        std::map<unsigned long long, std::vector<int>> blocks;
        int r = 0;
        for (unsigned w = 0; w < (1u << nsite); ++w) {
            if (__builtin_popcount(w) != N) continue;
            unsigned long long k = 0;
            for (int sub = 0; sub < nsub; ++sub) {
                int c = 0;
                for (int i = 0; i < nsite; ++i)
                    if (((w >> i) & 1) && ctx->site_subsys[i] == sub) ++c;
                k = k * 32 + (unsigned)c;
            }
            blocks[k].push_back(r++);
        }
        std::vector<const std::vector<int> *> order;
        for (auto &kv : blocks) order.push_back(&kv.second);
        std::stable_sort(order.begin(), order.end(),
                         [](const std::vector<int> *a, const std::vector<int> *b) { return a->size() > b->size(); });
        std::vector<int> local(n, -1), blk(n, -1);
        for (size_t b = 0; b < order.size(); ++b)
            for (size_t i = 0; i < order[b]->size(); ++i) {
                local[(*order[b])[i]] = (int)i;
                blk[(*order[b])[i]] = (int)b;
            }
        std::vector<int> off(1, 0), rows, ptr(1, 0);
        std::vector<HopEnt<float>> mvf;
        std::vector<HopEnt<double>> mvd;
        int maxrows = 0, mvmax = 0;
        for (size_t b = 0; b < order.size(); ++b) {
            const size_t m0 = mvf.size();
            for (int row : *order[b]) {
                rows.push_back(row);
                for (int s = 0; s < cnt[row]; ++s) {
                    const int tr = tgt[(size_t)s * n + row];
                    if (tr < 0 || tr >= n || blk[tr] != (int)b)
                        return fail(ctx, MO_ED_ERR_STATE, "down-spin move leaves its conserved block");
                    const double v = val[(size_t)s * n + row];
                    HopEnt<float> ef;
                    ef.t = local[tr];
                    ef.v = (float)v;
                    HopEnt<double> ed;
                    ed.t = local[tr];
                    ed.pad = 0;
                    ed.v = v;
                    mvf.push_back(ef);
                    mvd.push_back(ed);
                }
                ptr.push_back((int)mvf.size());
            }
            off.push_back((int)rows.size());
            maxrows = std::max(maxrows, (int)order[b]->size());
            mvmax = std::max(mvmax, (int)(mvf.size() - m0));
        }
        auto up = [&](auto **dst, const auto &v) -> int {
            using E = std::remove_const_t<std::remove_reference_t<decltype(v[0])>>;
            MOED_CUDA(ctx, cudaMalloc((void **)dst, sizeof(E) * std::max<size_t>(1, v.size())));
            MOED_CUDA(ctx, cudaMemcpyAsync((void *)*dst, v.data(), sizeof(E) * v.size(), cudaMemcpyHostToDevice,
                                           ctx->stream));
            return MO_ED_OK;
        };
        if (int rc = up(&sp->dblk_off, off)) return rc;
        if (int rc = up(&sp->dblk_rows, rows)) return rc;
        if (int rc = up(&sp->dblk_mv_f, mvf)) return rc;
        if (int rc = up(&sp->dblk_mv_d, mvd)) return rc;
        if (int rc = up(&sp->dblk_ptr, ptr)) return rc;   // last: marks the tables complete
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        sp->dblk_n = (int)order.size();
        sp->dblk_max = maxrows;
        sp->dblk_mvmax = mvmax;
        sp->dblk_h_off = off;
    }
    if (sp->dblk_chunks.count(ld)) return MO_ED_OK;
    const int units = ld / 32;
    std::vector<int2> ch(sp->dblk_n);
    int total = 0;
    for (int b = 0; b < sp->dblk_n; ++b) {
        const long long nr = sp->dblk_h_off[b + 1] - sp->dblk_h_off[b];
        const int per = (int)std::max(1LL, std::min<long long>(units, kChunkElems / (32 * nr)));
        ch[b] = make_int2(total, per);
        total += (units + per - 1) / per;
    }
    int2 *d = nullptr;
    MOED_CUDA(ctx, cudaMalloc(&d, sizeof(int2) * std::max<size_t>(1, ch.size())));
    MOED_CUDA(ctx, cudaMemcpyAsync(d, ch.data(), sizeof(int2) * ch.size(), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    sp->dblk_chunks[ld] = d;
    sp->dblk_nchunks[ld] = total;
    return MO_ED_OK;
}

// Up-spin gather schedule.  The moves of the 32 columns of a chunk are the
// edges of a bipartite multigraph between lanes (output columns) and shared-
// memory banks (target mod 32).  A proper edge colouring with Delta colours
// (Delta = the largest lane or bank degree; Koenig's theorem) gives Delta
// slots in which every lane has at most one move and every bank at most one
// reader: each slot is one conflict-free shared-memory access per staged row.
// Colouring: for edge (l, b), take a colour a free at l and c free at b; if a
// is also free at b use it, else swap a and c along the alternating path that
// starts at b (it cannot reach l), which frees a at b.
namespace {
struct EdgeColouring {
    int delta;
    std::vector<int> at;   // [node][colour] -> edge or -1; nodes 0..31 lanes, 32..63 banks
    std::vector<int> col;  // edge -> colour
    explicit EdgeColouring(int d) : delta(d), at(64 * d, -1) {}
    int free_colour(int node) const
    {
        for (int c = 0; c < delta; ++c)
            if (at[node * delta + c] < 0) return c;
        return -1;
    }
};
}  // namespace

static void colour_chunk(const std::vector<int> &lane, const std::vector<int> &bank, int delta,
                         std::vector<int> &colour)
{
    const int ne = (int)lane.size();
    EdgeColouring g(delta);
    g.col.assign(ne, -1);
    auto other = [&](int e, int node) { return node < 32 ? 32 + bank[e] : lane[e]; };
    for (int e = 0; e < ne; ++e) {
        const int l = lane[e], b = 32 + bank[e];
        const int a = g.free_colour(l), c = g.free_colour(b);
        if (g.at[b * delta + a] >= 0) {
            // alternating a/c path from b: collect its edges, then swap their colours
            std::vector<int> path;
            int node = b, want = a;
            while (true) {
                const int pe = g.at[node * delta + want];
                if (pe < 0) break;
                path.push_back(pe);
                node = other(pe, node);
                want = (want == a) ? c : a;
            }
            for (int pe : path) {
                const int pc = g.col[pe];
                g.at[lane[pe] * delta + pc] = -1;
                g.at[(32 + bank[pe]) * delta + pc] = -1;
            }
            for (int pe : path) {
                const int nc = (g.col[pe] == a) ? c : a;
                g.col[pe] = nc;
                g.at[lane[pe] * delta + nc] = pe;
                g.at[(32 + bank[pe]) * delta + nc] = pe;
            }
        }
        g.col[e] = a;
        g.at[l * delta + a] = e;
        g.at[b * delta + a] = e;
    }
    colour = g.col;
}

static int build_up_schedule(mo_ed_ctx *ctx, Species *s)
{
    const int nsite = ctx->nsite, N = s->N, n = s->n, nch = s->n_pad / 32;
    std::vector<int> words;
    std::vector<int> rank((size_t)1 << nsite, -1);
    for (unsigned w = 0; w < (1u << nsite); ++w)
        if (__builtin_popcount(w) == N) {
            rank[w] = (int)words.size();
            words.push_back((int)w);
        }
    auto parity_below_h = [](unsigned w, int bit) { return __builtin_popcount(w & ((1u << bit) - 1u)) & 1; };
    const int ncpl = ctx->mdl.ncpl;
    std::vector<int2> hdr(nch);
    std::vector<unsigned> ent;
    std::vector<int> el, eb, colour;
    std::vector<unsigned> ecode;
    int smax = 0;
    for (int c = 0; c < nch; ++c) {
        el.clear();
        eb.clear();
        ecode.clear();
        int deg_l[32] = {0}, deg_b[32] = {0};
        for (int l = 0; l < 32; ++l) {
            const int u = 32 * c + l;
            if (u >= n) continue;
            const unsigned w = (unsigned)words[u];
            for (int i = 0; i < ncpl; ++i) {   // the move rule of k_hops
                const int o = ctx->cpl_orb[i], k = ctx->cpl_bath[i];
                const int ob = (w >> o) & 1, kb = (w >> k) & 1;
                int src, dst;
                if (kb && !ob) {
                    src = k;
                    dst = o;
                } else if (ob && !kb) {
                    src = o;
                    dst = k;
                } else {
                    continue;
                }
                const int s1 = parity_below_h(w, src);
                const unsigned w1 = w & ~(1u << src);
                const int s2 = parity_below_h(w1, dst);
                const int t = rank[w1 | (1u << dst)];
                el.push_back(l);
                eb.push_back(t & 31);
                ecode.push_back(0x80000000u | ((unsigned)((s1 ^ s2) & 1) << 22) | ((unsigned)i << 16) |
                                (unsigned)t);
                deg_l[l]++;
                deg_b[t & 31]++;
            }
        }
        int delta = 0;
        for (int q = 0; q < 32; ++q) delta = std::max(delta, std::max(deg_l[q], deg_b[q]));
        hdr[c] = make_int2((int)ent.size(), delta);
        if (delta == 0) continue;
        colour_chunk(el, eb, delta, colour);
        const size_t base = ent.size();
        ent.resize(base + (size_t)32 * delta, 0u);
        for (size_t e = 0; e < el.size(); ++e) {
            unsigned &slot = ent[base + (size_t)32 * colour[e] + el[e]];
            if (colour[e] < 0 || colour[e] >= delta || slot != 0u)
                return fail(ctx, MO_ED_ERR_STATE, "gather schedule colouring failed");
            slot = ecode[e];
        }
        smax = std::max(smax, delta);
    }
    s->sched_slots_max = smax;
    if (ent.empty()) ent.push_back(0u);
    MOED_CUDA(ctx, cudaMalloc(&s->sched_hdr, sizeof(int2) * std::max(nch, 1)));
    MOED_CUDA(ctx, cudaMalloc(&s->sched_ent, sizeof(unsigned) * ent.size()));
    if (nch > 0)
        MOED_CUDA(ctx, cudaMemcpyAsync(s->sched_hdr, hdr.data(), sizeof(int2) * nch, cudaMemcpyHostToDevice,
                                       ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(s->sched_ent, ent.data(), sizeof(unsigned) * ent.size(),
                                   cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // before the host vectors move
    s->h_sched_hdr = std::move(hdr);
    s->h_sched_ent = std::move(ent);
    return MO_ED_OK;
}

int species_sched(mo_ed_ctx *ctx, Species *sp, int R)
{
    if (sp->sched_rf.count(R)) return MO_ED_OK;
    const std::vector<int2> &hdr = sp->h_sched_hdr;
    const std::vector<unsigned> &ent = sp->h_sched_ent;
    std::vector<HopEnt<float>> ef(ent.size());
    std::vector<HopEnt<double>> ed(ent.size());
    auto offset = [R](int t) { return ((t >> 5) * R) * 32 + (t & 31); };
    for (size_t c = 0; c < hdr.size(); ++c) {
        const int first = hdr[c].x, nslot = hdr[c].y;
        for (int sl = 0; sl < nslot; ++sl) {
            const unsigned *e = &ent[(size_t)first + (size_t)32 * sl];
            unsigned used = 0u;
            for (int l = 0; l < 32; ++l)
                if (e[l] & 0x80000000u) used |= 1u << (e[l] & 31u);
            for (int l = 0; l < 32; ++l) {
                const size_t o = (size_t)first + (size_t)32 * sl + l;
                int t;
                double v;
                if (e[l] & 0x80000000u) {
                    t = (int)(e[l] & 0xffffu);
                    v = ctx->cpl_val[(e[l] >> 16) & 63u];
                    if (e[l] & (1u << 22)) v = -v;
                } else {
                    t = __builtin_ctz(~used);   // a bank no lane of this slot reads (column t of tile 0)
                    used |= 1u << t;
                    v = 0.0;
                }
                ef[o].t = offset(t);
                ef[o].v = (float)v;
                ed[o].t = offset(t);
                ed[o].pad = 0;
                ed[o].v = v;
            }
        }
    }
    HopEnt<float> *df = nullptr;
    HopEnt<double> *dd = nullptr;
    MOED_CUDA(ctx, cudaMalloc(&df, sizeof(HopEnt<float>) * ef.size()));
    sp->sched_rf[R] = df;
    MOED_CUDA(ctx, cudaMalloc(&dd, sizeof(HopEnt<double>) * ed.size()));
    sp->sched_rd[R] = dd;
    MOED_CUDA(ctx, cudaMemcpyAsync(df, ef.data(), sizeof(HopEnt<float>) * ef.size(), cudaMemcpyHostToDevice,
                                   ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dd, ed.data(), sizeof(HopEnt<double>) * ed.size(), cudaMemcpyHostToDevice,
                                   ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MO_ED_OK;
}

int get_species(mo_ed_ctx *ctx, int N, Species **out)
{
    auto it = ctx->species.find(N);
    if (it != ctx->species.end()) {
        *out = it->second.get();
        return MO_ED_OK;
    }
    const int nsite = ctx->nsite;
    std::unique_ptr<Species> s(new Species);
    s->nsite = nsite;
    s->N = N;
    s->n = (int)binom(nsite, N);
    s->n_pad = (s->n + 31) / 32 * 32;
    s->hw = std::max(ctx->mdl.ncpl, 1);
    const int n = s->n, np = s->n_pad;
    const size_t nh = (size_t)n * s->hw;
    MOED_CUDA(ctx, cudaMalloc(&s->words, sizeof(int) * n));
    MOED_CUDA(ctx, cudaMalloc(&s->rank, sizeof(int) << nsite));
    MOED_CUDA(ctx, cudaMalloc(&s->hop_cnt, sizeof(int) * n));
    MOED_CUDA(ctx, cudaMalloc(&s->hop_tgt, sizeof(int) * nh));
    MOED_CUDA(ctx, cudaMalloc(&s->hop_val_d, sizeof(double) * nh));
    MOED_CUDA(ctx, cudaMalloc(&s->hop_val_f, sizeof(float) * nh));
    MOED_CUDA(ctx, cudaMalloc(&s->tab_f, sizeof(HopEnt<float>) * (size_t)np * s->hw));
    MOED_CUDA(ctx, cudaMalloc(&s->tab_d, sizeof(HopEnt<double>) * (size_t)np * s->hw));
    MOED_CUDA(ctx, cudaMalloc(&s->info, sizeof(int) * np));
    MOED_CUDA(ctx, cudaMalloc(&s->diag_d, sizeof(double) * np));
    MOED_CUDA(ctx, cudaMalloc(&s->diag_f, sizeof(float) * np));

    const int T = 256;
    k_unrank<<<(n + T - 1) / T, T, 0, ctx->stream>>>(nsite, N, n, s->words);
    MOED_CHECK_LAUNCH(ctx);
    k_rank<<<((1 << nsite) + T - 1) / T, T, 0, ctx->stream>>>(nsite, N, s->rank);
    MOED_CHECK_LAUNCH(ctx);

    CplList cl;
    memset(&cl, 0, sizeof(cl));
    cl.n = ctx->mdl.ncpl;
    for (int i = 0; i < cl.n; ++i) {
        cl.orb[i] = ctx->cpl_orb[i];
        cl.bath[i] = ctx->cpl_bath[i];
        cl.val[i] = ctx->cpl_val[i];
    }
    DevBuf dmax, dek;
    if (int rc = dev_alloc(ctx, dmax, sizeof(int))) return rc;
    if (int rc = dev_alloc(ctx, dek, sizeof(double) * nsite)) return rc;
    MOED_CUDA(ctx, cudaMemsetAsync(dmax.p, 0, sizeof(int), ctx->stream));
    MOED_CUDA(ctx, cudaMemcpyAsync(dek.p, ctx->ek.data(), sizeof(double) * nsite,
                                   cudaMemcpyHostToDevice, ctx->stream));
    if (cl.n == 0) {
        MOED_CUDA(ctx, cudaMemsetAsync(s->hop_cnt, 0, sizeof(int) * n, ctx->stream));
        MOED_CUDA(ctx, cudaMemsetAsync(s->hop_tgt, 0, sizeof(int) * nh, ctx->stream));
        MOED_CUDA(ctx, cudaMemsetAsync(s->hop_val_d, 0, sizeof(double) * nh, ctx->stream));
        MOED_CUDA(ctx, cudaMemsetAsync(s->hop_val_f, 0, sizeof(float) * nh, ctx->stream));
    }
    k_hops<<<(np + T - 1) / T, T, 0, ctx->stream>>>(n, np, ctx->mdl.nimp - 1, cl, s->words, s->rank,
                                                    s->hop_cnt, s->hop_tgt, s->hop_val_d, s->hop_val_f,
                                                    s->info, (int *)dmax.p);
    MOED_CHECK_LAUNCH(ctx);
    {
        const long long tot = (long long)np * s->hw;
        k_chunk_tables<<<(unsigned)((tot + T - 1) / T), T, 0, ctx->stream>>>(n, np, s->hw, s->hop_cnt, s->hop_tgt,
                                                                             s->hop_val_d, s->tab_f, s->tab_d);
        MOED_CHECK_LAUNCH(ctx);
    }
    k_species_diag<<<(np + T - 1) / T, T, 0, ctx->stream>>>(n, np, nsite, ctx->norb, s->words,
                                                            (const double *)dek.p, ctx->U - 3 * ctx->J,
                                                            s->diag_d, s->diag_f);
    MOED_CHECK_LAUNCH(ctx);
    {   // largest bath group (words sharing their bath bits)
        std::map<unsigned, int> gs;
        for (unsigned w = 0; w < (1u << nsite); ++w)
            if (__builtin_popcount(w) == N) s->max_group = std::max(s->max_group, ++gs[w >> ctx->norb]);
    }
    MOED_CUDA(ctx, cudaMemcpyAsync(&s->max_cnt, dmax.p, sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (int rc = build_up_schedule(ctx, s.get())) return rc;
    *out = s.get();
    ctx->species[N] = std::move(s);
    return MO_ED_OK;
}

int get_sector(mo_ed_ctx *ctx, int ne_up, int ne_down, Sector *out)
{
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    if (ne_up < 0 || ne_up > ctx->nsite || ne_down < 0 || ne_down > ctx->nsite)
        return fail(ctx, MO_ED_ERR_SECTOR, "sector (" + std::to_string(ne_up) + "," +
                                               std::to_string(ne_down) + ") out of range");
    out->ne_up = ne_up;
    out->ne_down = ne_down;
    if (int rc = get_species(ctx, ne_up, &out->up)) return rc;
    if (int rc = get_species(ctx, ne_down, &out->dn)) return rc;
    return MO_ED_OK;
}

int find_sector(mo_ed_ctx *ctx, int ne_up, int ne_down, Sector *out)
{
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    if (ne_up < 0 || ne_up > ctx->nsite || ne_down < 0 || ne_down > ctx->nsite)
        return fail(ctx, MO_ED_ERR_SECTOR, "sector (" + std::to_string(ne_up) + "," +
                                               std::to_string(ne_down) + ") out of range");
    auto iu = ctx->species.find(ne_up), id = ctx->species.find(ne_down);
    if (iu == ctx->species.end() || id == ctx->species.end())
        return fail(ctx, MO_ED_ERR_STATE, "sector (" + std::to_string(ne_up) + "," +
                                              std::to_string(ne_down) + ") tables not built yet");
    out->ne_up = ne_up;
    out->ne_down = ne_down;
    out->up = iu->second.get();
    out->dn = id->second.get();
    return MO_ED_OK;
}

int basis_get_dev(mo_ed_ctx *ctx, const Sector &s, long long n, const long long *d_idx,
                  unsigned *d_state)
{
    if (n <= 0) return MO_ED_OK;
    const int T = 256;
    k_basis_get<<<(unsigned)((n + T - 1) / T), T, 0, ctx->stream>>>(n, d_idx, d_state, s.up->words,
                                                                     s.dn->words, s.up->n,
                                                                     ctx->nsite);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

int basis_idx_dev(mo_ed_ctx *ctx, const Sector &s, long long n, const unsigned *d_state,
                  long long *d_idx)
{
    if (n <= 0) return MO_ED_OK;
    const int T = 256;
    k_basis_idx<<<(unsigned)((n + T - 1) / T), T, 0, ctx->stream>>>(n, d_state, d_idx, s.up->rank,
                                                                     s.dn->rank, s.up->n,
                                                                     ctx->nsite);
    MOED_CHECK_LAUNCH(ctx);
    return MO_ED_OK;
}

}  // namespace moed
